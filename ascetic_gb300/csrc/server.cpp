// Query server: BFS / SSSP / CC / PageRank queries against several resident
// graphs on one GPU under one device-memory budget.
//
// Two engines answer queries:
//  - ASC_SERVE_BATCHED (continuous batching): BFS and SSSP queries join the
//    per-(graph, algorithm) multi-source batch as soon as a source slot (and,
//    for BFS, a level plane within the budget) is free, advance in shared
//    iterations (one edge read serves every source of the batch; batches of
//    different graphs run on their own streams at the same time), and leave
//    when their own frontier is empty. CC and PageRank queries run whole on a
//    second worker; identical pending ones share one run. The two workers take
//    turns on the device (one batch iteration, then one whole run, when both
//    have work).
//  - ASC_SERVE_FIFO: the plain engine, one query at a time in arrival order.
// Admission accounts every device allocation against the budget: the graphs'
// static regions and offsets, per-graph single-query state, batch state and
// level planes. A query that can never fit fails with ASC_ERR_BUDGET.
// No reference counterpart: the reference answers one query per process run.
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "common.h"

namespace {

using Clock = std::chrono::steady_clock;

enum QState { Q_PENDING = 0, Q_RUNNING = 1, Q_DONE = 2 };

struct Query {
    uint64_t ticket = 0;
    uint32_t graph = 0;
    asc_algo algo = ASC_BFS;
    uint32_t source = 0;
    asc_params params;
    void *out = nullptr;
    QState state = Q_PENDING;
    asc_status status = ASC_OK;
    Clock::time_point t_submit, t_start, t_end;
    uint32_t batch = 1;
    int32_t iterations = 0;
    bool cancel = false;
    bool mem_wait = false;  // has waited for device memory (counted once)
    std::string err;        // why the query failed (the worker's error message)
};

struct GraphSlot {
    asc_graph *g = nullptr;
    uint64_t base_bytes = 0;        // static region + offsets (allocated at open)
    uint64_t ws_bytes = 0;          // single-query state once allocated
    bool ws_pr = false;
    asc::BatchEngine *batch[2] = {nullptr, nullptr};  // BFS, SSSP
    uint64_t batch_bytes[2] = {0, 0};
    uint32_t planes = 0;            // BFS level planes allocated
    // set while the batch worker uses the engine outside the lock (launch,
    // collect and the copy-out of finished slots): nobody may free it then,
    // even when it has just become idle
    bool in_use[2] = {false, false};
    Query *slot_q[2][64] = {{nullptr}};
    std::deque<Query *> pend[2];    // BFS, SSSP waiting for a slot
};

}  // namespace

struct asc_server {
    asc_server_config cfg;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    // The two workers take turns on the device: one of them at a time has
    // device work in flight or allocates and frees device memory (gpu_holder:
    // 0 batch worker, 1 single worker, -1 neither); when both want it they
    // alternate (gpu_last). Streams of the batch worker still overlap each
    // other. The turn-taking went in after the GPU raised MMU faults (Xid 31)
    // in a few sweeps of hundreds of queries with both workers' work in flight
    // at once; one worker alone (the plain engine) never faulted.
    std::condition_variable cv_gpu;
    int gpu_holder = -1, gpu_last = -1;
    bool gpu_want[2] = {false, false};
    std::vector<GraphSlot> graphs;
    std::map<uint64_t, Query *> queries;
    std::deque<Query *> single;     // CC / PR (batched mode) or everything (FIFO)
    uint64_t next_ticket = 1;
    uint64_t used_bytes = 0;
    bool stop = false;
    bool started = false;
    int single_graph = -1;          // graph the single worker is running, -1 when idle
    int device = -1;                // the device every graph of this server was opened on
    std::thread batch_worker, single_worker;
    std::vector<double> lat_ms;
    uint64_t submitted = 0, completed = 0, failed = 0, cancelled = 0, batches = 0, batch_sources = 0;
    uint64_t engines_created = 0, engines_freed = 0, workspaces_freed = 0, memory_waits = 0;
    Clock::time_point first_submit, last_done;
    bool any_submit = false;
    asc_status fatal = ASC_OK;
};

namespace {

uint64_t budget_left(asc_server *s) {
    if (!s->cfg.device_budget_bytes) return ~0ull;
    return s->cfg.device_budget_bytes > s->used_bytes ? s->cfg.device_budget_bytes - s->used_bytes : 0;
}

constexpr size_t kLatencyWindow = size_t(1) << 20;

void finish(asc_server *s, Query *q, asc_status st) {
    q->status = st;
    q->state = Q_DONE;
    q->t_end = Clock::now();
    s->last_done = q->t_end;
    if (st == ASC_OK) {
        s->completed++;
        // latencies of the most recent kLatencyWindow completions (a server that
        // runs for long does not grow without bound)
        if (s->lat_ms.size() >= kLatencyWindow) s->lat_ms.erase(s->lat_ms.begin(), s->lat_ms.begin() + kLatencyWindow / 2);
        s->lat_ms.push_back(std::chrono::duration<double, std::milli>(q->t_end - q->t_submit).count());
    } else if (st == ASC_ERR_CANCELLED) {
        s->cancelled++;
    } else {
        s->failed++;
    }
}

// Device bytes held by batch engines and planes (what draining batches frees).
uint64_t batch_held(const asc_server *s) {
    uint64_t b = 0;
    for (const auto &gs : s->graphs) {
        b += gs.batch_bytes[0] + gs.batch_bytes[1];
        b += (uint64_t)gs.planes * 4ull * gs.g->V;
    }
    return b;
}

// Device bytes no reclaim frees: the graphs' static regions and offsets.
uint64_t bases_total(const asc_server *s) {
    uint64_t b = 0;
    for (const auto &gs : s->graphs) b += gs.base_bytes;
    return b;
}

// Frees the batch engines that have nothing running or waiting.
void evict_idle_locked(asc_server *s) {
    for (auto &gs : s->graphs)
        for (int k = 0; k < 2; k++) {
            asc::BatchEngine *b = gs.batch[k];
            if (!b || gs.in_use[k] || asc::batch_busy(b) || !gs.pend[k].empty()) continue;
            asc::batch_destroy(b);
            s->engines_freed++;
            gs.batch[k] = nullptr;
            s->used_bytes -= gs.batch_bytes[k];
            gs.batch_bytes[k] = 0;
            if (k == 0) {
                s->used_bytes -= (uint64_t)gs.planes * 4ull * gs.g->V;
                gs.planes = 0;
            }
        }
}

// Frees what no query is using: idle batch engines with nobody waiting and
// the single-query state of graphs the single worker is not running (keep is
// a graph whose state the caller is about to use). Returns the bytes freed.
uint64_t reclaim_locked(asc_server *s, int keep) {
    const uint64_t before = s->used_bytes;
    evict_idle_locked(s);
    for (uint32_t gi = 0; gi < s->graphs.size(); gi++) {
        GraphSlot &gs = s->graphs[gi];
        if ((int)gi == keep || (int)gi == s->single_graph || !gs.ws_bytes || !gs.g->ws) continue;
        asc::free_workspace(gs.g);
        s->workspaces_freed++;
        s->used_bytes -= gs.ws_bytes;
        gs.ws_bytes = 0;
        gs.ws_pr = false;
    }
    return before - s->used_bytes;
}

// Waits for the device turn of worker `who` (lk holds s->mu).
void gpu_acquire(asc_server *s, std::unique_lock<std::mutex> &lk, int who) {
    s->gpu_want[who] = true;
    s->cv_gpu.wait(lk, [&] { return s->gpu_holder < 0 && !(s->gpu_want[1 - who] && s->gpu_last == who); });
    s->gpu_want[who] = false;
    s->gpu_holder = who;
}

void gpu_release(asc_server *s, int who) {
    if (s->gpu_holder != who) return;
    s->gpu_holder = -1;
    s->gpu_last = who;
    s->cv_gpu.notify_all();
}

// Between two iterations of a whole run: the single worker hands the device to
// the batch worker for one iteration when that one is waiting for it.
void single_yield(void *ctx) {
    asc_server *s = static_cast<asc_server *>(ctx);
    std::unique_lock<std::mutex> lk(s->mu);
    if (!s->gpu_want[0]) return;
    gpu_release(s, 1);
    gpu_acquire(s, lk, 1);
}

bool batchable(const asc_server *s, const Query *q) {
    return s->cfg.mode == ASC_SERVE_BATCHED && (q->algo == ASC_BFS || q->algo == ASC_SSSP);
}

// One pass of the batch worker under the lock: admit waiting queries into free
// slots (allocating batch state and planes within the budget). Returns the
// engines with work.
void admit_locked(asc_server *s, std::vector<std::pair<uint32_t, int>> &work) {
    const uint32_t max_batch = s->cfg.max_batch ? std::min(s->cfg.max_batch, 64u) : 64u;
    for (uint32_t gi = 0; gi < s->graphs.size(); gi++) {
        GraphSlot &gs = s->graphs[gi];
        for (int k = 0; k < 2; k++) {
            auto &pend = gs.pend[k];
            while (!pend.empty() && pend.front()->cancel) {
                Query *q = pend.front();
                pend.pop_front();
                finish(s, q, ASC_ERR_CANCELLED);
            }
            if (!pend.empty() && !gs.batch[k]) {
                const bool sssp = k == 1;
                // SSSP keeps a row of distances per vertex, one column per
                // slot: rows of 64 sources, or of 32 or 16 where max_batch asks
                // for no more or where 64 columns of this graph could never fit
                // the budget beside the graphs (idle batches and single-query
                // state are freed for a waiting batch)
                uint32_t stride = 64;
                if (sssp) {
                    while (stride > 16 && stride / 2 >= max_batch) stride /= 2;
                    while (stride > 16 && s->cfg.device_budget_bytes &&
                           asc::batch_state_bytes(gs.g, true, stride) + bases_total(s) > s->cfg.device_budget_bytes)
                        stride /= 2;
                }
                uint64_t need = asc::batch_state_bytes(gs.g, sssp, stride);
                if (need <= budget_left(s)) {
                    asc::BatchEngine *b = nullptr;
                    asc_status st = asc::batch_create(gs.g, sssp, stride, &b);
                    if (st == ASC_OK) {
                        gs.batch[k] = b;
                        s->engines_created++;
                        gs.batch_bytes[k] = need;
                        s->used_bytes += need;
                    } else {
                        while (!pend.empty()) {
                            finish(s, pend.front(), st);
                            pend.pop_front();
                        }
                    }
                } else if (s->cfg.device_budget_bytes && need + bases_total(s) > s->cfg.device_budget_bytes) {
                    // a batch of this graph can never fit: its queries run one at a time
                    while (!pend.empty()) {
                        s->single.push_back(pend.front());
                        pend.pop_front();
                    }
                    s->cv_work.notify_all();
                }
            }
            asc::BatchEngine *b = gs.batch[k];
            if (!b) continue;
            const uint32_t slots = std::min(max_batch, asc::batch_slots(b));
            for (uint32_t slot = 0; slot < slots && !pend.empty(); slot++) {
                if (gs.slot_q[k][slot]) continue;
                if (k == 0 && !asc::batch_has_plane(b, slot)) {
                    if (asc::batch_plane_bytes(gs.g) > budget_left(s)) break;
                    s->used_bytes += asc::batch_plane_bytes(gs.g);
                    gs.planes++;
                }
                Query *q = pend.front();
                pend.pop_front();
                asc_status st = asc::batch_admit(b, slot, q->source);
                if (st != ASC_OK) {
                    finish(s, q, st);
                    continue;
                }
                q->state = Q_RUNNING;
                q->t_start = Clock::now();
                gs.slot_q[k][slot] = q;
            }
            if (asc::batch_busy(b)) work.push_back({gi, k});
        }
    }
}

void batch_loop(asc_server *s) {
    // the graphs' device (asc_server_add_graph admits graphs of one device only)
    if (s->device >= 0) cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        gpu_acquire(s, lk, 0);
        std::vector<std::pair<uint32_t, int>> work;
        admit_locked(s, work);
        if (work.empty()) {
            if (s->stop) {
                gpu_release(s, 0);
                return;
            }
            bool stalled = false;
            for (const auto &gs : s->graphs) stalled = stalled || !gs.pend[0].empty() || !gs.pend[1].empty();
            if (stalled) {
                // queries wait for batch memory while no batch runs: free what
                // is idle, else wait for the single worker's run, else run the
                // waiting queries one at a time
                if (reclaim_locked(s, -1) > 0) {
                    gpu_release(s, 0);
                    continue;
                }
                if (s->single_graph >= 0) {
                    gpu_release(s, 0);
                    s->cv_work.wait_for(lk, std::chrono::milliseconds(1));
                    continue;
                }
                for (auto &gs : s->graphs)
                    for (int k = 0; k < 2; k++)
                        while (!gs.pend[k].empty()) {
                            s->single.push_back(gs.pend[k].front());
                            gs.pend[k].pop_front();
                        }
                evict_idle_locked(s);
                s->cv_work.notify_all();
                gpu_release(s, 0);
                continue;
            }
            s->cv_done.notify_all();
            gpu_release(s, 0);
            s->cv_work.wait(lk);
            continue;
        }
        for (const auto &w : work) s->graphs[w.first].in_use[w.second] = true;
        lk.unlock();
        // one iteration of every busy batch, each on its own stream: all are
        // launched before any is waited for, so their work overlaps on the GPU
        std::vector<uint64_t> fin(work.size(), 0);
        std::vector<asc_status> sts(work.size(), ASC_OK);
        for (size_t i = 0; i < work.size(); i++) {
            GraphSlot &gs = s->graphs[work[i].first];
            sts[i] = asc::batch_launch(gs.batch[work[i].second]);
        }
        for (size_t i = 0; i < work.size(); i++) {
            GraphSlot &gs = s->graphs[work[i].first];
            if (sts[i] == ASC_OK) sts[i] = asc::batch_collect(gs.batch[work[i].second], &fin[i]);
        }
        // finished sources: copy their values out
        std::vector<std::pair<Query *, asc_status>> done;
        std::vector<std::string> why(work.size());
        for (size_t i = 0; i < work.size(); i++) {
            GraphSlot &gs = s->graphs[work[i].first];
            const int k = work[i].second;
            uint64_t f = fin[i];
            if (sts[i] != ASC_OK) {
                // every source of the batch fails with the error; the engine is
                // emptied so that it is freed below, not launched again
                char msg[512];
                asc_last_error(msg, sizeof(msg));
                why[i] = std::string("graph ") + std::to_string(work[i].first) + (k ? " SSSP" : " BFS") +
                         " batch: " + msg;
                asc::batch_abort(gs.batch[k]);
                for (uint32_t slot = 0; slot < 64; slot++)
                    if (gs.slot_q[k][slot]) f |= 1ull << slot;
            }
            uint32_t width = 0;
            for (uint32_t slot = 0; slot < 64; slot++) width += gs.slot_q[k][slot] != nullptr;
            while (f) {
                const uint32_t slot = __builtin_ctzll(f);
                f &= f - 1;
                Query *q = gs.slot_q[k][slot];
                if (!q) continue;
                asc_status st = sts[i];
                if (st == ASC_OK && q->out) {
                    st = asc::batch_fetch(gs.batch[k], slot, q->out, false);
                    if (st != ASC_OK) {
                        char msg[512];
                        asc_last_error(msg, sizeof(msg));
                        q->err = msg;
                    }
                } else if (st != ASC_OK) {
                    q->err = why[i];
                }
                q->batch = width;
                done.push_back({q, st});
                gs.slot_q[k][slot] = nullptr;
            }
        }
        lk.lock();
        for (const auto &w : work) s->graphs[w.first].in_use[w.second] = false;
        // a batch whose launch failed is freed (its device state is undefined);
        // its waiting queries get a new engine
        for (size_t i = 0; i < work.size(); i++) {
            GraphSlot &gs = s->graphs[work[i].first];
            const int k = work[i].second;
            if (sts[i] == ASC_OK || !gs.batch[k]) continue;
            asc::batch_destroy(gs.batch[k]);
            gs.batch[k] = nullptr;
            s->used_bytes -= gs.batch_bytes[k];
            gs.batch_bytes[k] = 0;
            if (k == 0) {
                s->used_bytes -= (uint64_t)gs.planes * 4ull * gs.g->V;
                gs.planes = 0;
            }
            s->engines_freed++;
        }
        for (auto &d : done) finish(s, d.first, d.second);
        s->batches += work.size();
        if (!done.empty()) s->cv_done.notify_all();
        gpu_release(s, 0);
    }
}

void single_loop(asc_server *s) {
    if (s->device >= 0) cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        while (!s->single.empty() && s->single.front()->cancel) {
            finish(s, s->single.front(), ASC_ERR_CANCELLED);
            s->single.pop_front();
            s->cv_done.notify_all();
        }
        if (s->single.empty()) {
            gpu_release(s, 1);
            if (s->stop) return;
            s->cv_work.wait(lk);
            continue;
        }
        if (s->gpu_holder != 1) {
            gpu_acquire(s, lk, 1);
            continue;  // the queue may have changed meanwhile
        }
        Query *q = s->single.front();
        s->single.pop_front();
        GraphSlot &gs = s->graphs[q->graph];
        const bool pr = q->algo == ASC_PR;
        // budget: the graph's single-query state (and PageRank buffers)
        uint64_t have = gs.ws_bytes;
        uint64_t need = asc::workspace_bytes(gs.g, pr || gs.ws_pr);
        if (need > have) {
            if (need - have > budget_left(s)) {
                if (s->cfg.device_budget_bytes && need > s->cfg.device_budget_bytes) {
                    finish(s, q, ASC_ERR_BUDGET);
                    s->cv_done.notify_all();
                    gpu_release(s, 1);
                    continue;
                }
                reclaim_locked(s, (int)q->graph);
                s->cv_work.notify_all();
                if (need - have > budget_left(s)) {
                    if (batch_held(s) == 0) {
                        finish(s, q, ASC_ERR_BUDGET);
                        s->cv_done.notify_all();
                        gpu_release(s, 1);
                        continue;
                    }
                    // running batches still hold memory: retry when they drain
                    // (the device turn goes to the batch worker meanwhile)
                    if (!q->mem_wait) s->memory_waits++;
                    q->mem_wait = true;
                    s->single.push_front(q);
                    gpu_release(s, 1);
                    s->cv_work.wait_for(lk, std::chrono::milliseconds(1));
                    continue;
                }
            }
            s->used_bytes += need - have;
            gs.ws_bytes = need;
            gs.ws_pr = gs.ws_pr || pr;
        }
        // identical pending queries (same graph, algorithm, source-free
        // semantics and parameters) share this run
        std::vector<Query *> group{q};
        if (s->cfg.mode == ASC_SERVE_BATCHED && (q->algo == ASC_CC || q->algo == ASC_PR)) {
            for (auto it = s->single.begin(); it != s->single.end();) {
                Query *o = *it;
                if (o->graph == q->graph && o->algo == q->algo && !o->cancel &&
                    memcmp(&o->params, &q->params, sizeof(asc_params)) == 0) {
                    group.push_back(o);
                    it = s->single.erase(it);
                } else {
                    ++it;
                }
            }
        }
        for (Query *x : group) {
            x->state = Q_RUNNING;
            x->t_start = Clock::now();
        }
        s->single_graph = (int)q->graph;
        lk.unlock();
        asc_stats st;
        // beside the batch worker, a whole run steps its iterations from the
        // host and gives the device turn to a waiting batch iteration between
        // them, so a long run (PageRank on the largest graph: hundreds of ms)
        // does not hold the batches up
        asc_params prm = q->params;
        if (s->cfg.mode == ASC_SERVE_BATCHED) {
            prm.flags |= ASC_RUN_HOST_LOOP;
            asc::t_iteration_hook.fn = single_yield;
            asc::t_iteration_hook.ctx = s;
        }
        asc_status rc = asc_run(gs.g, q->algo, q->source, &prm, q->out, &st);
        asc::t_iteration_hook = asc::IterationHook();
        std::string why;
        if (rc != ASC_OK) {
            char msg[512];
            asc_last_error(msg, sizeof(msg));
            why = std::string("graph ") + std::to_string(q->graph) + " whole run: " + msg;
        }
        if (rc == ASC_OK && group.size() > 1) {
            size_t bytes = (size_t)gs.g->V *
                           (q->algo == ASC_PR ? ((q->params.pr_mode == ASC_PR_STD && q->params.precision == ASC_F32) ? 4 : 8)
                                              : 4);
            for (size_t i = 1; i < group.size(); i++)
                if (group[i]->out && q->out) memcpy(group[i]->out, q->out, bytes);
        }
        lk.lock();
        s->single_graph = -1;
        // the run's state as allocated (an estimate is accounted before a
        // graph's first run)
        if (gs.g->ws && gs.g->ws->device_bytes != gs.ws_bytes) {
            s->used_bytes = s->used_bytes - gs.ws_bytes + gs.g->ws->device_bytes;
            gs.ws_bytes = gs.g->ws->device_bytes;
        }
        s->cv_work.notify_all();
        for (Query *x : group) {
            x->iterations = st.iterations;
            x->batch = (uint32_t)group.size();
            x->err = why;
            finish(s, x, rc);
        }
        s->cv_done.notify_all();
        gpu_release(s, 1);
    }
}

void start_workers(asc_server *s) {
    if (s->started) return;
    s->started = true;
    if (s->cfg.mode == ASC_SERVE_BATCHED) s->batch_worker = std::thread(batch_loop, s);
    s->single_worker = std::thread(single_loop, s);
}

}  // namespace

using namespace asc;

extern "C" {

void asc_server_config_default(asc_server_config *c) {
    if (!c) return;
    memset(c, 0, sizeof(*c));
    c->device_budget_bytes = 0;
    c->max_batch = 64;
    c->queue_capacity = 1u << 20;
    c->mode = ASC_SERVE_BATCHED;
}

asc_status asc_server_create(const asc_server_config *cfg, asc_server **out) {
    if (!out) return fail(ASC_ERR_INVALID, "asc_server_create: out is NULL");
    asc_server *s = new asc_server();
    if (cfg) s->cfg = *cfg;
    else asc_server_config_default(&s->cfg);
    if (s->cfg.mode != ASC_SERVE_BATCHED && s->cfg.mode != ASC_SERVE_FIFO) {
        delete s;
        return fail(ASC_ERR_INVALID, "unknown server mode %u", s->cfg.mode);
    }
    if (!s->cfg.queue_capacity) s->cfg.queue_capacity = 1u << 20;
    *out = s;
    return ASC_OK;
}

asc_status asc_server_add_graph(asc_server *s, asc_graph *g, uint32_t *graph_id) {
    if (!s || !g || !graph_id) return fail(ASC_ERR_INVALID, "asc_server_add_graph: null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->started) return fail(ASC_ERR_INVALID, "add graphs before the first query");
    // the workers run every graph's kernels with one device current
    if (s->device >= 0 && g->device != s->device)
        return fail(ASC_ERR_INVALID, "graph was opened on device %d, this server's graphs on device %d", g->device,
                    s->device);
    asc_graph_info info;
    asc_graph_info_get(g, &info);
    GraphSlot gs;
    gs.g = g;
    gs.base_bytes = info.device_edge_bytes + g->device_vertex_bytes;
    if (g->ws) {
        gs.ws_bytes = g->ws->device_bytes;
        gs.ws_pr = g->ws->pr_rank != nullptr;
    }
    if (s->cfg.device_budget_bytes && s->used_bytes + gs.base_bytes + gs.ws_bytes > s->cfg.device_budget_bytes)
        return fail(ASC_ERR_BUDGET, "graph needs %llu device bytes, %llu of the budget left",
                    (unsigned long long)(gs.base_bytes + gs.ws_bytes), (unsigned long long)budget_left(s));
    s->used_bytes += gs.base_bytes + gs.ws_bytes;
    s->device = g->device;
    *graph_id = (uint32_t)s->graphs.size();
    s->graphs.push_back(gs);
    return ASC_OK;
}

asc_status asc_server_submit(asc_server *s, uint32_t graph_id, asc_algo algo, uint32_t source,
                             const asc_params *params, void *out, uint64_t *ticket) {
    if (!s || !ticket) return fail(ASC_ERR_INVALID, "asc_server_submit: null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    if (graph_id >= s->graphs.size()) return fail(ASC_ERR_INVALID, "unknown graph %u", graph_id);
    if ((unsigned)algo > (unsigned)ASC_PR) return fail(ASC_ERR_INVALID, "unknown algorithm");
    asc_graph *g = s->graphs[graph_id].g;
    if ((algo == ASC_BFS || algo == ASC_SSSP) && source >= g->V)
        return fail(ASC_ERR_INVALID, "source %u is not a vertex", source);
    if (algo == ASC_SSSP && g->edge_words != 2 && g->wbits == 0)
        return fail(ASC_ERR_UNSUPPORTED, "SSSP needs a weighted graph");
    if ((algo == ASC_BFS || algo == ASC_SSSP || algo == ASC_CC) && g->is_csc)
        return fail(ASC_ERR_UNSUPPORTED, "BFS/SSSP/CC need an out-edge graph");
    if (s->queries.size() >= s->cfg.queue_capacity) return fail(ASC_ERR_BUSY, "server queue is full");
    Query *q = new Query();
    q->ticket = s->next_ticket++;
    q->graph = graph_id;
    q->algo = algo;
    q->source = source;
    if (params) q->params = *params;
    else asc_params_default(&q->params);
    q->params.flags &= ~(uint32_t)(ASC_RUN_PHASE_TIMING | ASC_RUN_DEVICE_OUT);
    if (!out) q->params.flags |= ASC_RUN_NO_OUTPUT;
    q->out = out;
    q->t_submit = Clock::now();
    if (!s->any_submit) {
        s->any_submit = true;
        s->first_submit = q->t_submit;
    }
    s->queries[q->ticket] = q;
    s->submitted++;
    if (batchable(s, q)) s->graphs[graph_id].pend[algo == ASC_SSSP ? 1 : 0].push_back(q);
    else s->single.push_back(q);
    start_workers(s);
    *ticket = q->ticket;
    s->cv_work.notify_all();
    return ASC_OK;
}

asc_status asc_server_wait(asc_server *s, uint64_t ticket, int64_t timeout_ms, asc_query_info *info) {
    if (!s) return fail(ASC_ERR_INVALID, "asc_server_wait: null server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->queries.find(ticket);
    if (it == s->queries.end()) return fail(ASC_ERR_INVALID, "unknown ticket %llu", (unsigned long long)ticket);
    Query *q = it->second;
    auto pred = [&] { return q->state == Q_DONE; };
    if (timeout_ms < 0) s->cv_done.wait(lk, pred);
    else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred))
        return fail(ASC_ERR_TIMEOUT, "query %llu still running", (unsigned long long)ticket);
    if (info) {
        memset(info, 0, sizeof(*info));
        info->status = q->status;
        info->iterations = q->iterations;
        info->batch_size = q->batch;
        info->queue_ms = std::chrono::duration<double, std::milli>(q->t_start - q->t_submit).count();
        info->latency_ms = std::chrono::duration<double, std::milli>(q->t_end - q->t_submit).count();
    }
    asc_status st = q->status;
    const std::string why = q->err;
    s->queries.erase(it);
    delete q;
    if (st != ASC_OK && st != ASC_ERR_CANCELLED)
        return fail(st, "query %llu failed%s%s", (unsigned long long)ticket, why.empty() ? "" : ": ", why.c_str());
    return st;
}

asc_status asc_server_cancel(asc_server *s, uint64_t ticket) {
    if (!s) return fail(ASC_ERR_INVALID, "asc_server_cancel: null server");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->queries.find(ticket);
    if (it == s->queries.end()) return fail(ASC_ERR_INVALID, "unknown ticket");
    if (it->second->state == Q_PENDING) it->second->cancel = true;
    s->cv_work.notify_all();
    return ASC_OK;
}

asc_status asc_server_stats_get(asc_server *s, asc_server_stats *out) {
    if (!s || !out) return fail(ASC_ERR_INVALID, "asc_server_stats_get: null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    memset(out, 0, sizeof(*out));
    out->submitted = s->submitted;
    out->completed = s->completed;
    out->failed = s->failed;
    out->cancelled = s->cancelled;
    out->batch_iterations = s->batches;
    out->device_bytes = s->used_bytes;
    out->engines_created = s->engines_created;
    out->engines_freed = s->engines_freed;
    out->workspaces_freed = s->workspaces_freed;
    out->memory_waits = s->memory_waits;
    std::vector<double> l = s->lat_ms;
    if (!l.empty()) {
        std::sort(l.begin(), l.end());
        auto pct = [&](double p) { return l[std::min(l.size() - 1, (size_t)(p * (l.size() - 1) + 0.5))]; };
        out->p50_ms = pct(0.50);
        out->p99_ms = pct(0.99);
        double sum = 0;
        for (double x : l) sum += x;
        out->mean_ms = sum / l.size();
        out->max_ms = l.back();
    }
    if (s->any_submit && s->completed) {
        double span = std::chrono::duration<double>(s->last_done - s->first_submit).count();
        out->queries_per_s = span > 0 ? s->completed / span : 0;
        out->span_s = span;
    }
    return ASC_OK;
}

asc_status asc_server_destroy(asc_server *s) {
    if (!s) return ASC_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        for (auto &kv : s->queries)
            if (kv.second->state == Q_PENDING) kv.second->cancel = true;
        s->cv_work.notify_all();
    }
    if (s->batch_worker.joinable()) s->batch_worker.join();
    if (s->single_worker.joinable()) s->single_worker.join();
    for (auto &gs : s->graphs)
        for (auto &b : gs.batch) batch_destroy(b);
    for (auto &kv : s->queries) delete kv.second;
    delete s;
    return ASC_OK;
}

}  // extern "C"
