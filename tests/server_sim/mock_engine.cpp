// Host-only stand-in for the engine entry points the query server calls
// (batch engines, whole runs, workspaces), so that csrc/server.cpp can be
// compiled and driven on a machine without a GPU. Test infrastructure only.
//
// The stand-in keeps the server's contracts observable:
//  * device bytes: every "allocation" (batch state, level planes, single-query
//    state, PageRank buffers) is added to a counter that must never exceed the
//    server's budget;
//  * device turns: a batch iteration is "in flight" from its launch to its
//    collection and a whole run between its iterations; the two workers must
//    never have work in flight, or allocate or free, while the other does;
//  * values: a batch source and a whole run of the same query produce the same
//    deterministic values, so a test can check every output buffer.
#include <string.h>

#include <atomic>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <mutex>
#include <thread>

#include "common.h"
#include "sim.h"

namespace {

thread_local char t_err[512];

std::atomic<uint64_t> g_bytes{0};            // device bytes held right now
std::atomic<int> g_batch_inflight{0};        // batch iterations launched and not yet collected
std::atomic<int> g_single_inflight{0};       // whole runs with an iteration in flight
std::atomic<uint64_t> g_violations{0};
std::atomic<uint64_t> g_budget{0};
std::atomic<uint64_t> g_fail_source{0xffffffffull};
std::mutex g_msg_mu;
char g_first_violation[256];

void violation(const char *what) {
    if (g_violations.fetch_add(1) == 0) {
        std::lock_guard<std::mutex> lk(g_msg_mu);
        snprintf(g_first_violation, sizeof(g_first_violation), "%s", what);
    }
}

void add_bytes(uint64_t b) {
    const uint64_t now = g_bytes.fetch_add(b) + b;
    if (g_budget.load() && now > g_budget.load()) violation("device bytes above the server budget");
}

void sub_bytes(uint64_t b) { g_bytes.fetch_sub(b); }

// a batch iteration's launch, collection or copy-out: no whole-run iteration in flight
void check_batch_side() {
    if (g_single_inflight.load()) violation("batch worker used the device during a whole run's iteration");
}
// a whole-run iteration: no batch iteration in flight
void check_single_side() {
    if (g_batch_inflight.load()) violation("whole run used the device during a batch iteration");
}
// an allocation or free (either worker): nothing in flight at all
void check_quiet() {
    if (g_single_inflight.load() || g_batch_inflight.load())
        violation("device memory allocated or freed with device work in flight");
}

void spin_us(int us) { std::this_thread::sleep_for(std::chrono::microseconds(us)); }

}  // namespace

// values of a query: identical for a batch source and a whole run
uint32_t sim_value(asc_algo algo, uint32_t source, uint64_t v) {
    switch (algo) {
    case ASC_BFS: return (uint32_t)(source * 2654435761u + v) % 97u;
    case ASC_SSSP: return (uint32_t)(source * 40503u + 3 * v) % 1009u;
    case ASC_CC: return (uint32_t)(v % 13u);
    default: return 0;
    }
}

// iterations a source stays in a batch
static uint32_t sim_iters(uint32_t source) { return 1 + source % 5; }

void sim_reset(uint64_t budget, uint32_t fail_source) {
    g_bytes = 0;
    g_batch_inflight = 0;
    g_single_inflight = 0;
    g_violations = 0;
    g_budget = budget;
    g_fail_source = fail_source;
    g_first_violation[0] = 0;
}

uint64_t sim_violations(char *first, size_t n) {
    std::lock_guard<std::mutex> lk(g_msg_mu);
    snprintf(first, n, "%s", g_first_violation);
    return g_violations.load();
}

uint64_t sim_bytes() { return g_bytes.load(); }

asc_graph *sim_graph(uint64_t V) {
    asc_graph *g = new asc_graph();
    g->V = V;
    g->E = 16 * V;
    g->device = 0;
    g->edge_words = 2;  // weighted: SSSP allowed
    return g;
}

void sim_graph_free(asc_graph *g) {
    asc::free_workspace(g);
    delete g;
}

extern "C" cudaError_t cudaSetDevice(int) { return cudaSuccess; }

extern "C" size_t asc_last_error(char *buf, size_t n) {
    if (buf && n) snprintf(buf, n, "%s", t_err);
    return strlen(t_err);
}

extern "C" void asc_params_default(asc_params *p) {
    memset(p, 0, sizeof(*p));
    p->damping = 0.85;
    p->tolerance = 1e-9;
}

extern "C" asc_status asc_graph_info_get(const asc_graph *g, asc_graph_info *info) {
    memset(info, 0, sizeof(*info));
    info->vertices = g->V;
    info->edges = g->E;
    info->device_edge_bytes = 2 * g->V;  // the static region stands in as 2 bytes per vertex
    return ASC_OK;
}

// whole run: a few host-stepped iterations, the iteration hook between them
extern "C" asc_status asc_run(asc_graph *g, asc_algo algo, uint32_t source, const asc_params *p, void *out,
                              asc_stats *st) {
    check_quiet();
    if (!g->ws) {  // single-query state, allocated on a graph's first run
        g->ws = new asc::Workspace();
        g->ws->device_bytes = asc::workspace_bytes(g, false);
        g->ws->V = g->V;
        add_bytes(g->ws->device_bytes);
    }
    if (algo == ASC_PR && !g->ws->pr_rank) {
        check_quiet();
        g->ws->pr_rank = g;  // marks the buffers as present
        g->ws->device_bytes += 32 * g->V;
        add_bytes(32 * g->V);
    }
    const int iters = algo == ASC_PR ? 6 : 3;
    for (int i = 0; i < iters; i++) {
        g_single_inflight.fetch_add(1);
        check_single_side();
        spin_us(150);
        check_single_side();
        g_single_inflight.fetch_sub(1);
        asc::iteration_boundary();
    }
    if (out && !(p && (p->flags & ASC_RUN_NO_OUTPUT))) {
        if (algo == ASC_PR) {
            float *o = static_cast<float *>(out);
            for (uint64_t v = 0; v < g->V; v++) o[v] = (float)(v % 11) * 0.5f;
        } else {
            uint32_t *o = static_cast<uint32_t *>(out);
            for (uint64_t v = 0; v < g->V; v++) o[v] = sim_value(algo, source, v);
        }
    }
    if (st) {
        memset(st, 0, sizeof(*st));
        st->iterations = iters;
    }
    return ASC_OK;
}

namespace asc {

thread_local IterationHook t_iteration_hook;

asc_status fail(asc_status s, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(t_err, sizeof(t_err), fmt, ap);
    va_end(ap);
    return s;
}

struct BatchEngine {
    asc_graph *g = nullptr;
    bool sssp = false;
    uint32_t stride = 64;
    uint64_t bytes = 0;
    bool plane[64] = {false};
    uint32_t src[64] = {0};
    uint32_t left[64] = {0};
    uint64_t active = 0, pending = 0;
    bool inflight = false;
    bool failed = false;
};

uint64_t batch_state_bytes(asc_graph *g, bool sssp, uint32_t stride) {
    return 40 * g->V + (sssp ? 4ull * g->V * stride + 4 * g->V : 0);
}

uint64_t batch_plane_bytes(asc_graph *g) { return 4ull * g->V; }

uint64_t workspace_bytes(asc_graph *g, bool pagerank) {
    uint64_t b = g->ws ? g->ws->device_bytes : 12 * g->V;
    if (pagerank && (!g->ws || !g->ws->pr_rank)) b += 32 * g->V;
    return b;
}

void free_workspace(asc_graph *g) {
    if (!g->ws) return;
    check_quiet();
    sub_bytes(g->ws->device_bytes);
    delete g->ws;
    g->ws = nullptr;
}

asc_status batch_create(asc_graph *g, bool sssp, uint32_t stride, BatchEngine **out) {
    check_quiet();
    BatchEngine *b = new BatchEngine();
    b->g = g;
    b->sssp = sssp;
    b->stride = stride;
    b->bytes = batch_state_bytes(g, sssp, stride);
    add_bytes(b->bytes);
    *out = b;
    return ASC_OK;
}

void batch_destroy(BatchEngine *b) {
    if (!b) return;
    check_quiet();
    if (b->inflight) violation("batch engine freed with an iteration in flight");
    sub_bytes(b->bytes);
    for (int i = 0; i < 64; i++)
        if (b->plane[i]) sub_bytes(batch_plane_bytes(b->g));
    delete b;
}

bool batch_has_plane(BatchEngine *b, uint32_t slot) { return b->sssp || b->plane[slot]; }

asc_status batch_admit(BatchEngine *b, uint32_t slot, uint32_t source) {
    if (slot >= batch_slots(b)) return fail(ASC_ERR_INVALID, "slot %u out of range", slot);
    if (b->active & (1ull << slot)) return fail(ASC_ERR_INVALID, "slot %u is busy", slot);
    if (!b->sssp && !b->plane[slot]) {
        check_quiet();
        b->plane[slot] = true;
        add_bytes(batch_plane_bytes(b->g));
    }
    b->src[slot] = source;
    b->left[slot] = sim_iters(source);
    b->active |= 1ull << slot;
    b->pending |= 1ull << slot;
    return ASC_OK;
}

bool batch_busy(const BatchEngine *b) { return b->active != 0; }

uint32_t batch_slots(const BatchEngine *b) { return b->sssp ? b->stride : 64u; }

void batch_abort(BatchEngine *b) {
    b->active = 0;
    b->pending = 0;
}

asc_status batch_launch(BatchEngine *b) {
    check_batch_side();
    if (b->inflight) return fail(ASC_ERR_INVALID, "batch launched twice");
    b->pending = 0;
    for (int s = 0; s < 64; s++)
        if ((b->active >> s) & 1 && b->src[s] == g_fail_source.load())
            return fail(ASC_ERR_CUDA, "injected launch failure for source %u", b->src[s]);
    b->inflight = true;
    g_batch_inflight.fetch_add(1);
    return ASC_OK;
}

asc_status batch_collect(BatchEngine *b, uint64_t *finished) {
    check_batch_side();
    spin_us(80);
    check_batch_side();
    uint64_t fin = 0;
    for (int s = 0; s < 64; s++)
        if ((b->active >> s) & 1) {
            if (--b->left[s] == 0) fin |= 1ull << s;
        }
    b->active &= ~fin;
    *finished = fin;
    b->inflight = false;
    g_batch_inflight.fetch_sub(1);
    return ASC_OK;
}

asc_status batch_fetch(BatchEngine *b, uint32_t slot, void *out, bool) {
    check_batch_side();
    uint32_t *o = static_cast<uint32_t *>(out);
    const asc_algo algo = b->sssp ? ASC_SSSP : ASC_BFS;
    for (uint64_t v = 0; v < b->g->V; v++) o[v] = sim_value(algo, b->src[slot], v);
    return ASC_OK;
}

}  // namespace asc
