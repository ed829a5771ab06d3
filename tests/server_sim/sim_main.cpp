// Drives csrc/server.cpp against the host-only stand-in engine
// (mock_engine.cpp): streams of BFS/SSSP/CC/PageRank queries over several
// graphs, under an ample and under a tight device budget, with and without
// spacing between arrivals, with cancellations, with an injected launch
// failure, and in FIFO mode. Every query must complete with its values (or,
// where a failure is injected, fail with that failure's message), within a
// deadline; the stand-in must never see device bytes above the budget, nor
// the two workers using the device at the same time. Exit status 0 on success.
// Test infrastructure only.
#include <stdio.h>
#include <string.h>

#include <chrono>
#include <random>
#include <string>
#include <thread>
#include <vector>

#include "sim.h"

namespace {

int g_fails = 0;

#define CHECK(c, ...)                                                     \
    do {                                                                  \
        if (!(c)) {                                                       \
            fprintf(stderr, "FAIL %s:%d: ", __FILE__, __LINE__);          \
            fprintf(stderr, __VA_ARGS__);                                 \
            fputc('\n', stderr);                                          \
            g_fails++;                                                    \
        }                                                                 \
    } while (0)

struct Job {
    uint32_t gi = 0;
    asc_algo algo = ASC_BFS;
    uint32_t src = 0;
    uint64_t ticket = 0;
    bool cancelled = false;
    std::vector<uint32_t> out;
    std::vector<float> fout;
};

struct Scenario {
    const char *name;
    uint32_t mode;
    bool tight;
    int queries;
    int gap_us;        // arrival spacing (0: all at once)
    int cancel_every;  // cancel every n-th query right after submitting it (0: none)
    bool inject;       // one source's batch launch fails
};

void run(const Scenario &sc, uint32_t seed) {
    const std::vector<uint64_t> Vs = {4096, 16384, 65536};
    const uint32_t fail_source = sc.inject ? 777 : 0xffffffffu;
    uint64_t budget = 0;
    if (sc.tight) {
        // the graphs' static regions, one 16-row SSSP batch of the largest graph
        // and its single-query state: batches and whole runs must take turns
        // with the memory
        uint64_t bases = 0;
        for (uint64_t V : Vs) bases += 2 * V;
        budget = bases + (40 + 4 * 16 + 4) * Vs.back() + 12 * Vs.back() + 4096;
    }
    sim_reset(budget, fail_source);
    std::vector<asc_graph *> gs;
    for (uint64_t V : Vs) gs.push_back(sim_graph(V));
    asc_server_config cfg;
    asc_server_config_default(&cfg);
    cfg.device_budget_bytes = budget;
    cfg.mode = sc.mode;
    asc_server *srv = nullptr;
    CHECK(asc_server_create(&cfg, &srv) == ASC_OK, "%s: create", sc.name);
    std::vector<uint32_t> ids(gs.size());
    for (size_t i = 0; i < gs.size(); i++) CHECK(asc_server_add_graph(srv, gs[i], &ids[i]) == ASC_OK, "%s: add", sc.name);

    std::mt19937 rng(seed);
    asc_params pr;
    asc_params_default(&pr);
    pr.pr_mode = ASC_PR_STD;
    pr.precision = ASC_F32;
    std::vector<Job> jobs(sc.queries);
    for (int i = 0; i < sc.queries; i++) {
        Job &j = jobs[i];
        j.gi = rng() % gs.size();
        const uint32_t r = rng() % 10;
        j.algo = r < 5 ? ASC_BFS : (r < 8 ? ASC_SSSP : (r < 9 ? ASC_CC : ASC_PR));
        j.src = (uint32_t)(rng() % Vs[j.gi]);
        if (sc.inject && i % 50 == 7) j.src = fail_source;  // a few queries of the failing source
        void *out;
        if (j.algo == ASC_PR) {
            j.fout.assign(Vs[j.gi], -1.0f);
            out = j.fout.data();
        } else {
            j.out.assign(Vs[j.gi], 0xffffffffu);
            out = j.out.data();
        }
        const asc_status st =
            asc_server_submit(srv, ids[j.gi], j.algo, j.src, j.algo == ASC_PR ? &pr : nullptr, out, &j.ticket);
        CHECK(st == ASC_OK, "%s: submit %d", sc.name, i);
        if (sc.cancel_every && i % sc.cancel_every == 0) {
            asc_server_cancel(srv, j.ticket);
            j.cancelled = true;
        }
        if (sc.gap_us) std::this_thread::sleep_for(std::chrono::microseconds(sc.gap_us));
    }
    int ok = 0, cancelled = 0, failed = 0;
    for (int i = 0; i < sc.queries; i++) {
        Job &j = jobs[i];
        asc_query_info info;
        const asc_status st = asc_server_wait(srv, j.ticket, 60000, &info);
        if (st == ASC_ERR_TIMEOUT) {
            CHECK(false, "%s: query %d did not complete within 60 s", sc.name, i);
            continue;
        }
        if (st == ASC_ERR_CANCELLED) {
            CHECK(j.cancelled, "%s: query %d cancelled without a cancel", sc.name, i);
            cancelled++;
            continue;
        }
        if (st != ASC_OK) {
            char msg[512];
            asc_last_error(msg, sizeof(msg));
            CHECK(sc.inject && strstr(msg, "injected launch failure") && (j.algo == ASC_BFS || j.algo == ASC_SSSP),
                  "%s: query %d failed: %s", sc.name, i, msg);
            failed++;
            continue;
        }
        ok++;
        CHECK(!(sc.inject && j.src == fail_source && sc.mode == ASC_SERVE_BATCHED &&
                (j.algo == ASC_BFS || j.algo == ASC_SSSP) && info.iterations == 0),
              "%s: query %d of the failing source succeeded in a batch", sc.name, i);
        const uint64_t V = Vs[j.gi];
        bool good = true;
        for (uint64_t v = 0; v < V && good; v++) {
            if (j.algo == ASC_PR) good = j.fout[v] == (float)(v % 11) * 0.5f;
            else good = j.out[v] == sim_value(j.algo, j.src, v);
        }
        CHECK(good, "%s: query %d (graph %u, algo %d, source %u) has wrong values", sc.name, i, j.gi, (int)j.algo,
              j.src);
    }
    asc_server_stats ss;
    CHECK(asc_server_stats_get(srv, &ss) == ASC_OK, "%s: stats", sc.name);
    CHECK(ss.completed == (uint64_t)ok, "%s: completed %llu, counted %d", sc.name, (unsigned long long)ss.completed, ok);
    CHECK(!budget || ss.device_bytes <= budget, "%s: server accounts %llu bytes over a budget of %llu", sc.name,
          (unsigned long long)ss.device_bytes, (unsigned long long)budget);
    asc_server_destroy(srv);
    char first[256];
    const uint64_t nv = sim_violations(first, sizeof(first));
    CHECK(nv == 0, "%s: %llu contract violations, first: %s", sc.name, (unsigned long long)nv, first);
    if (sc.inject) CHECK(failed > 0, "%s: the injected failure failed no query", sc.name);
    else CHECK(failed == 0, "%s: %d queries failed", sc.name, failed);
    printf("%-28s ok %5d cancelled %4d failed %3d  engines %llu/%llu  states freed %llu  waits %llu\n", sc.name, ok,
           cancelled, failed, (unsigned long long)ss.engines_created, (unsigned long long)ss.engines_freed,
           (unsigned long long)ss.workspaces_freed, (unsigned long long)ss.memory_waits);
    for (asc_graph *g : gs) sim_graph_free(g);
}

}  // namespace

int main() {
    const Scenario scenarios[] = {
        {"batched, ample, burst", ASC_SERVE_BATCHED, false, 1500, 0, 0, false},
        {"batched, tight, burst", ASC_SERVE_BATCHED, true, 1500, 0, 0, false},
        {"batched, tight, spaced", ASC_SERVE_BATCHED, true, 600, 300, 0, false},
        {"batched, tight, cancels", ASC_SERVE_BATCHED, true, 800, 50, 9, false},
        {"batched, injected failure", ASC_SERVE_BATCHED, false, 600, 100, 0, true},
        {"fifo, tight", ASC_SERVE_FIFO, true, 300, 0, 0, false},
    };
    uint32_t seed = 1;
    for (const Scenario &sc : scenarios) run(sc, seed++);
    if (g_fails) {
        fprintf(stderr, "%d checks failed\n", g_fails);
        return 1;
    }
    printf("all scenarios passed\n");
    return 0;
}
