// Internal declarations shared by the host code and the CUDA engine.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>
#include <vector>

#include "ascetic.h"

namespace asc {

struct BatchEngine;
struct StagePlan;
struct PartPlan;

// Thread-local last-error message (asc_last_error).
void set_error(const char *fmt, ...);
asc_status fail(asc_status s, const char *fmt, ...);
asc_status cuda_fail(cudaError_t e, const char *what, const char *file, int line);

#define ASC_CUDA(call)                                                                  \
    do {                                                                                \
        cudaError_t _asc_e = (call);                                                    \
        if (_asc_e != cudaSuccess) return ::asc::cuda_fail(_asc_e, #call, __FILE__, __LINE__); \
    } while (0)

#define ASC_TRY(call)                                  \
    do {                                               \
        asc_status _asc_s = (call);                    \
        if (_asc_s != ASC_OK) return _asc_s;           \
    } while (0)

// Engine tunables (block size is fixed at compile time, the rest per graph).
constexpr int kBlock = 256;

struct Tuning {
    uint32_t huge_degree = 512;   // lists longer than this are cut into segments
    uint32_t segment_edges = 2048;  // edges per segment work item
    uint32_t ctas_per_sm = 0;     // persistent expansion grid = SMs x this (0: as many as stay resident)
    uint32_t dense_div = 64;      // walk a region in id order (frontier bitmap) when its list
                                  // holds more than 1/dense_div of the region's vertices; 0 = never
    uint32_t delta = 0;           // SSSP near-far step: distances >= threshold wait in the far set,
                                  // the threshold advances to (min far distance + delta); 0 = off
    uint32_t bu_div = 64;         // BFS on CSR graphs: a step whose frontier holds more than V / bu_div
                                  // vertices runs bottom-up over the in-edges; 0 = top-down only
};

// Per-run device state, sized for one graph and reused across its runs.
struct Workspace {
    uint64_t V = 0;
    uint32_t *val = nullptr;         // u32 values (BFS/SSSP/CC)
    uint32_t *bitmap[2] = {nullptr, nullptr};  // frontier membership by parity, one bit per vertex
    uint32_t *visited = nullptr;     // BFS: one bit per vertex already reached
    uint32_t *huge_bits = nullptr;   // one bit per vertex with more than huge_degree edges
    uint32_t *far_bits = nullptr;    // SSSP: vertices waiting for the threshold to reach them
    uint32_t *queue[2] = {nullptr, nullptr};   // [V]: static entries from 0, on-demand from S
    uint64_t *segs[2] = {nullptr, nullptr};    // segment items (v << 32 | k)
    uint64_t segcap_static = 0, segcap_ondemand = 0;
    uint32_t *ctl = nullptr;         // device control block (counters, work cursors, stats)
    uint32_t *h_ctl = nullptr;       // pinned mirror for per-iteration readback
    // PageRank buffers (allocated on the first PR run)
    void *pr_rank = nullptr;         // f64 or f32 [V]
    void *pr_contrib[2] = {nullptr, nullptr};
    void *pr_sum = nullptr;          // segment partial sums [V]
    size_t pr_elem = 0;
    uint32_t *huge_list = nullptr;   // vertices with degree > huge_degree, static first
    uint32_t n_huge_static = 0, n_huge_total = 0;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    std::vector<cudaEvent_t> phase_events;
    struct BatchEngine *batch[2] = {nullptr, nullptr};  // asc_run_batch engines (BFS, SSSP)
    cudaGraphExec_t loop_exec[3] = {nullptr, nullptr, nullptr};  // BFS, SSSP, CC iteration loops
    uint32_t loop_cap[3] = {0, 0, 0};
    Tuning tune;
    int num_sms = 0;
    uint64_t device_bytes = 0;
    unsigned long long *frag_counts = nullptr;  // per 4096-edge fragment, allocated on first use
    unsigned long long *frag_active = nullptr;  // frag_counts during a counting run, else null
    // gather-and-copy comparison engine (ASC_RUN_GATHER_COPY), allocated on first use
    uint32_t *g_stage = nullptr;     // device staging: gathered on-demand edges, edge_words words each
    uint32_t *g_items = nullptr;     // device: per item (vertex, staged offset, length, first segment)
    uint32_t *h_stage = nullptr;     // page-locked host staging
    uint32_t *h_items = nullptr;     // page-locked host items
    uint32_t *h_list = nullptr;      // page-locked copy of the on-demand frontier list
    uint64_t *h_segs = nullptr;      // page-locked copy of the on-demand segment items
    uint64_t g_cap = 0;              // staging capacity in edges (and in items)
    StagePlan *stage = nullptr;      // chunk plan of staged PageRank passes, made on first use
    PartPlan *part = nullptr;        // partitions of the whole-partition comparison engine
    uint32_t *in_ptr = nullptr;      // in-edge offsets on the device (bottom-up BFS steps)
    uint32_t *in_edges = nullptr;    // in-edges on the device (only when every out-edge is resident)
    uint32_t *in_none = nullptr;     // one bit per vertex without in-edges
    bool bu_active = false;          // this run's region arguments enable bottom-up steps
};

}  // namespace asc

struct asc_graph {
    uint64_t V = 0, E = 0;
    uint32_t edge_words = 1;      // 1: u32 destination (or packed dst/weight), 2: {dst, weight}
    uint32_t wbits = 0;           // > 0: weighted edges packed as (dst << wbits) | weight in one u32
    uint32_t ebits = 32;          // edge_words == 1: bits per edge word in h_edges / d_static (< 32:
                                  // a bit stream, edge i at bits [i*ebits, (i+1)*ebits))
    uint32_t file_edge_bytes = 4; // bytes per edge of the source layout (the budget's unit)
    bool is_csc = false;
    uint32_t max_degree = 0;
    uint32_t max_weight = 0;
    // host (pinned)
    uint32_t *h_ptr = nullptr;    // V+1 offsets (u32: E < 2^32)
    uint32_t *h_edges = nullptr;  // E * edge_words (or the ebits stream), mapped for device reads
    uint32_t *h_outdeg = nullptr; // V (CSC graphs)
    // device
    const uint32_t *d_host_edges = nullptr;  // device address of h_edges (zero-copy reads)
    uint32_t *managed_edges = nullptr;       // ASC_BUDGET_MANAGED: managed copy read instead
    uint32_t *d_ptr = nullptr;
    uint32_t *d_static = nullptr;  // edge prefix [0, static_edges)
    uint32_t *d_stage[2] = {nullptr, nullptr};  // staging buffers of dense on-demand passes
    uint64_t stage_words = 0;      // u32 words in each staging buffer (0: no staging)
    // in-edges of a CSR graph (bottom-up BFS steps), built on first use
    uint32_t *h_in_ptr = nullptr;  // V+1 offsets (host)
    uint32_t *h_in_none = nullptr;  // V/32+2 words: bit set where a vertex has no in-edges (host)
    // lists cut into segments for a (huge_degree, segment_edges), found on the
    // first workspace of that tuning and reused by later ones (a server frees
    // and re-creates the workspaces of idle graphs and batches, whose tunings
    // differ); the most recent few tunings are kept
    struct LongLists {
        uint32_t huge_degree = 0, segment_edges = 0;
        std::vector<uint32_t> list, bits;  // long-list vertices; one bit per vertex (V/32+2 words)
        uint64_t seg_static = 0, seg_ondemand = 0;  // segments of the static / on-demand long lists
        uint32_t n_static = 0;
    };
    std::vector<LongLists> long_lists;
    std::mutex long_lists_mu;
    uint32_t *h_in_edges = nullptr;  // source ids, a bit stream of in_ebits per edge (pinned, mapped)
    const uint32_t *d_host_in_edges = nullptr;
    uint32_t in_ebits = 32;
    uint32_t *d_in_heads = nullptr;  // first in-edge per vertex in HBM (from the byte budget), a bit stream
    uint64_t in_head_words = 0;
    bool in_heads_ready = false;
    uint32_t *d_outdeg = nullptr;
    uint64_t static_edges = 0;
    uint32_t static_vertices = 0;  // S: vertices [0, S) have all edges in the prefix
    int device = 0;
    cudaStream_t stream = nullptr;
    asc::Workspace *ws = nullptr;
    uint64_t device_vertex_bytes = 0;
    bool has_tuning = false;      // tuning chosen by asc_graph_set_tuning / asc_graph_tune
    asc::Tuning tuning;
};

namespace asc {
// u32 words holding edges [0, n) of a graph's edge array (plus one word of
// padding for bit streams, so a straddling read never leaves the buffer)
inline uint64_t edge_store_words(const asc_graph *g, uint64_t n) {
    if (g->edge_words == 2) return 2 * n;
    if (g->ebits == 32) return n;
    return (n * g->ebits + 31) / 32 + 1;
}
// bytes that n edges occupy in the stored layout (what n on-demand edges move over the link)
inline uint64_t edge_store_bytes(const asc_graph *g, uint64_t n) {
    if (g->edge_words == 2) return 8 * n;
    return (n * g->ebits + 7) / 8;
}
// engine.cu
asc_status run_traversal(asc_graph *g, asc_algo algo, uint32_t source, const asc_params &p, void *out,
                         asc_stats *st);
asc_status run_pagerank(asc_graph *g, const asc_params &p, void *out, asc_stats *st);
asc_status run_batch(asc_graph *g, asc_algo algo, const uint32_t *sources, uint32_t n, const asc_params &p,
                     void *out, asc_stats *st);
void free_workspace(asc_graph *g);
// continuous multi-source batches (engine.cu)
uint64_t batch_state_bytes(asc_graph *g, bool sssp, uint32_t stride);
uint64_t batch_plane_bytes(asc_graph *g);
asc_status batch_create(asc_graph *g, bool sssp, uint32_t stride, BatchEngine **out);
void batch_destroy(BatchEngine *b);
bool batch_has_plane(BatchEngine *b, uint32_t slot);
asc_status batch_admit(BatchEngine *b, uint32_t slot, uint32_t source);
bool batch_busy(const BatchEngine *b);
void batch_abort(BatchEngine *b);
// Self-checking build (ASC_SELF_CHECK): the first failed device index check since the last call.
asc_status self_check_result();
// Called on the calling thread between the iterations of a host-stepped run
// (and between PageRank passes), with none of the run's device work in flight:
// the query server hands the device to its other worker there. Unset outside it.
struct IterationHook {
    void (*fn)(void *) = nullptr;
    void *ctx = nullptr;
};
extern thread_local IterationHook t_iteration_hook;
inline void iteration_boundary() {
    if (t_iteration_hook.fn) t_iteration_hook.fn(t_iteration_hook.ctx);
}
// Source slots of a batch: 64, or the row width of a narrower SSSP batch.
uint32_t batch_slots(const BatchEngine *b);
asc_status batch_launch(BatchEngine *b);
asc_status batch_collect(BatchEngine *b, uint64_t *finished);
asc_status batch_fetch(BatchEngine *b, uint32_t slot, void *out, bool device_out);
uint64_t workspace_bytes(asc_graph *g, bool pagerank);
// graph.cpp
asc_status compute_static_split(asc_graph *g, const asc_budget *b, uint32_t param_size);
asc_status build_in_edges(asc_graph *g);
}  // namespace asc
