/*
 * ascetic.h: C ABI of the GB300-native out-of-GPU-memory graph iteration engine.
 *
 * The library (libascetic_gb300.so) keeps a static prefix of a graph's CSR edge
 * array resident on the GPU and reads the edges of the active vertices that the
 * prefix does not hold directly from pinned host memory over the host link
 * (NVLink-C2C on GB300), compacting them per iteration on the device.
 * BFS, SSSP, CC (min-label) and PageRank run as hand-written sm_103a kernels.
 *
 * Conventions
 *  - Every call returns an asc_status; nothing calls exit(). asc_last_error()
 *    gives the message of the last failure on the calling thread.
 *  - The caller owns every output buffer; the library owns device memory and
 *    frees it in asc_graph_close().
 *  - One asc_graph may be used by one thread at a time.
 *  - Value encoding follows the reference (GraphMeta.cuh:374-467): BFS level + 1,
 *    SSSP distance + 1, unreached = V + 1, CC minimum label, PR as double (or
 *    float when asked for).
 *
 * Reference interfaces replaced (file:line in the reference project):
 *  - ptgraph CLI flags --input/--type/--source/--adviseK  (main.cu:4-22,
 *    ArgumentParser.cu:15-48): the ptgraph binary built from
 *    ascetic_gb300/csrc/ptgraph.cpp, which calls only this header.
 *  - void bfs_opt(string path, uint src, double adviseRate)  (CalculateOpt.cuh:11)
 *  - void cc_opt(string path, double adviseRate)             (CalculateOpt.cuh:12)
 *  - void sssp_opt(string path, uint src, double adviseRate) (CalculateOpt.cuh:13)
 *  - void pr_opt(string path, double adviseRate)             (CalculateOpt.cuh:14)
 *  - GraphMeta<EdgeType>::readDataFromFile / initGraphHost / initGraphDevice
 *    (GraphMeta.cuh:151-297): asc_graph_open / asc_graph_from_csr.
 */
#ifndef ASCETIC_GB300_H
#define ASCETIC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum asc_status {
    ASC_OK = 0,
    ASC_ERR_INVALID = 1,      /* bad argument */
    ASC_ERR_BAD_FILE = 2,     /* unreadable, short or malformed graph file */
    ASC_ERR_BUDGET = 3,       /* the device budget or device memory cannot hold the run */
    ASC_ERR_CUDA = 4,         /* CUDA runtime failure */
    ASC_ERR_TIMEOUT = 5,      /* iteration limit or a bounded device wait ran out */
    ASC_ERR_CANCELLED = 6,    /* a queued or running query was cancelled */
    ASC_ERR_UNSUPPORTED = 7,  /* e.g. E >= 2^32, weights that could wrap u32, wrong file type */
    ASC_ERR_NO_DEVICE = 8,    /* no usable CUDA device */
    ASC_ERR_NOMEM = 9,        /* host allocation failed */
    ASC_ERR_BUSY = 10         /* server queue full */
} asc_status;

typedef enum asc_format {
    ASC_FMT_AUTO = 0,    /* detect from header and file size */
    ASC_FMT_BCSR = 1,    /* u64 V, u64 E, u64 ptr[V], u32 col[E]                     (.bcsr) */
    ASC_FMT_BWCSR = 2,   /* u64 V, u64 E, u64 ptr[V], {u32 dst, u32 w}[E]            (.bwcsr) */
    ASC_FMT_BCSC = 3,    /* u64 V, u64 E, u32 outDeg[V], u64 ptr[V], u32 src[E]     (.bcsc) */
    ASC_FMT_BCSR32 = 4   /* u32 V, u32 E, u32 ptr[V], u32 col[E] (legacy, bfs.cu:14-23) */
} asc_format;

typedef enum asc_algo { ASC_BFS = 0, ASC_SSSP = 1, ASC_CC = 2, ASC_PR = 3 } asc_algo;

typedef enum asc_budget_mode {
    /* Every mode but ALL and MANAGED gives a cap in edges that ends in the
     * reference's rule (GraphMeta.cuh:341-365): at most E and 2^32 - 1, rounded
     * down to whole fragments (fragment_edges, default 4096, as the reference's
     * fragmentSize), so the same cap puts the same prefix on the device. */
    ASC_BUDGET_ALL = 0,      /* whole edge array resident (no cap, no rounding) */
    ASC_BUDGET_FRAC = 1,     /* value = fraction of the source edge-array bytes (4 or 8 per edge as in
                                the file) for the static region */
    ASC_BUDGET_BYTES = 2,    /* value = bytes for the static region */
    ASC_BUDGET_ADVISE_K = 3, /* value = reference --adviseK: fraction of free device memory left
                                after the vertex arrays (GraphMeta.cuh:310-354); 0 = its auto formula */
    ASC_BUDGET_EDGES = 4,    /* value = static edge cap (the reference's max_partition_size before
                                its rounding) */
    ASC_BUDGET_MANAGED = 5   /* comparison engine, the reference's UVM baseline (bfs.cu:249-273): no
                                static region; the edge array lives in CUDA managed memory advised
                                read-mostly and the driver copies pages to the GPU as kernels touch
                                them. Device use is then up to the driver, outside any cap. */
} asc_budget_mode;

typedef struct asc_budget {
    uint32_t mode;           /* asc_budget_mode */
    uint32_t fragment_edges; /* static prefix rounded down to a multiple of this (0 = 4096,
                                the reference's fragment, GraphMeta.cuh:143,353-354) */
    double value;
    uint64_t stage_bytes;    /* bytes of the budget held as two staging buffers for dense
                                on-demand passes (0 = none). The static prefix gets the rest of
                                a FRAC, BYTES or ADVISE_K budget (an EDGES cap is the prefix
                                alone). Standard PageRank then copies the on-demand edges each
                                pass in chunks on a copy stream into the two buffers, overlapped
                                with the kernels that consume them, as the reference copies its
                                partitions into its staging area (CalculateOpt.cu:161-178,
                                GraphMeta.cuh:366-371). Ignored when every edge is static. */
} asc_budget;

typedef struct asc_graph asc_graph;

typedef struct asc_graph_info {
    uint64_t vertices;
    uint64_t edges;
    uint32_t edge_bytes;          /* bytes per edge of the source layout: 4 (destination or packed) or 8
                                     ({dst, weight}); edge_bits gives the stored width */
    uint32_t is_csc;              /* 1 for .bcsc (in-edges + out-degree block) */
    uint64_t static_edges;        /* edges in the device-resident prefix */
    uint64_t static_vertices;     /* vertices [0, static_vertices) have every edge in the prefix */
    uint64_t device_edge_bytes;   /* static region bytes (what the budget caps) */
    uint64_t device_vertex_bytes; /* offsets and per-run vertex state (outside the cap) */
    uint64_t host_pinned_bytes;   /* pinned host copy of the edge array (on-demand source) */
    uint32_t max_degree;
    uint32_t max_weight;          /* 0 for unweighted graphs */
    uint32_t weight_bits;         /* > 0: weighted edges stored packed as (dst << bits) | weight, bits the
                                     width of the largest weight (whenever destination and weight bits
                                     fit in 32): half the bytes per edge or less, twice the edges or
                                     more in the same static-region bytes */
    uint32_t edge_bits;           /* stored bits per edge: 64 ({dst, weight}), 32, or at most 30 when
                                     every edge word fits (a bit stream of edge_bits per edge, in HBM
                                     and in pinned host memory: more static edges per budget byte,
                                     fewer bytes over the host link; ASC_EDGE_PACKING=0 in the
                                     environment keeps 32) */
    uint64_t staging_bytes;       /* device staging buffers (asc_budget.stage_bytes; included in
                                     device_edge_bytes) */
    uint64_t in_head_bytes;       /* CSR graphs with edges on demand: the first in-edge of every vertex,
                                     bits(V - 1) each, held in HBM for bottom-up BFS steps (most unreached
                                     vertices find their parent there, so those steps barely touch the
                                     host link); taken from a FRAC / BYTES / ADVISE_K budget like the
                                     staging buffers, beside an EDGES cap; included in device_edge_bytes */
} asc_graph_info;

typedef enum asc_pr_mode {
    ASC_PR_REF = 0,  /* reference PageRank: 0.15 + 0.85*sum, per-vertex stop at |delta| <= 0.001,
                        FP64 (gpu_kernels.cuh:533-594) */
    ASC_PR_STD = 1   /* standard PageRank: damping, (1-d)/V teleport, dangling mass spread uniformly,
                        stop at FP64 L1 residual < tolerance or max_iterations */
} asc_pr_mode;

typedef enum asc_precision { ASC_F64 = 0, ASC_F32 = 1 } asc_precision;

enum {
    ASC_RUN_NO_OUTPUT = 1u << 0,   /* do not copy the values out (out may be NULL) */
    ASC_RUN_DEVICE_OUT = 1u << 1,  /* out is a device pointer */
    ASC_RUN_PHASE_TIMING = 1u << 2, /* time static and on-demand kernels separately (CUDA events);
                                       implies a host-driven iteration loop */
    ASC_RUN_HOST_LOOP = 1u << 3,    /* drive iterations from the host (one readback per iteration)
                                       instead of the CUDA-graph loop */
    ASC_RUN_FRAGMENT_COUNTS = 1u << 4, /* BFS/SSSP/CC: add the edges this run reads to per-fragment
                                          counters (4096 edges a fragment; read them with
                                          asc_graph_fragment_counts); implies ASC_RUN_HOST_LOOP */
    ASC_RUN_NO_STAGING = 1u << 6,      /* standard PageRank on a graph with staging buffers: read the
                                          on-demand edges in place (zero-copy) instead of staging */
    ASC_RUN_GATHER_COPY = 1u << 5,     /* BFS/SSSP/CC comparison engine, the reference's (and Subway's)
                                          transfer scheme: every iteration the on-demand frontier list
                                          goes to the host, host threads gather its edges into a
                                          page-locked staging buffer, one copy moves them to the
                                          device and a kernel expands them there (GraphMeta.cuh:469-578,
                                          CalculateOpt.cu:146-178); the static region runs as usual.
                                          Same values; implies ASC_RUN_HOST_LOOP */
    ASC_RUN_PARTITION_COPY = 1u << 7   /* BFS/SSSP/CC comparison engine, the reference's whole-partition
                                          baseline (bfs.cu:6-168, gpu_kernels.cu:302-519): the on-demand
                                          region is cut into partitions of one staging buffer (vertex
                                          boundaries; a list longer than a buffer is an error, as in the
                                          reference), and every iteration each partition holding an
                                          active vertex is copied whole and its active vertices expanded
                                          from the copy; the static region runs as usual. Needs a graph
                                          opened with asc_budget.stage_bytes. Same values; implies
                                          ASC_RUN_HOST_LOOP */
};

typedef struct asc_params {
    uint32_t pr_mode;        /* asc_pr_mode (default ASC_PR_REF) */
    uint32_t precision;      /* asc_precision of the PR ranks and sums (default ASC_F64);
                                ASC_F32 keeps FP64 dangling and residual reductions */
    double damping;          /* ASC_PR_STD (default 0.85) */
    double tolerance;        /* ASC_PR_STD L1 stop (default 1e-9) */
    int32_t max_iterations;  /* 0 = until convergence (PR std default 100) */
    uint32_t flags;          /* ASC_RUN_* */
} asc_params;

typedef struct asc_stats {
    int32_t iterations;
    int32_t status_detail;
    uint64_t frontier_vertices;  /* sum over iterations of processed frontier vertices */
    uint64_t ondemand_vertices;  /* of which on-demand (edges read from host memory) */
    uint64_t edges_processed;    /* sum over iterations of their degrees */
    uint64_t ondemand_edges;     /* of which read from host memory (moved over the host link) */
    uint64_t ondemand_bytes;     /* ondemand_edges x edge bytes */
    uint64_t reached_vertices;   /* BFS/SSSP: value < V + 1 */
    uint64_t reached_edges;      /* BFS/SSSP: sum of out-degrees of reached vertices (TEPS numerator) */
    double ms_total;             /* device time from the first to the last kernel of the run */
    double ms_static;            /* with ASC_RUN_PHASE_TIMING: static-region expansion kernels */
    double ms_ondemand;          /* with ASC_RUN_PHASE_TIMING: on-demand expansion kernels */
    double ms_copyout;           /* result copy to the caller's buffer */
    double residual;             /* PR std: last FP64 L1 residual */
    uint32_t kernel_launches;    /* kernels of this library launched by the run */
    uint32_t staged_chunks;      /* chunk copies into the staging buffers (staged PageRank passes);
                                    ondemand_bytes then counts the bytes those copies moved */
    uint64_t bottom_up_edges;    /* BFS: in-edges read by bottom-up steps (counted in ondemand_edges) */
    double ms_bottom_up;         /* with ASC_RUN_PHASE_TIMING: bottom-up BFS kernels */
    uint64_t bottom_up_vertices; /* BFS: unreached vertices the bottom-up steps examined */
} asc_stats;

/* ---- status and errors -------------------------------------------------- */
const char *asc_status_string(asc_status s);
/* Copies the calling thread's last error message into buf; returns its length. */
size_t asc_last_error(char *buf, size_t n);
const char *asc_version(void);
/* Number of usable CUDA devices (0 when none); never fails. */
int asc_device_count(void);
/* Free and total bytes of the current CUDA device (cudaMemGetInfo). */
asc_status asc_device_memory(uint64_t *free_bytes, uint64_t *total_bytes);
/* Page-locked host memory for result buffers: asc_run copies values into it at
 * the copy engine's full rate instead of through a pageable staging path.
 * Free it with asc_host_free. */
asc_status asc_host_alloc(uint64_t bytes, void **ptr);
asc_status asc_host_free(void *ptr);

/* ---- graphs -------------------------------------------------------------- */
void asc_budget_default(asc_budget *b);
/* Reads a reference-format file into pinned host memory and uploads the static
 * prefix chosen by the budget (replaces GraphMeta::readDataFromFile +
 * initGraphHost + initGraphDevice, GraphMeta.cuh:151-297). */
asc_status asc_graph_open(const char *path, asc_format fmt, const asc_budget *budget, asc_graph **out);
/* Builds a graph from caller arrays (copied): ptr has V+1 entries (ptr[V] = E);
 * edges holds E u32 destinations (edge_bytes 4) or E {dst, weight} pairs
 * (edge_bytes 8); outdeg (V entries) marks a CSC graph for PageRank, else NULL. */
asc_status asc_graph_from_csr(uint64_t V, uint64_t E, const uint64_t *ptr, const void *edges,
                              uint32_t edge_bytes, const uint32_t *outdeg, const asc_budget *budget,
                              asc_graph **out);
asc_status asc_graph_info_get(const asc_graph *g, asc_graph_info *info);
/* Releases every device and pinned buffer of the graph. NULL is ignored. */
asc_status asc_graph_close(asc_graph *g);

/* ---- runs ---------------------------------------------------------------- */
void asc_params_default(asc_params *p);
/* One query: BFS/SSSP from source, CC, or PR. out receives V values: uint32
 * for BFS/SSSP/CC, double (or float with precision ASC_F32) for PR. params
 * and stats may be NULL. */
asc_status asc_run(asc_graph *g, asc_algo algo, uint32_t source, const asc_params *params, void *out,
                   asc_stats *stats);

/* Up to 64 BFS or SSSP sources of one graph in one batch: every edge read
 * serves all sources (64-bit per-vertex source masks). out receives n rows of
 * V uint32 values, row i for sources[i], each identical to asc_run from that
 * source. Duplicate sources are allowed. No reference counterpart (the
 * reference runs one source per bfs_opt / sssp_opt call). */
asc_status asc_run_batch(asc_graph *g, asc_algo algo, const uint32_t *sources, uint32_t n, const asc_params *params,
                         void *out, asc_stats *stats);

/* Reference-shaped entry points (CalculateOpt.cuh:11-14): open the file with the
 * reference's --adviseK budget rule, run, close. out (nullable) receives the
 * values the reference keeps in valueD / valuePrD. */
asc_status asc_bfs_opt(const char *path, uint32_t source, double advise_rate, uint32_t *out,
                       asc_stats *stats);
asc_status asc_cc_opt(const char *path, double advise_rate, uint32_t *out, asc_stats *stats);
asc_status asc_sssp_opt(const char *path, uint32_t source, double advise_rate, uint32_t *out,
                        asc_stats *stats);
asc_status asc_pr_opt(const char *path, double advise_rate, double *out, asc_stats *stats);

/* ---- tuning ------------------------------------------------------------------- */
/* The engine's tunables for one graph: lists longer than huge_degree edges are
 * cut into segment_edges-edge work items; a region whose frontier holds more
 * than 1/dense_div of its vertices is walked in id order through the frontier
 * bitmap (0: never); ctas_per_sm sizes the persistent grids (0: as many as stay
 * resident); delta is the SSSP near-far step. ms is the measured time per run of the chosen setting (-1 when
 * it came from the cache). They apply to single-source runs; 64-source batches
 * keep the defaults. No reference counterpart (its launch shape is fixed
 * at 56 x 1024, GraphMeta.cuh:55-56). */
typedef struct asc_tuning {
    uint32_t huge_degree, segment_edges, dense_div, ctas_per_sm;
    uint32_t delta;  /* SSSP near-far step: relaxed distances at or above the threshold wait in a far
                        set; when the near frontier empties the threshold moves to the smallest far
                        distance + delta (0: plain frontier relaxation) */
    uint32_t bu_div; /* BFS on a CSR graph: an iteration whose frontier holds more than V / bu_div
                        vertices steps bottom-up, every unreached vertex scanning its in-edges for a
                        frontier parent (in-edges built once on the host, read in place; the device
                        holds their V + 1 offsets). Same levels. 0: top-down only. Default 64. */
    double ms;
} asc_tuning;
enum { ASC_TUNE_NO_CACHE = 1u << 0 };
asc_status asc_graph_get_tuning(const asc_graph *g, asc_tuning *t);
asc_status asc_graph_set_tuning(asc_graph *g, const asc_tuning *t);
/* Measures candidate settings on runs of algo (BFS/SSSP from the given
 * sources, CC from all vertices) and keeps the fastest for the graph's later
 * runs. Cached per GPU and graph shape unless ASC_TUNE_NO_CACHE. */
asc_status asc_graph_tune(asc_graph *g, asc_algo algo, const uint32_t *sources, uint32_t n, uint32_t flags,
                          asc_tuning *best);

/* ---- query server ----------------------------------------------------------- */
/* Serves BFS / SSSP / CC / PageRank queries against several resident graphs on
 * one GPU under one device-memory budget. In ASC_SERVE_BATCHED mode BFS and
 * SSSP queries are batched continuously: a query joins the running
 * multi-source batch of its graph as soon as a source slot and memory are
 * free, shares every later iteration with the other sources (one edge read
 * serves all of them), and completes when its own frontier is empty; its
 * values are identical to a solo asc_run. CC and PageRank queries run whole;
 * identical pending ones share one run. ASC_SERVE_FIFO is the plain engine:
 * one query at a time, in arrival order. The server is internally
 * synchronised; graphs stay owned by the caller and must outlive the server.
 * No reference counterpart (the reference answers one query per process). */
typedef struct asc_server asc_server;
enum { ASC_SERVE_BATCHED = 0, ASC_SERVE_FIFO = 1 };

typedef struct asc_server_config {
    uint64_t device_budget_bytes; /* every device allocation of the graphs and queries (0 = no cap) */
    uint32_t max_batch;           /* sources per batch, 1..64 (0 = 64); SSSP batches of at most 16 or
                                     32 sources keep rows of that width (less device memory) */
    uint32_t queue_capacity;      /* queries in flight before ASC_ERR_BUSY (0 = 2^20) */
    uint32_t mode;                /* ASC_SERVE_BATCHED or ASC_SERVE_FIFO */
    uint32_t reserved;
} asc_server_config;

typedef struct asc_query_info {
    int32_t status;       /* asc_status of the query */
    int32_t iterations;   /* iterations of the run that answered it (whole runs) */
    uint32_t batch_size;  /* sources sharing its batch when it finished, or queries sharing its run */
    uint32_t reserved;
    double queue_ms;      /* submit to start */
    double latency_ms;    /* submit to completion */
} asc_query_info;

typedef struct asc_server_stats {
    uint64_t submitted, completed, failed, cancelled;
    uint64_t batch_iterations;
    uint64_t device_bytes;  /* device bytes accounted against the budget */
    double p50_ms, p99_ms, mean_ms, max_ms;  /* completed-query latency (the most recent 2^19..2^20) */
    double queries_per_s;   /* completed / (last completion - first submit) */
    double span_s;
    uint64_t engines_created;   /* batch engines allocated */
    uint64_t engines_freed;     /* batch engines freed (idle, or after a failed launch) */
    uint64_t workspaces_freed;  /* single-query states of idle graphs freed for memory */
    uint64_t memory_waits;      /* whole runs that waited for device memory held by batches */
} asc_server_stats;

void asc_server_config_default(asc_server_config *c);
asc_status asc_server_create(const asc_server_config *cfg, asc_server **out);
/* Registers a graph (before the first query); its static region and offsets
 * count against the budget. */
asc_status asc_server_add_graph(asc_server *s, asc_graph *g, uint32_t *graph_id);
/* Queues a query; out (host memory, V values like asc_run, may be NULL) is
 * written before the query completes. */
asc_status asc_server_submit(asc_server *s, uint32_t graph_id, asc_algo algo, uint32_t source,
                             const asc_params *params, void *out, uint64_t *ticket);
/* Waits for a query (timeout_ms < 0: no limit) and releases its ticket;
 * returns the query's status. */
asc_status asc_server_wait(asc_server *s, uint64_t ticket, int64_t timeout_ms, asc_query_info *info);
/* Cancels a query that has not started (it completes with ASC_ERR_CANCELLED). */
asc_status asc_server_cancel(asc_server *s, uint64_t ticket);
asc_status asc_server_stats_get(asc_server *s, asc_server_stats *out);
/* Finishes running work, cancels queued queries and frees the server's state. */
asc_status asc_server_destroy(asc_server *s);

/* ---- synthetic graphs and files -------------------------------------------- */
enum {
    ASC_RMAT_WEIGHTS = 1u << 0,    /* emit {dst, weight} pairs, weight uniform in [wmin, wmax] */
    ASC_RMAT_SYMMETRIC = 1u << 1,  /* append the reverse of every edge before sorting */
    ASC_RMAT_TRANSPOSE = 1u << 2   /* emit the CSC (in-edge) arrays and the out-degrees */
};
/* Seeded RMAT edge list sorted by source into CSR (self-loops and duplicates
 * kept, each list in generation order; reversed edges follow the originals).
 * Deterministic for a seed on any host and thread count. Sizes: V = 2^scale,
 * E = V * edge_factor (x2 with ASC_RMAT_SYMMETRIC). ptr receives V+1 entries,
 * edges E u32 (or 2E with weights), outdeg V entries (ASC_RMAT_TRANSPOSE only). */
asc_status asc_rmat_csr(uint32_t scale, uint32_t edge_factor, uint64_t seed, double a, double b, double c,
                        uint32_t wmin, uint32_t wmax, uint32_t flags, uint64_t *ptr, void *edges,
                        uint32_t *outdeg);
/* Generates straight into a graph's pinned buffers (no extra host copy). */
asc_status asc_graph_rmat(uint32_t scale, uint32_t edge_factor, uint64_t seed, double a, double b, double c,
                          uint32_t wmin, uint32_t wmax, uint32_t flags, const asc_budget *budget,
                          asc_graph **out);
/* Host-link probe: best pinned host-to-device copy-engine bandwidth and best
 * bandwidth of SM loads from mapped pinned host memory, in GB/s (1e9 B/s),
 * over a buffer of the given size (measurement helper, no reference counterpart). */
asc_status asc_link_probe(uint64_t bytes, int iters, double *dma_h2d_gbs, double *sm_read_gbs);
/* Edges read per fragment of the edge array (fragment f holds edges
 * [4096 f, 4096 f + 4096)), summed over the runs made with
 * ASC_RUN_FRAGMENT_COUNTS since the last reset: the visit counters of the
 * reference's fragment swap (gpu_kernels.cu:666-739), kept as a measurement of
 * where reads fall. out receives min(n, ceil(E / 4096)) entries; *n_out (if not
 * NULL) the number of fragments. reset != 0 clears the counters afterwards. */
asc_status asc_graph_fragment_counts(asc_graph *g, uint64_t *out, uint64_t n, uint64_t *n_out, int reset);

/* Host-link read rate (GB/s of requested bytes, best of iters) when every warp
 * reads runs of run_bytes consecutive bytes at pseudo-random 4-byte-aligned
 * offsets of a pinned, mapped buffer of `bytes`: the ceiling the on-demand
 * expansion can reach for a given adjacency-list run length (short runs use
 * 32-byte sectors and link requests partly). No reference counterpart. */
asc_status asc_link_probe_runs(uint64_t bytes, uint32_t run_bytes, int iters, double *gbs);

/* ---- allocation-free BFS ------------------------------------------------- */
/* BFS over a CSR graph that the caller already holds in device memory, for
 * callers that cannot allocate device memory when they run a query: a process
 * whose device memory belongs to another allocator (for example a framework's
 * caching pool that reserved the whole GPU, where a cudaMalloc of our own would
 * fail or fragment that pool), or a latency-bound loop where cudaMalloc and
 * cudaFree, which may synchronize the device, are not allowed.
 * No counterpart in the reference (whose drivers always allocate, GraphMeta.cuh:237-297).
 *
 * Inputs: d_row_offsets (V+1 u32, device), d_col (E u32, device); output:
 * d_levels (V u32, device) in the reference encoding (level + 1, unreached V + 1).
 * stream is a cudaStream_t (NULL = the default stream); the call returns after
 * the BFS has finished on it.
 * Limits: V <= 1,048,576 and E <= 16,777,216; larger graphs return
 * ASC_ERR_BUDGET. The CSR is checked on the device first (ASC_ERR_INVALID).
 * Scratch: one fixed device array of about 9.6 MB in this library, held by
 * every GPU that loads it until the process exits; no cudaMalloc, cudaFree or
 * allocating library routine is called. The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress) with that device current, so
 * make that first call before any stream capture. The address is kept for the
 * life of the process, so it assumes the device's primary context does too:
 * after a cudaDeviceReset, or from a context other than the primary one, the
 * kept address is stale and the entry point must not be called. The array is
 * committed on a device when this library's device code is loaded there (with
 * lazy module loading, at the first call into the library that uses that
 * device): a caller whose own allocator will later reserve the rest of the
 * device makes one warm-up call before it does. All calls share the array
 * (counters are cleared at the start of each call): calls that overlap on the
 * GPU, on any stream or thread, race and must not be issued. */
asc_status asc_bfs_device_noalloc(uint64_t V, uint64_t E, const uint32_t *d_row_offsets, const uint32_t *d_col,
                                  uint32_t source, uint32_t *d_levels, void *stream);

/* Writes a graph file in a reference format from CSR arrays (ptr has V+1 entries). */
asc_status asc_write_graph(const char *path, asc_format fmt, uint64_t V, uint64_t E, const uint64_t *ptr,
                           const void *edges, const uint32_t *outdeg);

#ifdef __cplusplus
}
#endif
#endif
