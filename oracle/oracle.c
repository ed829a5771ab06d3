/*
 * CPU oracle for the out-of-GPU-memory iteration engine (TEST INFRASTRUCTURE).
 *
 * This file restates, in plain C, what the reference engine (Ascetic, `ptgraph`)
 * computes on its hot path, so that the CUDA engine can be checked against it.
 * Only tests, the smoke check and the CPU-baseline legs of the benchmark load it;
 * the product library never links or calls it.
 *
 * Parity pin: the restatement is checked against golden vectors produced by
 * running the reference's own kernel and host code (gpu_kernels.cuh,
 * GraphMeta.cuh) compiled for the CPU (see oracle/refemu/ and
 * tests/golden/make_golden.py), bit-exact for BFS/SSSP/CC and reference-PR.
 *
 * Graph layout used by every function: V vertices, row offsets ptr[0..V] with
 * ptr[V] = E (the file format stores V offsets; the sentinel reproduces the
 * reference's degree rule deg[V-1] = E - ptr[V-1], GraphMeta.cuh:216-226).
 * Unweighted edges are u32 destinations; weighted edges are AoS pairs
 * {u32 dst, u32 weight} (globals.cuh:10-13).
 *
 * Value encoding follows the reference (GraphMeta.cuh:374-467):
 *   BFS  value = level + 1, source = 1, unreached = V + 1
 *   SSSP value = dist + 1,  source = 1, unreached = V + 1
 *   CC   value = min vertex id that reaches the vertex (itself included)
 *   PR   double ranks
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>

#define ORC_OK 0
#define ORC_ERR_ARG 1
#define ORC_ERR_MEM 2

/* ------------------------------------------------------------------------ */
/* BFS: gpu_kernels.cuh:376-396 (bfs_kernelStatic) and :345-373 (dynamic part)
 * relax val[v] = min(val[v], val[u] + 1) from every active u until no value
 * changes. The unique fixpoint is the BFS level + 1, which a FIFO queue BFS
 * computes directly. */
int orc_bfs(uint64_t V, const uint64_t *ptr, const uint32_t *col, uint32_t src, uint32_t *out)
{
    if (V == 0) return ORC_OK;
    if (src >= V) return ORC_ERR_ARG;
    uint32_t inf = (uint32_t)(V + 1);
    for (uint64_t i = 0; i < V; i++) out[i] = inf;
    uint32_t *q = (uint32_t *)malloc(sizeof(uint32_t) * V);
    if (!q) return ORC_ERR_MEM;
    uint64_t head = 0, tail = 0;
    out[src] = 1;
    q[tail++] = src;
    while (head < tail) {
        uint32_t u = q[head++];
        uint32_t nv = out[u] + 1;
        for (uint64_t k = ptr[u]; k < ptr[u + 1]; k++) {
            uint32_t v = col[k];
            if (nv < out[v]) { out[v] = nv; q[tail++] = v; }
        }
    }
    free(q);
    return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* SSSP: gpu_kernels.cuh:483-532 relax val[v] = min(val[v], val[u] + w) with
 * u32 arithmetic, source value 1, every other value V + 1 (GraphMeta.cuh:440-447).
 * A vertex is only ever activated when its value drops below V + 1, so the
 * fixpoint is min(V + 1, dist + 1). Restated as binary-heap Dijkstra. The caller
 * guarantees V + 1 + max weight < 2^32 (no u32 wrap). */
typedef struct { uint32_t key; uint32_t v; } heap_item;

static void heap_push(heap_item *h, uint64_t *n, heap_item it)
{
    uint64_t i = (*n)++;
    while (i > 0) {
        uint64_t p = (i - 1) >> 1;
        if (h[p].key <= it.key) break;
        h[i] = h[p];
        i = p;
    }
    h[i] = it;
}

static heap_item heap_pop(heap_item *h, uint64_t *n)
{
    heap_item top = h[0];
    heap_item last = h[--(*n)];
    uint64_t i = 0, m = *n;
    for (;;) {
        uint64_t l = 2 * i + 1;
        if (l >= m) break;
        uint64_t c = (l + 1 < m && h[l + 1].key < h[l].key) ? l + 1 : l;
        if (h[c].key >= last.key) break;
        h[i] = h[c];
        i = c;
    }
    if (m > 0) h[i] = last;
    return top;
}

int orc_sssp(uint64_t V, const uint64_t *ptr, const uint32_t *adj, uint32_t src, uint32_t *out)
{
    if (V == 0) return ORC_OK;
    if (src >= V) return ORC_ERR_ARG;
    uint32_t inf = (uint32_t)(V + 1);
    for (uint64_t i = 0; i < V; i++) out[i] = inf;
    uint64_t E = ptr[V];
    /* lazy-deletion heap: at most one push per successful relaxation */
    heap_item *h = (heap_item *)malloc(sizeof(heap_item) * (E + 1));
    if (!h) return ORC_ERR_MEM;
    uint64_t n = 0;
    out[src] = 1;
    heap_item s = { 1, src };
    heap_push(h, &n, s);
    while (n > 0) {
        heap_item it = heap_pop(h, &n);
        if (it.key != out[it.v]) continue;
        uint32_t u = it.v;
        for (uint64_t k = ptr[u]; k < ptr[u + 1]; k++) {
            uint32_t v = adj[2 * k], w = adj[2 * k + 1];
            uint32_t nv = it.key + w;
            if (nv < out[v]) {
                out[v] = nv;
                heap_item x = { nv, v };
                heap_push(h, &n, x);
            }
        }
    }
    free(h);
    return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* CC: gpu_kernels.cuh:441-481 push val[u] along out-edges with atomicMin from
 * val[i] = i, all active (GraphMeta.cuh:448-452). The fixpoint gives each vertex
 * the smallest id among the vertices that reach it (itself included); on a
 * symmetric graph that is the minimum id of its connected component.
 * Restated as: visit sources in increasing id order and label every still
 * unlabelled vertex they reach. A labelled vertex stops the walk because all it
 * reaches was already labelled by a smaller id. */
int orc_cc(uint64_t V, const uint64_t *ptr, const uint32_t *col, uint32_t *out)
{
    if (V == 0) return ORC_OK;
    const uint32_t UNSET = 0xffffffffu;
    for (uint64_t i = 0; i < V; i++) out[i] = UNSET;
    uint32_t *stack = (uint32_t *)malloc(sizeof(uint32_t) * V);
    if (!stack) return ORC_ERR_MEM;
    for (uint64_t r = 0; r < V; r++) {
        if (out[r] != UNSET) continue;
        uint64_t sp = 0;
        out[r] = (uint32_t)r;
        stack[sp++] = (uint32_t)r;
        while (sp > 0) {
            uint32_t u = stack[--sp];
            for (uint64_t k = ptr[u]; k < ptr[u + 1]; k++) {
                uint32_t v = col[k];
                if (out[v] == UNSET) { out[v] = (uint32_t)r; stack[sp++] = v; }
            }
        }
    }
    free(stack);
    return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* Reference PageRank (pr_opt, CalculateOpt.cu:547-721):
 *   rank[i] = 1/V, every vertex active              (GraphMeta.cuh:415-419)
 *   repeat while any vertex is active:
 *     for active v: sum[v] = sum over in-edges (CSC order) of
 *                   rank[u] / outDeg[u]              (gpu_kernels.cuh:554-594)
 *     for active v: t = 0.15 + 0.85 * sum[v]; if |t - rank[v]| > 0.001 then
 *                   rank[v] = t (stays active) else deactivate for good
 *                                                    (gpu_kernels.cuh:533-552)
 * The sums read the ranks of the previous pass (the apply kernel runs after
 * every sum kernel), so this is a Jacobi iteration. nvcc contracts
 * 0.15 + 0.85 * s into one fused multiply-add, which fma() reproduces exactly.
 * ptr/col are the CSC (in-edge) arrays of a .bcsc file. */
int orc_pr_ref(uint64_t V, const uint64_t *ptr, const uint32_t *col, const uint32_t *outdeg,
               double *rank, int32_t *iters_out)
{
    if (V == 0) { if (iters_out) *iters_out = 0; return ORC_OK; }
    double *sum = (double *)calloc(V, sizeof(double));
    uint8_t *active = (uint8_t *)malloc(V);
    uint32_t *list = (uint32_t *)malloc(sizeof(uint32_t) * V);
    if (!sum || !active || !list) { free(sum); free(active); free(list); return ORC_ERR_MEM; }
    for (uint64_t i = 0; i < V; i++) { rank[i] = 1.0 / (double)V; active[i] = 1; }
    uint64_t nact = V;
    int32_t iters = 0;
    while (nact > 0) {
        iters++;
        uint64_t n = 0;
        for (uint64_t v = 0; v < V; v++) if (active[v]) list[n++] = (uint32_t)v;
        for (uint64_t i = 0; i < n; i++) {
            uint32_t v = list[i];
            double s = 0;
            for (uint64_t k = ptr[v]; k < ptr[v + 1]; k++) {
                uint32_t u = col[k];
                s += rank[u] / (double)outdeg[u];
            }
            sum[v] = s;
        }
        nact = 0;
        for (uint64_t i = 0; i < n; i++) {
            uint32_t v = list[i];
            double t = fma(0.85, sum[v], 0.15);
            double diff = t > rank[v] ? (t - rank[v]) : (rank[v] - t);
            if (diff > 0.001) { rank[v] = t; nact++; }
            else active[v] = 0;
            sum[v] = 0;
        }
    }
    free(sum); free(active); free(list);
    if (iters_out) *iters_out = iters;
    return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* Standard PageRank (the precision-study semantics): damping d, uniform start
 * 1/V, teleport (1-d)/V, the rank of vertices without out-edges spread
 * uniformly, stop when the L1 change is below tol or after max_iter passes.
 *   r'[v] = (1-d)/V + d * (sum_{u in in(v)} r[u]/outDeg[u] + dangling/V)
 * All FP64, pull over the CSC arrays. */
int orc_pr_std(uint64_t V, const uint64_t *ptr, const uint32_t *col, const uint32_t *outdeg,
               double damping, double tol, int32_t max_iter,
               double *rank, int32_t *iters_out, double *residual_out)
{
    if (V == 0) { if (iters_out) *iters_out = 0; if (residual_out) *residual_out = 0; return ORC_OK; }
    double *nxt = (double *)malloc(sizeof(double) * V);
    double *contrib = (double *)malloc(sizeof(double) * V);
    if (!nxt || !contrib) { free(nxt); free(contrib); return ORC_ERR_MEM; }
    double inv_v = 1.0 / (double)V;
    for (uint64_t i = 0; i < V; i++) rank[i] = inv_v;
    int32_t it = 0;
    double res = 0;
    while (it < max_iter) {
        double dangling = 0;
        for (uint64_t u = 0; u < V; u++) {
            if (outdeg[u] == 0) { dangling += rank[u]; contrib[u] = 0; }
            else contrib[u] = rank[u] / (double)outdeg[u];
        }
        double base = (1.0 - damping) * inv_v + damping * dangling * inv_v;
        res = 0;
        for (uint64_t v = 0; v < V; v++) {
            double s = 0;
            for (uint64_t k = ptr[v]; k < ptr[v + 1]; k++) s += contrib[col[k]];
            double r = base + damping * s;
            res += fabs(r - rank[v]);
            nxt[v] = r;
        }
        memcpy(rank, nxt, sizeof(double) * V);
        it++;
        if (res < tol) break;
    }
    free(nxt); free(contrib);
    if (iters_out) *iters_out = it;
    if (residual_out) *residual_out = res;
    return ORC_OK;
}

/* orc_pr_std on host threads, for graphs where one core takes minutes: each
 * pass computes the contributions (and per-thread dangling partials), then
 * every vertex's sum over its in-edges serially in CSC order exactly as
 * orc_pr_std (and per-thread residual partials). Partials are combined in
 * thread order, so a run is deterministic for a thread count; the dangling
 * mass and residual differ from the serial sums only in rounding order. */
typedef struct {
    int phase;
    uint64_t lo, hi;
    const uint64_t *ptr;
    const uint32_t *col;
    const uint32_t *outdeg;
    const double *rank;
    double *nxt, *contrib;
    double base, damping, part;
} pr_job;

static void *pr_worker(void *arg)
{
    pr_job *j = (pr_job *)arg;
    double acc = 0;
    if (j->phase == 0) {
        for (uint64_t u = j->lo; u < j->hi; u++) {
            if (j->outdeg[u] == 0) { acc += j->rank[u]; j->contrib[u] = 0; }
            else j->contrib[u] = j->rank[u] / (double)j->outdeg[u];
        }
    } else {
        for (uint64_t v = j->lo; v < j->hi; v++) {
            double s = 0;
            for (uint64_t k = j->ptr[v]; k < j->ptr[v + 1]; k++) s += j->contrib[j->col[k]];
            double r = j->base + j->damping * s;
            acc += fabs(r - j->rank[v]);
            j->nxt[v] = r;
        }
    }
    j->part = acc;
    return NULL;
}

int orc_pr_std_mt(uint64_t V, const uint64_t *ptr, const uint32_t *col, const uint32_t *outdeg,
                  double damping, double tol, int32_t max_iter, int nthreads,
                  double *rank, int32_t *iters_out, double *residual_out)
{
    if (nthreads < 1) nthreads = 1;
    if (V == 0) { if (iters_out) *iters_out = 0; if (residual_out) *residual_out = 0; return ORC_OK; }
    double *nxt = (double *)malloc(sizeof(double) * V);
    double *contrib = (double *)malloc(sizeof(double) * V);
    pr_job *jobs = (pr_job *)calloc((size_t)nthreads, sizeof(pr_job));
    pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
    if (!nxt || !contrib || !jobs || !th) { free(nxt); free(contrib); free(jobs); free(th); return ORC_ERR_MEM; }
    double inv_v = 1.0 / (double)V;
    for (uint64_t i = 0; i < V; i++) rank[i] = inv_v;
    for (int t = 0; t < nthreads; t++) {
        jobs[t].lo = V * (uint64_t)t / (uint64_t)nthreads;
        jobs[t].hi = V * (uint64_t)(t + 1) / (uint64_t)nthreads;
        jobs[t].ptr = ptr; jobs[t].col = col; jobs[t].outdeg = outdeg;
        jobs[t].rank = rank; jobs[t].nxt = nxt; jobs[t].contrib = contrib; jobs[t].damping = damping;
    }
    int32_t it = 0;
    double res = 0;
    while (it < max_iter) {
        double sums[2] = {0, 0};
        for (int phase = 0; phase < 2; phase++) {
            double base = (1.0 - damping) * inv_v + damping * sums[0] * inv_v;
            for (int t = 0; t < nthreads; t++) { jobs[t].phase = phase; jobs[t].base = base; }
            for (int t = 1; t < nthreads; t++) pthread_create(&th[t], NULL, pr_worker, &jobs[t]);
            pr_worker(&jobs[0]);
            for (int t = 1; t < nthreads; t++) pthread_join(th[t], NULL);
            for (int t = 0; t < nthreads; t++) sums[phase] += jobs[t].part;
        }
        res = sums[1];
        memcpy(rank, nxt, sizeof(double) * V);
        it++;
        if (res < tol) break;
    }
    free(nxt); free(contrib); free(jobs); free(th);
    if (iters_out) *iters_out = it;
    if (residual_out) *residual_out = res;
    return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* Static/on-demand split (GraphMeta.cuh:341-372): the static region is the
 * prefix edge[0, mps) of the edge array with mps rounded down to a multiple of
 * 4096 edges; vertex v is static when its whole edge list lies inside it. The
 * reference tests ptr[v] < mps && ptr[v] + deg - 1 < mps in u64 arithmetic
 * (a degree-0 vertex at offset 0 wraps and counts as non-static).
 * Outputs the static flags, the number of static edges and the rounded mps. */
int orc_static_split(uint64_t V, const uint64_t *ptr, uint64_t static_edges_cap,
                     uint8_t *is_static, uint64_t *mps_out, uint64_t *edges_in_static_out)
{
    uint64_t E = ptr[V];
    uint64_t mps = static_edges_cap;
    if (mps > E) mps = E;
    if (mps > 0xffffffffull) mps = 0xffffffffull;
    mps -= mps % 4096;
    uint64_t in_static = 0;
    for (uint64_t v = 0; v < V; v++) {
        uint64_t deg = ptr[v + 1] - ptr[v];
        if (ptr[v] < mps && (ptr[v] + deg - 1) < mps) { is_static[v] = 1; in_static += deg; }
        else is_static[v] = 0;
    }
    if (mps_out) *mps_out = mps;
    if (edges_in_static_out) *edges_in_static_out = in_static;
    return ORC_OK;
}

/* Graph500-style TEPS numerator: the sum of out-degrees of the reached
 * vertices (value < unreached). */
uint64_t orc_reached_edges(uint64_t V, const uint64_t *ptr, const uint32_t *val, uint32_t unreached)
{
    uint64_t s = 0;
    for (uint64_t v = 0; v < V; v++) if (val[v] < unreached) s += ptr[v + 1] - ptr[v];
    return s;
}

/* ------------------------------------------------------------------------ */
/* Multi-threaded CPU run of the reference's own iteration scheme (frontier of
 * active vertices, relax with atomic min, mark the improved destinations active
 * for the next pass; gpu_kernels.cuh:376-396, CalculateOpt.cu:60-191) on host
 * threads. Used as the timed CPU arm of the benchmark. mode 0 = BFS (+1),
 * mode 1 = SSSP (+w, adj holds pairs), mode 2 = CC (push own value, all start
 * active). Returns the number of passes in *iters_out. */
typedef struct {
    int mode;
    uint64_t V;
    const uint64_t *ptr;
    const uint32_t *edges;
    _Atomic uint32_t *val;
    _Atomic uint8_t *next_flag;
    const uint32_t *frontier;
    uint64_t nfront;
    _Atomic uint64_t cursor;
    uint32_t **out_lists;
    uint64_t *out_counts;
    int nthreads;
} mt_ctx;

typedef struct { mt_ctx *c; int tid; uint32_t *local; uint64_t cap; } mt_arg;

static void mt_relax_pass(mt_ctx *c, int tid, uint32_t *local, uint64_t *nloc)
{
    const uint64_t GRAIN = 256;
    uint64_t n = 0;
    for (;;) {
        uint64_t b = atomic_fetch_add_explicit(&c->cursor, GRAIN, memory_order_relaxed);
        if (b >= c->nfront) break;
        uint64_t e = b + GRAIN < c->nfront ? b + GRAIN : c->nfront;
        for (uint64_t i = b; i < e; i++) {
            uint32_t u = c->frontier[i];
            uint32_t vu = atomic_load_explicit(&c->val[u], memory_order_relaxed);
            for (uint64_t k = c->ptr[u]; k < c->ptr[u + 1]; k++) {
                uint32_t v, nv;
                if (c->mode == 1) { v = c->edges[2 * k]; nv = vu + c->edges[2 * k + 1]; }
                else { v = c->edges[k]; nv = (c->mode == 0) ? vu + 1 : vu; }
                uint32_t old = atomic_load_explicit(&c->val[v], memory_order_relaxed);
                while (nv < old) {
                    if (atomic_compare_exchange_weak_explicit(&c->val[v], &old, nv,
                                                              memory_order_relaxed, memory_order_relaxed)) {
                        if (atomic_exchange_explicit(&c->next_flag[v], 1, memory_order_relaxed) == 0)
                            local[n++] = v;
                        break;
                    }
                }
            }
        }
    }
    (void)tid;
    *nloc = n;
}

static void *mt_worker(void *p)
{
    mt_arg *a = (mt_arg *)p;
    mt_ctx *c = a->c;
    uint64_t n = 0;
    mt_relax_pass(c, a->tid, a->local, &n);
    c->out_lists[a->tid] = a->local;
    c->out_counts[a->tid] = n;
    return NULL;
}

int orc_relax_mt(int mode, uint64_t V, const uint64_t *ptr, const uint32_t *edges, uint32_t src,
                 int nthreads, uint32_t *out, int32_t *iters_out)
{
    if (V == 0) { if (iters_out) *iters_out = 0; return ORC_OK; }
    if (mode != 2 && src >= V) return ORC_ERR_ARG;
    if (nthreads < 1) nthreads = 1;
    _Atomic uint32_t *val = (_Atomic uint32_t *)out;
    _Atomic uint8_t *flag = (_Atomic uint8_t *)calloc(V, 1);
    uint32_t *front = (uint32_t *)malloc(sizeof(uint32_t) * V);
    uint32_t **locals = (uint32_t **)calloc((size_t)nthreads, sizeof(uint32_t *));
    uint64_t *counts = (uint64_t *)calloc((size_t)nthreads, sizeof(uint64_t));
    uint32_t **lists = (uint32_t **)calloc((size_t)nthreads, sizeof(uint32_t *));
    pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
    mt_arg *args = (mt_arg *)calloc((size_t)nthreads, sizeof(mt_arg));
    int ok = flag && front && locals && counts && lists && th && args;
    for (int t = 0; ok && t < nthreads; t++) {
        /* each vertex enters a thread's list at most once per pass */
        locals[t] = (uint32_t *)malloc(sizeof(uint32_t) * V);
        if (!locals[t]) ok = 0;
    }
    if (!ok) {
        if (locals) for (int t = 0; t < nthreads; t++) free(locals[t]);
        free((void *)flag); free(front); free(locals); free(counts); free(lists); free(th); free(args);
        return ORC_ERR_MEM;
    }
    uint64_t nfront = 0;
    if (mode == 2) {
        for (uint64_t i = 0; i < V; i++) { out[i] = (uint32_t)i; front[nfront++] = (uint32_t)i; }
    } else {
        for (uint64_t i = 0; i < V; i++) out[i] = (uint32_t)(V + 1);
        out[src] = 1;
        front[nfront++] = src;
    }
    mt_ctx c;
    memset(&c, 0, sizeof(c));
    c.mode = mode; c.V = V; c.ptr = ptr; c.edges = edges; c.val = val; c.next_flag = flag;
    c.out_lists = lists; c.out_counts = counts; c.nthreads = nthreads;
    int32_t iters = 0;
    while (nfront > 0) {
        iters++;
        c.frontier = front; c.nfront = nfront;
        atomic_store(&c.cursor, 0);
        for (int t = 0; t < nthreads; t++) {
            args[t].c = &c; args[t].tid = t; args[t].local = locals[t];
            if (t == 0) continue;
            pthread_create(&th[t], NULL, mt_worker, &args[t]);
        }
        mt_worker(&args[0]);
        for (int t = 1; t < nthreads; t++) pthread_join(th[t], NULL);
        nfront = 0;
        for (int t = 0; t < nthreads; t++) {
            for (uint64_t i = 0; i < counts[t]; i++) {
                uint32_t v = lists[t][i];
                front[nfront++] = v;
                atomic_store_explicit(&flag[v], 0, memory_order_relaxed);
            }
        }
    }
    for (int t = 0; t < nthreads; t++) free(locals[t]);
    free((void *)flag); free(front); free(locals); free(counts); free(lists); free(th); free(args);
    if (iters_out) *iters_out = iters;
    return ORC_OK;
}
