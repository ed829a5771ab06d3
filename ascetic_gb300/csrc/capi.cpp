// C-ABI entry points: errors, parameter defaults, run dispatch, and the
// reference-shaped bfs_opt / cc_opt / sssp_opt / pr_opt (CalculateOpt.cuh:11-14).
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include "common.h"

namespace asc {

static thread_local char g_err[1024];

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

asc_status fail(asc_status s, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return s;
}

asc_status cuda_fail(cudaError_t e, const char *what, const char *file, int line) {
    const char *base = strrchr(file, '/');
    set_error("CUDA error %d (%s) in %s at %s:%d", (int)e, cudaGetErrorString(e), what, base ? base + 1 : file,
              line);
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return ASC_ERR_BUDGET;
    }
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return ASC_ERR_NO_DEVICE;
    return ASC_ERR_CUDA;
}

static asc_status check_algo(asc_graph *g, asc_algo algo, uint32_t source) {
    switch (algo) {
        case ASC_BFS:
        case ASC_SSSP:
            if (g->is_csc) return fail(ASC_ERR_UNSUPPORTED, "BFS/SSSP read out-edges; this graph holds in-edges (bcsc)");
            if (algo == ASC_SSSP && g->edge_words != 2 && g->wbits == 0)
                return fail(ASC_ERR_UNSUPPORTED, "SSSP needs a weighted graph ({dst, weight} edges, bwcsr)");
            if (source >= g->V)
                return fail(ASC_ERR_INVALID, "source %u is not a vertex (V = %llu)", source, (unsigned long long)g->V);
            return ASC_OK;
        case ASC_CC:
            if (g->is_csc) return fail(ASC_ERR_UNSUPPORTED, "CC pushes along out-edges; this graph is bcsc");
            return ASC_OK;
        case ASC_PR:  // pull over in-edges (bcsc) or scatter over out-edges (bcsr / bwcsr)
            return ASC_OK;
    }
    return fail(ASC_ERR_INVALID, "unknown algorithm %d", (int)algo);
}

}  // namespace asc

using namespace asc;

extern "C" {

const char *asc_status_string(asc_status s) {
    switch (s) {
        case ASC_OK: return "ok";
        case ASC_ERR_INVALID: return "invalid argument";
        case ASC_ERR_BAD_FILE: return "bad graph file";
        case ASC_ERR_BUDGET: return "device budget exceeded";
        case ASC_ERR_CUDA: return "CUDA error";
        case ASC_ERR_TIMEOUT: return "timeout";
        case ASC_ERR_CANCELLED: return "cancelled";
        case ASC_ERR_UNSUPPORTED: return "unsupported";
        case ASC_ERR_NO_DEVICE: return "no CUDA device";
        case ASC_ERR_NOMEM: return "host out of memory";
        case ASC_ERR_BUSY: return "busy";
    }
    return "unknown status";
}

size_t asc_last_error(char *buf, size_t n) {
    size_t len = strlen(g_err);
    if (buf && n) {
        size_t c = len < n - 1 ? len : n - 1;
        memcpy(buf, g_err, c);
        buf[c] = 0;
    }
    return len;
}

const char *asc_version(void) { return "ascetic-gb300 0.1 (sm_103a)"; }

int asc_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

asc_status asc_host_alloc(uint64_t bytes, void **ptr) {
    if (!ptr) return fail(ASC_ERR_INVALID, "asc_host_alloc: ptr is NULL");
    *ptr = nullptr;
    const cudaError_t e = cudaHostAlloc(ptr, bytes ? bytes : 1, cudaHostAllocPortable);
    if (e != cudaSuccess) {
        *ptr = nullptr;
        cudaGetLastError();
        return fail(ASC_ERR_NOMEM, "cudaHostAlloc of %llu bytes failed: %s", (unsigned long long)bytes,
                    cudaGetErrorString(e));
    }
    return ASC_OK;
}

asc_status asc_host_free(void *ptr) {
    if (ptr) ASC_CUDA(cudaFreeHost(ptr));
    return ASC_OK;
}

asc_status asc_device_memory(uint64_t *free_bytes, uint64_t *total_bytes) {
    size_t f = 0, t = 0;
    ASC_CUDA(cudaMemGetInfo(&f, &t));
    if (free_bytes) *free_bytes = f;
    if (total_bytes) *total_bytes = t;
    return ASC_OK;
}

void asc_params_default(asc_params *p) {
    if (!p) return;
    memset(p, 0, sizeof(*p));
    p->pr_mode = ASC_PR_REF;
    p->precision = ASC_F64;
    p->damping = 0.85;
    p->tolerance = 1e-9;
    p->max_iterations = 0;
    p->flags = 0;
}

asc_status asc_run(asc_graph *g, asc_algo algo, uint32_t source, const asc_params *params, void *out,
                   asc_stats *stats) {
    if (!g) return fail(ASC_ERR_INVALID, "asc_run: graph is NULL");
    asc_params p;
    if (params) p = *params;
    else asc_params_default(&p);
    if (!out && !(p.flags & ASC_RUN_NO_OUTPUT)) return fail(ASC_ERR_INVALID, "asc_run: out is NULL");
    ASC_TRY(check_algo(g, algo, source));
    if (algo == ASC_PR) {
        if (p.pr_mode != ASC_PR_REF && p.pr_mode != ASC_PR_STD) return fail(ASC_ERR_INVALID, "bad pr_mode");
        if (p.pr_mode == ASC_PR_REF && p.precision != ASC_F64)
            return fail(ASC_ERR_UNSUPPORTED, "the reference PageRank runs in FP64 only");
        if (!(p.damping > 0 && p.damping < 1)) return fail(ASC_ERR_INVALID, "damping must be in (0, 1)");
        ASC_TRY(run_pagerank(g, p, out, stats));
        return self_check_result();
    }
    ASC_TRY(run_traversal(g, algo, source, p, out, stats));
    return self_check_result();
}

asc_status asc_run_batch(asc_graph *g, asc_algo algo, const uint32_t *sources, uint32_t n,
                         const asc_params *params, void *out, asc_stats *stats) {
    if (!g || !sources) return fail(ASC_ERR_INVALID, "asc_run_batch: graph and sources are required");
    if (n == 0 || n > 64) return fail(ASC_ERR_INVALID, "asc_run_batch: %u sources, the batch holds 1 to 64", n);
    if (algo != ASC_BFS && algo != ASC_SSSP)
        return fail(ASC_ERR_UNSUPPORTED, "asc_run_batch runs BFS or SSSP sources");
    asc_params p;
    if (params) p = *params;
    else asc_params_default(&p);
    if (!out && !(p.flags & ASC_RUN_NO_OUTPUT)) return fail(ASC_ERR_INVALID, "asc_run_batch: out is NULL");
    for (uint32_t i = 0; i < n; i++) ASC_TRY(check_algo(g, algo, sources[i]));
    return run_batch(g, algo, sources, n, p, out, stats);
}

static asc_status opt_common(const char *path, asc_format fmt, double advise, asc_algo algo, uint32_t source,
                             void *out, asc_stats *stats) {
    asc_budget b;
    asc_budget_default(&b);
    b.mode = ASC_BUDGET_ADVISE_K;
    b.value = advise;
    asc_graph *g = nullptr;
    ASC_TRY(asc_graph_open(path, fmt, &b, &g));
    asc_params p;
    asc_params_default(&p);
    if (!out) p.flags |= ASC_RUN_NO_OUTPUT;
    asc_status s = asc_run(g, algo, source, &p, out, stats);
    asc_graph_close(g);
    return s;
}

asc_status asc_bfs_opt(const char *path, uint32_t source, double advise_rate, uint32_t *out, asc_stats *stats) {
    return opt_common(path, ASC_FMT_AUTO, advise_rate, ASC_BFS, source, out, stats);
}

asc_status asc_cc_opt(const char *path, double advise_rate, uint32_t *out, asc_stats *stats) {
    return opt_common(path, ASC_FMT_AUTO, advise_rate, ASC_CC, 0, out, stats);
}

asc_status asc_sssp_opt(const char *path, uint32_t source, double advise_rate, uint32_t *out, asc_stats *stats) {
    return opt_common(path, ASC_FMT_AUTO, advise_rate, ASC_SSSP, source, out, stats);
}

asc_status asc_pr_opt(const char *path, double advise_rate, double *out, asc_stats *stats) {
    return opt_common(path, ASC_FMT_AUTO, advise_rate, ASC_PR, 0, out, stats);
}

}  // extern "C"
