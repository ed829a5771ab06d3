// Host side of the graph object: reference file formats, validation, pinned
// host copies, the static/on-demand split, the one-time static upload, and the
// seeded RMAT generator.
//
// Reference behaviour followed:
//  - file layouts and reading: GraphMeta.cuh:151-171 (64-bit header and offsets,
//    V offsets without a sentinel), bfs.cu:14-23 (legacy 32-bit layout),
//    converter/converter.cpp:77-420 (writers);
//  - degree rule deg[V-1] = E - ptr[V-1]: GraphMeta.cuh:216-226;
//  - budget and split: GraphMeta.cuh:310-372 (static prefix rounded down to
//    4096-edge fragments, a vertex is static when its whole list is inside);
//  - one-time static upload: GraphMeta.cuh:254-255.
#include <errno.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>

#include <algorithm>
#include <new>
#include <atomic>
#include <thread>

#include "common.h"

namespace asc {

namespace {

constexpr uint64_t kU32Max = 0xffffffffull;

asc_status pinned_alloc(void **p, size_t bytes) {
    *p = nullptr;
    cudaError_t e = cudaHostAlloc(p, bytes ? bytes : 16, cudaHostAllocMapped | cudaHostAllocPortable);
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return fail(ASC_ERR_NOMEM, "cudaHostAlloc of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
    }
    return ASC_OK;
}

asc_status ensure_device(int *dev) {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        return fail(ASC_ERR_NO_DEVICE, "no CUDA device available (%s)",
                    e == cudaSuccess ? "count is 0" : cudaGetErrorString(e));
    }
    ASC_CUDA(cudaGetDevice(dev));
    return ASC_OK;
}

unsigned host_threads(uint64_t work) {
    unsigned hw = std::thread::hardware_concurrency();
    if (hw == 0) hw = 4;
    hw = std::min(hw, 64u);
    uint64_t by_work = work / (1u << 20) + 1;
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(hw, by_work));
}

template <class F> void parallel_for(uint64_t n, unsigned threads, F f) {
    if (threads <= 1 || n < 2) {
        f(0, 0, n);
        return;
    }
    std::vector<std::thread> th;
    uint64_t chunk = (n + threads - 1) / threads;
    for (unsigned t = 0; t < threads; t++) {
        uint64_t b = std::min(n, t * chunk), e = std::min(n, b + chunk);
        th.emplace_back([=] { f(t, b, e); });
    }
    for (auto &x : th) x.join();
}

// Scans the graph once: offsets must not decrease, destinations must be < V
// (a destination out of range would make the kernels write outside the value
// array), and it records the largest degree and weight.
asc_status validate_and_measure(asc_graph *g) {
    const uint64_t V = g->V, E = g->E;
    const uint32_t *p = g->h_ptr;
    for (uint64_t v = 0; v < V; v++)
        if (p[v] > p[v + 1])
            return fail(ASC_ERR_BAD_FILE, "row offsets decrease at vertex %llu (%u > %u)",
                        (unsigned long long)v, p[v], p[v + 1]);
    uint32_t maxdeg = 0;
    for (uint64_t v = 0; v < V; v++) maxdeg = std::max(maxdeg, p[v + 1] - p[v]);
    g->max_degree = maxdeg;
    unsigned T = host_threads(E);
    std::vector<uint64_t> bad(T, ~0ull);
    std::vector<uint32_t> maxw(T, 0);
    const uint32_t words = g->edge_words;
    const uint32_t *ed = g->h_edges;
    parallel_for(E, T, [&](unsigned t, uint64_t b, uint64_t e) {
        uint32_t mw = 0;
        for (uint64_t i = b; i < e; i++) {
            if (ed[i * words] >= V) {
                bad[t] = i;
                return;
            }
            if (words == 2) mw = std::max(mw, ed[i * 2 + 1]);
        }
        maxw[t] = mw;
    });
    for (unsigned t = 0; t < T; t++)
        if (bad[t] != ~0ull)
            return fail(ASC_ERR_BAD_FILE, "edge %llu points to vertex %u >= V = %llu", (unsigned long long)bad[t],
                        ed[bad[t] * words], (unsigned long long)V);
    g->max_weight = 0;
    for (unsigned t = 0; t < T; t++) g->max_weight = std::max(g->max_weight, maxw[t]);
    if (g->edge_words == 2 && (uint64_t)V + 1 + g->max_weight > kU32Max)
        return fail(ASC_ERR_UNSUPPORTED, "weights up to %u could wrap the u32 distance (V + 1 + w >= 2^32)",
                    g->max_weight);
    if (g->is_csc) {
        // an in-edge from u means u has an out-edge, so outDeg[u] > 0 for every
        // source that appears; the reference divides by it (gpu_kernels.cuh:554-594)
        for (uint64_t i = 0; i < E; i++)
            if (g->h_outdeg[ed[i]] == 0)
                return fail(ASC_ERR_BAD_FILE, "in-edge %llu comes from vertex %u whose out-degree is 0",
                            (unsigned long long)i, ed[i]);
    }
    return ASC_OK;
}

asc_status alloc_host_arrays(asc_graph *g) {
    ASC_TRY(pinned_alloc((void **)&g->h_ptr, sizeof(uint32_t) * (g->V + 1)));
    ASC_TRY(pinned_alloc((void **)&g->h_edges, sizeof(uint32_t) * g->edge_words * g->E));
    if (g->is_csc) ASC_TRY(pinned_alloc((void **)&g->h_outdeg, sizeof(uint32_t) * (g->V ? g->V : 1)));
    void *dp = nullptr;
    ASC_CUDA(cudaHostGetDevicePointer(&dp, g->h_edges, 0));
    g->d_host_edges = (const uint32_t *)dp;
    return ASC_OK;
}

asc_status check_sizes(uint64_t V, uint64_t E) {
    if (V == 0) return fail(ASC_ERR_INVALID, "graph has no vertices");
    if (V >= kU32Max - 1) return fail(ASC_ERR_UNSUPPORTED, "V = %llu needs 64-bit vertex ids", (unsigned long long)V);
    if (E > kU32Max) return fail(ASC_ERR_UNSUPPORTED, "E = %llu needs 64-bit row offsets", (unsigned long long)E);
    return ASC_OK;
}

bool read_exact(FILE *f, void *dst, uint64_t bytes) {
    char *d = (char *)dst;
    while (bytes > 0) {
        size_t chunk = (size_t)std::min<uint64_t>(bytes, 1ull << 28);
        size_t got = fread(d, 1, chunk, f);
        if (got != chunk) return false;
        d += got;
        bytes -= got;
    }
    return true;
}

const char *ext_of(const char *path) {
    const char *dot = strrchr(path, '.');
    return dot ? dot + 1 : "";
}

// Chooses the layout from the header and the file size (and the extension when
// two layouts fit the same size).
asc_status detect_format(const char *path, uint64_t size, const uint8_t *hdr, asc_format *fmt) {
    uint64_t V = 0, E = 0;
    memcpy(&V, hdr, 8);
    memcpy(&E, hdr + 8, 8);
    uint32_t V32 = 0, E32 = 0;
    memcpy(&V32, hdr, 4);
    memcpy(&E32, hdr + 4, 4);
    std::vector<asc_format> fit;
    if (size >= 16 && V < (1ull << 40) && E < (1ull << 40)) {
        if (size == 16 + 8 * V + 4 * E) fit.push_back(ASC_FMT_BCSR);
        if (size == 16 + 8 * V + 8 * E) fit.push_back(ASC_FMT_BWCSR);
        if (size == 16 + 12 * V + 4 * E) fit.push_back(ASC_FMT_BCSC);
    }
    if (size >= 8 && size == 8 + 4ull * V32 + 4ull * E32) fit.push_back(ASC_FMT_BCSR32);
    if (fit.empty())
        return fail(ASC_ERR_BAD_FILE, "%s: size %llu matches no graph layout (header V=%llu E=%llu)", path,
                    (unsigned long long)size, (unsigned long long)V, (unsigned long long)E);
    if (fit.size() == 1) {
        *fmt = fit[0];
        return ASC_OK;
    }
    const char *ext = ext_of(path);
    struct { const char *e; asc_format f; } hints[] = {
        {"bcsr", ASC_FMT_BCSR}, {"bwcsr", ASC_FMT_BWCSR}, {"bcsc", ASC_FMT_BCSC}, {"bcsr32", ASC_FMT_BCSR32}};
    for (auto &h : hints)
        if (strcmp(ext, h.e) == 0 && std::find(fit.begin(), fit.end(), h.f) != fit.end()) {
            *fmt = h.f;
            return ASC_OK;
        }
    return fail(ASC_ERR_BAD_FILE, "%s: layout is ambiguous from the size alone; pass the format", path);
}

}  // namespace

asc_status compute_static_split(asc_graph *g, const asc_budget *b, uint32_t param_size) {
    asc_budget def;
    asc_budget_default(&def);
    if (!b) b = &def;
    const uint64_t E = g->E, V = g->V;
    // device bytes per edge (a bit stream of ebits per edge when narrower than 32)
    const double eb = g->edge_words == 2 ? 8.0 : g->ebits / 8.0;
    const double fb = g->file_edge_bytes ? (double)g->file_edge_bytes : eb;  // budget unit
    uint64_t frag = b->fragment_edges ? b->fragment_edges : 4096;
    uint64_t st = E;
    // A CSR graph keeps the first in-edge of every vertex in HBM for bottom-up
    // BFS steps (a bit stream of bits(V - 1) per vertex), and a budget may hold
    // staging buffers; both come out of a byte budget, the static prefix gets
    // the rest. An EDGES cap is the prefix alone. Neither is kept when every
    // edge fits.
    uint32_t in_bits = 1;
    while (in_bits < 32 && (1ull << in_bits) < V) in_bits++;
    const char *pack_env = getenv("ASC_EDGE_PACKING");
    if (in_bits > 30 || (pack_env && pack_env[0] == '0')) in_bits = 32;
    g->in_ebits = in_bits;
    const uint64_t head_words = g->is_csc || !V ? 0 : (in_bits == 32 ? V : (V * in_bits + 31) / 32 + 1);
    double heads = 4.0 * (double)head_words;
    double stage = (double)b->stage_bytes;
    auto prefix_of = [&](double budget_bytes) -> uint64_t {
        if (budget_bytes / eb >= (double)E) {
            stage = heads = 0;  // every edge fits
            return E;
        }
        double rest = budget_bytes;
        if (stage > rest) stage = rest;  // asked for: the staging buffers first
        rest -= stage;
        if (heads > rest) heads = 0;  // a budget too small for the heads keeps none
        rest -= heads;
        return (uint64_t)(rest / eb);
    };
    // every capped mode ends in the reference's rule (GraphMeta.cuh:341-353):
    // the cap in edges, at most E and 2^32 - 1, rounded down to whole fragments
    bool round_down = true;
    switch (b->mode) {
        case ASC_BUDGET_ALL:
            st = E;
            round_down = false;
            stage = heads = 0;
            break;
        case ASC_BUDGET_FRAC:
            if (!(b->value >= 0)) return fail(ASC_ERR_INVALID, "budget fraction %g is negative", b->value);
            // the fraction of the source edge-array bytes, spent on device-format edges
            if (b->value * fb >= eb) st = E;
            else st = prefix_of(b->value * (double)E * fb);
            break;
        case ASC_BUDGET_BYTES:
            if (!(b->value >= 0)) return fail(ASC_ERR_INVALID, "budget bytes %g is negative", b->value);
            st = prefix_of(b->value);
            break;
        case ASC_BUDGET_ADVISE_K: {
            // GraphMeta.cuh:318-354, in 64-bit arithmetic (the reference keeps
            // total_gpu_size in a u32, which wraps on devices with > 16 GiB free)
            size_t freeb = 0, totalb = 0;
            ASC_CUDA(cudaMemGetInfo(&freeb, &totalb));
            uint64_t reduce = (uint64_t)param_size * 4ull * V;
            uint64_t total_edges = freeb > reduce ? (uint64_t)((double)(freeb - reduce) / eb) : 0;
            double k;
            if (b->value > 0) k = b->value;
            else {
                k = total_edges ? (10.0 - (double)E / (double)total_edges) / 9.0 : 0.5;
                if (k < 0) k = 0.5;
                if (k > 1) k = 1.0;
            }
            st = (uint64_t)((float)k * (double)total_edges);
            if (st < E) st = prefix_of((double)st * eb);
            break;
        }
        case ASC_BUDGET_EDGES:
            if (!(b->value >= 0)) return fail(ASC_ERR_INVALID, "budget edges %g is negative", b->value);
            st = b->value >= (double)E ? E : (uint64_t)b->value;
            break;
        case ASC_BUDGET_MANAGED:
            st = 0;
            round_down = false;
            stage = heads = 0;
            break;
        default:
            return fail(ASC_ERR_INVALID, "unknown budget mode %u", b->mode);
    }
    if (round_down) {
        if (st > E) st = E;
        if (st > kU32Max) st = kU32Max;
        st -= st % frag;
    }
    g->static_edges = st;
    // two staging buffers of half the reserve each, 16-byte multiples, when
    // edges remain on demand; none when the budget leaves less than 8 KiB
    g->stage_words = 0;
    if (stage >= 8192 && st < E && b->mode != ASC_BUDGET_ALL && b->mode != ASC_BUDGET_MANAGED)
        g->stage_words = ((uint64_t)stage / 2) / 16 * 4;
    g->in_head_words = heads > 0 && st < E ? head_words : 0;
    // S = number of leading vertices whose whole list lies in [0, st); offsets
    // never decrease, so the static vertices are a prefix of the ids.
    uint64_t lo = 0, hi = V;  // find the first v with ptr[v+1] > st
    while (lo < hi) {
        uint64_t mid = (lo + hi) / 2;
        if (g->h_ptr[mid + 1] <= st) lo = mid + 1;
        else hi = mid;
    }
    g->static_vertices = (uint32_t)lo;
    return ASC_OK;
}

// Uploads offsets, out-degrees and the static prefix (GraphMeta.cuh:254-264).
static asc_status upload(asc_graph *g) {
    ASC_CUDA(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
    ASC_CUDA(cudaMalloc(&g->d_ptr, sizeof(uint32_t) * (g->V + 1)));
    ASC_CUDA(cudaMemcpy(g->d_ptr, g->h_ptr, sizeof(uint32_t) * (g->V + 1), cudaMemcpyHostToDevice));
    g->device_vertex_bytes = sizeof(uint32_t) * (g->V + 1);
    uint64_t sb = g->static_edges ? 4ull * edge_store_words(g, g->static_edges) : 0;
    ASC_CUDA(cudaMalloc(&g->d_static, sb ? sb : 16));
    if (sb) ASC_CUDA(cudaMemcpy(g->d_static, g->h_edges, sb, cudaMemcpyHostToDevice));
    for (int i = 0; i < 2 && g->stage_words; i++) ASC_CUDA(cudaMalloc(&g->d_stage[i], 4 * g->stage_words));
    if (g->in_head_words) {  // filled on the graph's first BFS, with the in-edges
        ASC_CUDA(cudaMalloc(&g->d_in_heads, 4 * g->in_head_words));
        g->in_heads_ready = false;
    }
    if (g->is_csc) {
        ASC_CUDA(cudaMalloc(&g->d_outdeg, sizeof(uint32_t) * g->V));
        ASC_CUDA(cudaMemcpy(g->d_outdeg, g->h_outdeg, sizeof(uint32_t) * g->V, cudaMemcpyHostToDevice));
        g->device_vertex_bytes += sizeof(uint32_t) * g->V;
    }
    return ASC_OK;
}

// Weighted edges are packed into one u32, (dst << wbits) | weight, wbits the
// bits of the largest weight, when destination and weight bits fit in 32:
// half the bytes per edge over the host link and twice the edges in the same
// static-region bytes; values are unchanged. The AoS host copy is released.
static asc_status pack_weighted(asc_graph *g) {
    if (g->edge_words != 2) return ASC_OK;
    uint32_t vbits = 1;
    while (vbits < 32 && (1ull << vbits) < g->V) vbits++;
    uint32_t wbits = 1;  // as few as the largest weight needs: the high bits stay free for a bit stream
    while (wbits < 32 && (1ull << wbits) <= (uint64_t)g->max_weight) wbits++;
    if (vbits + wbits > 32) return ASC_OK;
    uint32_t *packed = nullptr;
    ASC_TRY(pinned_alloc((void **)&packed, sizeof(uint32_t) * (g->E ? g->E : 1)));
    const uint32_t *aos = g->h_edges;
    parallel_for(g->E, host_threads(g->E), [&](unsigned, uint64_t b, uint64_t e) {
        for (uint64_t i = b; i < e; i++) packed[i] = (aos[2 * i] << wbits) | aos[2 * i + 1];
    });
    cudaFreeHost(g->h_edges);
    g->h_edges = packed;
    void *dp = nullptr;
    ASC_CUDA(cudaHostGetDevicePointer(&dp, g->h_edges, 0));
    g->d_host_edges = (const uint32_t *)dp;
    g->edge_words = 1;
    g->wbits = wbits;
    return ASC_OK;
}

// ASC_BUDGET_MANAGED: the kernels read the edges through a managed copy
// advised read-mostly, so the driver moves (duplicates) pages to the GPU on
// first touch, as the reference's UVM baseline does (bfs.cu:263-268).
static asc_status make_managed(asc_graph *g) {
    const size_t bytes = sizeof(uint32_t) * (g->E ? edge_store_words(g, g->E) : 1);
    ASC_CUDA(cudaMallocManaged(&g->managed_edges, bytes));
    if (g->E) memcpy(g->managed_edges, g->h_edges, bytes);
    cudaMemLocation loc;
    loc.type = cudaMemLocationTypeDevice;
    loc.id = g->device;
    ASC_CUDA(cudaMemAdvise(g->managed_edges, bytes, cudaMemAdviseSetReadMostly, loc));
    g->d_host_edges = g->managed_edges;
    return ASC_OK;
}

// Edge words that need fewer than 32 bits (the largest destination, or the
// largest packed destination/weight word, below 2^ebits) are stored as a bit
// stream of ebits per edge, edge i at bits [i*ebits, (i+1)*ebits): the static
// region then holds 32/ebits times the edges per byte and the on-demand edges
// cross the host link in ebits/32 of the bytes; values are unchanged. Kept at
// 32 bits when it would save under 2 bits per edge, for two-word edges, and
// when the environment sets ASC_EDGE_PACKING=0.
static asc_status narrow_edges(asc_graph *g) {
    if (g->edge_words != 1 || !g->E) return ASC_OK;
    const char *env = getenv("ASC_EDGE_PACKING");
    if (env && env[0] == '0') return ASC_OK;
    const uint32_t *src = g->h_edges;
    const unsigned nt = host_threads(g->E);
    std::vector<uint32_t> part(nt, 0);
    parallel_for(g->E, nt, [&](unsigned t, uint64_t b, uint64_t e) {
        uint32_t m = 0;
        for (uint64_t i = b; i < e; i++) m = std::max(m, src[i]);
        part[t] = m;
    });
    uint32_t maxw = 0;
    for (uint32_t m : part) maxw = std::max(maxw, m);
    uint32_t bits = 1;
    while (bits < 32 && (1ull << bits) <= maxw) bits++;
    if (bits > 30) return ASC_OK;
    g->ebits = bits;
    const uint64_t words = edge_store_words(g, g->E);
    uint32_t *packed = nullptr;
    ASC_TRY(pinned_alloc((void **)&packed, sizeof(uint32_t) * words));
    // 32 consecutive edges fill exactly `bits` words, so 32-edge groups pack independently
    const uint64_t groups = (g->E + 31) / 32;
    parallel_for(groups, host_threads(groups * 32), [&](unsigned, uint64_t b, uint64_t e) {
        for (uint64_t grp = b; grp < e; grp++) {
            uint32_t *out = packed + grp * bits;
            // a last, partial group ends inside the buffer's final words
            for (uint32_t k = 0; k < bits && grp * bits + k < words; k++) out[k] = 0;
            const uint64_t i0 = grp * 32, n = std::min<uint64_t>(32, g->E - i0);
            for (uint32_t j = 0; j < n; j++) {
                const uint32_t v = src[i0 + j], pos = j * bits, w = pos >> 5, sh = pos & 31;
                out[w] |= v << sh;
                if (sh + bits > 32) out[w + 1] |= v >> (32 - sh);
            }
        }
    });
    packed[words - 1] = 0;
    cudaFreeHost(g->h_edges);
    g->h_edges = packed;
    void *dp = nullptr;
    ASC_CUDA(cudaHostGetDevicePointer(&dp, g->h_edges, 0));
    g->d_host_edges = (const uint32_t *)dp;
    return ASC_OK;
}

// n words of src (each < 2^bits) as a bit stream of `bits` per word in new
// pinned, mapped memory (one padding word at the end).
static asc_status pack_stream(const uint32_t *src, uint64_t n, uint32_t bits, uint32_t **out) {
    const uint64_t words = bits == 32 ? (n ? n : 1) : (n * bits + 31) / 32 + 1;
    uint32_t *packed = nullptr;
    ASC_TRY(pinned_alloc((void **)&packed, sizeof(uint32_t) * words));
    if (bits == 32) {
        parallel_for(n, host_threads(n), [&](unsigned, uint64_t b, uint64_t e) {
            memcpy(packed + b, src + b, sizeof(uint32_t) * (e - b));
        });
        *out = packed;
        return ASC_OK;
    }
    const uint64_t groups = (n + 31) / 32;  // 32 words fill exactly `bits` stream words
    parallel_for(groups, host_threads(groups * 32), [&](unsigned, uint64_t b, uint64_t e) {
        for (uint64_t grp = b; grp < e; grp++) {
            uint32_t *o = packed + grp * bits;
            // a last, partial group ends inside the buffer's final words
            for (uint32_t k = 0; k < bits && grp * bits + k < words; k++) o[k] = 0;
            const uint64_t i0 = grp * 32, m = std::min<uint64_t>(32, n - i0);
            for (uint32_t j = 0; j < m; j++) {
                const uint32_t v = src[i0 + j], pos = j * bits, w = pos >> 5, sh = pos & 31;
                o[w] |= v << sh;
                if (sh + bits > 32) o[w + 1] |= v >> (32 - sh);
            }
        }
    });
    packed[words - 1] = 0;
    *out = packed;
    return ASC_OK;
}

// Destination of out-edge i in the stored layout.
static inline uint32_t host_edge_dst(const asc_graph *g, uint64_t i) {
    if (g->edge_words == 2) return g->h_edges[2 * i];
    uint32_t w;
    if (g->ebits == 32) {
        w = g->h_edges[i];
    } else {
        const uint64_t bit = i * g->ebits;
        const uint32_t *q = g->h_edges + (bit >> 5);
        const uint32_t sh = (uint32_t)bit & 31u;
        uint64_t x = q[0] >> sh;
        if (sh + g->ebits > 32) x |= (uint64_t)q[1] << (32 - sh);
        w = (uint32_t)x & ((1u << g->ebits) - 1u);
    }
    return w >> g->wbits;
}

static asc_status finish_graph(asc_graph *g, const asc_budget *budget, asc_graph **out) {
    ASC_TRY(validate_and_measure(g));
    g->file_edge_bytes = 4 * g->edge_words;
    ASC_TRY(pack_weighted(g));
    ASC_TRY(narrow_edges(g));
    ASC_TRY(compute_static_split(g, budget, g->is_csc ? 17 : (g->file_edge_bytes == 8 ? 15 : 13)));
    if (budget && budget->mode == ASC_BUDGET_MANAGED) ASC_TRY(make_managed(g));
    ASC_TRY(upload(g));
    *out = g;
    return ASC_OK;
}

static void destroy(asc_graph *g) {
    if (!g) return;
    free_workspace(g);
    if (g->d_ptr) cudaFree(g->d_ptr);
    if (g->d_static) cudaFree(g->d_static);
    for (uint32_t *p : g->d_stage)
        if (p) cudaFree(p);
    if (g->d_in_heads) cudaFree(g->d_in_heads);
    if (g->d_outdeg) cudaFree(g->d_outdeg);
    if (g->managed_edges) cudaFree(g->managed_edges);
    if (g->h_ptr) cudaFreeHost(g->h_ptr);
    if (g->h_edges) cudaFreeHost(g->h_edges);
    if (g->h_outdeg) cudaFreeHost(g->h_outdeg);
    if (g->h_in_edges) cudaFreeHost(g->h_in_edges);
    delete[] g->h_in_ptr;
    delete[] g->h_in_none;
    if (g->stream) cudaStreamDestroy(g->stream);
    delete g;
}

// ---------------------------------------------------------------- RMAT --------
namespace {

inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

struct Rmat {
    uint32_t scale;
    uint64_t E;  // generated edges (before symmetrisation)
    uint64_t seed_key;
    uint64_t ta, tab, tabc;  // quadrant thresholds on 32-bit draws
    uint32_t wmin, wspan;
    bool weights;

    // Edge i of the generated list: a counter-based stream keyed by (seed, i),
    // so the result does not depend on how the edges are split over threads.
    inline void edge(uint64_t i, uint32_t &s, uint32_t &d, uint32_t &w) const {
        uint64_t st = mix64(seed_key ^ (i * 0x9E3779B97F4A7C15ull)) ;
        uint32_t src = 0, dst = 0;
        uint64_t r = 0;
        for (uint32_t l = 0; l < scale; l++) {
            if ((l & 1) == 0) {
                st += 0x9E3779B97F4A7C15ull;
                r = mix64(st);
            }
            uint64_t u = (l & 1) ? (r >> 32) : (r & 0xffffffffull);
            uint32_t sb = u >= tab, db = (u >= ta && u < tab) || u >= tabc;
            src = (src << 1) | sb;
            dst = (dst << 1) | db;
        }
        s = src;
        d = dst;
        if (weights) {
            st += 0x9E3779B97F4A7C15ull;
            w = wmin + (uint32_t)(mix64(st) % wspan);
        } else {
            w = 0;
        }
    }
};

// Builds CSR (or CSC) from the generated list with a stable two-pass counting
// sort: pass 1 counts per thread chunk, pass 2 regenerates and places each edge,
// so every list keeps generation order. ptr32 or ptr64 receives V+1 offsets.
asc_status rmat_build(uint32_t scale, uint32_t ef, uint64_t seed, double a, double b, double c, uint32_t wmin,
                      uint32_t wmax, uint32_t flags, uint64_t *ptr64, uint32_t *ptr32, uint32_t *edges,
                      uint32_t *outdeg) {
    if (scale == 0 || scale > 31) return fail(ASC_ERR_INVALID, "RMAT scale %u out of range [1, 31]", scale);
    if (!(a >= 0 && b >= 0 && c >= 0 && a + b + c <= 1.0))
        return fail(ASC_ERR_INVALID, "RMAT probabilities a=%g b=%g c=%g are invalid", a, b, c);
    const bool weights = flags & ASC_RMAT_WEIGHTS, sym = flags & ASC_RMAT_SYMMETRIC,
               tr = flags & ASC_RMAT_TRANSPOSE;
    if (weights && (wmin > wmax || wmax == 0xffffffffu))
        return fail(ASC_ERR_INVALID, "weight range [%u, %u] is invalid", wmin, wmax);
    const uint64_t V = 1ull << scale;
    const uint64_t E0 = V * ef;
    const uint64_t Et = sym ? 2 * E0 : E0;
    if (Et > kU32Max) return fail(ASC_ERR_UNSUPPORTED, "RMAT with %llu edges needs 64-bit offsets",
                                  (unsigned long long)Et);
    Rmat R;
    R.scale = scale;
    R.E = E0;
    R.seed_key = mix64(seed + 0x632BE59BD9B4E019ull);
    const double two32 = 4294967296.0;
    R.ta = (uint64_t)(a * two32);
    R.tab = (uint64_t)((a + b) * two32);
    R.tabc = (uint64_t)((a + b + c) * two32);
    R.weights = weights;
    R.wmin = wmin;
    R.wspan = weights ? (wmax - wmin + 1) : 1;
    const uint32_t words = weights ? 2 : 1;

    // thread count bounded so the per-thread histograms stay within 4 GiB
    unsigned T = host_threads(Et);
    T = (unsigned)std::min<uint64_t>(T, std::max<uint64_t>(1, (4ull << 30) / (4 * V)));
    T = std::min(T, 32u);
    std::vector<uint32_t> hist;
    try {
        hist.assign((size_t)T * V, 0);
    } catch (...) {
        return fail(ASC_ERR_NOMEM, "RMAT histogram allocation failed");
    }
    std::vector<std::atomic<uint32_t>> odeg_dummy;
    uint64_t chunk = (Et + T - 1) / T;
    auto virt = [&](uint64_t i, uint32_t &s, uint32_t &d, uint32_t &w) {
        if (i < E0) R.edge(i, s, d, w);
        else {
            R.edge(i - E0, d, s, w);  // reversed copy
        }
    };
    // pass 1: per-chunk counts of the sort key; out-degree counts for CSC
    if (tr && outdeg) memset(outdeg, 0, sizeof(uint32_t) * V);
    {
        std::vector<std::thread> th;
        for (unsigned t = 0; t < T; t++)
            th.emplace_back([&, t] {
                uint32_t *h = hist.data() + (size_t)t * V;
                uint64_t b0 = std::min(Et, t * chunk), e0 = std::min(Et, b0 + chunk);
                for (uint64_t i = b0; i < e0; i++) {
                    uint32_t s, d, w;
                    virt(i, s, d, w);
                    h[tr ? d : s]++;
                    if (tr && outdeg) __atomic_fetch_add(&outdeg[s], 1u, __ATOMIC_RELAXED);
                }
            });
        for (auto &x : th) x.join();
    }
    // offsets: ptr[v] = sum of all counts of keys < v; per-chunk cursors in place
    {
        std::vector<uint64_t> vsum(V + 1, 0);
        parallel_for(V, host_threads(V * T), [&](unsigned, uint64_t b0, uint64_t e0) {
            for (uint64_t v = b0; v < e0; v++) {
                uint64_t s = 0;
                for (unsigned t = 0; t < T; t++) s += hist[(size_t)t * V + v];
                vsum[v] = s;
            }
        });
        uint64_t run = 0;
        for (uint64_t v = 0; v < V; v++) {
            uint64_t c0 = vsum[v];
            vsum[v] = run;
            run += c0;
        }
        vsum[V] = run;
        for (uint64_t v = 0; v <= V; v++) {
            if (ptr64) ptr64[v] = vsum[v];
            if (ptr32) ptr32[v] = (uint32_t)vsum[v];
        }
        parallel_for(V, host_threads(V * T), [&](unsigned, uint64_t b0, uint64_t e0) {
            for (uint64_t v = b0; v < e0; v++) {
                uint64_t cur = vsum[v];
                for (unsigned t = 0; t < T; t++) {
                    uint32_t c0 = hist[(size_t)t * V + v];
                    hist[(size_t)t * V + v] = (uint32_t)cur;
                    cur += c0;
                }
            }
        });
    }
    // pass 2: regenerate and place
    {
        std::vector<std::thread> th;
        for (unsigned t = 0; t < T; t++)
            th.emplace_back([&, t] {
                uint32_t *h = hist.data() + (size_t)t * V;
                uint64_t b0 = std::min(Et, t * chunk), e0 = std::min(Et, b0 + chunk);
                for (uint64_t i = b0; i < e0; i++) {
                    uint32_t s, d, w;
                    virt(i, s, d, w);
                    uint32_t key = tr ? d : s, val = tr ? s : d;
                    uint64_t pos = h[key]++;
                    edges[pos * words] = val;
                    if (weights) edges[pos * 2 + 1] = w;
                }
            });
        for (auto &x : th) x.join();
    }
    return ASC_OK;
}

}  // namespace
}  // namespace asc

namespace asc {

// In-edges of a CSR graph for bottom-up BFS steps: a counting sort of the
// out-edges by destination (host threads), each in-list sorted by source id,
// stored as a bit stream of bits(V - 1) per edge in pinned memory that the
// device reads in place. Built once per graph, on its first BFS that may step
// bottom-up.
asc_status build_in_edges(asc_graph *g) {
    if (g->h_in_edges || g->is_csc) return ASC_OK;
    const uint64_t V = g->V, E = g->E;
    std::vector<uint32_t> cnt(V + 1, 0);
    const unsigned nt = host_threads(E);
    parallel_for(E, nt, [&](unsigned, uint64_t b, uint64_t e) {
        for (uint64_t i = b; i < e; i++) __atomic_fetch_add(&cnt[host_edge_dst(g, i)], 1u, __ATOMIC_RELAXED);
    });
    uint32_t *in_ptr = new (std::nothrow) uint32_t[V + 1];
    if (!in_ptr) return fail(ASC_ERR_NOMEM, "in-edge offsets: %llu vertices", (unsigned long long)V);
    uint64_t run = 0;
    for (uint64_t v = 0; v < V; v++) {
        in_ptr[v] = (uint32_t)run;
        run += cnt[v];
        cnt[v] = in_ptr[v];  // becomes the scatter cursor
    }
    in_ptr[V] = (uint32_t)run;
    std::vector<uint32_t> raw;
    try {
        raw.resize(E ? E : 1);
    } catch (...) {
        delete[] in_ptr;
        return fail(ASC_ERR_NOMEM, "in-edges: %llu edges", (unsigned long long)E);
    }
    parallel_for(E, nt, [&](unsigned, uint64_t b, uint64_t e) {
        if (b >= e) return;
        // the source of edge b: the last vertex whose list starts at or before b
        uint64_t u = std::upper_bound(g->h_ptr, g->h_ptr + V + 1, (uint32_t)b) - g->h_ptr - 1;
        for (uint64_t i = b; i < e; i++) {
            while (g->h_ptr[u + 1] <= i) u++;
            const uint32_t d = host_edge_dst(g, i);
            raw[__atomic_fetch_add(&cnt[d], 1u, __ATOMIC_RELAXED)] = (uint32_t)u;
        }
    });
    parallel_for(V, host_threads(E), [&](unsigned, uint64_t b, uint64_t e) {
        for (uint64_t v = b; v < e; v++) std::sort(raw.begin() + in_ptr[v], raw.begin() + in_ptr[v + 1]);
    });
    const uint32_t bits = g->in_ebits;  // chosen with the split (bits(V - 1), or 32 without packing)
    uint32_t *packed = nullptr;
    asc_status st = pack_stream(raw.data(), E, bits, &packed);
    if (st != ASC_OK) {
        delete[] in_ptr;
        return st;
    }
    void *dp = nullptr;
    cudaError_t ce = cudaHostGetDevicePointer(&dp, packed, 0);
    if (ce != cudaSuccess) {
        delete[] in_ptr;
        cudaFreeHost(packed);
        return cuda_fail(ce, "cudaHostGetDevicePointer(in-edges)", __FILE__, __LINE__);
    }
    g->h_in_ptr = in_ptr;
    g->h_in_edges = packed;
    g->d_host_in_edges = (const uint32_t *)dp;
    if (g->d_in_heads && !g->in_heads_ready) {
        // first in-edge of every vertex, vertex-indexed; a vertex without
        // in-edges holds its own id (never a frontier vertex when it is probed,
        // since only unreached vertices probe)
        std::vector<uint32_t> first(V ? V : 1, 0);
        parallel_for(V, host_threads(V), [&](unsigned, uint64_t b, uint64_t e) {
            for (uint64_t v = b; v < e; v++) first[v] = in_ptr[v + 1] > in_ptr[v] ? raw[in_ptr[v]] : (uint32_t)v;
        });
        uint32_t *hp = nullptr;
        ASC_TRY(pack_stream(first.data(), V, bits, &hp));
        cudaError_t he = cudaMemcpy(g->d_in_heads, hp, 4 * g->in_head_words, cudaMemcpyHostToDevice);
        cudaFreeHost(hp);
        if (he != cudaSuccess) return cuda_fail(he, "cudaMemcpy(in-edge heads)", __FILE__, __LINE__);
        g->in_heads_ready = true;
    }
    return ASC_OK;
}

}  // namespace asc

using namespace asc;

extern "C" {

void asc_budget_default(asc_budget *b) {
    if (!b) return;
    b->mode = ASC_BUDGET_ALL;
    b->fragment_edges = 4096;
    b->value = 0;
    b->stage_bytes = 0;
}

asc_status asc_graph_open(const char *path, asc_format fmt, const asc_budget *budget, asc_graph **out) {
    if (!path || !out) return fail(ASC_ERR_INVALID, "asc_graph_open: path and out are required");
    *out = nullptr;
    FILE *f = fopen(path, "rb");
    if (!f) return fail(ASC_ERR_BAD_FILE, "%s: cannot open (%s)", path, strerror(errno));
    struct stat sb;
    if (fstat(fileno(f), &sb) != 0) {
        fclose(f);
        return fail(ASC_ERR_BAD_FILE, "%s: cannot stat", path);
    }
    uint64_t size = (uint64_t)sb.st_size;
    uint8_t hdr[16] = {0};
    size_t got = fread(hdr, 1, 16, f);
    if (got < 8) {
        fclose(f);
        return fail(ASC_ERR_BAD_FILE, "%s: shorter than any graph header", path);
    }
    if (fmt == ASC_FMT_AUTO) {
        asc_status s = detect_format(path, size, hdr, &fmt);
        if (s != ASC_OK) {
            fclose(f);
            return s;
        }
    }
    uint64_t V, E, hdr_bytes;
    if (fmt == ASC_FMT_BCSR32) {
        uint32_t v32, e32;
        memcpy(&v32, hdr, 4);
        memcpy(&e32, hdr + 4, 4);
        V = v32;
        E = e32;
        hdr_bytes = 8;
    } else if (fmt >= ASC_FMT_BCSR && fmt <= ASC_FMT_BCSC) {
        if (got < 16) {
            fclose(f);
            return fail(ASC_ERR_BAD_FILE, "%s: shorter than the 16-byte header", path);
        }
        memcpy(&V, hdr, 8);
        memcpy(&E, hdr + 8, 8);
        hdr_bytes = 16;
    } else {
        fclose(f);
        return fail(ASC_ERR_INVALID, "unknown format %d", (int)fmt);
    }
    asc_status s = check_sizes(V, E);
    if (s != ASC_OK) {
        fclose(f);
        return s;
    }
    uint64_t ptr_bytes = fmt == ASC_FMT_BCSR32 ? 4 * V : 8 * V;
    uint64_t ew = fmt == ASC_FMT_BWCSR ? 2 : 1;
    uint64_t expect = hdr_bytes + ptr_bytes + 4 * ew * E + (fmt == ASC_FMT_BCSC ? 4 * V : 0);
    if (size < expect) {
        fclose(f);
        return fail(ASC_ERR_BAD_FILE, "%s: file has %llu bytes, the %s layout with V=%llu E=%llu needs %llu", path,
                    (unsigned long long)size, fmt == ASC_FMT_BCSR ? "bcsr" : fmt == ASC_FMT_BWCSR ? "bwcsr"
                                              : fmt == ASC_FMT_BCSC ? "bcsc" : "bcsr32",
                    (unsigned long long)V, (unsigned long long)E, (unsigned long long)expect);
    }
    // the file's layout and size check out: now the device is needed
    int dev;
    s = ensure_device(&dev);
    if (s != ASC_OK) {
        fclose(f);
        return s;
    }
    asc_graph *g = new asc_graph();
    g->V = V;
    g->E = E;
    g->edge_words = (uint32_t)ew;
    g->is_csc = fmt == ASC_FMT_BCSC;
    g->device = dev;
    s = alloc_host_arrays(g);
    if (s != ASC_OK) {
        fclose(f);
        destroy(g);
        return s;
    }
    fseeko(f, (off_t)hdr_bytes, SEEK_SET);
    bool ok = true;
    if (g->is_csc) ok = read_exact(f, g->h_outdeg, 4 * V);
    // offsets: V entries in the file (u64 or u32), sentinel E appended
    if (ok) {
        const uint64_t CH = 1 << 20;
        std::vector<uint64_t> buf(CH);
        for (uint64_t v0 = 0; ok && v0 < V; v0 += CH) {
            uint64_t n = std::min(CH, V - v0);
            if (fmt == ASC_FMT_BCSR32) {
                ok = read_exact(f, g->h_ptr + v0, 4 * n);
            } else {
                ok = read_exact(f, buf.data(), 8 * n);
                for (uint64_t i = 0; ok && i < n; i++) {
                    if (buf[i] > E) {
                        fclose(f);
                        uint64_t bad = buf[i];
                        destroy(g);
                        return fail(ASC_ERR_BAD_FILE, "%s: row offset %llu of vertex %llu exceeds E = %llu", path,
                                    (unsigned long long)bad, (unsigned long long)(v0 + i), (unsigned long long)E);
                    }
                    g->h_ptr[v0 + i] = (uint32_t)buf[i];
                }
            }
        }
        g->h_ptr[V] = (uint32_t)E;
    }
    if (ok) ok = read_exact(f, g->h_edges, 4 * ew * E);
    fclose(f);
    if (!ok) {
        destroy(g);
        return fail(ASC_ERR_BAD_FILE, "%s: read failed (short file)", path);
    }
    s = finish_graph(g, budget, out);
    if (s != ASC_OK) destroy(g);
    return s;
}

asc_status asc_graph_from_csr(uint64_t V, uint64_t E, const uint64_t *ptr, const void *edges, uint32_t edge_bytes,
                              const uint32_t *outdeg, const asc_budget *budget, asc_graph **out) {
    if (!out || !ptr || (!edges && E)) return fail(ASC_ERR_INVALID, "asc_graph_from_csr: null argument");
    *out = nullptr;
    if (edge_bytes != 4 && edge_bytes != 8) return fail(ASC_ERR_INVALID, "edge_bytes must be 4 or 8");
    if (outdeg && edge_bytes != 4) return fail(ASC_ERR_INVALID, "a CSC graph has 4-byte in-edges");
    ASC_TRY(check_sizes(V, E));
    if (ptr[V] != E) return fail(ASC_ERR_INVALID, "ptr[V] = %llu differs from E = %llu",
                                 (unsigned long long)ptr[V], (unsigned long long)E);
    int dev;
    ASC_TRY(ensure_device(&dev));
    asc_graph *g = new asc_graph();
    g->V = V;
    g->E = E;
    g->edge_words = edge_bytes / 4;
    g->is_csc = outdeg != nullptr;
    g->device = dev;
    asc_status s = alloc_host_arrays(g);
    if (s == ASC_OK) {
        for (uint64_t v = 0; v <= V; v++) {
            if (ptr[v] > E) {
                s = fail(ASC_ERR_INVALID, "ptr[%llu] = %llu exceeds E", (unsigned long long)v,
                         (unsigned long long)ptr[v]);
                break;
            }
            g->h_ptr[v] = (uint32_t)ptr[v];
        }
    }
    if (s == ASC_OK) {
        if (E) memcpy(g->h_edges, edges, (size_t)edge_bytes * E);
        if (outdeg) memcpy(g->h_outdeg, outdeg, sizeof(uint32_t) * V);
        s = finish_graph(g, budget, out);
    }
    if (s != ASC_OK) destroy(g);
    return s;
}

asc_status asc_graph_rmat(uint32_t scale, uint32_t edge_factor, uint64_t seed, double a, double b, double c,
                          uint32_t wmin, uint32_t wmax, uint32_t flags, const asc_budget *budget,
                          asc_graph **out) {
    if (!out) return fail(ASC_ERR_INVALID, "asc_graph_rmat: out is required");
    *out = nullptr;
    if (scale == 0 || scale > 31) return fail(ASC_ERR_INVALID, "RMAT scale %u out of range [1, 31]", scale);
    if ((flags & ASC_RMAT_TRANSPOSE) && (flags & ASC_RMAT_WEIGHTS))
        return fail(ASC_ERR_INVALID, "a CSC graph for PageRank carries no weights");
    uint64_t V = 1ull << scale;
    uint64_t E = V * edge_factor * ((flags & ASC_RMAT_SYMMETRIC) ? 2 : 1);
    ASC_TRY(check_sizes(V, E));
    int dev;
    ASC_TRY(ensure_device(&dev));
    asc_graph *g = new asc_graph();
    g->V = V;
    g->E = E;
    g->edge_words = (flags & ASC_RMAT_WEIGHTS) ? 2 : 1;
    g->is_csc = (flags & ASC_RMAT_TRANSPOSE) != 0;
    g->device = dev;
    asc_status s = alloc_host_arrays(g);
    if (s == ASC_OK)
        s = rmat_build(scale, edge_factor, seed, a, b, c, wmin, wmax, flags, nullptr, g->h_ptr, g->h_edges,
                       g->h_outdeg);
    if (s == ASC_OK) s = finish_graph(g, budget, out);
    if (s != ASC_OK) destroy(g);
    return s;
}

asc_status asc_rmat_csr(uint32_t scale, uint32_t edge_factor, uint64_t seed, double a, double b, double c,
                        uint32_t wmin, uint32_t wmax, uint32_t flags, uint64_t *ptr, void *edges,
                        uint32_t *outdeg) {
    if (!ptr || !edges) return fail(ASC_ERR_INVALID, "asc_rmat_csr: ptr and edges are required");
    if ((flags & ASC_RMAT_TRANSPOSE) && !outdeg)
        return fail(ASC_ERR_INVALID, "asc_rmat_csr: ASC_RMAT_TRANSPOSE needs outdeg");
    if ((flags & ASC_RMAT_TRANSPOSE) && (flags & ASC_RMAT_WEIGHTS))
        return fail(ASC_ERR_INVALID, "a CSC graph for PageRank carries no weights");
    return rmat_build(scale, edge_factor, seed, a, b, c, wmin, wmax, flags, ptr, nullptr, (uint32_t *)edges,
                      outdeg);
}

asc_status asc_graph_info_get(const asc_graph *g, asc_graph_info *info) {
    if (!g || !info) return fail(ASC_ERR_INVALID, "asc_graph_info_get: null argument");
    memset(info, 0, sizeof(*info));
    info->vertices = g->V;
    info->edges = g->E;
    info->edge_bytes = 4 * g->edge_words;
    info->is_csc = g->is_csc;
    info->static_edges = g->static_edges;
    info->static_vertices = g->static_vertices;
    info->staging_bytes = 2 * 4 * g->stage_words;
    info->in_head_bytes = 4 * g->in_head_words;
    info->device_edge_bytes = (g->static_edges ? 4ull * edge_store_words(g, g->static_edges) : 0) +
                              info->staging_bytes + info->in_head_bytes;
    info->device_vertex_bytes = g->device_vertex_bytes + (g->ws ? g->ws->device_bytes : 0);
    info->host_pinned_bytes = 4ull * edge_store_words(g, g->E);
    info->max_degree = g->max_degree;
    info->max_weight = g->max_weight;
    info->weight_bits = g->wbits;
    info->edge_bits = g->edge_words == 2 ? 64 : g->ebits;
    return ASC_OK;
}

asc_status asc_graph_close(asc_graph *g) {
    destroy(g);
    return ASC_OK;
}

asc_status asc_write_graph(const char *path, asc_format fmt, uint64_t V, uint64_t E, const uint64_t *ptr,
                           const void *edges, const uint32_t *outdeg) {
    if (!path || !ptr || (!edges && E)) return fail(ASC_ERR_INVALID, "asc_write_graph: null argument");
    if (fmt == ASC_FMT_AUTO) return fail(ASC_ERR_INVALID, "asc_write_graph needs an explicit format");
    if (fmt == ASC_FMT_BCSC && !outdeg) return fail(ASC_ERR_INVALID, "the bcsc layout needs out-degrees");
    FILE *f = fopen(path, "wb");
    if (!f) return fail(ASC_ERR_BAD_FILE, "%s: cannot create (%s)", path, strerror(errno));
    bool ok = true;
    if (fmt == ASC_FMT_BCSR32) {
        if (V > kU32Max || E > kU32Max) {
            fclose(f);
            return fail(ASC_ERR_UNSUPPORTED, "the 32-bit layout cannot hold V=%llu E=%llu", (unsigned long long)V,
                        (unsigned long long)E);
        }
        uint32_t h[2] = {(uint32_t)V, (uint32_t)E};
        ok = fwrite(h, 4, 2, f) == 2;
        std::vector<uint32_t> p32(V);
        for (uint64_t v = 0; v < V; v++) p32[v] = (uint32_t)ptr[v];
        ok = ok && fwrite(p32.data(), 4, V, f) == V;
        ok = ok && fwrite(edges, 4, E, f) == E;
    } else {
        uint64_t h[2] = {V, E};
        ok = fwrite(h, 8, 2, f) == 2;
        if (fmt == ASC_FMT_BCSC) ok = ok && fwrite(outdeg, 4, V, f) == V;
        ok = ok && fwrite(ptr, 8, V, f) == V;
        uint64_t words = fmt == ASC_FMT_BWCSR ? 2 : 1;
        ok = ok && fwrite(edges, 4 * words, E, f) == E;
    }
    if (fclose(f) != 0) ok = false;
    if (!ok) return fail(ASC_ERR_BAD_FILE, "%s: write failed", path);
    return ASC_OK;
}

}  // extern "C"
