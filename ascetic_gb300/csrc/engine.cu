// The out-of-GPU-memory iteration engine: frontier kernels for BFS, SSSP, CC
// and PageRank over a device-resident static prefix of the edge array plus
// on-demand edges read straight from pinned host memory.
//
// What each iteration does, against the reference driver (CalculateOpt.cu:60-191):
//  - split of the active set into static and on-demand vertices, compaction
//    into lists, and the active counts (setStaticAndOverloadLabelBool,
//    thrust::reduce/exclusive_scan, setStaticActiveNodeArray,
//    setOverloadNodePointerSwap, gpu_kernels.cu:111-122, gpu_kernels.cuh:411-438)
//    happen here as a by-product of relaxation: the thread that lowers a value
//    and wins the vertex's bit in the next-frontier bitmap appends it, with one
//    warp-aggregated atomic per warp, to the static list, the on-demand list,
//    or (long lists) the segment list;
//  - the host gather of on-demand edges and the partitioned H2D copies
//    (GraphMeta.cuh:469-578, CalculateOpt.cu:146-178) are replaced by the
//    on-demand expansion kernel reading each active list directly from the
//    mapped pinned copy over the host link, so only active edges cross it;
//  - relaxation rules are those of bfs_kernelStatic / sssp_kernel /
//    cc_kernelStaticSwap (gpu_kernels.cuh:376-505, 441-481): atomicMin of
//    val[u]+1, val[u]+w, val[u]; PageRank sums follow prSumKernel_* and
//    prKernel_Opt (gpu_kernels.cuh:533-594).
//
// Load balance: each expansion launch is a persistent grid pulling work items
// from an atomic cursor. A work item is either a tile of 256 frontier vertices
// (the CTA scans their degrees and walks the tile's concatenated edge range,
// so consecutive threads read consecutive column indices) or one segment of a
// vertex whose degree exceeds the huge-degree threshold (a CTA-wide stride
// over up to segment_edges edges of that list).
#include <cooperative_groups.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <thread>
#include <vector>
#include <string>
#include <sys/stat.h>

#include "common.h"

namespace asc {

namespace {

constexpr unsigned kFull = 0xffffffffu;
// Minimum resident CTAs per SM asked of the expansion kernels (register cap):
// 8 x 256 threads fill an SM, 32 registers each. Measured on RMAT scale 24 with
// bit-packed edges: 65.6 GTEPS at 8, 64.5 at 6, 57.3 at 4 (64 registers, half
// the warps: the loads over the host link want every warp the SM can hold).
// The same for the PageRank pull/scatter kernels (8: FP32 standard PageRank on
// RMAT scale 23 in 181 ms against 195 at the compiler's choice of 40 registers).
// The batched SSSP kernel takes 5 (48 registers; at 6 or 8 it spills more than
// a few bytes); the batched BFS kernels are left to the compiler (32 registers).
#ifndef ASC_PR_MIN_BLOCKS
#define ASC_PR_MIN_BLOCKS 8
#endif
#ifndef ASC_MS_MIN_BLOCKS
#define ASC_MS_MIN_BLOCKS 5
#endif
#ifndef ASC_EXPAND_MIN_BLOCKS
#define ASC_EXPAND_MIN_BLOCKS 8
#endif
constexpr int kWarps = kBlock / 32;

// Self-checking build (nvcc -DASC_SELF_CHECK): indices the kernels take from
// device data (frontier lists, segment items, decoded edges, level-plane
// pointers, list and segment capacities) are checked before use; the first bad
// one is recorded as (site << 32 | index), its access is skipped, and the run
// or batch iteration that launched the kernel fails with ASC_ERR_CUDA naming
// the site. Without the macro the checks compile to nothing.
#ifdef ASC_SELF_CHECK
__device__ unsigned long long g_self_check;
__device__ __noinline__ bool self_check_fail(uint32_t site, uint64_t idx) {
    atomicCAS(&g_self_check, 0ull, ((unsigned long long)site << 32) | (idx & 0xffffffffull));
    return true;
}
#define ASC_BAD(cond, site, idx) ((cond) ? self_check_fail((site), (idx)) : false)
#else
#define ASC_BAD(cond, site, idx) false
#endif

enum Alg { kBFS = 0, kSSSP = 1, kCC = 2 };

// Control block (u32 words). Per parity p: [8p+0..3] counts of the frontier
// built for that parity (static list, on-demand list, static segments,
// on-demand segments), [8p+4..5] work cursors of the launches that build it,
// [8p+6..7] vertices of each region in that frontier (its bitmap's bits).
// Stats at word 16 (u64): edges static, edges on-demand, frontier vertices
// static, frontier vertices on-demand, reached vertices, reached edges. PageRank FP64 accumulators at word 32:
// residual[2], dangling[2].
// Word 28 counts iterations, word 29 flags an iteration cap hit and word 30
// counts loop-body executions when the loop runs as a CUDA graph. Word 31 is
// the SSSP near-far threshold, word 36 the minimum far distance of a pass.
// Words 42-43 (u64): in-edges that bottom-up BFS steps read from host memory;
// words 44-45 (u64): unreached vertices those steps examined.
enum { CTL_BLOCK = 8, CTL_STATS = 16, CTL_ITERS = 28, CTL_TIMEOUT = 29, CTL_BODIES = 30, CTL_THRESH = 31,
       CTL_PR = 32, CTL_MINFAR = 36, CTL_BU_EDGES = 42, CTL_BU_VERTS = 44, CTL_WORDS = 64 };

struct RegionArgs {
    const uint32_t *ptr;
    const uint32_t *edges;        // region edge base, indexed by global edge offset
    uint32_t *val;
    uint32_t *bitmap;             // next-frontier bitmap (written)
    uint32_t *visited;            // BFS: reached-vertex bitmap (claims)
    const uint32_t *huge_bits;    // one bit per vertex whose list is cut into segments
    uint32_t *far_bits;           // SSSP near-far: vertices whose distance is at or above *thresh
    const uint32_t *thresh;
    const uint32_t *bitmap_in;    // this iteration's frontier bitmap (null: no id-order mode)
    const uint32_t *q_in;         // this region's input list (null: dense range)
    const uint64_t *seg_in;       // this region's input segments
    const uint32_t *cnt_in;       // counts of the input frontier
    uint32_t region;              // 0 static, 1 on-demand
    uint32_t dense_begin, dense_end;
    uint32_t *q_out;              // output lists: static at 0, on-demand at S
    uint64_t *seg_out;            // output segments: static at 0, on-demand at segcap_static
    uint32_t *cnt_out;
    uint32_t *work;
    unsigned long long *stats;
    uint32_t S;
    uint32_t huge;
    uint32_t seg_len;
    uint32_t segcap_static;
    uint32_t segcap_ondemand;
    uint32_t V;
    uint32_t dense_div;
    uint32_t wbits;               // > 0: u32 edges packed as (dst << wbits) | weight
    uint32_t ebits;               // bits per stored edge word: 32, or a bit stream of ebits per edge
    unsigned long long *frag;     // non-null: add edges read per 4096-edge fragment
    // bottom-up BFS steps (null in_ptr: top-down only)
    const uint32_t *in_ptr;       // in-edge offsets (device)
    const uint32_t *in_edges;     // in-edge source ids, a bit stream of in_ebits per edge (pinned host)
    uint32_t in_ebits;
    uint32_t bu_div;              // a step whose input frontier holds more than V / bu_div vertices is bottom-up
    uint32_t in_resident;         // in_edges is device memory (a graph without a cap), else pinned host
    const uint32_t *in_heads;     // first in-edge of every vertex in HBM (a bit stream of in_ebits), or null
    const uint32_t *in_none;      // one bit per vertex without in-edges (never reached but as a source)
    // standard PageRank pull, on-demand region: tiles copy their in-edge range
    // through shared memory (see pr_vertices); edge_words bounds those reads
    uint32_t stage_edges;
    uint64_t edge_words;
};

// True when this BFS iteration steps bottom-up: its input frontier (the
// region bit counts of the previous step, upper bounds) holds more than
// V / bu_div vertices. The top-down and bottom-up kernels of an iteration both
// evaluate it from the same counts and exactly one of them does the work.
__device__ __forceinline__ bool bottom_up_step(const RegionArgs &a) {
    return a.in_ptr && a.bu_div && ((uint64_t)a.cnt_in[6] + a.cnt_in[7]) * a.bu_div > a.V;
}

// Adds the n edges read from [b, b + n) to their 4096-edge fragments' counters.
__device__ __forceinline__ void count_fragments(unsigned long long *frag, uint64_t b, uint32_t n) {
    if (!n) return;
    const uint64_t e = b + n;
    for (uint64_t f = b >> 12; f <= (e - 1) >> 12; f++) {
        const uint64_t lo = max(b, f << 12), hi = min(e, (f + 1) << 12);
        atomicAdd(frag + f, (unsigned long long)(hi - lo));
    }
}

// Edge layouts of the expansion kernels (their WORDS template argument):
// 1 = one u32 per edge, 2 = {dst, weight} pairs, kBitsLayout = one word per
// edge stored as a bit stream of ebits per edge.
constexpr int kBitsLayout = 3;

// ebits bits of a bit stream: edge idx at bits [idx*ebits, (idx+1)*ebits),
// little-endian across words; the buffer carries a padding word, so p[1]
// stays inside it.
__device__ __forceinline__ uint32_t bit_stream_word(const uint32_t *base, uint64_t idx, uint32_t ebits) {
    const uint64_t bit = idx * ebits;
    const uint32_t *p = base + (bit >> 5);
    const uint32_t sh = (uint32_t)bit & 31u;
    uint32_t x = __ldg(p) >> sh;
    if (sh + ebits > 32) x |= __ldg(p + 1) << (32 - sh);
    return x & ((1u << ebits) - 1u);
}

template <int WORDS>
__device__ __forceinline__ uint32_t layout_word(const uint32_t *base, uint64_t idx, uint32_t ebits) {
    return WORDS == kBitsLayout ? bit_stream_word(base, idx, ebits) : __ldg(base + idx);
}

// Edge word idx of a one-word-per-edge array: a plain load, or a bit-stream
// read when ebits < 32 (kernels with the layout as a template argument call
// bit_stream_word directly, without the per-edge test).
__device__ __forceinline__ uint32_t edge_word(const uint32_t *base, uint64_t idx, uint32_t ebits) {
    if (ebits == 32) return __ldg(base + idx);
    const uint64_t bit = idx * ebits;
    const uint32_t *p = base + (bit >> 5);
    const uint32_t sh = (uint32_t)bit & 31u;
    uint32_t x = __ldg(p) >> sh;
    if (sh + ebits > 32) x |= __ldg(p + 1) << (32 - sh);
    return x & ((1u << ebits) - 1u);
}

// How a PageRank tile picks its vertices: from the active list, or every
// vertex of a range (frontiers walked through their bitmap use chunks).
enum TileMode { kList = 0, kRange = 1 };

struct Smem {
    uint32_t pref[kBlock + 1];
    uint32_t start[kBlock];
    uint32_t vu[kBlock];
    uint32_t warp[kWarps + 1];
    uint32_t work;
};

__device__ __forceinline__ uint32_t block_excl_scan(uint32_t x, uint32_t &total, uint32_t *s_warp) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t incl = x;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t y = __shfl_up_sync(kFull, incl, d);
        if (lane >= d) incl += y;
    }
    if (lane == 31) s_warp[w] = incl;
    __syncthreads();
    if (w == 0) {
        uint32_t t = lane < kWarps ? s_warp[lane] : 0;
        uint32_t ti = t;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            uint32_t y = __shfl_up_sync(kFull, ti, d);
            if (lane >= d) ti += y;
        }
        if (lane < kWarps) s_warp[lane] = ti - t;
        if (lane == kWarps - 1) s_warp[kWarps] = ti;
    }
    __syncthreads();
    total = s_warp[kWarps];
    return s_warp[w] + incl - x;
}

template <int ALG, int WORDS>
__device__ __forceinline__ void load_edge(const RegionArgs &a, uint32_t vu, uint64_t idx, uint32_t &v, uint32_t &nv) {
    if (WORDS == 2) {
        uint2 e = __ldg(reinterpret_cast<const uint2 *>(a.edges) + idx);
        v = e.x;
        nv = ALG == kSSSP ? vu + e.y : (ALG == kBFS ? vu + 1 : vu);
    } else {
        const uint32_t e = layout_word<WORDS>(a.edges, idx, a.ebits);
        v = e >> a.wbits;
        nv = ALG == kBFS ? vu + 1 : (ALG == kSSSP ? vu + (e & ((1u << a.wbits) - 1u)) : vu);
    }
}

// Counts, per region, the vertices whose next-frontier bit this warp won
// (shared-memory counters, flushed once per CTA). Every lane calls it.
__device__ __forceinline__ void count_next(const RegionArgs &a, bool won, uint32_t v, uint32_t *s_next) {
    const unsigned m0 = __ballot_sync(kFull, won && v < a.S);
    const unsigned m1 = __ballot_sync(kFull, won && v >= a.S);
    if ((threadIdx.x & 31) == 0) {
        if (m0) atomicAdd(&s_next[0], (uint32_t)__popc(m0));
        if (m1) atomicAdd(&s_next[1], (uint32_t)__popc(m1));
    }
}

template <int ALG>
__device__ __forceinline__ uint32_t probe(const RegionArgs &a, uint32_t v) {
    return ALG == kBFS ? a.visited[v >> 5] : a.val[v];
}

#ifndef ASC_CLAIM_RED
#define ASC_CLAIM_RED 1
#endif
// Lowers val[v] to nv; true when this thread counts v into the next frontier.
// cur is the earlier probe: reached bits and values only ever grow / shrink,
// so a stale probe can only cost an extra atomic, never a missed update.
// BFS is level-synchronous: every update of an iteration writes the same
// level, so a thread whose probe found v unreached stores it and no atomicMin
// is needed (the result equals the atomicMin relaxation's fixpoint).
// With kClaimRed the atomics are fire-and-forget (no thread waits for a
// returned old value): two threads with stale probes may both store v's level
// (the same value) and both count v, so the per-region next-frontier counts
// are upper bounds. They only choose between list and bitmap walks and stop
// the loop when zero, which stays exact: a count is zero only when no thread
// set a bit. Otherwise the returned old bit decides, and counts are exact.
constexpr bool kClaimRed = ASC_CLAIM_RED != 0;
template <int ALG>
__device__ __forceinline__ bool lower(const RegionArgs &a, uint32_t v, uint32_t nv, uint32_t cur) {
    const uint32_t bit = 1u << (v & 31);
    if (ALG == kBFS) {
        if (nv == 0xffffffffu || (cur & bit)) return false;
        if (kClaimRed) atomicOr(&a.visited[v >> 5], bit);
        else if (atomicOr(&a.visited[v >> 5], bit) & bit) return false;
        a.val[v] = nv;
        atomicOr(&a.bitmap[v >> 5], bit);
        return true;
    }
    if (nv >= cur) return false;
    if (ALG == kSSSP && a.far_bits) {
        uint32_t old = atomicMin(&a.val[v], nv);
        if (nv >= old) return false;
        if (nv >= *a.thresh) {
            atomicOr(&a.far_bits[v >> 5], bit);  // waits until the threshold reaches it
            return false;
        }
        // now near: drop it from the far set, or a later promotion expands it twice
        if (a.far_bits[v >> 5] & bit) atomicAnd(&a.far_bits[v >> 5], ~bit);
    } else {
        // fire-and-forget: if another thread lowered v further since the probe,
        // it set v's bit too, so the next frontier is the same either way
        atomicMin(&a.val[v], nv);
    }
    if (kClaimRed) {
        atomicOr(&a.bitmap[v >> 5], bit);
        return true;
    }
    return (atomicOr(&a.bitmap[v >> 5], bit) & bit) == 0;
}

// Each thread handles kUnroll edges per pass: all column loads are issued
// first, then all destination-value loads, then the updates, so a thread keeps
// kUnroll independent reads in flight (on-demand column reads cross the host link).
// (measured with bit-packed edges at 8 CTAs per SM: 4 -> 65.7 GTEPS, 6 -> 64.3,
// 8 -> 62.2; more loads per thread spill at 32 registers)
#ifndef ASC_EXPAND_UNROLL
#define ASC_EXPAND_UNROLL 4
#endif
constexpr int kUnroll = ASC_EXPAND_UNROLL;

// Expands up to kBlock frontier vertices, one per thread (act = false where a
// thread has none): a block scan of their degrees lays the edges out as one
// range, which all threads walk kUnroll edges at a time.
template <int ALG, int WORDS>
__device__ void expand_vertices(const RegionArgs &a, bool act, uint32_t u, Smem &sm, uint32_t *s_next) {
    uint32_t deg = 0, start = 0, vu = 0;
    if (act && ASC_BAD(u >= a.V, 1, u)) act = false;
    if (act) {
        start = a.ptr[u];
        deg = a.ptr[u + 1] - start;
        if (deg > a.huge) {
            deg = 0;  // long lists are handled as segments
            act = false;
        }
        vu = a.val[u];
        if (a.frag) count_fragments(a.frag, start, deg);
    }
    uint32_t total;
    uint32_t excl = block_excl_scan(deg, total, sm.warp);
    sm.pref[threadIdx.x] = excl;
    sm.start[threadIdx.x] = start;
    sm.vu[threadIdx.x] = vu;
    if (threadIdx.x == 0) sm.pref[kBlock] = total;
    const uint32_t nact = __syncthreads_count(act);
    // each pass issues kUnroll column loads per thread before any update
    auto load_pass = [&](uint32_t base, uint32_t (&v)[kUnroll], uint32_t (&nv)[kUnroll]) {
#pragma unroll
        for (int k = 0; k < kUnroll; k++) {
            const uint32_t e = base + k * kBlock + threadIdx.x;
            v[k] = 0;
            nv[k] = 0xffffffffu;  // never lower than a value: no update
            if (e < total) {
                int lo = 0, hi = kBlock;
                while (hi - lo > 1) {
                    int mid = (lo + hi) >> 1;
                    if (sm.pref[mid] <= e) lo = mid;
                    else hi = mid;
                }
                load_edge<ALG, WORDS>(a, sm.vu[lo], (uint64_t)sm.start[lo] + (e - sm.pref[lo]), v[k], nv[k]);
                if (ASC_BAD(v[k] >= a.V, 2, v[k])) {
                    v[k] = 0;
                    nv[k] = 0xffffffffu;
                }
            }
        }
    };
    for (uint32_t base = 0; base < total; base += kUnroll * kBlock) {
        uint32_t v[kUnroll], nv[kUnroll], cur[kUnroll];
        load_pass(base, v, nv);
#pragma unroll
        for (int k = 0; k < kUnroll; k++) cur[k] = nv[k] != 0xffffffffu ? probe<ALG>(a, v[k]) : 0;
#pragma unroll
        for (int k = 0; k < kUnroll; k++) count_next(a, lower<ALG>(a, v[k], nv[k], cur[k]), v[k], s_next);
    }
    if (threadIdx.x == 0) {
        atomicAdd(&a.stats[a.region], (unsigned long long)total);
        atomicAdd(&a.stats[2 + a.region], (unsigned long long)nact);
    }
    __syncthreads();
}

// One bitmap word of a region walked through its bitmap, bits outside
// [dense_begin, dense_end) cleared (u0 is 32-aligned).
__device__ __forceinline__ uint32_t region_word(const RegionArgs &a, uint32_t u0) {
    if (u0 >= a.dense_end) return 0u;
    uint32_t word = a.bitmap_in[u0 >> 5];
    if (u0 < a.dense_begin) word &= 0xffffffffu << (a.dense_begin - u0);
    if (a.dense_end - u0 < 32u) word &= (1u << (a.dense_end - u0)) - 1u;
    return word;
}

// One tile of frontier vertices, one per thread: kBlock consecutive entries
// of the region's list, or (bitmap) kBlock consecutive vertex ids walked
// through the frontier bitmap (tiles start 32-aligned; a tile with no active
// vertex costs one bitmap read per warp).
template <int ALG, int WORDS>
__device__ __forceinline__ void expand_tile(const RegionArgs &a, uint32_t tile, uint32_t n_in, bool bitmap, Smem &sm,
                                            uint32_t *s_next) {
    bool act;
    uint32_t u;
    if (bitmap) {
        u = (a.dense_begin & ~31u) + tile * kBlock + threadIdx.x;
        act = (region_word(a, u & ~31u) >> (u & 31)) & 1u;
        if (!__syncthreads_or(act)) return;
    } else {
        const uint32_t i = tile * kBlock + threadIdx.x;
        act = i < n_in;
        u = act ? a.q_in[i] : 0;
    }
    expand_vertices<ALG, WORDS>(a, act, u, sm, s_next);
}

template <int ALG, int WORDS>
__device__ void expand_segment(const RegionArgs &a, uint64_t item, uint32_t *s_next) {
    const uint32_t u = (uint32_t)(item >> 32), k0 = (uint32_t)item;
    if (ASC_BAD(u >= a.V, 3, u)) return;
    const uint32_t b0 = a.ptr[u], e0 = a.ptr[u + 1];
    const uint64_t b = (uint64_t)b0 + (uint64_t)k0 * a.seg_len;
    const uint64_t e = min((uint64_t)e0, b + a.seg_len);
    const uint32_t n = (uint32_t)(e - b);
    const uint32_t vu = a.val[u];
    auto load_pass = [&](uint32_t base, uint32_t (&v)[kUnroll], uint32_t (&nv)[kUnroll]) {
#pragma unroll
        for (int k = 0; k < kUnroll; k++) {
            const uint32_t j = base + k * kBlock + threadIdx.x;
            v[k] = 0;
            nv[k] = 0xffffffffu;
            if (j < n) load_edge<ALG, WORDS>(a, vu, b + j, v[k], nv[k]);
            if (j < n && ASC_BAD(v[k] >= a.V, 2, v[k])) {
                v[k] = 0;
                nv[k] = 0xffffffffu;
            }
        }
    };
    for (uint32_t base = 0; base < n; base += kUnroll * kBlock) {
        uint32_t v[kUnroll], nv[kUnroll], cur[kUnroll];
        load_pass(base, v, nv);
#pragma unroll
        for (int k = 0; k < kUnroll; k++) cur[k] = nv[k] != 0xffffffffu ? probe<ALG>(a, v[k]) : 0;
#pragma unroll
        for (int k = 0; k < kUnroll; k++) count_next(a, lower<ALG>(a, v[k], nv[k], cur[k]), v[k], s_next);
    }
    if (threadIdx.x == 0) {
        atomicAdd(&a.stats[a.region], (unsigned long long)n);
        if (k0 == 0) atomicAdd(&a.stats[2 + a.region], 1ull);
        if (a.frag) count_fragments(a.frag, b, n);
    }
}

// Work of one region for the bitmap-built frontier: segments first, then a
// region whose frontier holds more than 1/dense_div of its vertices is walked
// in id order through its bitmap (its list was not built), kBlock ids per
// item, so the lists of neighbouring active vertices are read as one
// contiguous run; otherwise through its list, kBlock entries per item.
__device__ __forceinline__ void region_items_bits(const RegionArgs &a, uint32_t &n_in, uint32_t &nseg,
                                                  uint32_t &items, bool &bitmap) {
    const uint32_t range = a.dense_end - a.dense_begin;
    const uint32_t bits = a.cnt_in[6 + a.region];
    nseg = a.cnt_in[2 + a.region];
    bitmap = a.bitmap_in && a.dense_div && bits > range / a.dense_div;
    n_in = bitmap ? 0 : a.cnt_in[a.region];
    const uint32_t nvert = bitmap ? a.dense_end - (a.dense_begin & ~31u) : n_in;
    items = nseg + (nvert + kBlock - 1) / kBlock;
}

template <int ALG, int WORDS>
__device__ __forceinline__ void expand_item(const RegionArgs &a, uint32_t w, uint32_t n_in, uint32_t nseg,
                                            bool bitmap, Smem &sm, uint32_t *s_next) {
    if (w < nseg) expand_segment<ALG, WORDS>(a, a.seg_in[w], s_next);
    else expand_tile<ALG, WORDS>(a, w - nseg, n_in, bitmap, sm, s_next);
}

__device__ __forceinline__ void flush_next(const RegionArgs &a, uint32_t *s_next) {
    __syncthreads();
    if (threadIdx.x == 0) {
        if (s_next[0]) atomicAdd(&a.cnt_out[6], s_next[0]);
        if (s_next[1]) atomicAdd(&a.cnt_out[7], s_next[1]);
    }
}

template <int ALG, int WORDS>
__global__ void __launch_bounds__(kBlock, ASC_EXPAND_MIN_BLOCKS) expand_kernel(RegionArgs a) {
    if (ALG == kBFS && bottom_up_step(a)) return;
    __shared__ Smem sm;
    __shared__ uint32_t s_next[2];
    if (threadIdx.x < 2) s_next[threadIdx.x] = 0;
    uint32_t n_in, nseg, total;
    bool bitmap;
    region_items_bits(a, n_in, nseg, total, bitmap);
    for (;;) {
        if (threadIdx.x == 0) sm.work = atomicAdd(a.work, 1u);
        __syncthreads();
        const uint32_t w = sm.work;
        __syncthreads();
        if (w >= total) break;
        expand_item<ALG, WORDS>(a, w, n_in, nseg, bitmap, sm, s_next);
    }
    flush_next(a, s_next);
}

// Both regions in one launch. Work items alternate between the on-demand and
// the static region while both have items left, so every SM mixes HBM-bound
// static work with link-bound on-demand work; on-demand segments and tiles
// are handed out first within their region.
struct FusedArgs {
    RegionArgs r0, r1;
    uint32_t *work;
};

template <int ALG, int WORDS>
__global__ void __launch_bounds__(kBlock, ASC_EXPAND_MIN_BLOCKS) expand_fused_kernel(FusedArgs x) {
    if (ALG == kBFS && bottom_up_step(x.r0)) return;
    __shared__ Smem sm;
    __shared__ uint32_t s_next[2];
    if (threadIdx.x < 2) s_next[threadIdx.x] = 0;
    uint32_t n0, s0, i0, n1, s1, i1;
    bool m0, m1;
    region_items_bits(x.r0, n0, s0, i0, m0);
    region_items_bits(x.r1, n1, s1, i1, m1);
    const uint32_t m = min(i0, i1), total = i0 + i1;
    for (;;) {
        if (threadIdx.x == 0) sm.work = atomicAdd(x.work, 1u);
        __syncthreads();
        const uint32_t w = sm.work;
        __syncthreads();
        if (w >= total) break;
        bool od;
        uint32_t local;
        if (w < 2 * m) {
            od = (w & 1) == 0;
            local = w >> 1;
        } else {
            od = i1 > i0;
            local = m + (w - 2 * m);
        }
        if (od) expand_item<ALG, WORDS>(x.r1, local, n1, s1, m1, sm, s_next);
        else expand_item<ALG, WORDS>(x.r0, local, n0, s0, m0, sm, s_next);
    }
    flush_next(x.r0, s_next);
}

// Bottom-up BFS step (direction-optimizing BFS): every vertex not yet reached
// scans its in-edges, in source-id order, for a parent in this iteration's
// frontier and stops at the first one; a vertex found takes the parent's value
// + 1 (the level-synchronous top-down step gives every unreached vertex with a
// frontier in-neighbour the same value, so levels are identical) and joins the
// next frontier. When the frontier is a large part of the graph, most unreached
// vertices find a parent among their first in-edges, so the step reads far
// fewer edge bytes over the host link than expanding the frontier's out-lists.
// One warp per 32-vertex bitmap word, lane = vertex: the warp writes the
// word's reached and next-frontier bits whole. In-edges are read in place from
// pinned host memory, kBuUnroll per lane before any frontier probe.
#ifndef ASC_BU_UNROLL
#define ASC_BU_UNROLL 4
#endif
constexpr int kBuUnroll = ASC_BU_UNROLL;

// Words a warp takes per pass: all of their bitmap words, heads and frontier
// probes are loaded before any is used, so a warp keeps that many independent
// load chains in flight.
#ifndef ASC_BU_WORDS
#define ASC_BU_WORDS 4
#endif
constexpr int kBuWords = ASC_BU_WORDS;
// CTAs per SM the bottom-up kernel is compiled for; its grid is one wave of
// them. RMAT scale 24, 25% budget: 352.4 GTEPS at 8 (32 registers), 336.4 at 6
// (40), 303.8 at 4 (48); with 2 in-edges per scan step instead of 4, 351.0; with
// 2 words per pass, 335.6 (all at 6 except the first). At 8, 2 in-edges per scan
// step measured 330.6 against 343.5 for 4.
#ifndef ASC_BU_MIN_BLOCKS
#define ASC_BU_MIN_BLOCKS 8
#endif
constexpr int kBuMinBlocks = ASC_BU_MIN_BLOCKS;

__global__ void __launch_bounds__(kBlock, kBuMinBlocks) bottom_up_kernel(RegionArgs a, uint32_t nwords) {
    if (!bottom_up_step(a)) return;
    __shared__ uint32_t s_next[2];
    __shared__ unsigned long long s_scanned, s_examined;
    if (threadIdx.x < 2) s_next[threadIdx.x] = 0;
    if (threadIdx.x == 0) s_scanned = s_examined = 0;
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warps = gridDim.x * (kBlock / 32);
    unsigned long long scanned = 0, examined = 0;
    for (uint32_t w0 = kBuWords * (blockIdx.x * (kBlock / 32) + (threadIdx.x >> 5)); w0 < nwords;
         w0 += kBuWords * warps) {
        // vertices without in-edges can never be reached: about half of an
        // RMAT graph, nearly all of its unreachable vertices
        uint32_t vis[kBuWords], done[kBuWords];
#pragma unroll
        for (int k = 0; k < kBuWords; k++) {
            const bool in = w0 + k < nwords;
            vis[k] = in ? a.visited[w0 + k] : 0xffffffffu;
            done[k] = in ? vis[k] | a.in_none[w0 + k] : 0xffffffffu;
        }
        // the first in-edge is held in HBM, vertex-indexed (a coalesced read;
        // a vertex without in-edges holds its own id, never in the frontier):
        // most unreached vertices find their parent there and read nothing else
        uint32_t head[kBuWords];
        bool todo[kBuWords], hit[kBuWords];
#pragma unroll
        for (int k = 0; k < kBuWords; k++) {
            const uint32_t v = 32 * (w0 + k) + lane;
            todo[k] = done[k] != 0xffffffffu && v < a.V && !((done[k] >> lane) & 1u);
            head[k] = todo[k] && a.in_heads ? edge_word(a.in_heads, v, a.in_ebits) : 0u;
            if (ASC_BAD(head[k] >= a.V, 16, head[k])) head[k] = v;
        }
#pragma unroll
        for (int k = 0; k < kBuWords; k++)
            hit[k] = todo[k] && a.in_heads && ((a.bitmap_in[head[k] >> 5] >> (head[k] & 31)) & 1u);
#pragma unroll
        for (int k = 0; k < kBuWords; k++) {
            if (done[k] == 0xffffffffu) continue;  // the whole warp: nothing to look for in this word
            const uint32_t w = w0 + k, v = 32 * w + lane;
            examined += todo[k];
            uint32_t parent = hit[k] ? head[k] : 0xffffffffu;
            uint32_t h = 0, e = 0;
            if (todo[k] && !hit[k]) {
                h = a.in_ptr[v];
                e = a.in_ptr[v + 1];
                if (a.in_heads && h < e) h++;  // the head was in-edge h
            }
            if (parent == 0xffffffffu) {
                for (uint32_t i = h; i < e; i += kBuUnroll) {
                    uint32_t u[kBuUnroll];
                    bool in[kBuUnroll];
#pragma unroll
                    for (int q = 0; q < kBuUnroll; q++) {
                        u[q] = i + q < e ? edge_word(a.in_edges, (uint64_t)i + q, a.in_ebits) : 0xffffffffu;
                        if (u[q] != 0xffffffffu && ASC_BAD(u[q] >= a.V, 17, u[q])) u[q] = 0xffffffffu;
                    }
#pragma unroll
                    for (int q = 0; q < kBuUnroll; q++)
                        in[q] = u[q] != 0xffffffffu && ((a.bitmap_in[u[q] >> 5] >> (u[q] & 31)) & 1u);
                    int at = -1;
#pragma unroll
                    for (int q = kBuUnroll - 1; q >= 0; q--)
                        if (in[q]) at = q;
                    if (at >= 0) {
                        parent = u[at];
                        scanned += (i - h) + (uint32_t)at + 1;
                        break;
                    }
                }
                if (parent == 0xffffffffu) scanned += e - h;
            }
            const bool won = parent != 0xffffffffu;
            const unsigned found = __ballot_sync(kFull, won);
            // every frontier vertex holds the same value (the step is level-
            // synchronous): one lane reads its parent's, the warp shares it
            uint32_t nv = 0;
            if (found) {
                const int leader = __ffs(found) - 1;
                if ((int)lane == leader) nv = a.val[parent] + 1;
                nv = __shfl_sync(kFull, nv, leader);
            }
            if (won) a.val[v] = nv;
            if (lane == 0 && found) {
                a.visited[w] = vis[k] | found;
                a.bitmap[w] = found;
            }
            count_next(a, won, v, s_next);
        }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        scanned += __shfl_down_sync(kFull, scanned, d);
        examined += __shfl_down_sync(kFull, examined, d);
    }
    if (lane == 0 && scanned) atomicAdd(&s_scanned, scanned);
    if (lane == 0 && examined) atomicAdd(&s_examined, examined);
    flush_next(a, s_next);
    if (threadIdx.x == 0 && s_examined)
        atomicAdd((unsigned long long *)(a.stats + (CTL_BU_VERTS - CTL_STATS) / 2), s_examined);
    // in-edges are read in place from host memory (resident only on a graph
    // without a cap): the run's on-demand edges and its bottom-up edges
    if (threadIdx.x == 0 && s_scanned) {
        atomicAdd(&a.stats[a.in_resident ? 0 : 1], s_scanned);
        atomicAdd((unsigned long long *)(a.stats + (CTL_BU_EDGES - CTL_STATS) / 2), s_scanned);
    }
}

// Gather-and-copy comparison engine: expands on-demand edges that host
// threads gathered into a device staging buffer. Item i is (vertex, offset of
// its edges in the staging buffer, edge count, 1 for a vertex's first item);
// a warp takes an item, its lanes 32 edges at a time. Staged edges are plain
// words (WORDS 1: destination or packed destination/weight) or pairs (2).
struct StagedArgs {
    RegionArgs a;
    const uint32_t *stage;
    const uint32_t *items;
    uint32_t n_items;
};

template <int ALG, int WORDS>
__global__ void __launch_bounds__(kBlock) expand_staged_kernel(StagedArgs x) {
    __shared__ uint32_t s_next[2];
    if (threadIdx.x < 2) s_next[threadIdx.x] = 0;
    __syncthreads();
    const RegionArgs &a = x.a;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t i = warp; i < x.n_items; i += nwarps) {
        const uint32_t u = x.items[4 * i], off = x.items[4 * i + 1], len = x.items[4 * i + 2];
        const uint32_t vu = a.val[u];
        for (uint32_t j0 = 0; j0 < len; j0 += 32) {
            const uint32_t j = j0 + lane;
            uint32_t v = 0, nv = 0xffffffffu;
            if (j < len) {
                if (WORDS == 2) {
                    const uint2 e = reinterpret_cast<const uint2 *>(x.stage)[(uint64_t)off + j];
                    v = e.x;
                    nv = ALG == kSSSP ? vu + e.y : (ALG == kBFS ? vu + 1 : vu);
                } else {
                    const uint32_t e = x.stage[(uint64_t)off + j];
                    v = e >> a.wbits;
                    nv = ALG == kBFS ? vu + 1 : (ALG == kSSSP ? vu + (e & ((1u << a.wbits) - 1u)) : vu);
                }
            }
            const uint32_t cur = nv != 0xffffffffu ? probe<ALG>(a, v) : 0;
            count_next(a, lower<ALG>(a, v, nv, cur), v, s_next);
        }
        if (lane == 0) {
            atomicAdd(&a.stats[1], (unsigned long long)len);
            if (x.items[4 * i + 3]) atomicAdd(&a.stats[3], 1ull);
        }
    }
    flush_next(a, s_next);
}

// Builds the next frontier from its bitmap (one thread per 32-vertex word):
// vertices with long lists become segment items; the others are appended to
// their region's list only when that region will be walked as a list (warp
// scan of the per-word counts, one atomic per warp). cnt_out[6..7] hold the
// region bit counts the expansion flushed; cnt_out[0..3] receive the lists.
__global__ void build_frontier_kernel(RegionArgs a, const uint32_t *next_bits, uint32_t nwords) {
    const int lane = threadIdx.x & 31;
    const uint32_t range0 = a.S, range1 = a.V - a.S;
    const bool list0 = !(a.dense_div && a.cnt_out[6] > range0 / a.dense_div);
    const bool list1 = !(a.dense_div && a.cnt_out[7] > range1 / a.dense_div);
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < nwords; base += stride) {
        const uint32_t w = base + threadIdx.x;
        uint32_t word = 0, hw = 0;
        if (w < nwords) {
            word = next_bits[w];
            hw = word & a.huge_bits[w];
        }
        // long lists: one thread per vertex appends its segments (rare)
        while (hw) {
            const int b = __ffs(hw) - 1;
            hw &= hw - 1;
            const uint32_t v = 32 * w + b;
            const uint32_t deg = a.ptr[v + 1] - a.ptr[v];
            const uint32_t nseg = (deg + a.seg_len - 1) / a.seg_len;
            const bool od = v >= a.S;
            const uint32_t sb = atomicAdd(&a.cnt_out[2 + od], nseg);
            if (ASC_BAD((uint64_t)sb + nseg > (od ? a.segcap_ondemand : a.segcap_static), 13, sb)) continue;
            uint64_t *dst = a.seg_out + (od ? a.segcap_static : 0) + sb;
            for (uint32_t k = 0; k < nseg; k++) dst[k] = ((uint64_t)v << 32) | k;
        }
        if (w < nwords) word &= ~a.huge_bits[w];
        // region split of this word: bits of vertices below S are static
        uint32_t smask;
        const uint32_t v0 = 32 * w;
        if (v0 + 32 <= a.S) smask = 0xffffffffu;
        else if (v0 >= a.S) smask = 0;
        else smask = (1u << (a.S - v0)) - 1u;
        const uint32_t w0 = list0 ? (word & smask) : 0, w1 = list1 ? (word & ~smask) : 0;
        const uint32_t c0 = __popc(w0), c1 = __popc(w1);
        uint32_t i0 = c0, i1 = c1;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y0 = __shfl_up_sync(kFull, i0, d), y1 = __shfl_up_sync(kFull, i1, d);
            if (lane >= d) {
                i0 += y0;
                i1 += y1;
            }
        }
        const uint32_t t0 = __shfl_sync(kFull, i0, 31), t1 = __shfl_sync(kFull, i1, 31);
        uint32_t b0 = 0, b1 = 0;
        if (lane == 0) {
            if (t0) b0 = atomicAdd(&a.cnt_out[0], t0);
            if (t1) b1 = atomicAdd(&a.cnt_out[1], t1);
        }
        b0 = __shfl_sync(kFull, b0, 0) + i0 - c0;
        b1 = __shfl_sync(kFull, b1, 0) + i1 - c1;
        uint32_t x = w0;
        while (x) {
            const int b = __ffs(x) - 1;
            x &= x - 1;
            if (!ASC_BAD(b0 >= a.S, 14, b0)) a.q_out[b0] = v0 + b;
            b0++;
        }
        x = w1;
        while (x) {
            const int b = __ffs(x) - 1;
            x &= x - 1;
            if (!ASC_BAD(a.S + b1 >= a.V, 15, b1)) a.q_out[a.S + b1] = v0 + b;
            b1++;
        }
    }
}

// SSSP near-far, step 1: when the pass left the near frontier empty, the
// smallest distance in the far set (atomicMin into the control block).
__global__ void far_min_kernel(RegionArgs a, uint32_t nwords, uint32_t *minfar) {
    if (a.cnt_out[6] | a.cnt_out[7]) return;
    uint32_t m = 0xffffffffu;
    for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < nwords; w += gridDim.x * blockDim.x) {
        uint32_t word = a.far_bits[w];
        while (word) {
            const int b = __ffs(word) - 1;
            word &= word - 1;
            m = min(m, a.val[32 * w + b]);
        }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) m = min(m, __shfl_down_sync(kFull, m, d));
    if ((threadIdx.x & 31) == 0 && m != 0xffffffffu) atomicMin(minfar, m);
}

// SSSP near-far, step 2: the threshold moves to (min far distance + delta) and
// every far vertex below it joins the next frontier (bit and region count).
__global__ void far_promote_kernel(RegionArgs a, uint32_t nwords, const uint32_t *minfar, uint32_t *thresh,
                                   uint32_t delta) {
    if (a.cnt_out[6] | a.cnt_out[7]) return;
    const uint32_t mf = *minfar;
    if (mf == 0xffffffffu) return;
    const uint32_t t = mf > 0xffffffffu - delta ? 0xffffffffu : mf + delta;
    if (blockIdx.x == 0 && threadIdx.x == 0) *thresh = t;
    uint32_t n0 = 0, n1 = 0;
    for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < nwords; w += gridDim.x * blockDim.x) {
        const uint32_t word = a.far_bits[w];
        if (!word) continue;
        uint32_t x = word, promo = 0;
        while (x) {
            const int b = __ffs(x) - 1;
            x &= x - 1;
            if (a.val[32 * w + b] < t) promo |= 1u << b;
        }
        if (!promo) continue;
        a.far_bits[w] = word & ~promo;
        a.bitmap[w] |= promo;
        const uint32_t v0 = 32 * w;
        const uint32_t smask = v0 + 32 <= a.S ? 0xffffffffu : (v0 >= a.S ? 0 : (1u << (a.S - v0)) - 1u);
        n0 += __popc(promo & smask);
        n1 += __popc(promo & ~smask);
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        n0 += __shfl_down_sync(kFull, n0, d);
        n1 += __shfl_down_sync(kFull, n1, d);
    }
    if ((threadIdx.x & 31) == 0) {
        if (n0) atomicAdd(&a.cnt_out[6], n0);
        if (n1) atomicAdd(&a.cnt_out[7], n1);
    }
}

// First frontier of a traversal: one source, or every vertex (CC); sets its
// bits and region counts in the parity-0 block.
__global__ void seed_bits_kernel(RegionArgs a, uint32_t src, uint32_t all, uint32_t nwords) {
    if (!all) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            a.bitmap[src >> 5] |= 1u << (src & 31);
            if (a.visited) a.visited[src >> 5] |= 1u << (src & 31);
            a.cnt_out[src < a.S ? 6 : 7] = 1;
        }
        return;
    }
    uint32_t n0 = 0, n1 = 0;
    for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < nwords; w += gridDim.x * blockDim.x) {
        const uint32_t v0 = 32 * w;
        uint32_t m = v0 + 32 <= a.V ? 0xffffffffu : (v0 < a.V ? (1u << (a.V - v0)) - 1u : 0);
        a.bitmap[w] = m;
        uint32_t smask = v0 + 32 <= a.S ? 0xffffffffu : (v0 >= a.S ? 0 : (1u << (a.S - v0)) - 1u);
        n0 += __popc(m & smask);
        n1 += __popc(m & ~smask);
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        n0 += __shfl_down_sync(kFull, n0, d);
        n1 += __shfl_down_sync(kFull, n1, d);
    }
    if ((threadIdx.x & 31) == 0) {
        if (n0) atomicAdd(&a.cnt_out[6], n0);
        if (n1) atomicAdd(&a.cnt_out[7], n1);
    }
}

// End of one CUDA-graph loop body (two iterations: parity 0 then parity 1).
// Block 1 holds what the first half produced (the second half's input),
// block 0 what the second half produced. Keeps looping while block 0 is
// non-empty, counts the iterations that had input, and stops at the cap.
__global__ void loop_cond_kernel(cudaGraphConditionalHandle h, uint32_t *ctl, uint32_t cap) {
    const uint32_t *b0 = ctl, *b1 = ctl + CTL_BLOCK;
    const bool second = (b1[6] | b1[7]) != 0;
    bool more = (b0[6] | b0[7]) != 0;
    const uint32_t it = ctl[CTL_ITERS] + 1 + (second ? 1 : 0);
    ctl[CTL_ITERS] = it;
    ctl[CTL_BODIES] += 1;
    if (more && it >= cap) {
        ctl[CTL_TIMEOUT] = 1;
        more = false;
    }
    cudaGraphSetConditional(h, more ? 1u : 0u);
}

template <int ALG>
__global__ void init_values_kernel(uint32_t *val, uint32_t V, uint32_t src) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < V; i += gridDim.x * blockDim.x)
        val[i] = ALG == kCC ? i : (i == src ? 1u : V + 1u);
}

// Reached vertices and the sum of their out-degrees (TEPS numerator).
__global__ void reached_kernel(const uint32_t *val, const uint32_t *ptr, uint32_t V, unsigned long long *out) {
    unsigned long long cnt = 0, edges = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < V; i += gridDim.x * blockDim.x)
        if (val[i] < V + 1) {
            cnt++;
            edges += ptr[i + 1] - ptr[i];
        }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        cnt += __shfl_down_sync(kFull, cnt, d);
        edges += __shfl_down_sync(kFull, edges, d);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&out[0], cnt);
        atomicAdd(&out[1], edges);
    }
}

// BFS: reached vertices are the reached-vertex bitmap's bits (no level read).
// A warp takes kReachedWords consecutive 32-vertex words at a time, lane =
// vertex: all of their bitmap words and then all the offsets of their reached
// vertices are loaded before any is summed, so each warp keeps several
// independent loads in flight instead of a chain per word.
constexpr int kReachedWords = 4;

__global__ void reached_bits_kernel(const uint32_t *visited, const uint32_t *ptr, uint32_t V, uint32_t nwords,
                                    unsigned long long *out) {
    unsigned long long cnt = 0, edges = 0;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t w0 = kReachedWords * (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)); w0 < nwords;
         w0 += kReachedWords * warps) {
        uint32_t bits[kReachedWords], lo[kReachedWords], hi[kReachedWords];
#pragma unroll
        for (int k = 0; k < kReachedWords; k++) bits[k] = w0 + k < nwords ? visited[w0 + k] : 0u;
#pragma unroll
        for (int k = 0; k < kReachedWords; k++) {
            const uint32_t v = 32 * (w0 + k) + lane;
            const bool in = ((bits[k] >> lane) & 1u) && v < V;
            lo[k] = in ? ptr[v] : 0u;
            hi[k] = in ? ptr[v + 1] : 0u;
            cnt += in;
        }
#pragma unroll
        for (int k = 0; k < kReachedWords; k++) edges += hi[k] - lo[k];
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        cnt += __shfl_down_sync(kFull, cnt, d);
        edges += __shfl_down_sync(kFull, edges, d);
    }
    if (lane == 0 && (cnt | edges)) {
        atomicAdd(&out[0], cnt);
        atomicAdd(&out[1], edges);
    }
}

// ------------------------------------------------------------- PageRank -----
//
// Ranks are FP64 in every mode; the contributions rank/outDeg that the edges
// carry are T (FP64, or FP32 for the precision pattern: 4 bytes per edge
// gather, and half the L2 footprint of the contribution array).
//
// How the sums of contributions accumulate (PrAcc<T>): FP64 contributions add
// in FP64, where the order of the atomics changes a sum by about 1e-16
// relative, far below the stop tolerance. FP32 contributions add in FP32 only
// in a fixed order (a thread's own edges, then a warp's segmented shuffle
// tree), and every partial that meets others through an atomic (across warps,
// tiles, segments or a scatter's edges) adds exactly, as 64-bit fixed point
// with 62 fraction bits. Integer addition is associative, so the atomics'
// order cannot change a sum: every pass recomputes bit-identical sums from
// identical contributions, and the FP64 L1 residual falls to the stop
// tolerance. (FP32 atomics in any order floor it near 1.5e-8 at RMAT scale
// 25, so that such a run always took the pass cap.) A sum is at most the total
// rank (1 in standard mode), so two integer bits are enough; a partial below
// 2^-62 rounds to the grid (an absolute error below 1.1e-19 each).
template <typename T>
struct PrAcc;
template <>
struct PrAcc<double> {
    typedef double type;
    static __device__ __forceinline__ double from(double x) { return x; }
    static __device__ __forceinline__ double value(double a) { return a; }
};
template <>
struct PrAcc<float> {
    typedef unsigned long long type;
    static __device__ __forceinline__ unsigned long long from(float x) { return __float2ull_rn(x * 0x1p62f); }
    static __device__ __forceinline__ double value(unsigned long long a) { return __ull2double_rn(a) * 0x1p-62; }
};

template <typename T>
struct PrArgs {
    typedef typename PrAcc<T>::type Acc;
    RegionArgs r;           // lists, segments, counts (pull over in-edges)
    const uint32_t *outdeg;
    double *rank;
    const T *c_old;
    T *c_new;
    Acc *sum;               // partial sums of segmented vertices
    double damping;
    const double *dangling_prev;   // std mode: dangling mass of the previous pass
    double *acc;            // std mode: [0] residual, [1] dangling of this pass
};

// The update of one vertex from its summed contributions s (FP64):
// reference mode prKernel_Opt (gpu_kernels.cuh:533-552), standard mode
// (1 - d) / V + d * (dangling mass / V + s) with the L1 residual and the
// dangling mass of this pass accumulated in FP64.
template <typename T>
__device__ __forceinline__ bool pr_update(double *rank, const T *c_old, T *c_new, uint32_t v, uint32_t od, double s,
                                          bool ref, double damping, double V, const double *dangling_prev,
                                          double &res, double &dang) {
    if (ref) {
        const double r = rank[v];
        const double t = fma(0.85, s, 0.15);
        const double diff = t > r ? t - r : r - t;
        if (diff > 0.001) {
            rank[v] = t;
            c_new[v] = od ? (T)(t / (double)od) : (T)0;
            return true;
        }
        c_new[v] = c_old[v];
        return false;
    }
    const double base = (1.0 - damping) / V + damping * (*dangling_prev) / V;
    const double r = rank[v];
    const double rn = base + damping * s;
    res += fabs(rn - r);
    if (od == 0) dang += rn;
    rank[v] = rn;
    c_new[v] = od ? (T)(rn / (double)od) : (T)0;
    return false;
}

template <typename T, bool REF>
__device__ __forceinline__ bool pr_apply(const PrArgs<T> &p, uint32_t v, double s, double &res, double &dang) {
    return pr_update<T>(p.rank, p.c_old, p.c_new, v, p.outdeg[v], s, REF, p.damping, (double)p.r.V,
                        p.dangling_prev, res, dang);
}

template <typename T>
__device__ __forceinline__ void block_reduce2_atomic(double a, double b, double *out, double *s_buf) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        a += __shfl_down_sync(kFull, a, d);
        b += __shfl_down_sync(kFull, b, d);
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        s_buf[2 * w] = a;
        s_buf[2 * w + 1] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double x = 0, y = 0;
        for (int i = 0; i < kWarps; i++) {
            x += s_buf[2 * i];
            y += s_buf[2 * i + 1];
        }
        if (x != 0) atomicAdd(&out[0], x);
        if (y != 0) atomicAdd(&out[1], y);
    }
    __syncthreads();
}

// Edges per thread per pass of the PageRank pull (all reads issued first).
#ifndef ASC_PR_UNROLL
#define ASC_PR_UNROLL 4
#endif
constexpr int kPrUnroll = ASC_PR_UNROLL;
// Edge words a pull tile copies into shared memory per chunk (8 KB).
#ifndef ASC_PR_STAGE_WORDS
#define ASC_PR_STAGE_WORDS 2048
#endif
constexpr uint32_t kPrStageWords = ASC_PR_STAGE_WORDS;

template <typename T>
struct PrSmem {
    alignas(16) uint32_t stage[kPrStageWords];
    uint32_t pref[kBlock + 1];
    uint32_t start[kBlock];
    uint32_t warp[kWarps + 1];
    typename PrAcc<T>::type sum[kBlock];
    double red[2 * kWarps];
    uint32_t work;
};

// Sums the in-edge contributions of a standard-PageRank tile (consecutive
// vertices, no long list, so their in-edges are one range [E0, E0 + total),
// E0 = the first vertex's offset) with the range read through shared memory:
// the CTA copies kPrStageWords edge words at a time with 16-byte loads, so
// the host link serves runs of several KB per tile instead of one 128-byte
// line per warp load, then every thread decodes its edges from shared memory
// and gathers their contributions, kPrUnroll edges in flight. The summation
// order is a fixed function of the range (same partials every pass).
template <typename T>
__device__ void pr_vertices_staged(const PrArgs<T> &p, uint32_t total, PrSmem<T> &sm) {
    const RegionArgs &a = p.r;
    const int lane = threadIdx.x & 31;
    const uint32_t eb = a.ebits;
    const uint64_t E0 = sm.start[0];
    uint4 *st4 = reinterpret_cast<uint4 *>(sm.stage);
    for (uint32_t c0 = 0; c0 < total;) {
        // words [w_lo, w_end): edges [c0, c1) of the tile, w_lo 16-byte aligned
        const uint64_t w_lo = (((E0 + c0) * eb) >> 5) & ~3ull;
        const uint64_t cap_edges = (w_lo + kPrStageWords) * 32 / eb;  // edges ending in the chunk
        const uint32_t c1 = (uint32_t)min((uint64_t)total, cap_edges - E0);
        const uint64_t w_end = ((E0 + c1) * eb + 31) >> 5;
        const uint32_t nq = (uint32_t)((w_end - w_lo + 3) >> 2);
        for (uint32_t i = threadIdx.x; i < nq; i += kBlock) {
            const uint64_t w = w_lo + 4ull * i;
            uint4 q;
            if (w + 4 <= a.edge_words) {
                q = __ldg(reinterpret_cast<const uint4 *>(a.edges + w));
            } else {  // the buffer's last words
                q.x = w < a.edge_words ? __ldg(a.edges + w) : 0u;
                q.y = w + 1 < a.edge_words ? __ldg(a.edges + w + 1) : 0u;
                q.z = w + 2 < a.edge_words ? __ldg(a.edges + w + 2) : 0u;
                q.w = 0u;
            }
            st4[i] = q;
        }
        __syncthreads();
        const uint64_t bit0 = w_lo * 32;
        for (uint32_t base = c0; base < c1; base += kPrUnroll * kBlock) {
            T x[kPrUnroll];
            int owner[kPrUnroll];
            uint32_t srcv[kPrUnroll];
#pragma unroll
            for (int k = 0; k < kPrUnroll; k++) {
                const uint32_t e = base + k * kBlock + threadIdx.x;
                owner[k] = -1 - lane;  // distinct per invalid lane
                srcv[k] = 0xffffffffu;
                if (e < c1) {
                    int lo = 0, hi = kBlock;
                    while (hi - lo > 1) {
                        int mid = (lo + hi) >> 1;
                        if (sm.pref[mid] <= e) lo = mid;
                        else hi = mid;
                    }
                    owner[k] = lo;
                    const uint32_t bit = (uint32_t)((E0 + e) * eb - bit0);
                    const uint32_t wi = bit >> 5, sh = bit & 31u;
                    uint32_t v = sm.stage[wi] >> sh;
                    if (eb < 32) {
                        if (sh + eb > 32) v |= sm.stage[wi + 1] << (32 - sh);
                        v &= (1u << eb) - 1u;
                    }
                    srcv[k] = v;
                    if (ASC_BAD(srcv[k] >= a.V, 22, srcv[k])) {
                        srcv[k] = 0xffffffffu;
                        owner[k] = -1 - lane;
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < kPrUnroll; k++) x[k] = srcv[k] != 0xffffffffu ? p.c_old[srcv[k]] : (T)0;
#pragma unroll
            for (int k = 0; k < kPrUnroll; k++) {
                T xs = x[k];
                const int ow = owner[k];
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    T y = __shfl_down_sync(kFull, xs, d);
                    int oy = __shfl_down_sync(kFull, ow, d);
                    if (lane + d < 32 && oy == ow) xs += y;
                }
                int oprev = __shfl_up_sync(kFull, ow, 1);
                if (ow >= 0 && (lane == 0 || oprev != ow)) atomicAdd(&sm.sum[ow], PrAcc<T>::from(xs));
            }
        }
        __syncthreads();  // the stage is rewritten by the next chunk
        c0 = c1;
    }
}

// Reference mode walks the active set like a traversal frontier (list, or
// the bitmap in id order when dense) and a vertex that stays active sets its
// bit in the next bitmap; standard mode walks every vertex of the region.
template <typename T, bool REF>
__device__ void pr_vertices(const PrArgs<T> &p, bool valid, uint32_t u, PrSmem<T> &sm, uint32_t *s_next) {
    typedef typename PrAcc<T>::type Acc;
    const RegionArgs &a = p.r;
    uint32_t deg = 0, start = 0;
    bool huge = false;
    if (valid) {
        start = a.ptr[u];
        deg = a.ptr[u + 1] - start;
        huge = deg > a.huge;
        if (huge) deg = 0;
    }
    uint32_t total;
    uint32_t excl = block_excl_scan(deg, total, sm.warp);
    sm.pref[threadIdx.x] = excl;
    sm.start[threadIdx.x] = start;
    sm.sum[threadIdx.x] = (Acc)0;
    if (threadIdx.x == 0) sm.pref[kBlock] = total;
    const uint32_t nact = __syncthreads_count(valid && !huge);
    const int lane = threadIdx.x & 31;
    // kPrUnroll edges per thread per pass (edge k of a pass is edge
    // base + k * kBlock + thread): every source id is loaded, then every
    // contribution gathered, before any is summed, so a thread has kPrUnroll
    // reads in flight instead of one
    const bool staged = !REF && a.stage_edges && !__syncthreads_or(valid && huge);
    if (staged) pr_vertices_staged<T>(p, total, sm);
    for (uint32_t base = 0; !staged && base < total; base += kPrUnroll * kBlock) {
        T x[kPrUnroll];
        int owner[kPrUnroll];
        uint32_t srcv[kPrUnroll];
#pragma unroll
        for (int k = 0; k < kPrUnroll; k++) {
            const uint32_t e = base + k * kBlock + threadIdx.x;
            owner[k] = -1 - lane;  // distinct per invalid lane
            srcv[k] = 0xffffffffu;
            if (e < total) {
                int lo = 0, hi = kBlock;
                while (hi - lo > 1) {
                    int mid = (lo + hi) >> 1;
                    if (sm.pref[mid] <= e) lo = mid;
                    else hi = mid;
                }
                owner[k] = lo;
                srcv[k] = edge_word(a.edges, (uint64_t)sm.start[lo] + (e - sm.pref[lo]), a.ebits);
                if (ASC_BAD(srcv[k] >= a.V, 21, srcv[k])) {
                    srcv[k] = 0xffffffffu;
                    owner[k] = -1 - lane;
                }
            }
        }
#pragma unroll
        for (int k = 0; k < kPrUnroll; k++) x[k] = srcv[k] != 0xffffffffu ? p.c_old[srcv[k]] : (T)0;
#pragma unroll
        for (int k = 0; k < kPrUnroll; k++) {
            // segmented suffix sum over lanes with the same owner (owners
            // ascend with the lane; a fixed shuffle tree, so the same edges
            // give the same partial every pass)
            T xs = x[k];
            const int ow = owner[k];
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                T y = __shfl_down_sync(kFull, xs, d);
                int oy = __shfl_down_sync(kFull, ow, d);
                if (lane + d < 32 && oy == ow) xs += y;
            }
            int oprev = __shfl_up_sync(kFull, ow, 1);
            if (ow >= 0 && (lane == 0 || oprev != ow)) atomicAdd(&sm.sum[ow], PrAcc<T>::from(xs));
        }
    }
    __syncthreads();
    double res = 0, dang = 0;
    bool won = false;
    if (valid && !huge) won = pr_apply<T, REF>(p, u, PrAcc<T>::value(sm.sum[threadIdx.x]), res, dang);
    if (REF) {
        if (won) atomicOr(&a.bitmap[u >> 5], 1u << (u & 31));
        count_next(a, won, u, s_next);
    } else {
        block_reduce2_atomic<T>(res, dang, p.acc, sm.red);
    }
    if (threadIdx.x == 0) {
        atomicAdd(&a.stats[a.region], (unsigned long long)total);
        atomicAdd(&a.stats[2 + a.region], (unsigned long long)nact);
    }
    __syncthreads();
}

template <typename T, bool REF>
__device__ __forceinline__ void pr_tile(const PrArgs<T> &p, uint32_t tile, uint32_t n_in, int mode, PrSmem<T> &sm,
                                        uint32_t *s_next) {
    const RegionArgs &a = p.r;
    const uint32_t i = tile * kBlock + threadIdx.x;
    bool valid;
    uint32_t u = 0;
    if (mode == kList) {
        valid = i < n_in;
        if (valid) u = a.q_in[i];
    } else {
        u = a.dense_begin + i;
        valid = u < a.dense_end;
    }
    pr_vertices<T, REF>(p, valid, u, sm, s_next);
}

template <typename T, bool REF>
__device__ void pr_bitmap_tile(const PrArgs<T> &p, uint32_t tile, PrSmem<T> &sm, uint32_t *s_next) {
    const uint32_t u = (p.r.dense_begin & ~31u) + tile * kBlock + threadIdx.x;
    const bool valid = (region_word(p.r, u & ~31u) >> (u & 31)) & 1u;
    if (__syncthreads_or(valid)) pr_vertices<T, REF>(p, valid, u, sm, s_next);
}

template <typename T>
__device__ void pr_segment(const PrArgs<T> &p, uint64_t item, PrSmem<T> &sm) {
    typedef typename PrAcc<T>::type Acc;
    const RegionArgs &a = p.r;
    const uint32_t u = (uint32_t)(item >> 32), k = (uint32_t)item;
    const uint32_t b0 = a.ptr[u], e0 = a.ptr[u + 1];
    const uint64_t b = (uint64_t)b0 + (uint64_t)k * a.seg_len;
    const uint64_t e = min((uint64_t)e0, b + a.seg_len);
    const uint32_t n = (uint32_t)(e - b);
    T x = (T)0;  // this thread's edges in order, then a fixed warp tree
    if (a.stage_edges) {
        // the segment's range through shared memory, as a staged tile: thread
        // t still adds edges t, t + kBlock, ... in order
        const uint32_t eb = a.ebits;
        uint4 *st4 = reinterpret_cast<uint4 *>(sm.stage);
        for (uint32_t c0 = 0; c0 < n;) {
            const uint64_t w_lo = (((b + c0) * eb) >> 5) & ~3ull;
            const uint64_t cap_edges = (w_lo + kPrStageWords) * 32 / eb;
            const uint32_t c1 = (uint32_t)min((uint64_t)n, cap_edges - b);
            const uint64_t w_end = ((b + c1) * eb + 31) >> 5;
            const uint32_t nq = (uint32_t)((w_end - w_lo + 3) >> 2);
            for (uint32_t i = threadIdx.x; i < nq; i += kBlock) {
                const uint64_t w = w_lo + 4ull * i;
                uint4 q;
                if (w + 4 <= a.edge_words) {
                    q = __ldg(reinterpret_cast<const uint4 *>(a.edges + w));
                } else {
                    q.x = w < a.edge_words ? __ldg(a.edges + w) : 0u;
                    q.y = w + 1 < a.edge_words ? __ldg(a.edges + w + 1) : 0u;
                    q.z = w + 2 < a.edge_words ? __ldg(a.edges + w + 2) : 0u;
                    q.w = 0u;
                }
                st4[i] = q;
            }
            __syncthreads();
            const uint64_t bit0 = w_lo * 32;
            const uint32_t first = c0 + ((threadIdx.x + kBlock - c0 % kBlock) % kBlock);
            for (uint32_t j0 = first; j0 < c1; j0 += kPrUnroll * kBlock) {
                uint32_t sv[kPrUnroll];
#pragma unroll
                for (int k = 0; k < kPrUnroll; k++) {
                    const uint32_t j = j0 + k * kBlock;
                    sv[k] = 0xffffffffu;
                    if (j < c1) {
                        const uint32_t bit = (uint32_t)((b + j) * eb - bit0);
                        const uint32_t wi = bit >> 5, sh = bit & 31u;
                        uint32_t v = sm.stage[wi] >> sh;
                        if (eb < 32) {
                            if (sh + eb > 32) v |= sm.stage[wi + 1] << (32 - sh);
                            v &= (1u << eb) - 1u;
                        }
                        sv[k] = ASC_BAD(v >= a.V, 23, v) ? 0xffffffffu : v;
                    }
                }
                T c[kPrUnroll];
#pragma unroll
                for (int k = 0; k < kPrUnroll; k++) c[k] = sv[k] != 0xffffffffu ? p.c_old[sv[k]] : (T)0;
#pragma unroll
                for (int k = 0; k < kPrUnroll; k++)
                    if (sv[k] != 0xffffffffu) x += c[k];
            }
            __syncthreads();
            c0 = c1;
        }
    }
    for (uint32_t j0 = threadIdx.x; !a.stage_edges && j0 < n; j0 += kPrUnroll * kBlock) {
        // kPrUnroll loads in flight, added in edge order
        uint32_t sv[kPrUnroll];
#pragma unroll
        for (int k = 0; k < kPrUnroll; k++) {
            const uint32_t j = j0 + k * kBlock;
            sv[k] = j < n ? edge_word(a.edges, b + j, a.ebits) : 0xffffffffu;
            if (sv[k] != 0xffffffffu && ASC_BAD(sv[k] >= a.V, 21, sv[k])) sv[k] = 0xffffffffu;
        }
        T c[kPrUnroll];
#pragma unroll
        for (int k = 0; k < kPrUnroll; k++) c[k] = sv[k] != 0xffffffffu ? p.c_old[sv[k]] : (T)0;
#pragma unroll
        for (int k = 0; k < kPrUnroll; k++)
            if (sv[k] != 0xffffffffu) x += c[k];
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) x += __shfl_down_sync(kFull, x, d);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sm.sum[w] = PrAcc<T>::from(x);
    __syncthreads();
    if (threadIdx.x == 0) {
        Acc s = (Acc)0;
        for (int i = 0; i < kWarps; i++) s += sm.sum[i];
        atomicAdd(&p.sum[u], s);
        atomicAdd(&a.stats[a.region], (unsigned long long)n);
        if (k == 0) atomicAdd(&a.stats[2 + a.region], 1ull);
    }
    __syncthreads();
}

template <typename T, bool REF>
__global__ void __launch_bounds__(kBlock, ASC_PR_MIN_BLOCKS) pr_pull_kernel(PrArgs<T> p) {
    __shared__ PrSmem<T> sm;
    __shared__ uint32_t s_next[2];
    if (threadIdx.x < 2) s_next[threadIdx.x] = 0;
    const RegionArgs &a = p.r;
    uint32_t n_in, nseg, total;
    bool bitmap = false;
    if (REF) {
        region_items_bits(a, n_in, nseg, total, bitmap);
    } else {
        n_in = 0;
        nseg = a.cnt_in[2 + a.region];
        total = nseg + (a.dense_end - a.dense_begin + kBlock - 1) / kBlock;
    }
    for (;;) {
        if (threadIdx.x == 0) sm.work = atomicAdd(a.work, 1u);
        __syncthreads();
        const uint32_t w = sm.work;
        __syncthreads();
        if (w >= total) break;
        if (w < nseg) pr_segment<T>(p, a.seg_in[w], sm);
        else if (REF && bitmap) pr_bitmap_tile<T, REF>(p, w - nseg, sm, s_next);
        else pr_tile<T, REF>(p, w - nseg, n_in, REF ? kList : kRange, sm, s_next);
    }
    if (REF) flush_next(a, s_next);
}

// Work items of one region for the pull pass (reference mode: its frontier;
// standard mode: every vertex of the region, long lists as segments).
template <bool REF>
__device__ __forceinline__ void pr_items(const RegionArgs &a, uint32_t &n_in, uint32_t &nseg, uint32_t &total,
                                         bool &bitmap) {
    bitmap = false;
    if (REF) {
        region_items_bits(a, n_in, nseg, total, bitmap);
    } else {
        n_in = 0;
        nseg = a.cnt_in[2 + a.region];
        total = nseg + (a.dense_end - a.dense_begin + kBlock - 1) / kBlock;
    }
}

template <typename T, bool REF>
__device__ __forceinline__ void pr_item(const PrArgs<T> &p, uint32_t w, uint32_t n_in, uint32_t nseg, bool bitmap,
                                        PrSmem<T> &sm, uint32_t *s_next) {
    if (w < nseg) pr_segment<T>(p, p.r.seg_in[w], sm);
    else if (REF && bitmap) pr_bitmap_tile<T, REF>(p, w - nseg, sm, s_next);
    else pr_tile<T, REF>(p, w - nseg, n_in, REF ? kList : kRange, sm, s_next);
}

// Both regions of a pull pass in one launch, items alternating between the
// on-demand and the static region while both have some (as the traversal's
// fused expansion), so every SM overlaps host-link reads with HBM reads.
template <typename T, bool REF>
__global__ void __launch_bounds__(kBlock, ASC_PR_MIN_BLOCKS) pr_pull_fused_kernel(PrArgs<T> p0, PrArgs<T> p1) {
    __shared__ PrSmem<T> sm;
    __shared__ uint32_t s_next[2];
    if (threadIdx.x < 2) s_next[threadIdx.x] = 0;
    uint32_t n0, s0, i0, n1, s1, i1;
    bool b0, b1;
    pr_items<REF>(p0.r, n0, s0, i0, b0);
    pr_items<REF>(p1.r, n1, s1, i1, b1);
    const uint32_t m = min(i0, i1), total = i0 + i1;
    for (;;) {
        if (threadIdx.x == 0) sm.work = atomicAdd(p0.r.work, 1u);
        __syncthreads();
        const uint32_t w = sm.work;
        __syncthreads();
        if (w >= total) break;
        bool od;
        uint32_t local;
        if (w < 2 * m) {
            od = (w & 1) == 0;
            local = w >> 1;
        } else {
            od = i1 > i0;
            local = m + (w - 2 * m);
        }
        if (od) pr_item<T, REF>(p1, local, n1, s1, b1, sm, s_next);
        else pr_item<T, REF>(p0, local, n0, s0, b0, sm, s_next);
    }
    if (REF) flush_next(p0.r, s_next);
}

// Applies the segmented vertices once all their segments are summed. In
// reference mode the list is this pass's segment items (k == 0 marks the
// vertex); in standard mode it is the fixed list of long-list vertices.
template <typename T, bool REF>
__global__ void pr_apply_segmented_kernel(PrArgs<T> p, const uint64_t *items_static, const uint64_t *items_od,
                                          const uint32_t *huge_list, uint32_t n_huge) {
    __shared__ double red[2 * kWarps];
    const RegionArgs &a = p.r;
    uint32_t n0 = 0, n1 = 0;
    if (REF) {
        n0 = a.cnt_in[2];
        n1 = a.cnt_in[3];
    }
    const uint32_t n = REF ? n0 + n1 : n_huge;
    const uint32_t stride = gridDim.x * blockDim.x;
    double res = 0, dang = 0;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t i = base + threadIdx.x;
        bool won = false;
        uint32_t v = 0;
        if (i < n) {
            bool go = true;
            if (REF) {
                uint64_t it = i < n0 ? items_static[i] : items_od[i - n0];
                v = (uint32_t)(it >> 32);
                go = (uint32_t)it == 0;
            } else {
                v = huge_list[i];
            }
            if (go) {
                const double s = PrAcc<T>::value(p.sum[v]);
                p.sum[v] = 0;
                won = pr_apply<T, REF>(p, v, s, res, dang);
            }
        }
        if (REF) {
            // a long-list vertex that stays active joins the next bitmap
            if (won) atomicOr(&a.bitmap[v >> 5], 1u << (v & 31));
            const unsigned m0 = __ballot_sync(kFull, won && v < a.S), m1 = __ballot_sync(kFull, won && v >= a.S);
            if ((threadIdx.x & 31) == 0) {
                if (m0) atomicAdd(&a.cnt_out[6], (uint32_t)__popc(m0));
                if (m1) atomicAdd(&a.cnt_out[7], (uint32_t)__popc(m1));
            }
        }
    }
    if (!REF) block_reduce2_atomic<T>(res, dang, p.acc, red);
}

template <typename T>
__global__ void pr_init_kernel(double *rank, T *c0, T *c1, typename PrAcc<T>::type *sum, const uint32_t *outdeg,
                               uint32_t V, double *dang) {
    // dang points at a (residual, dangling) pair; the start vector adds to dangling
    __shared__ double red[2 * kWarps];
    double d = 0;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < V; base += stride) {
        const uint32_t i = base + threadIdx.x;
        if (i < V) {
            const double r = 1.0 / (double)V;
            const uint32_t od = outdeg[i];
            rank[i] = r;
            const T c = od ? (T)(r / (double)od) : (T)0;
            c0[i] = c;
            c1[i] = c;
            sum[i] = 0;
            if (od == 0) d += r;
        }
    }
    block_reduce2_atomic<T>(0.0, d, dang, red);
}

// FP32 results: the FP64 ranks rounded to float (into the caller's device
// buffer, or a staging buffer that is then copied out).
__global__ void pr_rank_to_float_kernel(const double *rank, float *out, uint32_t V) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < V; i += gridDim.x * blockDim.x)
        out[i] = (float)rank[i];
}

// Segment items of every long-list vertex (standard PageRank, fixed each pass).
__global__ void seed_huge_segments_kernel(RegionArgs a, const uint32_t *huge_list, uint32_t n_static, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t v = huge_list[i];
        const uint32_t deg = a.ptr[v + 1] - a.ptr[v];
        const uint32_t nseg = (deg + a.seg_len - 1) / a.seg_len;
        const bool od = i >= n_static;
        const uint32_t base = atomicAdd(&a.cnt_out[2 + od], nseg);
        if (ASC_BAD((uint64_t)base + nseg > (od ? a.segcap_ondemand : a.segcap_static), 20, base)) continue;
        uint64_t *dst = a.seg_out + (od ? a.segcap_static : 0) + base;
        for (uint32_t k = 0; k < nseg; k++) dst[k] = ((uint64_t)v << 32) | k;
    }
}

// --------------------------------------------------------------- host -------

// Sizes and allocates the frontier machinery of one run for graph g, with
// the graph's tuning or (graph_tuning false) the default thresholds.
asc_status alloc_workspace(asc_graph *g, Workspace *ws, bool graph_tuning = true) {
    ws->V = g->V;
    if (g->has_tuning && graph_tuning) ws->tune = g->tuning;
    ASC_CUDA(cudaDeviceGetAttribute(&ws->num_sms, cudaDevAttrMultiProcessorCount, g->device));
    {
        // persistent grids fill the GPU: as many CTAs per SM as stay resident
        int per_sm = 0;
        ASC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, expand_fused_kernel<kSSSP, 2>, kBlock, 0));
        const uint32_t resident = (uint32_t)std::max(1, per_sm);
        if (!g->has_tuning || !ws->tune.ctas_per_sm || ws->tune.ctas_per_sm > resident) ws->tune.ctas_per_sm = resident;
    }
    const uint64_t V = g->V;
    const uint32_t S = g->static_vertices;
    const Tuning &t = ws->tune;
    std::lock_guard<std::mutex> plan_lk(g->long_lists_mu);
    auto &cache = g->long_lists;
    auto hit = std::find_if(cache.begin(), cache.end(), [&](const asc_graph::LongLists &c) {
        return c.huge_degree == t.huge_degree && c.segment_edges == t.segment_edges;
    });
    if (hit == cache.end()) {
        constexpr size_t kKeep = 4;
        if (cache.size() >= kKeep) cache.erase(cache.begin());
        cache.emplace_back();
        hit = cache.end() - 1;
        asc_graph::LongLists &ll = *hit;
        for (uint64_t v = 0; v < V; v++) {
            uint32_t d = g->h_ptr[v + 1] - g->h_ptr[v];
            if (d > t.huge_degree) {
                uint64_t ns = (d + t.segment_edges - 1) / t.segment_edges;
                if (v < S) { ll.seg_static += ns; ll.n_static++; }
                else ll.seg_ondemand += ns;
                ll.list.push_back((uint32_t)v);
            }
        }
        ll.bits.assign(V / 32 + 2, 0);
        for (uint32_t v : ll.list) ll.bits[v >> 5] |= 1u << (v & 31);
        ll.huge_degree = t.huge_degree;
        ll.segment_edges = t.segment_edges;
    }
    const asc_graph::LongLists &ll = *hit;
    const std::vector<uint32_t> &huge = ll.list, &hbits = ll.bits;
    const uint64_t cs = ll.seg_static, co = ll.seg_ondemand;
    ws->n_huge_static = ll.n_static;
    ws->n_huge_total = (uint32_t)huge.size();
    ws->segcap_static = cs;
    ws->segcap_ondemand = co;
    uint64_t bytes = 0;
    auto dalloc = [&](void **p, size_t n) -> asc_status {
        n = n ? n : 16;
        ASC_CUDA(cudaMalloc(p, n));
        bytes += n;
        return ASC_OK;
    };
    ASC_TRY(dalloc((void **)&ws->val, 4 * V));
    for (int i = 0; i < 2; i++) ASC_TRY(dalloc((void **)&ws->bitmap[i], 4 * (V / 32 + 2)));
    ASC_TRY(dalloc((void **)&ws->visited, 4 * (V / 32 + 2)));
    ASC_TRY(dalloc((void **)&ws->huge_bits, 4 * (V / 32 + 2)));
    ASC_TRY(dalloc((void **)&ws->far_bits, 4 * (V / 32 + 2)));
    ASC_CUDA(cudaMemcpy(ws->huge_bits, hbits.data(), 4 * (V / 32 + 2), cudaMemcpyHostToDevice));
    for (int i = 0; i < 2; i++) {
        ASC_TRY(dalloc((void **)&ws->queue[i], 4 * V));
        ASC_TRY(dalloc((void **)&ws->segs[i], 8 * (cs + co)));
    }
    ASC_TRY(dalloc((void **)&ws->ctl, 4 * CTL_WORDS));
    ASC_TRY(dalloc((void **)&ws->huge_list, 4 * huge.size()));
    if (!huge.empty())
        ASC_CUDA(cudaMemcpy(ws->huge_list, huge.data(), 4 * huge.size(), cudaMemcpyHostToDevice));
    ASC_CUDA(cudaHostAlloc((void **)&ws->h_ctl, 4 * CTL_WORDS, cudaHostAllocDefault));
    for (auto &e : ws->ev) ASC_CUDA(cudaEventCreate(&e));
    ws->device_bytes = bytes;
    return ASC_OK;
}

asc_status ensure_workspace(asc_graph *g) {
    if (g->ws) return ASC_OK;
    g->ws = new Workspace();
    return alloc_workspace(g, g->ws);
}

// PageRank state for contributions of elem bytes: FP64 ranks, two
// contribution arrays (this pass's and the next's), 8-byte sums.
uint64_t pr_buffer_bytes(uint64_t V, size_t elem) { return (16 + 2 * (uint64_t)elem) * V; }

asc_status ensure_pr_buffers(asc_graph *g, size_t elem) {
    Workspace *ws = g->ws;
    if (ws->pr_rank && ws->pr_elem == elem) return ASC_OK;
    for (void *p : {ws->pr_rank, ws->pr_contrib[0], ws->pr_contrib[1], ws->pr_sum})
        if (p) cudaFree(p);
    if (ws->pr_rank && ws->pr_elem) ws->device_bytes -= pr_buffer_bytes(g->V, ws->pr_elem);
    ws->pr_rank = ws->pr_contrib[0] = ws->pr_contrib[1] = ws->pr_sum = nullptr;
    ws->pr_elem = 0;
    ASC_CUDA(cudaMalloc(&ws->pr_rank, 8 * g->V));
    ASC_CUDA(cudaMalloc(&ws->pr_contrib[0], elem * g->V));
    ASC_CUDA(cudaMalloc(&ws->pr_contrib[1], elem * g->V));
    ASC_CUDA(cudaMalloc(&ws->pr_sum, 8 * g->V));
    ws->pr_elem = elem;
    ws->device_bytes += pr_buffer_bytes(g->V, elem);
    return ASC_OK;
}

RegionArgs base_args(asc_graph *g, Workspace *ws, int parity_in) {
    RegionArgs a;
    memset(&a, 0, sizeof(a));
    a.ptr = g->d_ptr;
    a.val = ws->val;
    a.bitmap = ws->bitmap[1 - parity_in];
    a.bitmap_in = ws->bitmap[parity_in];
    a.visited = ws->visited;
    a.huge_bits = ws->huge_bits;
    a.dense_div = ws->tune.dense_div;
    a.wbits = g->wbits;
    a.ebits = g->edge_words == 1 ? g->ebits : 32;
    a.frag = ws->frag_active;
    if (ws->bu_active && ws->in_ptr) {
        a.in_ptr = ws->in_ptr;
        a.in_edges = ws->in_edges ? ws->in_edges : g->d_host_in_edges;
        a.in_resident = ws->in_edges != nullptr;
        a.in_heads = g->in_heads_ready ? g->d_in_heads : nullptr;
        a.in_none = ws->in_none;
        a.in_ebits = g->in_ebits;
        a.bu_div = ws->tune.bu_div;
    }
    a.S = g->static_vertices;
    a.V = (uint32_t)g->V;
    a.huge = ws->tune.huge_degree;
    a.seg_len = ws->tune.segment_edges;
    a.segcap_static = (uint32_t)ws->segcap_static;
    a.segcap_ondemand = (uint32_t)ws->segcap_ondemand;
    a.stats = (unsigned long long *)(ws->ctl + CTL_STATS);
    const int po = 1 - parity_in;
    a.cnt_in = ws->ctl + CTL_BLOCK * parity_in;
    a.cnt_out = ws->ctl + CTL_BLOCK * po;
    a.q_out = ws->queue[po];
    a.seg_out = ws->segs[po];
    return a;
}

RegionArgs base_args(asc_graph *g, int parity_in) { return base_args(g, g->ws, parity_in); }

RegionArgs region_args(asc_graph *g, Workspace *ws, int parity_in, int region, bool dense) {
    RegionArgs a = base_args(g, ws, parity_in);
    a.region = region;
    a.edges = region == 0 ? g->d_static : g->d_host_edges;
    a.dense_begin = region == 0 ? 0 : g->static_vertices;
    a.dense_end = region == 0 ? g->static_vertices : (uint32_t)g->V;
    if (dense) {
        a.q_in = nullptr;
    } else {
        a.q_in = ws->queue[parity_in] + (region == 0 ? 0 : g->static_vertices);
    }
    a.seg_in = ws->segs[parity_in] + (region == 0 ? 0 : ws->segcap_static);
    a.work = a.cnt_out + 4 + region;
    a.edge_words = region == 0 ? edge_store_words(g, g->static_edges) : edge_store_words(g, g->E);
    return a;
}

// Standard PageRank pulls the on-demand region's tiles through shared memory
// (pr_vertices_staged) on single-word edge layouts; ASC_PR_TILE_STAGE=0 reads
// every edge word with its own load instead (for comparison).
bool pr_tile_stage(const asc_graph *g) {
    const char *env = getenv("ASC_PR_TILE_STAGE");
    return g->edge_words == 1 && !(env && env[0] == '0');
}

RegionArgs region_args(asc_graph *g, int parity_in, int region, bool dense) {
    return region_args(g, g->ws, parity_in, region, dense);
}

// SSSP near-far on: the expansion parks distances at or above the threshold in
// the far set.
bool near_far(asc_graph *g, asc_algo algo) { return algo == ASC_SSSP && g->ws->tune.delta != 0; }

void attach_far(asc_graph *g, asc_algo algo, RegionArgs &a) {
    if (near_far(g, algo)) {
        a.far_bits = g->ws->far_bits;
        a.thresh = g->ws->ctl + CTL_THRESH;
    }
}

uint32_t grid_for(const Workspace *ws, uint64_t work_items) {
    uint64_t cap = (uint64_t)ws->num_sms * ws->tune.ctas_per_sm;
    return (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(cap, work_items));
}

// One wave of bottom-up CTAs (a warp per kBuWords bitmap words per pass).
uint32_t bu_grid(const Workspace *ws, uint64_t nwords) {
    const uint64_t blocks = (nwords + kBuWords * (kBlock / 32) - 1) / (kBuWords * (kBlock / 32));
    return (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(blocks, (uint64_t)ws->num_sms * kBuMinBlocks));
}

uint32_t fill_grid(const Workspace *ws, uint64_t n) {
    uint64_t blocks = (n + kBlock - 1) / kBlock;
    return (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(blocks, (uint64_t)ws->num_sms * 8));
}

// The near-far promotion after an expansion (no-ops when the near frontier is
// not empty or the far set is).
void launch_far(asc_graph *g, cudaStream_t s, const RegionArgs &out_args) {
    Workspace *ws = g->ws;
    const uint32_t nwords = (uint32_t)g->V / 32 + 1;
    far_min_kernel<<<fill_grid(ws, nwords), kBlock, 0, s>>>(out_args, nwords, ws->ctl + CTL_MINFAR);
    far_promote_kernel<<<fill_grid(ws, nwords), kBlock, 0, s>>>(out_args, nwords, ws->ctl + CTL_MINFAR,
                                                                 ws->ctl + CTL_THRESH, ws->tune.delta);
}


template <int ALG, int WORDS>
void launch_expand(asc_graph *g, const RegionArgs &a, uint32_t grid) {
    expand_kernel<ALG, WORDS><<<grid, kBlock, 0, g->stream>>>(a);
}

typedef void (*ExpandFn)(asc_graph *, const RegionArgs &, uint32_t);
typedef void (*FusedFn)(cudaStream_t, const FusedArgs &, uint32_t);

template <int ALG, int WORDS>
void launch_fused(cudaStream_t s, const FusedArgs &x, uint32_t grid) {
    expand_fused_kernel<ALG, WORDS><<<grid, kBlock, 0, s>>>(x);
}

// the expansion kernels' WORDS argument for a graph's stored edge layout
int edge_layout(const asc_graph *g) { return g->edge_words == 2 ? 2 : (g->ebits < 32 ? kBitsLayout : 1); }

FusedFn pick_fused(asc_algo algo, int layout) {
    if (algo == ASC_BFS)
        return layout == 2 ? launch_fused<kBFS, 2> : layout == kBitsLayout ? launch_fused<kBFS, kBitsLayout>
                                                                            : launch_fused<kBFS, 1>;
    if (algo == ASC_CC)
        return layout == 2 ? launch_fused<kCC, 2> : layout == kBitsLayout ? launch_fused<kCC, kBitsLayout>
                                                                           : launch_fused<kCC, 1>;
    return layout == 2 ? launch_fused<kSSSP, 2> : layout == kBitsLayout ? launch_fused<kSSSP, kBitsLayout>
                                                                         : launch_fused<kSSSP, 1>;
}

ExpandFn pick_expand(asc_algo algo, int layout) {
    if (algo == ASC_BFS)
        return layout == 2 ? launch_expand<kBFS, 2> : layout == kBitsLayout ? launch_expand<kBFS, kBitsLayout>
                                                                             : launch_expand<kBFS, 1>;
    if (algo == ASC_CC)
        return layout == 2 ? launch_expand<kCC, 2> : layout == kBitsLayout ? launch_expand<kCC, kBitsLayout>
                                                                            : launch_expand<kCC, 1>;
    return layout == 2 ? launch_expand<kSSSP, 2> : layout == kBitsLayout ? launch_expand<kSSSP, kBitsLayout>
                                                                          : launch_expand<kSSSP, 1>;
}

// Per-iteration phase timing with events on the engine's stream.
struct PhaseTimer {
    Workspace *ws;
    bool on;
    size_t used = 0;
    std::vector<int> kind;
    PhaseTimer(Workspace *w, bool enable) : ws(w), on(enable) {}
    asc_status begin(int k) {
        if (!on) return ASC_OK;
        if (ws->phase_events.size() < used + 2) {
            for (int i = 0; i < 64; i++) {
                cudaEvent_t e;
                ASC_CUDA(cudaEventCreate(&e));
                ws->phase_events.push_back(e);
            }
        }
        kind.push_back(k);
        return ASC_OK;
    }
    void record(cudaStream_t s) {
        if (on) cudaEventRecord(ws->phase_events[used++], s);
    }
    asc_status sum(double *ms_by_kind) {
        for (size_t i = 0; i < kind.size(); i++) {
            float ms = 0;
            ASC_CUDA(cudaEventElapsedTime(&ms, ws->phase_events[2 * i], ws->phase_events[2 * i + 1]));
            ms_by_kind[kind[i]] += ms;
        }
        used = 0;
        kind.clear();
        return ASC_OK;
    }
};

// Builds the iteration loop of one algorithm as a CUDA graph: a conditional
// WHILE node whose body runs two iterations (parity 0 then 1; an iteration
// with an empty input costs only empty launches) and loop_cond_kernel. The
// kernels read their frontier sizes from the control block, so nothing
// returns to the host between iterations.
asc_status build_loop_graph(asc_graph *g, asc_algo algo, uint32_t cap) {
    Workspace *ws = g->ws;
    const int slot = algo == ASC_BFS ? 0 : (algo == ASC_SSSP ? 1 : 2);
    if (ws->loop_exec[slot] && ws->loop_cap[slot] == cap) return ASC_OK;
    if (ws->loop_exec[slot]) {
        cudaGraphExecDestroy(ws->loop_exec[slot]);
        ws->loop_exec[slot] = nullptr;
    }
    FusedFn fused = pick_fused(algo, edge_layout(g));
    const uint32_t V = (uint32_t)g->V;
    const uint32_t grid = (uint32_t)(ws->num_sms * ws->tune.ctas_per_sm);
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t cs = nullptr;
    asc_status st = ASC_OK;
    auto chk = [&](cudaError_t e, const char *what) {
        if (e != cudaSuccess && st == ASC_OK) st = cuda_fail(e, what, __FILE__, __LINE__);
        return st == ASC_OK;
    };
    cudaGraphConditionalHandle handle;
    cudaGraphNodeParams cp = {};
    cudaGraphNode_t node;
    if (chk(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "stream") &&
        chk(cudaGraphCreate(&graph, 0), "cudaGraphCreate") &&
        chk(cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault), "handle")) {
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = handle;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        if (chk(cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp), "cudaGraphAddNode")) {
            cudaGraph_t body = cp.conditional.phGraph_out[0];
            if (chk(cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal),
                    "capture")) {
                for (int parity = 0; parity < 2; parity++) {
                    const int po = 1 - parity;
                    cudaMemsetAsync(ws->ctl + CTL_BLOCK * po, 0, 4 * CTL_BLOCK, cs);
                    cudaMemsetAsync(ws->bitmap[po], 0, 4 * (V / 32 + 2), cs);
                    FusedArgs x;
                    x.r0 = region_args(g, parity, 0, false);
                    x.r1 = region_args(g, parity, 1, false);
                    attach_far(g, algo, x.r0);
                    attach_far(g, algo, x.r1);
                    x.work = x.r0.cnt_out + 4;
                    if (near_far(g, algo)) cudaMemsetAsync(ws->ctl + CTL_MINFAR, 0xff, 4, cs);
                    fused(cs, x, grid);
                    if (algo == ASC_BFS && x.r0.in_ptr)
                        bottom_up_kernel<<<bu_grid(ws, V / 32 + 1), kBlock, 0, cs>>>(x.r0, V / 32 + 1);
                    if (near_far(g, algo)) launch_far(g, cs, x.r0);
                    build_frontier_kernel<<<fill_grid(ws, V / 32 + 1), kBlock, 0, cs>>>(x.r0, ws->bitmap[po],
                                                                                        V / 32 + 1);
                }
                loop_cond_kernel<<<1, 1, 0, cs>>>(handle, ws->ctl, cap);
                cudaGraph_t out = nullptr;
                chk(cudaStreamEndCapture(cs, &out), "end capture");
            }
        }
    }
    if (st == ASC_OK) chk(cudaGraphInstantiate(&exec, graph, 0), "cudaGraphInstantiate");
    if (graph) cudaGraphDestroy(graph);
    if (cs) cudaStreamDestroy(cs);
    if (st != ASC_OK) {
        if (exec) cudaGraphExecDestroy(exec);
        cudaGetLastError();
        return st;
    }
    ws->loop_exec[slot] = exec;
    ws->loop_cap[slot] = cap;
    return ASC_OK;
}

}  // namespace

// ------------------------------------------- staged dense on-demand passes --
//
// Standard PageRank reads every edge each pass. On a graph opened with staging
// buffers (asc_budget.stage_bytes, part of the device budget), the on-demand
// region is copied each pass in chunks by the copy engine, on a stream of its
// own, into the two device buffers (chunk k into buffer k % 2), while the
// kernels consume the chunk before it; the copy of chunk k + 2 waits only for
// the launch that read chunk k. Chunks end at vertex boundaries, except inside
// a long list (more than huge_degree edges, summed by segments), which is cut
// at segment boundaries; a chunk's tile range holds the vertices that start in
// it, so every vertex is summed exactly once. The static region is cut into as
// many slices by edges, and launch k runs static slice k with chunk k in one
// grid (items interleaved), so every launch mixes HBM-bound gathers with the
// staged chunk and the copies never wait for the static work. The reference
// moves its gathered partitions into its staging area one at a time with
// synchronous copies before each partition kernel (CalculateOpt.cu:161-178).
struct StagePiece {
    uint32_t v_lo = 0, v_hi = 0;  // tile range: the vertices that start in this piece
    uint64_t e_lo = 0, e_hi = 0;  // its edges [e_lo, e_hi)
    std::vector<uint64_t> segs;   // segment items (v << 32 | k) of long lists, in order
};

struct StageLaunch {
    uint32_t s_lo = 0, s_hi = 0;  // static slice tile range
    uint32_t c_lo = 0, c_hi = 0;  // chunk tile range
    uint64_t w_lo = 0, w_n = 0;   // u32 words the chunk's copy moves (0: no chunk)
    uint64_t seg_s = 0, seg_c = 0;  // offsets of the slice's and the chunk's segment items
    uint32_t nseg_s = 0, nseg_c = 0;
    // work items of the launch: segments plus tiles of kBlock vertices
    uint64_t items() const {
        return (uint64_t)nseg_s + nseg_c + (s_hi - s_lo + kBlock - 1) / kBlock + (c_hi - c_lo + kBlock - 1) / kBlock;
    }
};

struct StagePlan {
    uint32_t huge = 0, seg_len = 0;  // the tuning the plan was made for
    uint32_t chunks = 0;             // launches [0, chunks) carry a chunk
    std::vector<StageLaunch> launches;
    uint64_t copy_bytes = 0;         // moved per pass
    uint64_t *d_segs = nullptr;      // every launch's segment items
    uint32_t *d_cnt = nullptr;       // per launch, 8 words: [2] slice segments, [3] chunk segments
    uint32_t *d_work = nullptr;      // per launch work cursor
    cudaStream_t copy = nullptr;
    cudaEvent_t copied[2] = {nullptr, nullptr}, consumed[2] = {nullptr, nullptr};
};

void destroy_stage_plan(StagePlan *sp) {
    if (!sp) return;
    if (sp->copy) cudaStreamSynchronize(sp->copy);
    for (void *q : {(void *)sp->d_segs, (void *)sp->d_cnt, (void *)sp->d_work})
        if (q) cudaFree(q);
    for (int i = 0; i < 2; i++) {
        if (sp->copied[i]) cudaEventDestroy(sp->copied[i]);
        if (sp->consumed[i]) cudaEventDestroy(sp->consumed[i]);
    }
    if (sp->copy) cudaStreamDestroy(sp->copy);
    delete sp;
}

// u32 words of the stored edge array that hold edges [e_lo, e_hi).
void edge_words_of(const asc_graph *g, uint64_t e_lo, uint64_t e_hi, uint64_t &w_lo, uint64_t &w_n) {
    w_lo = w_n = 0;
    if (e_hi <= e_lo) return;
    if (g->edge_words == 2) {
        w_lo = 2 * e_lo;
        w_n = 2 * (e_hi - e_lo);
    } else if (g->ebits == 32) {
        w_lo = e_lo;
        w_n = e_hi - e_lo;
    } else {
        w_lo = (e_lo * g->ebits) >> 5;
        w_n = ((e_hi * g->ebits - 1) >> 5) - w_lo + 1;
    }
}

// Cuts vertices [v0, v1) into pieces whose edges satisfy fits(e_lo, e_hi).
// False when a single short list or segment does not fit by itself.
template <typename Fits>
bool plan_pieces(const uint32_t *ptr, uint32_t v0, uint32_t v1, uint32_t huge, uint32_t seg_len, Fits fits,
                 std::vector<StagePiece> &out) {
    StagePiece cur;
    cur.v_lo = v0;
    cur.e_lo = cur.e_hi = ptr[v0];
    auto close = [&](uint32_t v_hi, uint64_t next_e) {
        cur.v_hi = v_hi;
        out.push_back(std::move(cur));
        cur = StagePiece();
        cur.v_lo = v_hi;
        cur.e_lo = cur.e_hi = next_e;
    };
    for (uint32_t v = v0; v < v1; v++) {
        const uint64_t b = ptr[v], e = ptr[v + 1];
        if (e - b <= huge) {
            if (!fits(cur.e_lo, e)) {
                if (cur.e_hi == cur.e_lo) return false;
                close(v, b);
                if (!fits(cur.e_lo, e)) return false;
            }
            cur.e_hi = e;
            continue;
        }
        const uint64_t nseg = (e - b + seg_len - 1) / seg_len;
        for (uint64_t k = 0; k < nseg; k++) {
            const uint64_t sb = b + k * seg_len, se = std::min<uint64_t>(e, sb + seg_len);
            if (!fits(cur.e_lo, se)) {
                if (cur.e_hi == cur.e_lo) return false;
                // v belongs to the piece holding its first segment
                close(k == 0 ? v : v + 1, sb);
                if (!fits(cur.e_lo, se)) return false;
            }
            cur.segs.push_back(((uint64_t)v << 32) | k);
            cur.e_hi = se;
        }
    }
    cur.v_hi = v1;
    out.push_back(std::move(cur));
    return true;
}

// The chunk plan for the graph's current tuning; *ok false (and no plan) when
// a long-list segment or a short list does not fit a staging buffer.
asc_status ensure_stage_plan(asc_graph *g, bool *ok) {
    Workspace *ws = g->ws;
    *ok = false;
    if (!g->stage_words || g->static_edges >= g->E) return ASC_OK;
    const uint32_t huge = ws->tune.huge_degree, seg_len = ws->tune.segment_edges;
    if (ws->stage && ws->stage->huge == huge && ws->stage->seg_len == seg_len) {
        *ok = true;
        return ASC_OK;
    }
    destroy_stage_plan(ws->stage);
    ws->stage = nullptr;
    const uint32_t V = (uint32_t)g->V, S = g->static_vertices;
    std::vector<StagePiece> chunks, slices;
    const uint64_t cap_words = g->stage_words;
    if (!plan_pieces(g->h_ptr, S, V, huge, seg_len,
                     [&](uint64_t lo, uint64_t hi) {
                         uint64_t w0, wn;
                         edge_words_of(g, lo, hi, w0, wn);
                         return wn <= cap_words;
                     },
                     chunks))
        return ASC_OK;
    // every chunk read stays inside its copy: the short lists of its tile range
    // and its segments lie in its edges, which fit a buffer; the tile ranges
    // cover [S, V) once
    for (size_t k = 0; k < chunks.size(); k++) {
        const StagePiece &c = chunks[k];
        uint64_t w0, wn;
        edge_words_of(g, c.e_lo, c.e_hi, w0, wn);
        bool good = wn <= cap_words && c.v_lo == (k ? chunks[k - 1].v_hi : S) && c.v_hi >= c.v_lo;
        for (uint32_t v = c.v_lo; good && v < c.v_hi; v++) {
            const uint64_t b = g->h_ptr[v], e = g->h_ptr[v + 1];
            if (e - b <= huge) good = b >= c.e_lo && e <= c.e_hi;
        }
        for (uint64_t it : c.segs) {
            const uint32_t v = (uint32_t)(it >> 32), j = (uint32_t)it;
            const uint64_t b = (uint64_t)g->h_ptr[v] + (uint64_t)j * seg_len;
            good = good && b >= c.e_lo && std::min<uint64_t>(g->h_ptr[v + 1], b + seg_len) <= c.e_hi;
        }
        if (!good) return fail(ASC_ERR_INVALID, "internal: staging chunk %zu does not cover its reads", k);
    }
    if (chunks.back().v_hi != V) return fail(ASC_ERR_INVALID, "internal: staging chunks do not cover the region");
    const uint64_t static_edges = g->h_ptr[S];
    if (S > 0) {
        const uint64_t cap = std::max<uint64_t>({(static_edges + chunks.size() - 1) / chunks.size(),
                                                 (uint64_t)huge + 1, (uint64_t)seg_len});
        plan_pieces(g->h_ptr, 0, S, huge, seg_len, [&](uint64_t lo, uint64_t hi) { return hi - lo <= cap; },
                    slices);
    }
    StagePlan *sp = new StagePlan();
    sp->huge = huge;
    sp->seg_len = seg_len;
    sp->chunks = (uint32_t)chunks.size();
    const size_t L = std::max(chunks.size(), slices.size());
    std::vector<uint64_t> segs;
    std::vector<uint32_t> cnt(8 * L, 0);
    sp->launches.resize(L);
    for (size_t k = 0; k < L; k++) {
        StageLaunch &x = sp->launches[k];
        if (k < slices.size()) {
            x.s_lo = slices[k].v_lo;
            x.s_hi = slices[k].v_hi;
            x.seg_s = segs.size();
            x.nseg_s = (uint32_t)slices[k].segs.size();
            cnt[8 * k + 2] = x.nseg_s;
            segs.insert(segs.end(), slices[k].segs.begin(), slices[k].segs.end());
        }
        if (k < chunks.size()) {
            x.c_lo = chunks[k].v_lo;
            x.c_hi = chunks[k].v_hi;
            edge_words_of(g, chunks[k].e_lo, chunks[k].e_hi, x.w_lo, x.w_n);
            sp->copy_bytes += 4 * x.w_n;
            x.seg_c = segs.size();
            x.nseg_c = (uint32_t)chunks[k].segs.size();
            cnt[8 * k + 3] = x.nseg_c;
            segs.insert(segs.end(), chunks[k].segs.begin(), chunks[k].segs.end());
        }
    }
    asc_status st = ASC_OK;
    auto cu = [&](cudaError_t e, const char *what) {
        if (e != cudaSuccess && st == ASC_OK) st = cuda_fail(e, what, __FILE__, __LINE__);
    };
    cu(cudaMalloc(&sp->d_segs, 8 * std::max<size_t>(1, segs.size())), "cudaMalloc(stage segments)");
    cu(cudaMalloc(&sp->d_cnt, 4 * cnt.size()), "cudaMalloc(stage counts)");
    cu(cudaMalloc(&sp->d_work, 4 * L), "cudaMalloc(stage cursors)");
    if (st == ASC_OK && !segs.empty())
        cu(cudaMemcpy(sp->d_segs, segs.data(), 8 * segs.size(), cudaMemcpyHostToDevice), "cudaMemcpy(segments)");
    if (st == ASC_OK) cu(cudaMemcpy(sp->d_cnt, cnt.data(), 4 * cnt.size(), cudaMemcpyHostToDevice), "cudaMemcpy");
    if (st == ASC_OK) cu(cudaStreamCreateWithFlags(&sp->copy, cudaStreamNonBlocking), "cudaStreamCreate");
    for (int i = 0; i < 2 && st == ASC_OK; i++) {
        cu(cudaEventCreateWithFlags(&sp->copied[i], cudaEventDisableTiming), "cudaEventCreate");
        cu(cudaEventCreateWithFlags(&sp->consumed[i], cudaEventDisableTiming), "cudaEventCreate");
    }
    if (st != ASC_OK) {
        destroy_stage_plan(sp);
        return st;
    }
    ws->stage = sp;
    *ok = true;
    return ASC_OK;
}

// Whole-partition comparison engine (ASC_RUN_PARTITION_COPY), the reference's
// baseline of bfs.cu:6-168 / gpu_kernels.cu:302-519: the on-demand region in
// partitions of one staging buffer, cut at vertex boundaries only; each
// iteration copies every partition that holds a frontier vertex, whole, and
// expands that partition's frontier vertices from the copy.
struct PartPlan {
    std::vector<StageLaunch> parts;  // c_lo / c_hi (tile range), w_lo / w_n (copy)
    uint32_t *d_ranges = nullptr;    // per partition: tile range
    uint32_t *d_flags = nullptr;     // per partition: holds a frontier vertex this iteration
    uint32_t *h_flags = nullptr;     // page-locked mirror
    uint32_t *d_cnt = nullptr;       // per partition, 8 words: an id-order walk of its range, no segments
    uint32_t *d_work = nullptr;      // per partition work cursor
    cudaStream_t copy = nullptr;
    cudaEvent_t copied[2] = {nullptr, nullptr}, consumed[2] = {nullptr, nullptr};
};

void destroy_part_plan(PartPlan *pp) {
    if (!pp) return;
    if (pp->copy) cudaStreamSynchronize(pp->copy);
    for (void *q : {(void *)pp->d_ranges, (void *)pp->d_flags, (void *)pp->d_cnt, (void *)pp->d_work})
        if (q) cudaFree(q);
    if (pp->h_flags) cudaFreeHost(pp->h_flags);
    for (int i = 0; i < 2; i++) {
        if (pp->copied[i]) cudaEventDestroy(pp->copied[i]);
        if (pp->consumed[i]) cudaEventDestroy(pp->consumed[i]);
    }
    if (pp->copy) cudaStreamDestroy(pp->copy);
    delete pp;
}

asc_status ensure_part_plan(asc_graph *g) {
    Workspace *ws = g->ws;
    if (ws->part) return ASC_OK;
    if (!g->stage_words)
        return fail(ASC_ERR_INVALID, "the partition-copy engine needs staging buffers (asc_budget.stage_bytes)");
    const uint32_t V = (uint32_t)g->V, S = g->static_vertices;
    std::vector<StagePiece> parts;
    const uint64_t cap = g->stage_words;
    if (!plan_pieces(g->h_ptr, S, V, 0xffffffffu, 1u << 30,
                     [&](uint64_t lo, uint64_t hi) {
                         uint64_t w0, wn;
                         edge_words_of(g, lo, hi, w0, wn);
                         return wn <= cap;
                     },
                     parts))
        return fail(ASC_ERR_BUDGET, "an adjacency list is longer than a partition (%llu words)",
                    (unsigned long long)cap);
    PartPlan *pp = new PartPlan();
    const size_t n = parts.size();
    std::vector<uint32_t> ranges(2 * n), cnt(8 * n, 0);
    pp->parts.resize(n);
    for (size_t k = 0; k < n; k++) {
        StageLaunch &x = pp->parts[k];
        x.c_lo = parts[k].v_lo;
        x.c_hi = parts[k].v_hi;
        edge_words_of(g, parts[k].e_lo, parts[k].e_hi, x.w_lo, x.w_n);
        ranges[2 * k] = x.c_lo;
        ranges[2 * k + 1] = x.c_hi;
        cnt[8 * k + 7] = 1;  // with dense_div at its maximum: walk the range in id order
    }
    asc_status st = ASC_OK;
    auto cu = [&](cudaError_t e, const char *what) {
        if (e != cudaSuccess && st == ASC_OK) st = cuda_fail(e, what, __FILE__, __LINE__);
    };
    cu(cudaMalloc(&pp->d_ranges, 8 * n), "cudaMalloc(partition ranges)");
    cu(cudaMalloc(&pp->d_flags, 4 * n), "cudaMalloc(partition flags)");
    cu(cudaMalloc(&pp->d_cnt, 32 * n), "cudaMalloc(partition counts)");
    cu(cudaMalloc(&pp->d_work, 4 * n), "cudaMalloc(partition cursors)");
    cu(cudaHostAlloc((void **)&pp->h_flags, 4 * n, cudaHostAllocDefault), "cudaHostAlloc(partition flags)");
    if (st == ASC_OK) cu(cudaMemcpy(pp->d_ranges, ranges.data(), 8 * n, cudaMemcpyHostToDevice), "cudaMemcpy");
    if (st == ASC_OK) cu(cudaMemcpy(pp->d_cnt, cnt.data(), 32 * n, cudaMemcpyHostToDevice), "cudaMemcpy");
    if (st == ASC_OK) cu(cudaStreamCreateWithFlags(&pp->copy, cudaStreamNonBlocking), "cudaStreamCreate");
    for (int i = 0; i < 2 && st == ASC_OK; i++) {
        cu(cudaEventCreateWithFlags(&pp->copied[i], cudaEventDisableTiming), "cudaEventCreate");
        cu(cudaEventCreateWithFlags(&pp->consumed[i], cudaEventDisableTiming), "cudaEventCreate");
    }
    if (st != ASC_OK) {
        destroy_part_plan(pp);
        return st;
    }
    ws->part = pp;
    return ASC_OK;
}

// One CTA per partition (grid-stride): whether its tile range holds a vertex
// of this iteration's frontier.
__global__ void part_active_kernel(const uint32_t *bitmap_in, const uint32_t *ranges, uint32_t n,
                                   uint32_t *flags) {
    for (uint32_t k = blockIdx.x; k < n; k += gridDim.x) {
        const uint32_t lo = ranges[2 * k], hi = ranges[2 * k + 1];
        uint32_t any = 0;
        for (uint32_t u0 = (lo & ~31u) + 32 * threadIdx.x; u0 < hi; u0 += 32 * blockDim.x) {
            uint32_t w = bitmap_in[u0 >> 5];
            if (u0 < lo) w &= 0xffffffffu << (lo - u0);
            if (hi - u0 < 32u) w &= (1u << (hi - u0)) - 1u;
            any |= w;
        }
        any = __syncthreads_or(any != 0);
        if (threadIdx.x == 0) flags[k] = any;
    }
}

// Launch k's chunk: its copy on the copy stream once the launch that last read
// the same buffer is done, and the compute stream s waits for it. Returns the
// device address that the chunk's edge offsets index (the buffer less the
// chunk's first word), or the static prefix when launch k has no chunk.
const uint32_t *stage_chunk(asc_graph *g, StagePlan *sp, uint32_t k, cudaStream_t s, asc_status *st) {
    const StageLaunch &x = sp->launches[k];
    *st = ASC_OK;
    if (!x.w_n) return g->d_static;
    const int b = k & 1;
    cudaError_t e = cudaStreamWaitEvent(sp->copy, sp->consumed[b], 0);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(g->d_stage[b], g->h_edges + x.w_lo, 4 * x.w_n, cudaMemcpyHostToDevice, sp->copy);
    if (e == cudaSuccess) e = cudaEventRecord(sp->copied[b], sp->copy);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, sp->copied[b], 0);
    if (e != cudaSuccess) *st = cuda_fail(e, "staged chunk copy", __FILE__, __LINE__);
    return (const uint32_t *)((uintptr_t)g->d_stage[b] - 4 * (uintptr_t)x.w_lo);
}

asc_status stage_release(StagePlan *sp, uint32_t k, cudaStream_t s) {
    if (sp->launches[k].w_n) ASC_CUDA(cudaEventRecord(sp->consumed[k & 1], s));
    return ASC_OK;
}

// Region arguments of launch k: the static slice (region 0) or the chunk
// (region 1) with its tile range, segment items, counts and cursor.
void stage_region(const StagePlan *sp, uint32_t k, int region, const uint32_t *edges, RegionArgs &a) {
    const StageLaunch &x = sp->launches[k];
    a.dense_begin = region == 0 ? x.s_lo : x.c_lo;
    a.dense_end = region == 0 ? x.s_hi : x.c_hi;
    a.seg_in = sp->d_segs + (region == 0 ? x.seg_s : x.seg_c);
    a.cnt_in = sp->d_cnt + 8 * k;
    a.work = sp->d_work + k;
    if (region == 1) a.edges = edges;
}

void free_ws_buffers(Workspace *ws) {
    for (void *p : {(void *)ws->val, (void *)ws->visited, (void *)ws->huge_bits, (void *)ws->far_bits,
                    (void *)ws->frag_counts,
                    (void *)ws->bitmap[0],
                    (void *)ws->bitmap[1],
                    (void *)ws->queue[0],
                    (void *)ws->queue[1],
                    (void *)ws->segs[0], (void *)ws->segs[1], (void *)ws->ctl, (void *)ws->huge_list, ws->pr_rank,
                    ws->pr_contrib[0], ws->pr_contrib[1], ws->pr_sum, (void *)ws->in_ptr, (void *)ws->in_edges,
                    (void *)ws->in_none})
        if (p) cudaFree(p);
    if (ws->h_ctl) cudaFreeHost(ws->h_ctl);
    for (void *p : {(void *)ws->g_stage, (void *)ws->g_items})
        if (p) cudaFree(p);
    for (void *p : {(void *)ws->h_stage, (void *)ws->h_items, (void *)ws->h_list, (void *)ws->h_segs})
        if (p) cudaFreeHost(p);
    for (auto &e : ws->loop_exec)
        if (e) cudaGraphExecDestroy(e);
    for (auto e : ws->ev)
        if (e) cudaEventDestroy(e);
    for (auto e : ws->phase_events) cudaEventDestroy(e);
    destroy_stage_plan(ws->stage);
    ws->stage = nullptr;
    destroy_part_plan(ws->part);
    ws->part = nullptr;
}

void free_workspace(asc_graph *g) {
    Workspace *ws = g->ws;
    if (!ws) return;
    for (auto &b : ws->batch)
        if (b) {
            batch_destroy(b);
            b = nullptr;
        }
    free_ws_buffers(ws);
    delete ws;
    g->ws = nullptr;
}

asc_status run_traversal_impl(asc_graph *g, asc_algo algo, uint32_t source, const asc_params &p, void *out,
                              asc_stats *st);

uint64_t fragment_count(const asc_graph *g) { return (g->E + 4095) / 4096; }

asc_status run_traversal(asc_graph *g, asc_algo algo, uint32_t source, const asc_params &p, void *out,
                         asc_stats *st) {
    ASC_TRY(ensure_workspace(g));
    Workspace *ws = g->ws;
    if (p.flags & ASC_RUN_FRAGMENT_COUNTS) {
        if (!ws->frag_counts) {
            const size_t bytes = 8 * std::max<uint64_t>(1, fragment_count(g));
            ASC_CUDA(cudaMalloc(&ws->frag_counts, bytes));
            ASC_CUDA(cudaMemsetAsync(ws->frag_counts, 0, bytes, g->stream));
            ws->device_bytes += bytes;
        }
        ws->frag_active = ws->frag_counts;
    }
    // the gather engine expands the on-demand region from its frontier list
    const uint32_t div = ws->tune.dense_div;
    if (p.flags & ASC_RUN_GATHER_COPY) ws->tune.dense_div = 0;
    const asc_status rc = run_traversal_impl(g, algo, source, p, out, st);
    ws->tune.dense_div = div;
    ws->frag_active = nullptr;
    return rc;
}

typedef void (*StagedFn)(cudaStream_t, const StagedArgs &, uint32_t);

template <int ALG, int WORDS>
void launch_staged(cudaStream_t s, const StagedArgs &x, uint32_t grid) {
    expand_staged_kernel<ALG, WORDS><<<grid, kBlock, 0, s>>>(x);
}

StagedFn pick_staged(asc_algo algo, bool pairs) {
    if (algo == ASC_BFS) return pairs ? launch_staged<kBFS, 2> : launch_staged<kBFS, 1>;
    if (algo == ASC_CC) return pairs ? launch_staged<kCC, 2> : launch_staged<kCC, 1>;
    return pairs ? launch_staged<kSSSP, 2> : launch_staged<kSSSP, 1>;
}

// Host side of the gather-and-copy engine for one iteration: the on-demand
// list and segments come back to the host, host threads gather their edges
// (decoding the stored layout) into page-locked staging in parts of at most
// g_cap edges, and each part is copied over and expanded before the next.
asc_status gather_ondemand(asc_graph *g, asc_algo algo, int parity, const uint32_t *cnt, cudaEvent_t lists_ready,
                           uint32_t &launches) {
    Workspace *ws = g->ws;
    cudaStream_t s = g->stream;
    const uint32_t n_list = cnt[1], n_seg = cnt[3];
    ASC_CUDA(cudaEventSynchronize(lists_ready));
    if (!n_list && !n_seg) return ASC_OK;
    const uint32_t words = g->edge_words;
    const uint32_t seg_len = ws->tune.segment_edges;
    struct Item { uint32_t u; uint64_t b; uint32_t len, first; };
    std::vector<Item> items;
    items.reserve((size_t)n_list + n_seg);
    for (uint32_t i = 0; i < n_list; i++) {
        const uint32_t u = ws->h_list[i];
        items.push_back({u, g->h_ptr[u], g->h_ptr[u + 1] - g->h_ptr[u], 1u});
    }
    for (uint32_t i = 0; i < n_seg; i++) {
        const uint32_t u = (uint32_t)(ws->h_segs[i] >> 32), k = (uint32_t)ws->h_segs[i];
        const uint64_t b = (uint64_t)g->h_ptr[u] + (uint64_t)k * seg_len;
        const uint64_t e = std::min<uint64_t>(g->h_ptr[u + 1], b + seg_len);
        items.push_back({u, b, (uint32_t)(e - b), k == 0 ? 1u : 0u});
    }
    const uint32_t *he = g->h_edges;
    const uint32_t eb = g->ebits;
    auto word_at = [&](uint64_t idx) -> uint32_t {
        if (words == 2 || eb == 32) return he[idx];
        const uint64_t bit = idx * eb;
        const uint32_t sh = (uint32_t)(bit & 31);
        uint32_t x = he[bit >> 5] >> sh;
        if (sh + eb > 32) x |= he[(bit >> 5) + 1] << (32 - sh);
        return x & ((1u << eb) - 1u);
    };
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const StagedFn staged = pick_staged(algo, words == 2);
    size_t i0 = 0;
    while (i0 < items.size()) {
        // one part: items whose edges fit the staging buffer
        uint64_t tot = 0;
        size_t i1 = i0;
        while (i1 < items.size() && i1 - i0 < ws->g_cap && tot + items[i1].len <= ws->g_cap) tot += items[i1++].len;
        const size_t n = i1 - i0;
        std::vector<uint64_t> off(n + 1, 0);
        for (size_t k = 0; k < n; k++) off[k + 1] = off[k] + items[i0 + k].len;
        auto work = [&](unsigned t) {
            for (size_t k = t; k < n; k += hw) {
                const Item &it = items[i0 + k];
                uint32_t *dst = ws->h_stage + off[k] * words;
                if (words == 2) memcpy(dst, he + 2 * it.b, 8ull * it.len);
                else for (uint32_t j = 0; j < it.len; j++) dst[j] = word_at(it.b + j);
                uint32_t *q = ws->h_items + 4 * k;
                q[0] = it.u;
                q[1] = (uint32_t)off[k];
                q[2] = it.len;
                q[3] = it.first;
            }
        };
        std::vector<std::thread> th;
        for (unsigned t = 1; t < hw; t++) th.emplace_back(work, t);
        work(0);
        for (auto &x : th) x.join();
        ASC_CUDA(cudaMemcpyAsync(ws->g_stage, ws->h_stage, 4ull * words * tot, cudaMemcpyHostToDevice, s));
        ASC_CUDA(cudaMemcpyAsync(ws->g_items, ws->h_items, 16ull * n, cudaMemcpyHostToDevice, s));
        StagedArgs x;
        x.a = region_args(g, parity, 1, false);
        attach_far(g, algo, x.a);
        x.stage = ws->g_stage;
        x.items = ws->g_items;
        x.n_items = (uint32_t)n;
        staged(s, x, fill_grid(ws, 32ull * n));
        launches++;
        ASC_CUDA(cudaGetLastError());
        // the staging buffers are reused by the next part
        ASC_CUDA(cudaStreamSynchronize(s));
        i0 = i1;
    }
    return ASC_OK;
}

asc_status ensure_gather_buffers(asc_graph *g) {
    Workspace *ws = g->ws;
    if (ws->g_stage) return ASC_OK;
    const uint64_t od = g->E - std::min<uint64_t>(g->E, g->h_ptr[g->static_vertices]);
    // a part must hold the longest item: a list up to huge_degree edges or a segment
    const uint64_t need = std::max<uint64_t>(ws->tune.huge_degree, ws->tune.segment_edges);
    ws->g_cap = std::max<uint64_t>(need, std::min<uint64_t>(std::max<uint64_t>(od, 1), 1ull << 25));
    const uint64_t words = g->edge_words;
    ASC_CUDA(cudaMalloc(&ws->g_stage, 4 * words * ws->g_cap));
    ASC_CUDA(cudaMalloc(&ws->g_items, 16 * ws->g_cap));
    ASC_CUDA(cudaHostAlloc(&ws->h_stage, 4 * words * ws->g_cap, cudaHostAllocDefault));
    ASC_CUDA(cudaHostAlloc(&ws->h_items, 16 * ws->g_cap, cudaHostAllocDefault));
    ASC_CUDA(cudaHostAlloc(&ws->h_list, 4 * (g->V + 1), cudaHostAllocDefault));
    ASC_CUDA(cudaHostAlloc(&ws->h_segs, 8 * (ws->segcap_ondemand + 1), cudaHostAllocDefault));
    return ASC_OK;
}

// In-edge offsets on the device for bottom-up BFS steps, built on the
// graph's first BFS. The in-edges stay in pinned host memory, read in place,
// unless the graph has no cap (every out-edge resident): then they are
// resident too.
asc_status ensure_in_ptr(asc_graph *g) {
    Workspace *ws = g->ws;
    if (ws->in_ptr) return ASC_OK;
    ASC_TRY(build_in_edges(g));
    ASC_CUDA(cudaMalloc(&ws->in_ptr, 4 * (g->V + 1)));
    ASC_CUDA(cudaMemcpy(ws->in_ptr, g->h_in_ptr, 4 * (g->V + 1), cudaMemcpyHostToDevice));
    ws->device_bytes += 4 * (g->V + 1);
    {
        // one bit per vertex without in-edges (bits past V set: nothing to look
        // for there), built once per graph: a server that frees the state of an
        // idle graph uploads it again
        const uint64_t nw = g->V / 32 + 2;
        if (!g->h_in_none) {
            uint32_t *none = new uint32_t[nw]();
            for (uint64_t v = 0; v < 32 * nw; v++)
                if (v >= g->V || g->h_in_ptr[v + 1] == g->h_in_ptr[v]) none[v >> 5] |= 1u << (v & 31);
            g->h_in_none = none;
        }
        ASC_CUDA(cudaMalloc(&ws->in_none, 4 * nw));
        ASC_CUDA(cudaMemcpy(ws->in_none, g->h_in_none, 4 * nw, cudaMemcpyHostToDevice));
        ws->device_bytes += 4 * nw;
    }
    if (g->static_edges >= g->E) {
        const uint64_t words = g->in_ebits == 32 ? std::max<uint64_t>(1, g->E) : (g->E * g->in_ebits + 31) / 32 + 1;
        ASC_CUDA(cudaMalloc(&ws->in_edges, 4 * words));
        ASC_CUDA(cudaMemcpy(ws->in_edges, g->h_in_edges, 4 * words, cudaMemcpyHostToDevice));
        ws->device_bytes += 4 * words;
    }
    if (ws->loop_exec[0]) {  // the BFS loop was captured without bottom-up steps
        cudaGraphExecDestroy(ws->loop_exec[0]);
        ws->loop_exec[0] = nullptr;
    }
    return ASC_OK;
}

asc_status run_traversal_impl(asc_graph *g, asc_algo algo, uint32_t source, const asc_params &p, void *out,
                              asc_stats *st) {
    Workspace *ws = g->ws;
    const uint32_t V = (uint32_t)g->V;
    cudaStream_t s = g->stream;
    const bool all = algo == ASC_CC;
    uint32_t launches = 0;
    PhaseTimer pt(ws, (p.flags & ASC_RUN_PHASE_TIMING) != 0);
    // bottom-up steps: BFS on a CSR graph, in the CUDA-graph loop or the host
    // loop (the per-region timing, fragment counting and gather-and-copy runs
    // measure the top-down expansion alone)
    ws->bu_active = algo == ASC_BFS && ws->tune.bu_div && !g->is_csc &&
                    !(p.flags & (ASC_RUN_FRAGMENT_COUNTS | ASC_RUN_GATHER_COPY | ASC_RUN_PARTITION_COPY));
    if (ws->bu_active) ASC_TRY(ensure_in_ptr(g));
    ExpandFn expand = pick_expand(algo, edge_layout(g));
    FusedFn fused = pick_fused(algo, edge_layout(g));

    ASC_CUDA(cudaEventRecord(ws->ev[0], s));
    ASC_CUDA(cudaMemsetAsync(ws->ctl, 0, 4 * CTL_WORDS, s));
    for (int i = 0; i < 2; i++) ASC_CUDA(cudaMemsetAsync(ws->bitmap[i], 0, 4 * (V / 32 + 2), s));
    ASC_CUDA(cudaMemsetAsync(ws->visited, 0, 4 * (V / 32 + 2), s));
    const uint32_t ig = fill_grid(ws, V);
    if (algo == ASC_CC) init_values_kernel<kCC><<<ig, kBlock, 0, s>>>(ws->val, V, 0);
    else if (algo == ASC_BFS) init_values_kernel<kBFS><<<ig, kBlock, 0, s>>>(ws->val, V, source);
    else init_values_kernel<kSSSP><<<ig, kBlock, 0, s>>>(ws->val, V, source);
    if (near_far(g, algo)) {
        ASC_CUDA(cudaMemsetAsync(ws->far_bits, 0, 4 * (V / 32 + 2), s));
        ASC_CUDA(cudaStreamSynchronize(s));  // the staging word below is host memory
        ws->h_ctl[CTL_THRESH] = 1 + ws->tune.delta;
        ASC_CUDA(cudaMemcpyAsync(ws->ctl + CTL_THRESH, ws->h_ctl + CTL_THRESH, 4, cudaMemcpyHostToDevice, s));
    }
    // the seeded frontier lands in parity 0 (as the output of a virtual pass from parity 1)
    RegionArgs sa = base_args(g, 1);
    const uint32_t nwords = V / 32 + 1;
    seed_bits_kernel<<<all ? fill_grid(ws, nwords) : 1, kBlock, 0, s>>>(sa, source, all ? 1 : 0, nwords);
    build_frontier_kernel<<<fill_grid(ws, nwords), kBlock, 0, s>>>(sa, ws->bitmap[0], nwords);
    launches += 3;
    ASC_CUDA(cudaGetLastError());
    const int64_t cap = p.max_iterations > 0 ? p.max_iterations : (int64_t)4 * V + 64;
    // fragment counting runs the host-driven loop: the captured graph loop is
    // built without counters
    const bool gather = (p.flags & ASC_RUN_GATHER_COPY) != 0;
    if (gather) ASC_TRY(ensure_gather_buffers(g));
    const bool part = !gather && (p.flags & ASC_RUN_PARTITION_COPY) != 0;
    if (part) ASC_TRY(ensure_part_plan(g));
    uint64_t part_bytes = 0;
    uint32_t part_copies = 0;
    const bool use_graph = !(p.flags & (ASC_RUN_PHASE_TIMING | ASC_RUN_HOST_LOOP | ASC_RUN_FRAGMENT_COUNTS |
                                        ASC_RUN_GATHER_COPY | ASC_RUN_PARTITION_COPY));
    int iters = 0;
    double phase_ms[3] = {0, 0, 0};  // static top-down, on-demand top-down, bottom-up
    if (use_graph) {
        const uint32_t gcap = (uint32_t)std::min<int64_t>(cap, 0x7fffffff);
        ASC_TRY(build_loop_graph(g, algo, gcap));
        const int slot = algo == ASC_BFS ? 0 : (algo == ASC_SSSP ? 1 : 2);
        ASC_CUDA(cudaGraphLaunch(ws->loop_exec[slot], s));
        launches += 1;
    }
    uint32_t cnt[CTL_BLOCK] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (!use_graph) {
        ASC_CUDA(cudaMemcpyAsync(ws->h_ctl, ws->ctl, 4 * CTL_BLOCK, cudaMemcpyDeviceToHost, s));
        ASC_CUDA(cudaStreamSynchronize(s));
        memcpy(cnt, ws->h_ctl, sizeof(cnt));
    }
    int parity = 0;
    const uint32_t div = ws->tune.dense_div;
    auto region_work = [&](int region) -> uint64_t {
        const uint32_t range = region == 0 ? g->static_vertices : V - g->static_vertices;
        const bool bitmap_mode = div && cnt[6 + region] > range / div;
        return (uint64_t)cnt[2 + region] + ((bitmap_mode ? range : cnt[region]) + kBlock - 1) / kBlock;
    };
    while (cnt[6] | cnt[7]) {
        if (iters >= cap) return fail(ASC_ERR_TIMEOUT, "no fixpoint after %d iterations", iters);
        iters++;
        const int po = 1 - parity;
        ASC_CUDA(cudaMemsetAsync(ws->ctl + CTL_BLOCK * po, 0, 4 * CTL_BLOCK, s));
        ASC_CUDA(cudaMemsetAsync(ws->bitmap[po], 0, 4 * (V / 32 + 2), s));
        if (gather) {
            // the on-demand list and segments go to the host first, so the host
            // gathers while the static region expands on the device
            ASC_CUDA(cudaMemcpyAsync(ws->h_list, ws->queue[parity] + g->static_vertices, 4ull * cnt[1],
                                     cudaMemcpyDeviceToHost, s));
            ASC_CUDA(cudaMemcpyAsync(ws->h_segs, ws->segs[parity] + ws->segcap_static, 8ull * cnt[3],
                                     cudaMemcpyDeviceToHost, s));
            ASC_CUDA(cudaEventRecord(ws->ev[3], s));
            const uint64_t items0 = region_work(0);
            if (items0) {
                RegionArgs a = region_args(g, parity, 0, false);
                attach_far(g, algo, a);
                expand(g, a, grid_for(ws, items0));
                launches++;
            }
            ASC_TRY(gather_ondemand(g, algo, parity, cnt, ws->ev[3], launches));
        } else if (part) {
            // the static region in place, then every on-demand partition that
            // holds a frontier vertex: copied whole, its frontier expanded from
            // the copy (partition j of this run into buffer j % 2)
            const uint64_t items0 = region_work(0);
            if (items0) {
                RegionArgs a = region_args(g, parity, 0, false);
                attach_far(g, algo, a);
                expand(g, a, grid_for(ws, items0));
                launches++;
            }
            PartPlan *pp = ws->part;
            const uint32_t np = (uint32_t)pp->parts.size();
            if (cnt[7]) {
                part_active_kernel<<<std::min<uint32_t>(np, ws->num_sms * 8), kBlock, 0, s>>>(
                    ws->bitmap[parity], pp->d_ranges, np, pp->d_flags);
                ASC_CUDA(cudaMemsetAsync(pp->d_work, 0, 4ull * np, s));
                ASC_CUDA(cudaMemcpyAsync(pp->h_flags, pp->d_flags, 4ull * np, cudaMemcpyDeviceToHost, s));
                ASC_CUDA(cudaStreamSynchronize(s));
                launches++;
            }
            for (uint32_t k = 0; cnt[7] && k < np; k++) {
                if (!pp->h_flags[k]) continue;
                const StageLaunch &x = pp->parts[k];
                const int b = part_copies & 1;
                ASC_CUDA(cudaStreamWaitEvent(pp->copy, pp->consumed[b], 0));
                ASC_CUDA(cudaMemcpyAsync(g->d_stage[b], g->h_edges + x.w_lo, 4 * x.w_n, cudaMemcpyHostToDevice,
                                         pp->copy));
                ASC_CUDA(cudaEventRecord(pp->copied[b], pp->copy));
                ASC_CUDA(cudaStreamWaitEvent(s, pp->copied[b], 0));
                RegionArgs a = region_args(g, parity, 1, false);
                attach_far(g, algo, a);
                a.edges = (const uint32_t *)((uintptr_t)g->d_stage[b] - 4 * (uintptr_t)x.w_lo);
                a.dense_begin = x.c_lo;
                a.dense_end = x.c_hi;
                a.cnt_in = pp->d_cnt + 8ull * k;  // id-order walk of the range, no segments
                a.dense_div = 0xffffffffu;
                a.huge = 0xffffffffu;             // long lists too are expanded from the copy
                a.work = pp->d_work + k;
                expand(g, a, grid_for(ws, (x.c_hi - (x.c_lo & ~31u) + kBlock - 1) / kBlock));
                ASC_CUDA(cudaEventRecord(pp->consumed[b], s));
                launches++;
                part_copies++;
                part_bytes += 4 * x.w_n;
            }
        } else if (pt.on && ws->bu_active && ws->in_ptr && ((uint64_t)cnt[6] + cnt[7]) * ws->tune.bu_div > V) {
            // diagnostic: a bottom-up step, timed on its own
            RegionArgs a = region_args(g, parity, 0, false);
            ASC_TRY(pt.begin(2));
            pt.record(s);
            bottom_up_kernel<<<bu_grid(ws, nwords), kBlock, 0, s>>>(a, nwords);
            pt.record(s);
            launches++;
        } else if (pt.on) {
            // diagnostic: one launch per region, each timed on its own
            if (near_far(g, algo)) ASC_CUDA(cudaMemsetAsync(ws->ctl + CTL_MINFAR, 0xff, 4, s));
            for (int region = 0; region < 2; region++) {
                const uint64_t items = region_work(region);
                if (!items) continue;
                RegionArgs a = region_args(g, parity, region, false);
                attach_far(g, algo, a);
                ASC_TRY(pt.begin(region));
                pt.record(s);
                expand(g, a, grid_for(ws, items));
                pt.record(s);
                launches++;
            }
        } else {
            const uint64_t items = region_work(0) + region_work(1);
            FusedArgs x;
            x.r0 = region_args(g, parity, 0, false);
            x.r1 = region_args(g, parity, 1, false);
            attach_far(g, algo, x.r0);
            attach_far(g, algo, x.r1);
            x.work = x.r0.cnt_out + 4;
            if (near_far(g, algo)) ASC_CUDA(cudaMemsetAsync(ws->ctl + CTL_MINFAR, 0xff, 4, s));
            fused(s, x, grid_for(ws, items));
            launches++;
            if (algo == ASC_BFS && x.r0.in_ptr) {
                bottom_up_kernel<<<bu_grid(ws, nwords), kBlock, 0, s>>>(x.r0, nwords);
                launches++;
            }
        }
        {
            RegionArgs out_args = region_args(g, parity, 0, false);
            attach_far(g, algo, out_args);
            if (near_far(g, algo)) {
                launch_far(g, s, out_args);
                launches += 2;
            }
            build_frontier_kernel<<<fill_grid(ws, nwords), kBlock, 0, s>>>(out_args, ws->bitmap[po], nwords);
        }
        launches++;
        ASC_CUDA(cudaGetLastError());
        ASC_CUDA(cudaMemcpyAsync(ws->h_ctl, ws->ctl + CTL_BLOCK * po, 4 * CTL_BLOCK, cudaMemcpyDeviceToHost, s));
        ASC_CUDA(cudaStreamSynchronize(s));
        memcpy(cnt, ws->h_ctl, sizeof(cnt));
        if (pt.on) ASC_TRY(pt.sum(phase_ms));
        parity = po;
        iteration_boundary();
    }
    // a top-down BFS expands every reached vertex exactly once, so its
    // expansion counts already are the reached vertices and edges; SSSP
    // re-expands, and bottom-up steps reach vertices without expanding them,
    // so count them
    const bool count_reached = algo == ASC_SSSP || (algo == ASC_BFS && ws->bu_active);
    if (count_reached) {
        if (algo == ASC_BFS)
            reached_bits_kernel<<<fill_grid(ws, 32ull * nwords), kBlock, 0, s>>>(
                ws->visited, g->d_ptr, V, nwords, (unsigned long long *)(ws->ctl + CTL_STATS) + 4);
        else
            reached_kernel<<<fill_grid(ws, V), kBlock, 0, s>>>(ws->val, g->d_ptr, V,
                                                               (unsigned long long *)(ws->ctl + CTL_STATS) + 4);
        launches++;
    }
    ASC_CUDA(cudaEventRecord(ws->ev[1], s));
    ASC_CUDA(cudaGetLastError());
    if (out && !(p.flags & ASC_RUN_NO_OUTPUT)) {
        ASC_CUDA(cudaMemcpyAsync(out, ws->val, 4ull * V,
                                 (p.flags & ASC_RUN_DEVICE_OUT) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                 s));
    }
    ASC_CUDA(cudaEventRecord(ws->ev[2], s));
    ASC_CUDA(cudaMemcpyAsync(ws->h_ctl + CTL_STATS, ws->ctl + CTL_STATS, 4 * (CTL_BODIES + 1 - CTL_STATS),
                             cudaMemcpyDeviceToHost, s));
    ASC_CUDA(cudaMemcpyAsync(ws->h_ctl + CTL_BU_EDGES, ws->ctl + CTL_BU_EDGES, 16, cudaMemcpyDeviceToHost, s));
    ASC_CUDA(cudaStreamSynchronize(s));
    if (use_graph) {
        iters = (int)ws->h_ctl[CTL_ITERS];
        // per body: two expansions, two builds (and two near-far pairs, or two
        // bottom-up kernels), the loop test
        launches += (near_far(g, algo) ? 9 : (algo == ASC_BFS && ws->bu_active ? 7 : 5)) * ws->h_ctl[CTL_BODIES] - 1;
        if (ws->h_ctl[CTL_TIMEOUT]) return fail(ASC_ERR_TIMEOUT, "no fixpoint after %d iterations", iters);
    }
    if (st) {
        memset(st, 0, sizeof(*st));
        const unsigned long long *hs = (const unsigned long long *)(ws->h_ctl + CTL_STATS);
        const unsigned long long bu_edges = *(const unsigned long long *)(ws->h_ctl + CTL_BU_EDGES);
        st->iterations = iters;
        st->edges_processed = hs[0] + hs[1];
        st->ondemand_edges = hs[1];
        // out-edges in their stored width, in-edges of bottom-up steps in theirs
        const unsigned long long bu_od = ws->in_edges ? 0 : bu_edges;
        st->ondemand_bytes = edge_store_bytes(g, hs[1] - bu_od) + (bu_od * g->in_ebits + 7) / 8;
        if (part) {  // what the partition copies moved
            st->ondemand_bytes = part_bytes;
            st->staged_chunks = part_copies;
        }
        st->bottom_up_edges = bu_edges;
        st->bottom_up_vertices = *(const unsigned long long *)(ws->h_ctl + CTL_BU_VERTS);
        st->frontier_vertices = hs[2] + hs[3];
        st->ondemand_vertices = hs[3];
        if (algo == ASC_CC) {
            st->reached_vertices = V;
            st->reached_edges = g->E;
        } else if (algo == ASC_BFS && !count_reached) {
            st->reached_vertices = hs[2] + hs[3];
            st->reached_edges = hs[0] + hs[1];
        } else {
            st->reached_vertices = hs[4];
            st->reached_edges = hs[5];
        }
        float ms = 0;
        ASC_CUDA(cudaEventElapsedTime(&ms, ws->ev[0], ws->ev[1]));
        st->ms_total = ms;
        ASC_CUDA(cudaEventElapsedTime(&ms, ws->ev[1], ws->ev[2]));
        st->ms_copyout = ms;
        st->ms_static = phase_ms[0];
        st->ms_ondemand = phase_ms[1];
        st->ms_bottom_up = phase_ms[2];
        st->kernel_launches = launches;
    }
    return ASC_OK;
}

// Copies the FP64 ranks out as T: directly for FP64; for FP32 rounded to
// float on the device, into the caller's buffer (ASC_RUN_DEVICE_OUT) or into
// staging (a contribution array, free once the passes are over) copied out.
template <typename T>
asc_status copy_ranks_out(asc_graph *g, const double *rank, void *staging, void *out, uint32_t flags) {
    const uint32_t V = (uint32_t)g->V;
    cudaStream_t s = g->stream;
    const cudaMemcpyKind kind = (flags & ASC_RUN_DEVICE_OUT) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (sizeof(T) == 8) {
        ASC_CUDA(cudaMemcpyAsync(out, rank, 8 * (size_t)V, kind, s));
        return ASC_OK;
    }
    float *dst = (flags & ASC_RUN_DEVICE_OUT) ? (float *)out : (float *)staging;
    pr_rank_to_float_kernel<<<fill_grid(g->ws, V), kBlock, 0, s>>>(rank, dst, V);
    ASC_CUDA(cudaGetLastError());
    if (!(flags & ASC_RUN_DEVICE_OUT)) ASC_CUDA(cudaMemcpyAsync(out, staging, 4 * (size_t)V, kind, s));
    return ASC_OK;
}

template <typename T, bool REF>
static asc_status pagerank_impl(asc_graph *g, const asc_params &p, void *out, asc_stats *st) {
    Workspace *ws = g->ws;
    ASC_TRY(ensure_pr_buffers(g, sizeof(T)));
    const uint32_t V = (uint32_t)g->V;
    cudaStream_t s = g->stream;
    uint32_t launches = 0;
    PhaseTimer pt(ws, (p.flags & ASC_RUN_PHASE_TIMING) != 0);
    typedef typename PrAcc<T>::type Acc;
    // FP64 accumulators per pass parity q: acc[2q] residual, acc[2q+1] dangling mass
    double *acc = (double *)(ws->ctl + CTL_PR);
    double *rank = (double *)ws->pr_rank;
    T *c[2] = {(T *)ws->pr_contrib[0], (T *)ws->pr_contrib[1]};

    ASC_CUDA(cudaEventRecord(ws->ev[0], s));
    ASC_CUDA(cudaMemsetAsync(ws->ctl, 0, 4 * CTL_WORDS, s));
    // the start vector's dangling mass goes to the parity-1 pair, which pass 0 reads
    pr_init_kernel<T><<<fill_grid(ws, V), kBlock, 0, s>>>(rank, c[0], c[1], (Acc *)ws->pr_sum, g->d_outdeg, V,
                                                          acc + 2);
    launches++;
    RegionArgs sa = base_args(g, 1);  // seeds land in parity 0
    const uint32_t nwords = V / 32 + 1;
    if (REF) {
        // every vertex starts active: full bitmap, then lists/segments from it
        for (int i = 0; i < 2; i++) ASC_CUDA(cudaMemsetAsync(ws->bitmap[i], 0, 4 * (V / 32 + 2), s));
        seed_bits_kernel<<<fill_grid(ws, nwords), kBlock, 0, s>>>(sa, 0, 1, nwords);
        build_frontier_kernel<<<fill_grid(ws, nwords), kBlock, 0, s>>>(sa, ws->bitmap[0], nwords);
        launches += 2;
    } else if (ws->n_huge_total) {
        seed_huge_segments_kernel<<<fill_grid(ws, ws->n_huge_total), kBlock, 0, s>>>(
            sa, ws->huge_list, ws->n_huge_static, ws->n_huge_total);
        launches++;
    }
    ASC_CUDA(cudaGetLastError());
    ASC_CUDA(cudaMemcpyAsync(ws->h_ctl, ws->ctl, 4 * CTL_BLOCK, cudaMemcpyDeviceToHost, s));
    ASC_CUDA(cudaStreamSynchronize(s));
    uint32_t cnt[CTL_BLOCK];
    memcpy(cnt, ws->h_ctl, sizeof(cnt));

    // standard PageRank on a graph with staging buffers: the on-demand edges are
    // copied in chunks every pass, overlapped with the kernels
    bool staged = false;
    if (!REF && !pt.on && !(p.flags & ASC_RUN_NO_STAGING)) ASC_TRY(ensure_stage_plan(g, &staged));
    StagePlan *sp = staged ? ws->stage : nullptr;

    // REF: the active set alternates parity like a traversal frontier. STD:
    // every vertex every pass (dense ranges), fixed segment list in parity 0.
    int parity = 0;
    int it = 0;
    const int max_it = p.max_iterations > 0 ? p.max_iterations : (REF ? 1000000 : 100);
    double residual = 0;
    double phase_ms[2] = {0, 0};
    for (;;) {
        if (REF && !(cnt[6] | cnt[7])) break;
        if (it >= max_it) {
            if (REF) return fail(ASC_ERR_TIMEOUT, "reference PageRank still active after %d passes", it);
            break;
        }
        const int cp = it & 1;
        const int po = 1 - parity;
        ASC_CUDA(cudaMemsetAsync(ws->ctl + CTL_BLOCK * po, 0, 4 * CTL_BLOCK, s));
        if (REF) ASC_CUDA(cudaMemsetAsync(ws->bitmap[po], 0, 4 * (V / 32 + 2), s));
        if (!REF) ASC_CUDA(cudaMemsetAsync(acc + 2 * cp, 0, 16, s));
        PrArgs<T> pa;
        memset(&pa, 0, sizeof(pa));
        pa.outdeg = g->d_outdeg;
        pa.rank = rank;
        pa.c_old = c[cp];
        pa.c_new = c[1 - cp];
        pa.sum = (Acc *)ws->pr_sum;
        pa.damping = REF ? 0.85 : p.damping;
        pa.acc = acc + 2 * cp;
        pa.dangling_prev = acc + 2 * (1 - cp) + 1;
        uint64_t region_items[2];
        for (int region = 0; region < 2; region++) {
            const uint32_t range = region == 0 ? g->static_vertices : V - g->static_vertices;
            const bool bitmap_mode = REF && ws->tune.dense_div && cnt[6 + region] > range / ws->tune.dense_div;
            const uint32_t nvert = REF ? (bitmap_mode ? range : cnt[region]) : range;
            region_items[region] = (uint64_t)cnt[2 + region] + (nvert + kBlock - 1) / kBlock;
        }
        if (staged) {
            ASC_CUDA(cudaMemsetAsync(sp->d_work, 0, 4 * sp->launches.size(), s));
            for (uint32_t k = 0; k < (uint32_t)sp->launches.size(); k++) {
                asc_status cs;
                const uint32_t *chunk_edges = stage_chunk(g, sp, k, s, &cs);
                ASC_TRY(cs);
                PrArgs<T> p0 = pa, p1 = pa;
                p0.r = region_args(g, parity, 0, true);
                p1.r = region_args(g, parity, 1, true);
                stage_region(sp, k, 0, chunk_edges, p0.r);
                stage_region(sp, k, 1, chunk_edges, p1.r);
                pr_pull_fused_kernel<T, REF><<<grid_for(ws, sp->launches[k].items()), kBlock, 0, s>>>(p0, p1);
                ASC_TRY(stage_release(sp, k, s));
                launches++;
            }
        } else if (!pt.on) {
            // one launch for both regions (the timed split below runs them apart)
            if (region_items[0] + region_items[1]) {
                PrArgs<T> p0 = pa, p1 = pa;
                p0.r = region_args(g, parity, 0, !REF);
                p1.r = region_args(g, parity, 1, !REF);
                p1.r.stage_edges = !REF && pr_tile_stage(g);
                pr_pull_fused_kernel<T, REF>
                    <<<grid_for(ws, region_items[0] + region_items[1]), kBlock, 0, s>>>(p0, p1);
                launches++;
            }
        } else {
            for (int region = 0; region < 2; region++) {
                if (!region_items[region]) continue;
                pa.r = region_args(g, parity, region, !REF);
                pa.r.stage_edges = region == 1 && !REF && pr_tile_stage(g);
                ASC_TRY(pt.begin(region));
                pt.record(s);
                pr_pull_kernel<T, REF><<<grid_for(ws, region_items[region]), kBlock, 0, s>>>(pa);
                pt.record(s);
                launches++;
            }
        }
        const uint32_t nseg_items = REF ? cnt[2] + cnt[3] : ws->n_huge_total;
        if (nseg_items) {
            pa.r = region_args(g, parity, 0, !REF);
            pr_apply_segmented_kernel<T, REF><<<fill_grid(ws, nseg_items), kBlock, 0, s>>>(
                pa, ws->segs[parity], ws->segs[parity] + ws->segcap_static, ws->huge_list, ws->n_huge_total);
            launches++;
        }
        if (REF) {
            build_frontier_kernel<<<fill_grid(ws, nwords), kBlock, 0, s>>>(region_args(g, parity, 0, false),
                                                                            ws->bitmap[po], nwords);
            launches++;
        }
        ASC_CUDA(cudaGetLastError());
        if (REF)
            ASC_CUDA(cudaMemcpyAsync(ws->h_ctl, ws->ctl + CTL_BLOCK * po, 4 * CTL_BLOCK, cudaMemcpyDeviceToHost, s));
        else ASC_CUDA(cudaMemcpyAsync(ws->h_ctl, acc + 2 * cp, 16, cudaMemcpyDeviceToHost, s));
        ASC_CUDA(cudaStreamSynchronize(s));
        if (pt.on) ASC_TRY(pt.sum(phase_ms));
        it++;
        iteration_boundary();
        if (REF) {
            memcpy(cnt, ws->h_ctl, sizeof(cnt));
            parity = po;
        } else {
            memcpy(&residual, ws->h_ctl, 8);
            if (residual < p.tolerance) break;
        }
    }
    ASC_CUDA(cudaEventRecord(ws->ev[1], s));
    if (out && !(p.flags & ASC_RUN_NO_OUTPUT)) {
        ASC_TRY(copy_ranks_out<T>(g, rank, (void *)c[0], out, p.flags));
        launches += sizeof(T) == 4;
    }
    ASC_CUDA(cudaEventRecord(ws->ev[2], s));
    ASC_CUDA(cudaMemcpyAsync(ws->h_ctl + CTL_STATS, ws->ctl + CTL_STATS, 8 * 6, cudaMemcpyDeviceToHost, s));
    ASC_CUDA(cudaStreamSynchronize(s));
    if (st) {
        memset(st, 0, sizeof(*st));
        const unsigned long long *hs = (const unsigned long long *)(ws->h_ctl + CTL_STATS);
        st->iterations = it;
        st->edges_processed = hs[0] + hs[1];
        st->ondemand_edges = hs[1];
        st->ondemand_bytes = staged ? sp->copy_bytes * (uint64_t)it : edge_store_bytes(g, hs[1]);
        st->staged_chunks = staged ? sp->chunks * (uint32_t)it : 0;
        st->frontier_vertices = hs[2] + hs[3];
        st->ondemand_vertices = hs[3];
        st->reached_vertices = V;
        st->reached_edges = g->E;
        st->residual = residual;
        float ms = 0;
        ASC_CUDA(cudaEventElapsedTime(&ms, ws->ev[0], ws->ev[1]));
        st->ms_total = ms;
        ASC_CUDA(cudaEventElapsedTime(&ms, ws->ev[1], ws->ev[2]));
        st->ms_copyout = ms;
        st->ms_static = phase_ms[0];
        st->ms_ondemand = phase_ms[1];
        st->kernel_launches = launches;
    }
    return ASC_OK;
}

// -------------------------------------------- multi-source batches (<= 64) --
//
// Up to 64 BFS or SSSP sources of one graph advance together: each vertex
// carries a 64-bit mask of the sources for which it is in the frontier, so one
// read of an edge serves every source of the batch. BFS keeps 64-bit visited /
// frontier / next masks per vertex and is level-synchronous, so each source's
// levels equal a single-source BFS from it. Batched SSSP keeps a vertex-major
// [V][64] distance block (one 256-byte row per vertex) and relaxes the sources
// of a frontier vertex's mask lane by lane; its fixpoint per source is the
// single-source one. Expansion only ORs masks and marks touched vertices in a
// bitmap; an apply pass over the touched words turns them into the next
// frontier bitmap, and the compaction kernel of the single-query engine builds
// the lists and segments.
//
// Batches are continuous: source slots are filled and emptied between
// iterations. A query joins as soon as a slot (and, for BFS, a level plane) is
// free, advances with the other sources, and leaves when its own frontier is
// empty; levels are counted from the iteration the source joined, so every
// query's values equal a solo run. asc_run_batch is one fill of the slots.
struct BatchEngine {
    asc_graph *g = nullptr;
    bool sssp = false;
    uint32_t stride = 64;             // SSSP distance row length (sources per row)
    Workspace ws;                     // own frontier lists, bitmaps, counters
    unsigned long long *visit = nullptr, *front = nullptr, *next = nullptr;
    uint32_t *touched = nullptr;      // bitmap of vertices whose next mask went non-zero
    uint32_t *dist = nullptr;         // SSSP [V][stride]
    uint32_t *plane[64] = {nullptr};  // BFS per-slot level planes [V]
    uint32_t **d_plane = nullptr;     // device copy of plane[]
    int32_t *d_lvl_off = nullptr;     // per-slot level offset (level = iteration + offset)
    int32_t lvl_off[64] = {0};
    uint32_t *staging = nullptr;      // SSSP column gather [V]
    cudaStream_t stream = nullptr;
    int parity = 0;
    uint32_t it = 0;                  // iterations run so far
    uint64_t active = 0;              // slots in use
    uint32_t pend_n = 0, pend_slot[64], pend_src[64];
};

namespace {

enum { CTL_ALIVE = 34 };  // u64 (words 34-35): OR of the new frontier masks of an iteration

struct MsArgs {
    RegionArgs r0, r1;            // frontier lists/segments/bitmaps of both regions (val unused)
    unsigned long long *visit;    // BFS: sources that reached v
    unsigned long long *front;    // sources for which v is in the current frontier
    unsigned long long *next;     // sources that reached v in this iteration (atomicOr)
    uint32_t *touched;            // bitmap: v's next mask went non-zero this iteration
    uint32_t *work;
    uint32_t *dist;               // SSSP: [V][64]
    uint32_t V;
};

struct MsSmem {
    uint32_t pref[kBlock + 1];
    uint32_t start[kBlock];
    unsigned long long f[kBlock];
    uint32_t warp[kWarps + 1];
    uint32_t work;
};

// BFS relaxation of one edge for a whole mask: true when v's next mask was empty.
__device__ __forceinline__ bool ms_reach(const MsArgs &m, uint32_t v, unsigned long long f,
                                         unsigned long long vis) {
    const unsigned long long nb = f & ~vis;
    if (!nb) return false;
    return atomicOr(&m.next[v], nb) == 0ull;
}

__device__ __forceinline__ void mark_touched(const MsArgs &m, bool first, uint32_t v) {
    if (first) atomicOr(&m.touched[v >> 5], 1u << (v & 31));
}

#ifndef ASC_MS_UNROLL
#define ASC_MS_UNROLL 4
#endif
// Edges per thread per pass in the batched BFS expansion (all loads first).
// 64-source batch, RMAT scale 22 / 24: 5.45 / 18.27 ms at 4 (32 registers, 8
// CTAs per SM), 5.58 / 18.46 at 6 (40, 6 CTAs), 5.78 / 18.96 at 8 (48, 5 CTAs).
constexpr int kMsUnroll = ASC_MS_UNROLL;

template <int WORDS>
__device__ void ms_vertices(const MsArgs &m, const RegionArgs &a, bool act, uint32_t u, MsSmem &sm) {
    uint32_t deg = 0, start = 0;
    unsigned long long f = 0;
    if (act && ASC_BAD(u >= m.V, 4, u)) act = false;
    if (act) {
        start = a.ptr[u];
        deg = a.ptr[u + 1] - start;
        if (deg > a.huge) {
            deg = 0;
            act = false;
        }
        f = m.front[u];
    }
    uint32_t total;
    uint32_t excl = block_excl_scan(deg, total, sm.warp);
    sm.pref[threadIdx.x] = excl;
    sm.start[threadIdx.x] = start;
    sm.f[threadIdx.x] = f;
    if (threadIdx.x == 0) sm.pref[kBlock] = total;
    const uint32_t nact = __syncthreads_count(act);
    for (uint32_t base = 0; base < total; base += kMsUnroll * kBlock) {
        uint32_t v[kMsUnroll];
        unsigned long long fk[kMsUnroll], vis[kMsUnroll];
#pragma unroll
        for (int k = 0; k < kMsUnroll; k++) {
            const uint32_t e = base + k * kBlock + threadIdx.x;
            v[k] = 0;
            fk[k] = 0;
            if (e < total) {
                int lo = 0, hi = kBlock;
                while (hi - lo > 1) {
                    int mid = (lo + hi) >> 1;
                    if (sm.pref[mid] <= e) lo = mid;
                    else hi = mid;
                }
                const uint64_t idx = (uint64_t)sm.start[lo] + (e - sm.pref[lo]);
                v[k] = WORDS == 2 ? __ldg(a.edges + 2 * idx) : layout_word<WORDS>(a.edges, idx, a.ebits) >> a.wbits;
                fk[k] = sm.f[lo];
                if (ASC_BAD(v[k] >= m.V, 5, v[k])) {
                    v[k] = 0;
                    fk[k] = 0;
                }
            }
        }
#pragma unroll
        for (int k = 0; k < kMsUnroll; k++) vis[k] = fk[k] ? m.visit[v[k]] : ~0ull;
#pragma unroll
        for (int k = 0; k < kMsUnroll; k++) mark_touched(m, ms_reach(m, v[k], fk[k], vis[k]), v[k]);
    }
    if (threadIdx.x == 0) {
        atomicAdd(&a.stats[a.region], (unsigned long long)total);
        atomicAdd(&a.stats[2 + a.region], (unsigned long long)nact);
    }
    __syncthreads();
}

template <int WORDS>
__device__ void ms_segment(const MsArgs &m, const RegionArgs &a, uint64_t item) {
    const uint32_t u = (uint32_t)(item >> 32), k0 = (uint32_t)item;
    if (ASC_BAD(u >= m.V, 6, u)) return;
    const uint32_t b0 = a.ptr[u], e0 = a.ptr[u + 1];
    const uint64_t b = (uint64_t)b0 + (uint64_t)k0 * a.seg_len;
    const uint64_t e = min((uint64_t)e0, b + a.seg_len);
    const uint32_t n = (uint32_t)(e - b);
    const unsigned long long f = m.front[u];
    for (uint32_t base = 0; base < n; base += kMsUnroll * kBlock) {
        uint32_t v[kMsUnroll];
        unsigned long long vis[kMsUnroll];
        bool ok[kMsUnroll];
#pragma unroll
        for (int k = 0; k < kMsUnroll; k++) {
            const uint32_t j = base + k * kBlock + threadIdx.x;
            ok[k] = j < n;
            v[k] = ok[k] ? (WORDS == 2 ? __ldg(a.edges + 2 * (b + j)) : layout_word<WORDS>(a.edges, b + j, a.ebits) >> a.wbits)
                         : 0;
            if (ok[k] && ASC_BAD(v[k] >= m.V, 5, v[k])) {
                ok[k] = false;
                v[k] = 0;
            }
        }
#pragma unroll
        for (int k = 0; k < kMsUnroll; k++) vis[k] = ok[k] ? m.visit[v[k]] : ~0ull;
#pragma unroll
        for (int k = 0; k < kMsUnroll; k++) mark_touched(m, ok[k] && ms_reach(m, v[k], f, vis[k]), v[k]);
    }
    if (threadIdx.x == 0) {
        atomicAdd(&a.stats[a.region], (unsigned long long)n);
        if (k0 == 0) atomicAdd(&a.stats[2 + a.region], 1ull);
    }
}

template <int WORDS>
__device__ __forceinline__ void ms_item(const MsArgs &m, const RegionArgs &a, uint32_t w, uint32_t n_in,
                                        uint32_t nseg, bool bitmap, MsSmem &sm) {
    if (w < nseg) {
        ms_segment<WORDS>(m, a, a.seg_in[w]);
    } else if (!bitmap) {
        const uint32_t i = (w - nseg) * kBlock + threadIdx.x;
        const bool act = i < n_in;
        ms_vertices<WORDS>(m, a, act, act ? a.q_in[i] : 0, sm);
    } else {
        const uint32_t u = (a.dense_begin & ~31u) + (w - nseg) * kBlock + threadIdx.x;
        const bool act = (region_word(a, u & ~31u) >> (u & 31)) & 1u;
        if (__syncthreads_or(act)) ms_vertices<WORDS>(m, a, act, u, sm);
    }
}

template <int WORDS>
__global__ void __launch_bounds__(kBlock) ms_bfs_expand_kernel(MsArgs m) {
    __shared__ MsSmem sm;
    uint32_t n0, s0, i0, n1, s1, i1;
    bool m0, m1;
    region_items_bits(m.r0, n0, s0, i0, m0);
    region_items_bits(m.r1, n1, s1, i1, m1);
    const uint32_t mm = min(i0, i1), total = i0 + i1;
    for (;;) {
        if (threadIdx.x == 0) sm.work = atomicAdd(m.work, 1u);
        __syncthreads();
        const uint32_t w = sm.work;
        __syncthreads();
        if (w >= total) break;
        bool od;
        uint32_t local;
        if (w < 2 * mm) {
            od = (w & 1) == 0;
            local = w >> 1;
        } else {
            od = i1 > i0;
            local = mm + (w - 2 * mm);
        }
        if (od) ms_item<WORDS>(m, m.r1, local, n1, s1, m1, sm);
        else ms_item<WORDS>(m, m.r0, local, n0, s0, m0, sm);
    }
}

// Batched SSSP expansion: one CTA per work item (a tile of frontier vertices,
// or one segment of a long list); the distances of a vertex are one row of
// dist (64 sources: 256 bytes).
#ifndef ASC_MS_SSSP_SPARSE
#define ASC_MS_SSSP_SPARSE 4
#endif
// An edge whose source vertex is active for at most this many sources is
// relaxed lane-per-edge, one 4-byte load per source and row; up to
// kMsQuadSources lane-per-edge a 16-byte quad of sources at a time; above that
// a group of lanes per edge. 64- and 8-source batches on RMAT scale 24 (16 lanes
// per many-source edge): 4-byte loads up to 8 sources and half-warps above: 75 /
// 30 ms; quads for 5-8: 75 / 26 ms; quads up to 12 or 16: 79-81 / 26 ms; quads
// for all above 4: 150 / 26 ms; 4-byte loads up to 16, 32 or 64 sources: 82,
// 101, 179 ms (64 sources).
constexpr int kMsSparseSources = ASC_MS_SSSP_SPARSE;
// Sources whose values a lane of the few-source path loads before comparing.
constexpr int kMsGroup = kMsSparseSources < 8 ? kMsSparseSources : 8;

#ifndef ASC_MS_SSSP_ROWS
#define ASC_MS_SSSP_ROWS 2
#endif
// Edges a lane group of the many-source path loads the distance rows of before
// it compares any of them, so those row reads are in flight together.
constexpr int kMsRows = ASC_MS_SSSP_ROWS;
#ifndef ASC_MS_SSSP_QUAD_SOURCES
#define ASC_MS_SSSP_QUAD_SOURCES 8
#endif
#ifndef ASC_MS_SSSP_QUADS
#define ASC_MS_SSSP_QUADS 2
#endif
// Edges whose source vertex is active for more than kMsSparseSources and at
// most kMsQuadSources sources are relaxed lane-per-edge a 16-byte quad of
// sources at a time (kMsQuads quads in flight); above that a lane group per edge.
constexpr int kMsQuadSources = ASC_MS_SSSP_QUAD_SOURCES;
constexpr int kMsQuads = ASC_MS_SSSP_QUADS;
#ifndef ASC_MS_SSSP_PER_LANE
#define ASC_MS_SSSP_PER_LANE 8
#endif
// Sources per lane of a many-source edge; the lanes sharing the edge are the
// row width over this (4: one 16-byte load per lane, 16 lanes for a 64-source
// row; 8: two loads, 8 lanes; 16: four loads, 4 lanes). 64-source batch on RMAT
// scale 24: 76 ms at 4 per lane (two edges per group in flight), 69 at 8 (two
// in flight), 71 at 8 (one), 71 at 16 (one).
constexpr int kMsPerLane = ASC_MS_SSSP_PER_LANE;
static_assert(kMsPerLane == 4 || kMsPerLane == 8 || kMsPerLane == 16, "4, 8 or 16 sources per lane");
// Distance rows of a batch hold R = 16, 32 or 64 sources (R x 4 bytes per
// vertex): the 64-wide batch, or a narrower one where a device budget cannot
// hold 64 columns of a large graph.
__host__ __device__ constexpr bool ms_row_ok(int R) { return R == 16 || R == 32 || R == 64; }

struct MsSsspSmem {
    uint32_t pref[kBlock + 1];       // exclusive degree prefix of the tile's vertices
    uint32_t start[kBlock];          // first edge of each
    uint32_t vid[kBlock];            // vertex id of each
    unsigned long long f[kBlock];    // frontier mask of each
    uint32_t warp[kWarps + 1];
    uint32_t work;
    uint32_t dv[kWarps][32];         // per warp: many-source edges of the current chunk
    uint32_t dw[kWarps][32];
    uint32_t downer[kWarps][32];
};

__device__ __forceinline__ void ms_sssp_load_edge(const RegionArgs &a, uint64_t idx, uint32_t &v, uint32_t &w) {
    if (a.wbits) {
        const uint32_t e = edge_word(a.edges, idx, a.ebits);
        v = e >> a.wbits;
        w = e & ((1u << a.wbits) - 1u);
    } else {
        const uint2 e = __ldg(reinterpret_cast<const uint2 *>(a.edges) + idx);
        v = e.x;
        w = e.y;
    }
}

// Relaxes one edge (u -> v, weight w) for the sources in f, lane-per-edge:
// the lane reads the two distance rows a 16-byte quad (four sources) at a
// time, only the quads with an active source, kMsQuads quads in flight.
template <int R>
__device__ __forceinline__ void ms_sssp_lane_quads(const MsArgs &m, uint32_t u, uint32_t v, uint32_t w,
                                                   unsigned long long f) {
    const uint4 *urow = reinterpret_cast<const uint4 *>(m.dist + (uint64_t)u * R);
    uint32_t *vrow = m.dist + (uint64_t)v * R;
    uint32_t qm = 0;
#pragma unroll
    for (int q = 0; q < R / 4; q++) qm |= ((f >> (4 * q)) & 0xfull) ? 1u << q : 0u;
    unsigned long long imp = 0;
    while (qm) {
        int qx[kMsQuads];
        uint4 du[kMsQuads], cur[kMsQuads];
#pragma unroll
        for (int k = 0; k < kMsQuads; k++) {
            qx[k] = qm ? __ffs(qm) - 1 : -1;
            qm &= qm - 1;
            du[k] = make_uint4(0, 0, 0, 0);
            cur[k] = make_uint4(0, 0, 0, 0);
            if (qx[k] >= 0) {
                du[k] = urow[qx[k]];
                cur[k] = reinterpret_cast<const uint4 *>(vrow)[qx[k]];
            }
        }
#pragma unroll
        for (int k = 0; k < kMsQuads; k++) {
            if (qx[k] < 0) continue;
            const uint32_t a4 = (uint32_t)(f >> (4 * qx[k])) & 0xfu;
            uint32_t *r = vrow + 4 * qx[k];
            const uint32_t n0 = du[k].x + w, n1 = du[k].y + w, n2 = du[k].z + w, n3 = du[k].w + w;
            uint32_t bits = 0;
            if ((a4 & 1u) && n0 < cur[k].x) { atomicMin(r + 0, n0); bits |= 1u; }
            if ((a4 & 2u) && n1 < cur[k].y) { atomicMin(r + 1, n1); bits |= 2u; }
            if ((a4 & 4u) && n2 < cur[k].z) { atomicMin(r + 2, n2); bits |= 4u; }
            if ((a4 & 8u) && n3 < cur[k].w) { atomicMin(r + 3, n3); bits |= 8u; }
            imp |= (unsigned long long)bits << (4 * qx[k]);
        }
    }
    if (imp) {
        atomicOr(&m.next[v], imp);
        atomicOr(&m.touched[v >> 5], 1u << (v & 31));
    }
}

// One warp relaxes 32 consecutive edges of the tile's flattened edge range
// [e0, e0 + 32) ∩ [0, total). An edge whose source vertex is active for at most
// kMsQuadSources sources is relaxed by its own lane for each of them; the
// others are gathered into the warp's shared slots and relaxed by groups of
// R / kMsPerLane lanes, each lane kMsPerLane sources (16-byte loads of the
// source's and the destination's distance rows of R x 4 bytes), kMsRows edges
// per group in flight.
template <int R>
__device__ __forceinline__ void ms_sssp_chunk(const MsArgs &m, const RegionArgs &a, MsSsspSmem &sm, uint32_t e0,
                                              uint32_t total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t e = e0 + lane;
    const bool ok = e < total;
    uint32_t o = 0, v = 0, w = 0;
    unsigned long long f = 0;
    if (ok) {
        int lo = 0, hi = kBlock;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (sm.pref[mid] <= e) lo = mid;
            else hi = mid;
        }
        o = (uint32_t)lo;
        ms_sssp_load_edge(a, (uint64_t)sm.start[o] + (e - sm.pref[o]), v, w);
        f = sm.f[o];
        if (ASC_BAD(v >= m.V || (f >> 1 >> (R - 1)) != 0, 8, v)) {
            v = 0;
            f = 0;
        }
    }
    const int nsrc = __popcll(f);
    const bool dense = nsrc > kMsQuadSources, mid = nsrc > kMsSparseSources && !dense;
    if (ok && nsrc && nsrc <= kMsSparseSources) {
        // few sources: this lane relaxes its edge for each of them, loading the
        // values of kMsGroup sources before comparing any
        const uint32_t u = sm.vid[o];
        uint32_t *row = m.dist + (uint64_t)v * R;
        unsigned long long fm = f, imp = 0;
        while (fm) {
            uint32_t ds[kMsGroup], cur[kMsGroup];
            int sx[kMsGroup];
#pragma unroll
            for (int k = 0; k < kMsGroup; k++) {
                sx[k] = fm ? __ffsll((long long)fm) - 1 : -1;
                fm &= fm - 1;
                ds[k] = sx[k] >= 0 ? m.dist[(uint64_t)u * R + sx[k]] : 0u;
                cur[k] = sx[k] >= 0 ? row[sx[k]] : 0u;
            }
#pragma unroll
            for (int k = 0; k < kMsGroup; k++) {
                const uint32_t nd = ds[k] + w;
                // fire-and-forget lowering: a source lowered further meanwhile
                // (or whose loaded value was stale) is marked active for v all
                // the same, which costs at most one more relaxation and never
                // changes the fixpoint
                if (sx[k] >= 0 && nd < cur[k]) {
                    atomicMin(&row[sx[k]], nd);
                    imp |= 1ull << sx[k];
                }
            }
        }
        if (imp) {
            atomicOr(&m.next[v], imp);
            atomicOr(&m.touched[v >> 5], 1u << (v & 31));
        }
    }
    if (ok && mid) ms_sssp_lane_quads<R>(m, sm.vid[o], v, w, f);
    const uint32_t dm = __ballot_sync(kFull, ok && dense);
    if (!dm) return;
    if (ok && dense) {
        const uint32_t r = __popc(dm & ((1u << lane) - 1u));
        sm.dv[wid][r] = v;
        sm.dw[wid][r] = w;
        sm.downer[wid][r] = o;
    }
    __syncwarp();
    const uint32_t nd = __popc(dm);
    // R / kMsPerLane lanes per edge, kMsPerLane sources (kMsPerLane / 4 quads) per lane
    constexpr int S = kMsPerLane < R ? kMsPerLane : R, G = R / S, Q = S / 4, EPW = 32 / G;
    const uint32_t grp = (uint32_t)lane / G, l = (uint32_t)lane % G;
    for (uint32_t j0 = 0; j0 < nd; j0 += EPW * kMsRows) {
        uint32_t vk[kMsRows], wk[kMsRows], act[kMsRows];
        uint4 du[kMsRows][Q], cur[kMsRows][Q];
#pragma unroll
        for (int k = 0; k < kMsRows; k++) {
            const uint32_t j = j0 + EPW * k + grp;
            act[k] = 0;
            vk[k] = 0;
            wk[k] = 0;
#pragma unroll
            for (int q = 0; q < Q; q++) {
                du[k][q] = make_uint4(0, 0, 0, 0);
                cur[k][q] = make_uint4(0, 0, 0, 0);
            }
            if (j < nd) {
                const uint32_t ow = sm.downer[wid][j];
                vk[k] = sm.dv[wid][j];
                wk[k] = sm.dw[wid][j];
                act[k] = (uint32_t)(sm.f[ow] >> (S * l)) & (uint32_t)((1ull << S) - 1);
                if (act[k]) {
                    const uint4 *ur = reinterpret_cast<const uint4 *>(m.dist + (uint64_t)sm.vid[ow] * R);
                    const uint4 *vr = reinterpret_cast<const uint4 *>(m.dist + (uint64_t)vk[k] * R);
#pragma unroll
                    for (int q = 0; q < Q; q++) {
                        du[k][q] = ur[Q * l + q];
                        cur[k][q] = vr[Q * l + q];
                    }
                }
            }
        }
#pragma unroll
        for (int k = 0; k < kMsRows; k++) {
            const uint32_t j = j0 + EPW * k + grp;
            uint32_t imp = 0;
            if (act[k]) {
                uint32_t *row = m.dist + (uint64_t)vk[k] * R + S * l;
#pragma unroll
                for (int q = 0; q < Q; q++) {
                    const uint32_t n0 = du[k][q].x + wk[k], n1 = du[k][q].y + wk[k];
                    const uint32_t n2 = du[k][q].z + wk[k], n3 = du[k][q].w + wk[k];
                    const uint32_t a4 = act[k] >> (4 * q);
                    uint32_t *r = row + 4 * q;
                    if ((a4 & 1u) && n0 < cur[k][q].x) { atomicMin(r + 0, n0); imp |= 1u << (4 * q); }
                    if ((a4 & 2u) && n1 < cur[k][q].y) { atomicMin(r + 1, n1); imp |= 2u << (4 * q); }
                    if ((a4 & 4u) && n2 < cur[k][q].z) { atomicMin(r + 2, n2); imp |= 4u << (4 * q); }
                    if ((a4 & 8u) && n3 < cur[k][q].w) { atomicMin(r + 3, n3); imp |= 8u << (4 * q); }
                }
            }
            // the group's improved sources as one 64-bit mask
            unsigned long long im = (unsigned long long)imp << (S * l);
#pragma unroll
            for (int d = G / 2; d > 0; d >>= 1) im |= __shfl_xor_sync(kFull, im, d);
            if (l == 0 && j < nd && im) {
                atomicOr(&m.next[vk[k]], im);
                atomicOr(&m.touched[vk[k] >> 5], 1u << (vk[k] & 31));
            }
        }
    }
    __syncwarp();  // the slots are rewritten by the next chunk
}

// One work item of the batched SSSP: a tile of up to 256 list vertices or one
// segment of a long list. The tile's edges are walked as one flattened range,
// 32 per warp per pass, so short lists do not leave lanes idle and every warp
// has loads in flight.
template <int R>
__device__ void ms_sssp_item(const MsArgs &m, const RegionArgs &a, uint32_t w, uint32_t n_in, uint32_t nseg,
                             MsSsspSmem &sm) {
    bool act = false;
    uint32_t u = 0, start = 0, deg = 0;
    unsigned long long f = 0;
    bool seg = w < nseg;
    if (seg) {
        if (threadIdx.x == 0 && !ASC_BAD((uint32_t)(a.seg_in[w] >> 32) >= m.V, 7, a.seg_in[w] >> 32)) {
            const uint64_t item = a.seg_in[w];
            const uint32_t k0 = (uint32_t)item;
            u = (uint32_t)(item >> 32);
            const uint32_t b0 = a.ptr[u], e0 = a.ptr[u + 1];
            const uint64_t b = (uint64_t)b0 + (uint64_t)k0 * a.seg_len;
            start = (uint32_t)b;
            deg = (uint32_t)(min((uint64_t)e0, b + a.seg_len) - b);
            act = k0 == 0;  // the vertex counts once
            f = m.front[u];
        }
    } else {
        const uint32_t i = (w - nseg) * kBlock + threadIdx.x;
        if (i < n_in && !ASC_BAD(a.q_in[i] >= m.V, 7, a.q_in[i])) {
            u = a.q_in[i];
            start = a.ptr[u];
            deg = a.ptr[u + 1] - start;
            act = true;
            f = m.front[u];
        }
    }
    uint32_t total;
    const uint32_t excl = block_excl_scan(deg, total, sm.warp);
    sm.pref[threadIdx.x] = excl;
    sm.start[threadIdx.x] = start;
    sm.vid[threadIdx.x] = u;
    sm.f[threadIdx.x] = f;
    if (threadIdx.x == 0) sm.pref[kBlock] = total;
    const uint32_t nact = __syncthreads_count(act);
    for (uint32_t base = 0; base < total; base += kBlock)
        ms_sssp_chunk<R>(m, a, sm, base + (threadIdx.x & ~31u), total);
    if (threadIdx.x == 0) {
        atomicAdd(&a.stats[a.region], (unsigned long long)total);
        atomicAdd(&a.stats[2 + a.region], (unsigned long long)nact);
    }
    __syncthreads();
}

// Work items are per CTA: the static region's segments and list tiles and the
// on-demand region's, interleaved so link-bound and HBM-bound work overlap.
// The SSSP batch always builds lists (its RegionArgs carry dense_div = 0).
template <int R>
__global__ void __launch_bounds__(kBlock, ASC_MS_MIN_BLOCKS) ms_sssp_expand_kernel(MsArgs m) {
    static_assert(ms_row_ok(R), "rows of 16, 32 or 64 sources");
    __shared__ MsSsspSmem sm;
    uint32_t n0, s0, i0, n1, s1, i1;
    bool m0, m1;
    region_items_bits(m.r0, n0, s0, i0, m0);
    region_items_bits(m.r1, n1, s1, i1, m1);
    const uint32_t mm = min(i0, i1), total = i0 + i1;
    for (;;) {
        if (threadIdx.x == 0) sm.work = atomicAdd(m.work, 1u);
        __syncthreads();
        const uint32_t w = sm.work;
        __syncthreads();
        if (w >= total) break;
        bool od;
        uint32_t local;
        if (w < 2 * mm) {
            od = (w & 1) == 0;
            local = w >> 1;
        } else {
            od = i1 > i0;
            local = mm + (w - 2 * mm);
        }
        if (od) ms_sssp_item<R>(m, m.r1, local, n1, s1, sm);
        else ms_sssp_item<R>(m, m.r0, local, n0, s0, sm);
    }
}

// Apply pass over the touched bitmap: the new sources of a touched vertex
// become its frontier mask, BFS levels are written into the
// sources' planes, and the vertex's bit goes into the next frontier bitmap
// (with per-region counts for the compaction kernel). ORs every new mask into
// *alive so finished sources can be told apart.
template <bool BFS>
__global__ void ms_apply_kernel(MsArgs m, uint32_t **planes, const int32_t *lvl_off, uint32_t it,
                                unsigned long long *alive, uint32_t nwords) {
    // a warp takes 32 touched-bitmap words at a time and walks the non-empty
    // ones, lane = vertex: the level stores of one source go to 32 consecutive
    // entries of its plane (one coalesced store per source present in the word)
    const RegionArgs &a = m.r0;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    unsigned long long any = 0;
    uint32_t n0 = 0, n1 = 0;
    for (uint64_t g0 = (uint64_t)warp * 32; g0 < nwords; g0 += (uint64_t)nwarps * 32) {
        const uint64_t gw = g0 + lane;
        const uint32_t tw = gw < nwords ? m.touched[gw] : 0u;
        unsigned nz = __ballot_sync(kFull, tw != 0);
        while (nz) {
            const int j = __ffs(nz) - 1;
            nz &= nz - 1;
            const uint32_t w = (uint32_t)g0 + (uint32_t)j;
            const uint32_t word = __shfl_sync(kFull, tw, j);
            const uint32_t v = 32 * w + lane;
            unsigned long long nb = 0;
            if ((word >> lane) & 1u) {
                nb = m.next[v];
                m.next[v] = 0;
                if (BFS) {
                    nb &= ~m.visit[v];
                    m.visit[v] |= nb;
                }
                m.front[v] = nb;
                any |= nb;
            }
            if (BFS) {
                unsigned long long un = ((unsigned long long)__reduce_or_sync(kFull, (uint32_t)(nb >> 32)) << 32) |
                                        __reduce_or_sync(kFull, (uint32_t)nb);
                while (un) {
                    const int src = __ffsll((long long)un) - 1;
                    un &= un - 1;
                    if (((nb >> src) & 1ull) && !ASC_BAD(!planes[src], 12, src))
                        planes[src][v] = (uint32_t)((int32_t)it + lvl_off[src]);
                }
            }
            const unsigned nbits = __ballot_sync(kFull, nb != 0ull);
            if (lane == 0) {
                m.touched[w] = 0;
                if (nbits) {
                    a.bitmap[w] = nbits;
                    const uint32_t v0 = 32 * w;
                    const uint32_t smask =
                        v0 + 32 <= a.S ? 0xffffffffu : (v0 >= a.S ? 0 : (1u << (a.S - v0)) - 1u);
                    n0 += __popc(nbits & smask);
                    n1 += __popc(nbits & ~smask);
                }
            }
        }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) any |= __shfl_down_sync(kFull, any, d);
    if (lane == 0) {
        if (any) atomicOr(alive, any);
        if (n0) atomicAdd(&a.cnt_out[6], n0);
        if (n1) atomicAdd(&a.cnt_out[7], n1);
    }
}

struct Admit {
    uint32_t n;
    uint32_t slot[64];
    uint32_t src[64];
};

// Resets the per-slot state of newly admitted slots: BFS clears their bits in
// every visited mask and fills their level planes, SSSP resets their distance
// columns.
__global__ void cb_clear_kernel(unsigned long long *visit, uint32_t *dist, uint32_t stride, uint32_t **planes,
                                unsigned long long newmask, uint32_t V, uint32_t fill, uint32_t sssp) {
    if (sssp) {
        // stride / 4 lanes per distance row (16 for 64 sources): lane l owns
        // sources 4l..4l+3, one 16-byte store when all four are new, else a merge
        const uint32_t lanes = stride / 4;
        const uint32_t l = threadIdx.x % lanes;
        const uint32_t m4 = (uint32_t)(newmask >> (4 * l)) & 0xfu;
        if (!m4) return;
        const uint64_t h0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) / lanes;
        const uint64_t hs = ((uint64_t)gridDim.x * blockDim.x) / lanes;
        for (uint64_t v = h0; v < V; v += hs) {
            uint4 *p = reinterpret_cast<uint4 *>(dist + v * stride) + l;
            uint4 x = make_uint4(fill, fill, fill, fill);
            if (m4 != 0xfu) {
                const uint4 o = *p;
                if (!(m4 & 1u)) x.x = o.x;
                if (!(m4 & 2u)) x.y = o.y;
                if (!(m4 & 4u)) x.z = o.z;
                if (!(m4 & 8u)) x.w = o.w;
            }
            *p = x;
        }
        return;
    }
    for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (uint64_t)gridDim.x * blockDim.x) {
        unsigned long long t = newmask;
        visit[v] &= ~newmask;
        while (t) {
            const int s = __ffsll((long long)t) - 1;
            t &= t - 1;
            if (!ASC_BAD(!planes[s], 11, s)) planes[s][v] = fill;
        }
    }
}

// Admission, phase 1: a new source that is not in the current frontier gets a
// fresh frontier mask (front[] of non-members may hold stale bits).
__global__ void cb_admit_reset_kernel(Admit ad, unsigned long long *front, const uint32_t *bitmap_cur) {
    const uint32_t i = threadIdx.x;
    if (i < ad.n) {
        const uint32_t v = ad.src[i];
        if (!((bitmap_cur[v >> 5] >> (v & 31)) & 1u)) front[v] = 0;
    }
}

// Admission, phase 2: marks each source at level / distance 1 and adds it to
// the current frontier: a vertex that was not a member gets its bit and its
// region count, and joins its region list (or, for a long list, the segment
// list). A region walked through its bitmap ignores the list.
__global__ void cb_admit_kernel(Admit ad, MsArgs m, RegionArgs cur, uint32_t **planes, uint32_t stride,
                                uint32_t sssp) {
    const uint32_t i = threadIdx.x;
    if (i >= ad.n) return;
    const uint32_t s = ad.slot[i], v = ad.src[i];
    if (ASC_BAD(v >= m.V || s >= stride || (!sssp && !planes[s]), 9, v)) return;
    const unsigned long long bit = 1ull << s;
    if (sssp) m.dist[(uint64_t)v * stride + s] = 1;
    else {
        atomicOr(&m.visit[v], bit);
        planes[s][v] = 1;
    }
    atomicOr(&m.front[v], bit);
    const uint32_t vb = 1u << (v & 31);
    if (atomicOr(&cur.bitmap[v >> 5], vb) & vb) return;  // already in the frontier
    const bool od = v >= cur.S;
    atomicAdd(&cur.cnt_out[6 + od], 1u);
    const uint32_t deg = cur.ptr[v + 1] - cur.ptr[v];
    if (deg > cur.huge) {
        const uint32_t nseg = (deg + cur.seg_len - 1) / cur.seg_len;
        const uint32_t sb = atomicAdd(&cur.cnt_out[2 + od], nseg);
        if (ASC_BAD((uint64_t)sb + nseg > (od ? cur.segcap_ondemand : cur.segcap_static), 10, sb)) return;
        uint64_t *dst = cur.seg_out + (od ? cur.segcap_static : 0) + sb;
        for (uint32_t k = 0; k < nseg; k++) dst[k] = ((uint64_t)v << 32) | k;
    } else {
        const uint32_t pos = atomicAdd(&cur.cnt_out[od], 1u);
        if (ASC_BAD((od ? cur.S : 0) + pos >= (od ? cur.V : cur.S), 10, pos)) return;
        cur.q_out[(od ? cur.S : 0) + pos] = v;
    }
}

__global__ void cb_gather_column_kernel(const uint32_t *dist, uint32_t stride, uint32_t s, uint32_t *out, uint32_t V) {
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x)
        out[v] = dist[(uint64_t)v * stride + s];
}

}  // namespace

uint64_t batch_state_bytes(asc_graph *g, bool sssp, uint32_t stride) {
    const uint64_t V = g->V;
    uint64_t b = 24 * V + 4 * (V / 32 + 2) + 16 * V + 4 * 4 * (V / 32 + 2) + 8 * (g->E / 256 + 1024) + 4096;
    if (sssp) b += 4ull * V * stride + 4 * V;
    return b;
}

uint64_t batch_plane_bytes(asc_graph *g) { return 4ull * g->V; }

thread_local IterationHook t_iteration_hook;

// Self-checking build: the first index check that failed since the last call
// (after the launching stream was synchronized), as an error.
asc_status self_check_result() {
#ifdef ASC_SELF_CHECK
    unsigned long long v = 0;
    ASC_CUDA(cudaMemcpyFromSymbol(&v, g_self_check, sizeof(v)));
    if (v) {
        const unsigned long long zero = 0;
        ASC_CUDA(cudaMemcpyToSymbol(g_self_check, &zero, sizeof(zero)));
        return fail(ASC_ERR_CUDA, "self-check failed at site %u, index %u", (unsigned)(v >> 32), (unsigned)v);
    }
#endif
    return ASC_OK;
}

// Device bytes a graph's single-query state needs (an upper bound before the
// first run; exact afterwards), with the PageRank buffers when asked for.
uint64_t workspace_bytes(asc_graph *g, bool pagerank) {
    const uint64_t V = g->V, E = g->E;
    const Tuning t = g->ws ? g->ws->tune : (g->has_tuning ? g->tuning : Tuning());
    uint64_t b;
    if (g->ws) {
        b = g->ws->device_bytes;
    } else {
        // alloc_workspace: values, two queues, five bitmaps, control words, and
        // two segment lists plus the list of long-list vertices (a list of d >
        // huge_degree edges is ceil(d / segment_edges) <= d / segment_edges + 1
        // segments, and there are at most E / (huge_degree + 1) such lists)
        const uint64_t huge = E / ((uint64_t)t.huge_degree + 1) + 1;
        const uint64_t segs = E / std::max<uint32_t>(1, t.segment_edges) + huge;
        b = 12 * V + 20 * (V / 32 + 2) + 4 * CTL_WORDS + 16 * segs + 4 * huge + 8 * 16;
    }
    if (pagerank && (!g->ws || !g->ws->pr_rank)) b += 4ull * 8 * V;
    // in-edge offsets of bottom-up BFS steps, allocated on the first BFS (with
    // the in-edges themselves when every out-edge is resident)
    if (!g->is_csc && t.bu_div && (!g->ws || !g->ws->in_ptr)) {
        b += 4 * (V + 1) + 4 * (V / 32 + 2);
        if (g->static_edges >= E) b += 4 * (g->in_ebits == 32 ? std::max<uint64_t>(1, E) : (E * g->in_ebits + 31) / 32 + 1);
    }
    return b;
}

void batch_destroy(BatchEngine *b) {
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    free_ws_buffers(&b->ws);
    for (void *p : {(void *)b->visit, (void *)b->front, (void *)b->next, (void *)b->touched, (void *)b->dist,
                    (void *)b->d_plane, (void *)b->d_lvl_off, (void *)b->staging})
        if (p) cudaFree(p);
    for (auto p : b->plane)
        if (p) cudaFree(p);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

asc_status batch_create(asc_graph *g, bool sssp, uint32_t stride, BatchEngine **out) {
    BatchEngine *b = new BatchEngine();
    b->g = g;
    b->sssp = sssp;
    b->stride = stride;
    asc_status st = stride == 64 || (sssp && (stride == 16 || stride == 32))
                        ? ASC_OK
                        : fail(ASC_ERR_UNSUPPORTED, "batch rows of %u sources", stride);
    // 64-source batches keep the default thresholds: a graph's tuning is chosen on
    // single-source runs, and the batch kernels measured faster with the defaults
    if (st == ASC_OK) st = alloc_workspace(g, &b->ws, false);
    if (sssp) b->ws.tune.dense_div = 0;  // the SSSP batch walks lists only
    const uint64_t V = g->V;
    auto al = [&](void **p, size_t n) {
        if (st != ASC_OK) return;
        cudaError_t e = cudaMalloc(p, n ? n : 16);
        if (e != cudaSuccess) st = cuda_fail(e, "cudaMalloc", __FILE__, __LINE__);
    };
    al((void **)&b->visit, 8 * V);
    al((void **)&b->front, 8 * V);
    al((void **)&b->next, 8 * V);
    al((void **)&b->touched, 4 * (V / 32 + 2));
    al((void **)&b->d_plane, 8 * 64);
    al((void **)&b->d_lvl_off, 4 * 64);
    if (sssp) {
        al((void **)&b->dist, 4ull * V * stride);
        al((void **)&b->staging, 4 * V);
    }
    if (st == ASC_OK) {
        cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) st = cuda_fail(e, "cudaStreamCreate", __FILE__, __LINE__);
    }
    // empty start state: no frontier, zero masks
    if (st == ASC_OK) {
        cudaError_t e = cudaMemsetAsync(b->ws.ctl, 0, 4 * CTL_WORDS, b->stream);
        for (int i = 0; i < 2 && e == cudaSuccess; i++)
            e = cudaMemsetAsync(b->ws.bitmap[i], 0, 4 * (V / 32 + 2), b->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(b->touched, 0, 4 * (V / 32 + 2), b->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(b->visit, 0, 8 * V, b->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(b->front, 0, 8 * V, b->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(b->next, 0, 8 * V, b->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(b->d_plane, 0, 8 * 64, b->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
        if (e != cudaSuccess) st = cuda_fail(e, "batch init", __FILE__, __LINE__);
    }
    if (st != ASC_OK) {
        batch_destroy(b);
        return st;
    }
    *out = b;
    return ASC_OK;
}

bool batch_has_plane(BatchEngine *b, uint32_t slot) { return b->sssp || b->plane[slot] != nullptr; }

// Queues a source for slot (joins before the next iteration). BFS slots need
// their level plane; it is allocated here on first use.
asc_status batch_admit(BatchEngine *b, uint32_t slot, uint32_t source) {
    if (!b->sssp && !b->plane[slot]) {
        ASC_CUDA(cudaMalloc(&b->plane[slot], 4ull * b->g->V));
        ASC_CUDA(cudaMemcpyAsync(b->d_plane, b->plane, 8 * 64, cudaMemcpyHostToDevice, b->stream));
    }
    b->pend_slot[b->pend_n] = slot;
    b->pend_src[b->pend_n] = source;
    b->pend_n++;
    b->active |= 1ull << slot;
    return ASC_OK;
}

bool batch_busy(const BatchEngine *b) { return b->active != 0; }

// Drops every source of a batch whose launch or collection failed: the batch
// is idle afterwards (its state is undefined until new sources are admitted).
void batch_abort(BatchEngine *b) {
    b->active = 0;
    b->pend_n = 0;
}

uint32_t batch_slots(const BatchEngine *b) { return b->sssp ? b->stride : 64u; }

// Applies the queued admissions and launches one iteration on the batch's
// stream, ending with the readback of its counts (nothing waits here).
asc_status batch_launch(BatchEngine *b) {
    asc_graph *g = b->g;
    Workspace *ws = &b->ws;
    cudaStream_t s = b->stream;
    const uint32_t V = (uint32_t)g->V;
    const uint32_t nwords = V / 32 + 1;
    const int p = b->parity, po = 1 - p;
    MsArgs m;
    memset(&m, 0, sizeof(m));
    m.visit = b->visit;
    m.front = b->front;
    m.next = b->next;
    m.touched = b->touched;
    m.dist = b->dist;
    m.V = V;
    if (b->pend_n) {
        Admit ad;
        memset(&ad, 0, sizeof(ad));
        ad.n = b->pend_n;
        unsigned long long newmask = 0;
        for (uint32_t i = 0; i < b->pend_n; i++) {
            ad.slot[i] = b->pend_slot[i];
            ad.src[i] = b->pend_src[i];
            newmask |= 1ull << ad.slot[i];
            b->lvl_off[ad.slot[i]] = 2 - (int32_t)(b->it + 1);  // found in the next iteration: level 2
        }
        ASC_CUDA(cudaMemcpyAsync(b->d_lvl_off, b->lvl_off, 4 * 64, cudaMemcpyHostToDevice, s));
        cb_clear_kernel<<<fill_grid(ws, V), kBlock, 0, s>>>(b->visit, b->dist, b->stride, b->d_plane, newmask, V, V + 1,
                                                             b->sssp ? 1 : 0);
        RegionArgs cur = base_args(g, ws, 1 - p);  // the lists/bitmap/counts of parity p (this iteration's input)
        cb_admit_reset_kernel<<<1, 64, 0, s>>>(ad, b->front, ws->bitmap[p]);
        cb_admit_kernel<<<1, 64, 0, s>>>(ad, m, cur, b->d_plane, b->stride, b->sssp ? 1 : 0);
        ASC_CUDA(cudaGetLastError());
        b->pend_n = 0;
    }
    unsigned long long *alive = (unsigned long long *)(ws->ctl + CTL_ALIVE);
    ASC_CUDA(cudaMemsetAsync(ws->ctl + CTL_BLOCK * po, 0, 4 * CTL_BLOCK, s));
    ASC_CUDA(cudaMemsetAsync(alive, 0, 8, s));
    ASC_CUDA(cudaMemsetAsync(ws->bitmap[po], 0, 4 * (V / 32 + 2), s));
    m.r0 = region_args(g, ws, p, 0, false);
    m.r1 = region_args(g, ws, p, 1, false);
    m.work = m.r0.cnt_out + 4;
    const uint32_t grid = (uint32_t)(ws->num_sms * ws->tune.ctas_per_sm);
    b->it++;
    if (b->sssp && b->stride == 16) ms_sssp_expand_kernel<16><<<grid, kBlock, 0, s>>>(m);
    else if (b->sssp && b->stride == 32) ms_sssp_expand_kernel<32><<<grid, kBlock, 0, s>>>(m);
    else if (b->sssp) ms_sssp_expand_kernel<64><<<grid, kBlock, 0, s>>>(m);
    else if (g->edge_words == 2) ms_bfs_expand_kernel<2><<<grid, kBlock, 0, s>>>(m);
    else if (g->ebits < 32) ms_bfs_expand_kernel<kBitsLayout><<<grid, kBlock, 0, s>>>(m);
    else ms_bfs_expand_kernel<1><<<grid, kBlock, 0, s>>>(m);
    if (b->sssp) ms_apply_kernel<false><<<fill_grid(ws, nwords), kBlock, 0, s>>>(m, b->d_plane, b->d_lvl_off, b->it,
                                                                               alive, nwords);
    else ms_apply_kernel<true><<<fill_grid(ws, nwords), kBlock, 0, s>>>(m, b->d_plane, b->d_lvl_off, b->it, alive,
                                                                        nwords);
    build_frontier_kernel<<<fill_grid(ws, nwords), kBlock, 0, s>>>(m.r0, ws->bitmap[po], nwords);
    ASC_CUDA(cudaGetLastError());
    ASC_CUDA(cudaMemcpyAsync(ws->h_ctl + CTL_ALIVE, alive, 8, cudaMemcpyDeviceToHost, s));
    b->parity = po;
    return ASC_OK;
}

// Waits for the launched iteration and reports the slots whose sources have
// no frontier left (their values are final).
asc_status batch_collect(BatchEngine *b, uint64_t *finished) {
    ASC_CUDA(cudaStreamSynchronize(b->stream));
    ASC_TRY(self_check_result());
    unsigned long long al = 0;
    memcpy(&al, b->ws.h_ctl + CTL_ALIVE, 8);
    *finished = b->active & ~al;
    b->active &= al;
    return ASC_OK;
}

// Copies a finished slot's values (V u32) to host or device memory.
asc_status batch_fetch(BatchEngine *b, uint32_t slot, void *out, bool device_out = false) {
    const uint32_t V = (uint32_t)b->g->V;
    const cudaMemcpyKind kind = device_out ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (b->sssp) {
        cb_gather_column_kernel<<<fill_grid(&b->ws, V), kBlock, 0, b->stream>>>(b->dist, b->stride, slot, b->staging, V);
        ASC_CUDA(cudaGetLastError());
        ASC_CUDA(cudaMemcpyAsync(out, b->staging, 4ull * V, kind, b->stream));
    } else {
        ASC_CUDA(cudaMemcpyAsync(out, b->plane[slot], 4ull * V, kind, b->stream));
    }
    ASC_CUDA(cudaStreamSynchronize(b->stream));
    return ASC_OK;
}

// asc_run_batch: all n sources fill slots 0..n-1 of the graph's own batch
// engine (kept for later batches), then iterations run until every source is
// done; each finished slot's values are copied to row i of out.
asc_status run_batch(asc_graph *g, asc_algo algo, const uint32_t *sources, uint32_t n, const asc_params &p,
                     void *out, asc_stats *st) {
    ASC_TRY(ensure_workspace(g));
    Workspace *ws = g->ws;
    const int k = algo == ASC_SSSP ? 1 : 0;
    if (!ws->batch[k]) ASC_TRY(batch_create(g, k == 1, 64, &ws->batch[k]));
    BatchEngine *b = ws->batch[k];
    const uint32_t V = (uint32_t)g->V;
    cudaStream_t s = b->stream;
    ASC_CUDA(cudaMemsetAsync(b->ws.ctl + CTL_STATS, 0, 8 * 6, s));
    ASC_CUDA(cudaEventRecord(ws->ev[0], s));
    for (uint32_t i = 0; i < n; i++) ASC_TRY(batch_admit(b, i, sources[i]));
    const uint32_t it0 = b->it;
    const int64_t cap = p.max_iterations > 0 ? p.max_iterations : (int64_t)4 * V + 64;
    uint64_t done = 0;
    const bool want = out && !(p.flags & ASC_RUN_NO_OUTPUT);
    double copy_ms = 0;
    while (b->active) {
        if ((int64_t)(b->it - it0) >= cap) {
            // drop the unfinished slots so the engine is reusable
            b->active = 0;
            return fail(ASC_ERR_TIMEOUT, "batch has no fixpoint after %u iterations", b->it - it0);
        }
        ASC_TRY(batch_launch(b));
        uint64_t fin = 0;
        ASC_TRY(batch_collect(b, &fin));
        done |= fin;
        if (want) {
            cudaEvent_t e0 = ws->ev[2], e1 = ws->ev[3];
            ASC_CUDA(cudaEventRecord(e0, s));
            while (fin) {
                const uint32_t slot = __builtin_ctzll(fin);
                fin &= fin - 1;
                ASC_TRY(batch_fetch(b, slot, (uint32_t *)out + (uint64_t)slot * V,
                                    (p.flags & ASC_RUN_DEVICE_OUT) != 0));
            }
            ASC_CUDA(cudaEventRecord(e1, s));
            ASC_CUDA(cudaEventSynchronize(e1));
            float ms = 0;
            ASC_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            copy_ms += ms;
        }
    }
    ASC_CUDA(cudaEventRecord(ws->ev[1], s));
    ASC_CUDA(cudaMemcpyAsync(b->ws.h_ctl + CTL_STATS, b->ws.ctl + CTL_STATS, 8 * 6, cudaMemcpyDeviceToHost, s));
    ASC_CUDA(cudaStreamSynchronize(s));
    if (st) {
        memset(st, 0, sizeof(*st));
        const unsigned long long *hs = (const unsigned long long *)(b->ws.h_ctl + CTL_STATS);
        st->iterations = (int32_t)(b->it - it0);
        st->edges_processed = hs[0] + hs[1];
        st->ondemand_edges = hs[1];
        st->ondemand_bytes = edge_store_bytes(g, hs[1]);
        st->frontier_vertices = hs[2] + hs[3];
        st->ondemand_vertices = hs[3];
        float ms = 0;
        ASC_CUDA(cudaEventElapsedTime(&ms, ws->ev[0], ws->ev[1]));
        st->ms_total = ms - copy_ms;
        st->ms_copyout = copy_ms;
        st->kernel_launches = (uint32_t)(4 * (b->it - it0) + 3);
    }
    return ASC_OK;
}

// ------------------------------------------------- PageRank over CSR graphs --
//
// Graphs stored by out-edges (.bcsr / .bwcsr) run PageRank by scatter: every
// vertex adds rank/outDeg to each out-neighbour's sum with an atomic add (FP64
// contributions in FP64; FP32 contributions exactly, as the pull's 62-bit
// fixed point, so an FP32 scatter's sums do not depend on the order of the
// atomics), then one dense pass applies the update. The reference PageRank
// semantics (per-vertex deactivation at |delta| <= 0.001, Jacobi order) and
// the standard ones are the same as the pull kernels'.
namespace {

template <typename T>
struct PushArgs {
    typedef typename PrAcc<T>::type Acc;
    RegionArgs r0, r1;         // dense ranges and the fixed segment list
    const uint32_t *ptr;
    double *rank;
    const T *c_old;
    T *c_new;
    Acc *sum;
    uint32_t *active;          // reference mode: one bit per still-active vertex
    uint32_t *active_count;
    double damping;
    const double *dangling_prev;
    double *acc;
    uint32_t *work;
};

template <typename T>
struct PushSmem {
    uint32_t pref[kBlock + 1];
    uint32_t start[kBlock];
    typename PrAcc<T>::type c[kBlock];   // each tile vertex's contribution, as added
    uint32_t warp[kWarps + 1];
    uint32_t work;
};

template <typename T, int WORDS>
__device__ void push_tile(const PushArgs<T> &p, const RegionArgs &a, uint32_t tile, PushSmem<T> &sm) {
    typedef typename PrAcc<T>::type Acc;
    const uint32_t u = a.dense_begin + tile * kBlock + threadIdx.x;
    uint32_t deg = 0, start = 0;
    Acc c = (Acc)0;
    if (u < a.dense_end) {
        start = a.ptr[u];
        deg = a.ptr[u + 1] - start;
        if (deg > a.huge) deg = 0;
        c = PrAcc<T>::from(p.c_old[u]);
    }
    uint32_t total;
    const uint32_t excl = block_excl_scan(deg, total, sm.warp);
    sm.pref[threadIdx.x] = excl;
    sm.start[threadIdx.x] = start;
    sm.c[threadIdx.x] = c;
    if (threadIdx.x == 0) sm.pref[kBlock] = total;
    __syncthreads();
    for (uint32_t base = 0; base < total; base += kUnroll * kBlock) {
        uint32_t v[kUnroll];
        Acc ck[kUnroll];
#pragma unroll
        for (int k = 0; k < kUnroll; k++) {
            const uint32_t e = base + k * kBlock + threadIdx.x;
            v[k] = 0xffffffffu;
            ck[k] = (Acc)0;
            if (e < total) {
                int lo = 0, hi = kBlock;
                while (hi - lo > 1) {
                    int mid = (lo + hi) >> 1;
                    if (sm.pref[mid] <= e) lo = mid;
                    else hi = mid;
                }
                const uint64_t idx = (uint64_t)sm.start[lo] + (e - sm.pref[lo]);
                v[k] = WORDS == 2 ? __ldg(a.edges + 2 * idx) : edge_word(a.edges, idx, a.ebits) >> a.wbits;
                ck[k] = sm.c[lo];
                if (ASC_BAD(v[k] >= a.V, 18, v[k])) v[k] = 0xffffffffu;
            }
        }
#pragma unroll
        for (int k = 0; k < kUnroll; k++)
            if (v[k] != 0xffffffffu) atomicAdd(&p.sum[v[k]], ck[k]);
    }
    if (threadIdx.x == 0) {
        atomicAdd(&a.stats[a.region], (unsigned long long)total);
        atomicAdd(&a.stats[2 + a.region], (unsigned long long)min((uint32_t)kBlock, a.dense_end - a.dense_begin -
                                                                                       tile * kBlock));
    }
    __syncthreads();
}

template <typename T, int WORDS>
__device__ void push_segment(const PushArgs<T> &p, const RegionArgs &a, uint64_t item) {
    const uint32_t u = (uint32_t)(item >> 32), k0 = (uint32_t)item;
    if (ASC_BAD(u >= a.V, 19, u)) return;
    const uint64_t b = (uint64_t)a.ptr[u] + (uint64_t)k0 * a.seg_len;
    const uint64_t e = min((uint64_t)a.ptr[u + 1], b + a.seg_len);
    const uint32_t n = (uint32_t)(e - b);
    const typename PrAcc<T>::type c = PrAcc<T>::from(p.c_old[u]);
    for (uint32_t base = 0; base < n; base += kUnroll * kBlock) {
        uint32_t v[kUnroll];
#pragma unroll
        for (int k = 0; k < kUnroll; k++) {
            const uint32_t j = base + k * kBlock + threadIdx.x;
            v[k] = j < n ? (WORDS == 2 ? __ldg(a.edges + 2 * (b + j)) : edge_word(a.edges, b + j, a.ebits) >> a.wbits)
                         : 0xffffffffu;
            if (v[k] != 0xffffffffu && ASC_BAD(v[k] >= a.V, 18, v[k])) v[k] = 0xffffffffu;
        }
#pragma unroll
        for (int k = 0; k < kUnroll; k++)
            if (v[k] != 0xffffffffu) atomicAdd(&p.sum[v[k]], c);
    }
    if (threadIdx.x == 0) {
        atomicAdd(&a.stats[a.region], (unsigned long long)n);
        if (k0 == 0) atomicAdd(&a.stats[2 + a.region], 1ull);
    }
}

template <typename T, int WORDS>
__global__ void __launch_bounds__(kBlock, ASC_PR_MIN_BLOCKS) pr_scatter_kernel(PushArgs<T> p) {
    __shared__ PushSmem<T> sm;
    const uint32_t s0 = p.r0.cnt_in[2], s1 = p.r1.cnt_in[3];
    const uint32_t t0 = s0 + (p.r0.dense_end - p.r0.dense_begin + kBlock - 1) / kBlock;
    const uint32_t t1 = s1 + (p.r1.dense_end - p.r1.dense_begin + kBlock - 1) / kBlock;
    const uint32_t mm = min(t0, t1), total = t0 + t1;
    for (;;) {
        if (threadIdx.x == 0) sm.work = atomicAdd(p.work, 1u);
        __syncthreads();
        const uint32_t w = sm.work;
        __syncthreads();
        if (w >= total) break;
        bool od;
        uint32_t local;
        if (w < 2 * mm) {
            od = (w & 1) == 0;
            local = w >> 1;
        } else {
            od = t1 > t0;
            local = mm + (w - 2 * mm);
        }
        const RegionArgs &a = od ? p.r1 : p.r0;
        const uint32_t s = od ? s1 : s0;
        if (local < s) push_segment<T, WORDS>(p, a, a.seg_in[local]);
        else push_tile<T, WORDS>(p, a, local - s, sm);
    }
}

template <typename T, bool REF>
__global__ void pr_push_apply_kernel(PushArgs<T> p, uint32_t V) {
    __shared__ double red[2 * kWarps];
    double res = 0, dang = 0;
    uint32_t nact = 0;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < V; base += stride) {
        const uint32_t v = base + threadIdx.x;
        if (v >= V) continue;
        const double s = PrAcc<T>::value(p.sum[v]);
        p.sum[v] = 0;
        const uint32_t od = p.ptr[v + 1] - p.ptr[v];
        if (REF) {
            const uint32_t bit = 1u << (v & 31);
            if (!(p.active[v >> 5] & bit)) {
                p.c_new[v] = p.c_old[v];
                continue;
            }
            if (pr_update<T>(p.rank, p.c_old, p.c_new, v, od, s, true, 0.85, (double)V, nullptr, res, dang)) nact++;
            else atomicAnd(&p.active[v >> 5], ~bit);
        } else {
            pr_update<T>(p.rank, p.c_old, p.c_new, v, od, s, false, p.damping, (double)V, p.dangling_prev, res, dang);
        }
    }
    if (REF) {
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) nact += __shfl_down_sync(kFull, nact, d);
        if ((threadIdx.x & 31) == 0 && nact) atomicAdd(p.active_count, nact);
    } else {
        block_reduce2_atomic<T>(res, dang, p.acc, red);
    }
}

template <typename T>
__global__ void pr_push_init_kernel(double *rank, T *c0, T *c1, typename PrAcc<T>::type *sum, const uint32_t *ptr,
                                    uint32_t *active, uint32_t V, double *acc_pair) {
    __shared__ double red[2 * kWarps];
    double d = 0;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < V; base += stride) {
        const uint32_t i = base + threadIdx.x;
        if (i < V) {
            const double r = 1.0 / (double)V;
            const uint32_t od = ptr[i + 1] - ptr[i];
            rank[i] = r;
            const T c = od ? (T)(r / (double)od) : (T)0;
            c0[i] = c;
            c1[i] = c;
            sum[i] = 0;
            if (od == 0) d += r;
        }
        if (i < (V + 31) / 32) active[i] = 0xffffffffu;
    }
    block_reduce2_atomic<T>(0.0, d, acc_pair, red);
}

}  // namespace

template <typename T, bool REF, int WORDS>
static asc_status pagerank_push_impl(asc_graph *g, const asc_params &p, void *out, asc_stats *st) {
    Workspace *ws = g->ws;
    ASC_TRY(ensure_pr_buffers(g, sizeof(T)));
    const uint32_t V = (uint32_t)g->V;
    cudaStream_t s = g->stream;
    uint32_t launches = 0;
    double *acc = (double *)(ws->ctl + CTL_PR);   // residual/dangling pairs by pass parity
    uint32_t *active_count = ws->ctl + CTL_PR + 8;  // word 40
    typedef typename PrAcc<T>::type Acc;
    double *rank = (double *)ws->pr_rank;
    T *c[2] = {(T *)ws->pr_contrib[0], (T *)ws->pr_contrib[1]};
    uint32_t *active = ws->bitmap[1];

    ASC_CUDA(cudaEventRecord(ws->ev[0], s));
    ASC_CUDA(cudaMemsetAsync(ws->ctl, 0, 4 * CTL_WORDS, s));
    pr_push_init_kernel<T><<<fill_grid(ws, V), kBlock, 0, s>>>(rank, c[0], c[1], (Acc *)ws->pr_sum, g->d_ptr, active,
                                                               V, acc + 2);
    launches++;
    if (ws->n_huge_total) {
        seed_huge_segments_kernel<<<fill_grid(ws, ws->n_huge_total), kBlock, 0, s>>>(
            base_args(g, 1), ws->huge_list, ws->n_huge_static, ws->n_huge_total);
        launches++;
    }
    ASC_CUDA(cudaGetLastError());
    const int max_it = p.max_iterations > 0 ? p.max_iterations : (REF ? 1000000 : 100);
    const uint32_t grid = (uint32_t)(ws->num_sms * ws->tune.ctas_per_sm);
    bool staged = false;
    if (!REF && !(p.flags & ASC_RUN_NO_STAGING)) ASC_TRY(ensure_stage_plan(g, &staged));
    StagePlan *sp = staged ? ws->stage : nullptr;
    int it = 0;
    double residual = 0;
    for (;;) {
        if (it >= max_it) {
            if (REF) return fail(ASC_ERR_TIMEOUT, "reference PageRank still active after %d passes", it);
            break;
        }
        const int cp = it & 1;
        ASC_CUDA(cudaMemsetAsync(ws->ctl + CTL_BLOCK, 0, 4 * CTL_BLOCK, s));  // work cursors (block 1)
        ASC_CUDA(cudaMemsetAsync(REF ? (void *)active_count : (void *)(acc + 2 * cp), 0, REF ? 4 : 16, s));
        PushArgs<T> pa;
        memset(&pa, 0, sizeof(pa));
        pa.r0 = region_args(g, 0, 0, true);
        pa.r1 = region_args(g, 0, 1, true);
        pa.work = ws->ctl + CTL_BLOCK + 4;
        pa.ptr = g->d_ptr;
        pa.rank = rank;
        pa.c_old = c[cp];
        pa.c_new = c[1 - cp];
        pa.sum = (Acc *)ws->pr_sum;
        pa.active = active;
        pa.active_count = active_count;
        pa.damping = REF ? 0.85 : p.damping;
        pa.acc = acc + 2 * cp;
        pa.dangling_prev = acc + 2 * (1 - cp) + 1;
        if (staged) {
            ASC_CUDA(cudaMemsetAsync(sp->d_work, 0, 4 * sp->launches.size(), s));
            for (uint32_t k = 0; k < (uint32_t)sp->launches.size(); k++) {
                asc_status cs;
                const uint32_t *chunk_edges = stage_chunk(g, sp, k, s, &cs);
                ASC_TRY(cs);
                PushArgs<T> pk = pa;
                stage_region(sp, k, 0, chunk_edges, pk.r0);
                stage_region(sp, k, 1, chunk_edges, pk.r1);
                pk.work = sp->d_work + k;
                pr_scatter_kernel<T, WORDS><<<grid_for(ws, sp->launches[k].items()), kBlock, 0, s>>>(pk);
                ASC_TRY(stage_release(sp, k, s));
                launches++;
            }
        } else {
            pr_scatter_kernel<T, WORDS><<<grid, kBlock, 0, s>>>(pa);
            launches++;
        }
        pr_push_apply_kernel<T, REF><<<fill_grid(ws, V), kBlock, 0, s>>>(pa, V);
        launches++;
        ASC_CUDA(cudaGetLastError());
        ASC_CUDA(cudaMemcpyAsync(ws->h_ctl, REF ? (void *)active_count : (void *)(acc + 2 * cp), REF ? 4 : 16,
                                 cudaMemcpyDeviceToHost, s));
        ASC_CUDA(cudaStreamSynchronize(s));
        it++;
        iteration_boundary();
        if (REF) {
            if (ws->h_ctl[0] == 0) break;
        } else {
            memcpy(&residual, ws->h_ctl, 8);
            if (residual < p.tolerance) break;
        }
    }
    ASC_CUDA(cudaEventRecord(ws->ev[1], s));
    if (out && !(p.flags & ASC_RUN_NO_OUTPUT)) {
        ASC_TRY(copy_ranks_out<T>(g, rank, (void *)c[0], out, p.flags));
        launches += sizeof(T) == 4;
    }
    ASC_CUDA(cudaEventRecord(ws->ev[2], s));
    ASC_CUDA(cudaMemcpyAsync(ws->h_ctl + CTL_STATS, ws->ctl + CTL_STATS, 8 * 4, cudaMemcpyDeviceToHost, s));
    ASC_CUDA(cudaStreamSynchronize(s));
    if (st) {
        memset(st, 0, sizeof(*st));
        const unsigned long long *hs = (const unsigned long long *)(ws->h_ctl + CTL_STATS);
        st->iterations = it;
        st->edges_processed = hs[0] + hs[1];
        st->ondemand_edges = hs[1];
        st->ondemand_bytes = staged ? sp->copy_bytes * (uint64_t)it : edge_store_bytes(g, hs[1]);
        st->staged_chunks = staged ? sp->chunks * (uint32_t)it : 0;
        st->frontier_vertices = hs[2] + hs[3];
        st->ondemand_vertices = hs[3];
        st->reached_vertices = V;
        st->reached_edges = g->E;
        st->residual = residual;
        float ms = 0;
        ASC_CUDA(cudaEventElapsedTime(&ms, ws->ev[0], ws->ev[1]));
        st->ms_total = ms;
        ASC_CUDA(cudaEventElapsedTime(&ms, ws->ev[1], ws->ev[2]));
        st->ms_copyout = ms;
        st->kernel_launches = launches;
    }
    return ASC_OK;
}

asc_status run_pagerank(asc_graph *g, const asc_params &p, void *out, asc_stats *st) {
    ASC_TRY(ensure_workspace(g));
    if (!g->is_csc) {
        const bool w2 = g->edge_words == 2;
        if (p.pr_mode == ASC_PR_REF)
            return w2 ? pagerank_push_impl<double, true, 2>(g, p, out, st)
                      : pagerank_push_impl<double, true, 1>(g, p, out, st);
        if (p.precision == ASC_F32)
            return w2 ? pagerank_push_impl<float, false, 2>(g, p, out, st)
                      : pagerank_push_impl<float, false, 1>(g, p, out, st);
        return w2 ? pagerank_push_impl<double, false, 2>(g, p, out, st)
                  : pagerank_push_impl<double, false, 1>(g, p, out, st);
    }
    if (p.pr_mode == ASC_PR_REF) return pagerank_impl<double, true>(g, p, out, st);
    if (p.precision == ASC_F32) return pagerank_impl<float, false>(g, p, out, st);
    return pagerank_impl<double, false>(g, p, out, st);
}

}  // namespace asc

namespace {
__global__ void link_read_kernel(const uint4 *__restrict__ src, size_t n16, unsigned long long *sink) {
    // four independent 16-byte loads in flight per thread
    uint32_t acc = 0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * stride < n16; i += 4 * stride) {
        uint4 a = __ldg(src + i), b = __ldg(src + i + stride), c = __ldg(src + i + 2 * stride),
              d = __ldg(src + i + 3 * stride);
        acc ^= a.x ^ a.y ^ a.z ^ a.w ^ b.x ^ b.y ^ b.z ^ b.w ^ c.x ^ c.y ^ c.z ^ c.w ^ d.x ^ d.y ^ d.z ^ d.w;
    }
    for (; i < n16; i += stride) {
        uint4 v = __ldg(src + i);
        acc ^= v.x ^ v.y ^ v.z ^ v.w;
    }
    if (acc == 0x9e3779b9u) atomicAdd(sink, 1ull);  // keeps the loads live
}
__device__ __forceinline__ uint64_t probe_mix(uint64_t x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    return x ^ (x >> 33);
}

// Each warp reads `runs` runs of L consecutive words at pseudo-random word
// offsets in [0, n4 - L), four runs in flight, lanes striding the run: the
// access shape of short adjacency lists read over the host link.
__global__ void link_runs_kernel(const uint32_t *__restrict__ src, uint64_t n4, uint32_t L, uint32_t runs,
                                 unsigned long long *sink) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t acc = 0;
    for (uint32_t r = 0; r < runs; r += 4) {
        uint32_t v[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const uint64_t off = probe_mix(warp * 1000003ull + r + k) % (n4 - L);  // off + L < n4
            v[k] = 0;
            for (uint32_t j = lane; j < L; j += 32) v[k] ^= __ldg(src + off + j);
        }
        acc ^= v[0] ^ v[1] ^ v[2] ^ v[3];
    }
    if (acc == 0x9e3779b9u) atomicAdd(sink, 1ull);  // keeps the loads live
}
}  // namespace

extern "C" asc_status asc_link_probe_runs(uint64_t bytes, uint32_t run_bytes, int iters, double *gbs) {
    using namespace asc;
    if (bytes < (1u << 20) || iters < 1 || run_bytes < 4 || run_bytes % 4 || run_bytes > bytes / 16)
        return fail(ASC_ERR_INVALID, "asc_link_probe_runs: bytes >= 1 MiB, 4 <= run_bytes <= bytes/16, "
                                     "run_bytes a multiple of 4, iters >= 1");
    bytes &= ~(uint64_t)15;
    void *h = nullptr, *hd = nullptr;
    unsigned long long *sink = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    asc_status st = ASC_OK;
    double best = 0;
    int sms = 0, dev = 0;
    auto chk = [&](cudaError_t e, const char *what) {
        if (e != cudaSuccess && st == ASC_OK) st = cuda_fail(e, what, __FILE__, __LINE__);
        return st == ASC_OK;
    };
    if (chk(cudaHostAlloc(&h, bytes, cudaHostAllocMapped | cudaHostAllocPortable), "cudaHostAlloc") &&
        chk(cudaHostGetDevicePointer(&hd, h, 0), "cudaHostGetDevicePointer") &&
        chk(cudaMalloc(&sink, 8), "cudaMalloc") && chk(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "stream") &&
        chk(cudaEventCreate(&e0), "event") && chk(cudaEventCreate(&e1), "event") && chk(cudaGetDevice(&dev), "dev") &&
        chk(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "attr")) {
        memset(h, 1, bytes);
        const uint64_t n4 = bytes / 4;
        const uint32_t L = run_bytes / 4;
        const uint64_t warps = (uint64_t)sms * 8 * (256 / 32);
        // about one pass over the buffer, a multiple of 4 runs per warp
        const uint32_t runs = (uint32_t)std::max<uint64_t>(4, (n4 / (warps * L)) & ~3ull);
        for (int i = 0; i < iters + 1 && st == ASC_OK; i++) {
            float ms = 0;
            chk(cudaEventRecord(e0, s), "rec");
            link_runs_kernel<<<sms * 8, 256, 0, s>>>((const uint32_t *)hd, n4, L, runs, sink);
            chk(cudaGetLastError(), "launch");
            chk(cudaEventRecord(e1, s), "rec");
            chk(cudaEventSynchronize(e1), "sync");
            chk(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
            if (i > 0 && ms > 0) best = std::max(best, (double)warps * runs * run_bytes / (ms * 1e6));
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    if (sink) cudaFree(sink);
    if (h) cudaFreeHost(h);
    if (gbs) *gbs = best;
    return st;
}

extern "C" asc_status asc_link_probe(uint64_t bytes, int iters, double *dma_h2d_gbs, double *sm_read_gbs) {
    using namespace asc;
    if (bytes < (1u << 20) || iters < 1) return fail(ASC_ERR_INVALID, "asc_link_probe: bytes >= 1 MiB, iters >= 1");
    bytes &= ~(uint64_t)15;
    void *h = nullptr, *d = nullptr, *hd = nullptr;
    unsigned long long *sink = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    asc_status st = ASC_OK;
    double best_dma = 0, best_sm = 0;
    int sms = 0, dev = 0;
    auto chk = [&](cudaError_t e, const char *what) {
        if (e != cudaSuccess && st == ASC_OK) st = cuda_fail(e, what, __FILE__, __LINE__);
        return st == ASC_OK;
    };
    if (chk(cudaHostAlloc(&h, bytes, cudaHostAllocMapped | cudaHostAllocPortable), "cudaHostAlloc") &&
        chk(cudaHostGetDevicePointer(&hd, h, 0), "cudaHostGetDevicePointer") &&
        chk(cudaMalloc(&d, bytes), "cudaMalloc") && chk(cudaMalloc(&sink, 8), "cudaMalloc") &&
        chk(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "stream") &&
        chk(cudaEventCreate(&e0), "event") && chk(cudaEventCreate(&e1), "event") &&
        chk(cudaGetDevice(&dev), "dev") &&
        chk(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "attr")) {
        memset(h, 1, bytes);
        for (int i = 0; i < iters + 1 && st == ASC_OK; i++) {
            // one copy per quarter, issued back to back on one stream
            float ms = 0;
            chk(cudaEventRecord(e0, s), "rec");
            const uint64_t q = (bytes / 4) & ~(uint64_t)15;
            for (int k = 0; k < 4; k++) {
                uint64_t off = k * q, n = k == 3 ? bytes - off : q;
                chk(cudaMemcpyAsync((char *)d + off, (const char *)h + off, n, cudaMemcpyHostToDevice, s),
                    "memcpy");
            }
            chk(cudaEventRecord(e1, s), "rec");
            chk(cudaEventSynchronize(e1), "sync");
            chk(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
            if (i > 0 && ms > 0) best_dma = std::max(best_dma, bytes / (ms * 1e6));
        }
        for (int i = 0; i < iters + 1 && st == ASC_OK; i++) {
            float ms = 0;
            chk(cudaEventRecord(e0, s), "rec");
            link_read_kernel<<<sms * 16, 256, 0, s>>>((const uint4 *)hd, bytes / 16, sink);
            chk(cudaGetLastError(), "launch");
            chk(cudaEventRecord(e1, s), "rec");
            chk(cudaEventSynchronize(e1), "sync");
            chk(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
            if (i > 0 && ms > 0) best_sm = std::max(best_sm, bytes / (ms * 1e6));
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    if (sink) cudaFree(sink);
    if (d) cudaFree(d);
    if (h) cudaFreeHost(h);
    if (dma_h2d_gbs) *dma_h2d_gbs = best_dma;
    if (sm_read_gbs) *sm_read_gbs = best_sm;
    return st;
}

// ------------------------------------------------- allocation-free BFS -------
//
// asc_bfs_device_noalloc runs the same BFS expansion kernel over a CSR graph the
// caller already holds in device memory, for callers that cannot allocate
// device memory at query time: a process whose device memory is owned by
// another allocator (a framework's caching pool sized to the whole GPU, where
// a cudaMalloc of its own would fail or fragment the pool), or a latency-bound
// loop where cudaMalloc/cudaFree (which can synchronize the device) are not
// allowed. Its scratch state (frontier lists, segment lists, the next-frontier
// bitmap, counters) lives in one file-scope device array of fixed size, which
// every GPU that loads this library holds until the process exits.
namespace asc {
namespace {

constexpr uint64_t kNoAllocMaxV = 1ull << 20;   // vertices
constexpr uint64_t kNoAllocMaxE = 1ull << 24;   // edges
constexpr uint32_t kNoAllocHuge = 512;          // same degree buckets as the default Tuning
constexpr uint32_t kNoAllocSeg = 2048;
// segment items never exceed E/seg_len (full segments) + E/huge (one partial per long list)
constexpr uint64_t kNoAllocMaxSegs = kNoAllocMaxE / kNoAllocSeg + kNoAllocMaxE / kNoAllocHuge + 1;

constexpr uint64_t na_round(uint64_t x) { return (x + 255) & ~255ull; }
constexpr uint64_t kNaCtl = 0;
constexpr uint64_t kNaBitmap = na_round(kNaCtl + 4 * CTL_WORDS);
constexpr uint64_t kNaBitmap1 = na_round(kNaBitmap + 4 * (kNoAllocMaxV / 32 + 2));
constexpr uint64_t kNaVisited = na_round(kNaBitmap1 + 4 * (kNoAllocMaxV / 32 + 2));
constexpr uint64_t kNaHuge = na_round(kNaVisited + 4 * (kNoAllocMaxV / 32 + 2));
constexpr uint64_t kNaQueue0 = na_round(kNaHuge + 4 * (kNoAllocMaxV / 32 + 2));
constexpr uint64_t kNaQueue1 = na_round(kNaQueue0 + 4 * kNoAllocMaxV);
constexpr uint64_t kNaSegs0 = na_round(kNaQueue1 + 4 * kNoAllocMaxV);
constexpr uint64_t kNaSegs1 = na_round(kNaSegs0 + 8 * kNoAllocMaxSegs);
constexpr uint64_t kNaBytes = na_round(kNaSegs1 + 8 * kNoAllocMaxSegs);   // about 9.6 MB

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

// In host code g_noalloc_scratch names a host-side stand-in, not device memory;
// kernels get the device address looked up once per device. The cached address
// belongs to the device's primary context: a cudaDeviceReset or another context
// would leave it stale, which the header rules out for callers.
constexpr int kNaMaxDevices = 64;
std::mutex g_na_mutex;
unsigned char *g_na_addr[kNaMaxDevices] = {nullptr};

// Checks the caller's CSR on the device: offsets start at 0, never decrease,
// end at E, destinations are < V. flag[0] becomes nonzero on the first defect.
__global__ void noalloc_validate_kernel(const uint32_t *ptr, const uint32_t *col, uint32_t V, uint32_t E,
                                        uint32_t *flag) {
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t == 0 && (ptr[0] != 0 || ptr[V] != E)) atomicOr(flag, 1u);
    for (uint32_t v = t; v < V; v += stride)
        if (ptr[v] > ptr[v + 1]) atomicOr(flag, 2u);
    for (uint32_t i = t; i < E; i += stride)
        if (col[i] >= V) atomicOr(flag, 4u);
}

// One bit per vertex whose list is longer than the huge-degree threshold.
__global__ void noalloc_huge_bits_kernel(const uint32_t *ptr, uint32_t V, uint32_t huge, uint32_t *bits,
                                         uint32_t nwords) {
    for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < nwords; w += gridDim.x * blockDim.x) {
        uint32_t m = 0;
        for (uint32_t b = 0; b < 32; b++) {
            const uint32_t v = 32 * w + b;
            if (v < V && ptr[v + 1] - ptr[v] > huge) m |= 1u << b;
        }
        bits[w] = m;
    }
}

asc_status noalloc_scratch(unsigned char **out) {
    int dev = 0;
    ASC_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNaMaxDevices) return fail(ASC_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_addr[dev]) {
        void *p = nullptr;
        ASC_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_na_addr[dev] = (unsigned char *)p;
    }
    *out = g_na_addr[dev];
    return ASC_OK;
}

}  // namespace
}  // namespace asc

extern "C" asc_status asc_bfs_device_noalloc(uint64_t V, uint64_t E, const uint32_t *d_row_offsets,
                                             const uint32_t *d_col, uint32_t source, uint32_t *d_levels,
                                             void *stream) {
    using namespace asc;
    if (!d_row_offsets || !d_levels || (!d_col && E))
        return fail(ASC_ERR_INVALID, "asc_bfs_device_noalloc: null device pointer");
    if (V == 0 || V > kNoAllocMaxV)
        return fail(ASC_ERR_BUDGET, "asc_bfs_device_noalloc: V = %llu outside [1, %llu], the fixed scratch limit",
                    (unsigned long long)V, (unsigned long long)kNoAllocMaxV);
    if (E > kNoAllocMaxE)
        return fail(ASC_ERR_BUDGET, "asc_bfs_device_noalloc: E = %llu above %llu, the fixed scratch limit",
                    (unsigned long long)E, (unsigned long long)kNoAllocMaxE);
    if (source >= V) return fail(ASC_ERR_INVALID, "source %u is not a vertex (V = %llu)", source,
                                 (unsigned long long)V);
    unsigned char *base = nullptr;
    ASC_TRY(noalloc_scratch(&base));
    cudaStream_t s = (cudaStream_t)stream;
    uint32_t *ctl = (uint32_t *)(base + kNaCtl);
    uint32_t *bitmap[2] = {(uint32_t *)(base + kNaBitmap), (uint32_t *)(base + kNaBitmap1)};
    uint32_t *visited = (uint32_t *)(base + kNaVisited);
    uint32_t *huge_bits = (uint32_t *)(base + kNaHuge);
    uint32_t *queue[2] = {(uint32_t *)(base + kNaQueue0), (uint32_t *)(base + kNaQueue1)};
    uint64_t *segs[2] = {(uint64_t *)(base + kNaSegs0), (uint64_t *)(base + kNaSegs1)};
    const uint32_t V32 = (uint32_t)V, E32 = (uint32_t)E;
    const uint32_t nwords = V32 / 32 + 1;
    int dev = 0, sms = 0;
    ASC_CUDA(cudaGetDevice(&dev));
    ASC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const uint32_t fill = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((V + kBlock - 1) / kBlock, sms * 8ull));

    // the array keeps the previous call's contents: clear the counters and the
    // bitmaps first
    ASC_CUDA(cudaMemsetAsync(ctl, 0, 4 * CTL_WORDS, s));
    ASC_CUDA(cudaMemsetAsync(visited, 0, 4 * (V / 32 + 2), s));
    for (int i = 0; i < 2; i++) ASC_CUDA(cudaMemsetAsync(bitmap[i], 0, 4 * (V / 32 + 2), s));
    noalloc_validate_kernel<<<fill, kBlock, 0, s>>>(d_row_offsets, d_col, V32, E32, ctl + CTL_PR);
    ASC_CUDA(cudaGetLastError());
    uint32_t flag = 0;
    ASC_CUDA(cudaMemcpyAsync(&flag, ctl + CTL_PR, 4, cudaMemcpyDeviceToHost, s));
    ASC_CUDA(cudaStreamSynchronize(s));
    if (flag)
        return fail(ASC_ERR_INVALID, "asc_bfs_device_noalloc: malformed CSR (%s%s%s)",
                    flag & 1 ? "offsets must start at 0 and end at E; " : "",
                    flag & 2 ? "offsets decrease; " : "", flag & 4 ? "destination >= V" : "");
    noalloc_huge_bits_kernel<<<fill, kBlock, 0, s>>>(d_row_offsets, V32, kNoAllocHuge, huge_bits, nwords);

    RegionArgs a;
    memset(&a, 0, sizeof(a));
    a.ptr = d_row_offsets;
    a.edges = d_col;
    a.ebits = 32;
    a.val = d_levels;
    a.visited = visited;
    a.huge_bits = huge_bits;
    a.S = V32;  // the whole graph is device resident: one region
    a.V = V32;
    a.dense_begin = 0;
    a.dense_end = V32;
    a.dense_div = 64;
    a.huge = kNoAllocHuge;
    a.seg_len = kNoAllocSeg;
    a.segcap_static = (uint32_t)kNoAllocMaxSegs;
    a.stats = (unsigned long long *)(ctl + CTL_STATS);
    // seed: the source lands in parity 0
    a.cnt_out = ctl;
    a.q_out = queue[0];
    a.seg_out = segs[0];
    a.bitmap = bitmap[0];
    init_values_kernel<kBFS><<<fill, kBlock, 0, s>>>(d_levels, V32, source);
    seed_bits_kernel<<<1, kBlock, 0, s>>>(a, source, 0, nwords);
    build_frontier_kernel<<<fill, kBlock, 0, s>>>(a, bitmap[0], nwords);
    ASC_CUDA(cudaGetLastError());
    uint32_t cnt[CTL_BLOCK] = {0, 0, 0, 0, 0, 0, 0, 0};
    ASC_CUDA(cudaMemcpyAsync(cnt, ctl, sizeof(cnt), cudaMemcpyDeviceToHost, s));
    ASC_CUDA(cudaStreamSynchronize(s));
    int parity = 0;
    int64_t iters = 0;
    while (cnt[6] | cnt[7]) {
        if (++iters > (int64_t)V + 2) return fail(ASC_ERR_TIMEOUT, "no fixpoint after %lld iterations",
                                                  (long long)iters);
        const int po = 1 - parity;
        ASC_CUDA(cudaMemsetAsync(ctl + CTL_BLOCK * po, 0, 4 * CTL_BLOCK, s));
        ASC_CUDA(cudaMemsetAsync(bitmap[po], 0, 4 * (V / 32 + 2), s));
        a.region = 0;
        a.q_in = queue[parity];
        a.seg_in = segs[parity];
        a.bitmap_in = bitmap[parity];
        a.bitmap = bitmap[po];
        a.cnt_in = ctl + CTL_BLOCK * parity;
        a.cnt_out = ctl + CTL_BLOCK * po;
        a.q_out = queue[po];
        a.seg_out = segs[po];
        a.work = a.cnt_out + 4;
        const bool dense = cnt[6] > V32 / a.dense_div;
        const uint64_t items = (uint64_t)cnt[2] + ((dense ? V32 : cnt[0]) + kBlock - 1) / kBlock;
        const uint32_t grid = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(items, (uint64_t)sms * 4));
        expand_kernel<kBFS, 1><<<grid, kBlock, 0, s>>>(a);
        build_frontier_kernel<<<fill, kBlock, 0, s>>>(a, bitmap[po], nwords);
        ASC_CUDA(cudaGetLastError());
        ASC_CUDA(cudaMemcpyAsync(cnt, a.cnt_out, sizeof(cnt), cudaMemcpyDeviceToHost, s));
        ASC_CUDA(cudaStreamSynchronize(s));
        parity = po;
    }
    return ASC_OK;
}

// ------------------------------------------------------------- autotuner ----
//
// Picks the engine's tunables for one graph by measurement: the degree above
// which a list is cut into segments, the segment length, the frontier density
// above which a region is walked through its bitmap, and the CTAs per SM of
// the persistent grids. Coordinate descent from the current setting, each
// candidate timed over the given sources (CUDA events, best of two passes).
// Results are cached in a text file keyed by GPU and graph shape
// (ASC_TUNE_CACHE, default $HOME/.cache/ascetic_gb300_tune.txt).
namespace {

std::string tune_key(asc_graph *g, asc_algo algo) {
    cudaDeviceProp prop;
    std::string name = "gpu";
    if (cudaGetDeviceProperties(&prop, g->device) == cudaSuccess) name = prop.name;
    for (auto &c : name)
        if (c == ' ') c = '_';
    char buf[256];
    snprintf(buf, sizeof(buf), "%s:V%llu:E%llu:S%llu:W%u:B%u:C%u:A%d", name.c_str(), (unsigned long long)g->V,
             (unsigned long long)g->E, (unsigned long long)g->static_edges, g->edge_words, g->ebits,
             g->is_csc ? 1 : 0, (int)algo);
    return buf;
}

std::string tune_cache_path() {
    const char *p = getenv("ASC_TUNE_CACHE");
    if (p && *p) return p;
    const char *home = getenv("HOME");
    return std::string(home ? home : "/tmp") + "/.cache/ascetic_gb300_tune.txt";
}

bool tune_cache_lookup(const std::string &key, asc::Tuning *t) {
    FILE *f = fopen(tune_cache_path().c_str(), "r");
    if (!f) return false;
    char line[512], k[256];
    unsigned h, sg, d, c, dl, bu;
    double ms;
    bool found = false;
    // one entry per line: key and the eight fields; lines of another layout are skipped
    while (fgets(line, sizeof(line), f))
        if (sscanf(line, "%255s %u %u %u %u %u %u %lf", k, &h, &sg, &d, &c, &dl, &bu, &ms) == 8 && key == k) {
            t->huge_degree = h;
            t->segment_edges = sg;
            t->dense_div = d;
            t->ctas_per_sm = c;
            t->delta = dl;
            t->bu_div = bu;
            found = true;
        }
    fclose(f);
    return found;
}

void tune_cache_store(const std::string &key, const asc::Tuning &t, double ms) {
    std::string path = tune_cache_path();
    std::string dir = path.substr(0, path.find_last_of('/'));
    if (!dir.empty()) {
        std::string cmd = dir;  // create the cache directory when missing
        mkdir(cmd.c_str(), 0755);
    }
    FILE *f = fopen(path.c_str(), "a");
    if (!f) return;
    fprintf(f, "%s %u %u %u %u %u %u %.4f\n", key.c_str(), t.huge_degree, t.segment_edges, t.dense_div,
            t.ctas_per_sm, t.delta, t.bu_div, ms);
    fclose(f);
}

}  // namespace

namespace asc {

asc_status set_tuning(asc_graph *g, const Tuning &t) {
    if (t.huge_degree < 32 || t.huge_degree > (1u << 20) || t.segment_edges < 256 || t.segment_edges > (1u << 24))
        return fail(ASC_ERR_INVALID, "tuning out of range (huge %u, segment %u)", t.huge_degree, t.segment_edges);
    free_workspace(g);  // segment capacities depend on the thresholds
    g->tuning = t;
    g->has_tuning = true;
    return ASC_OK;
}

}  // namespace asc

extern "C" {

asc_status asc_graph_get_tuning(const asc_graph *g, asc_tuning *t) {
    if (!g || !t) return asc::fail(ASC_ERR_INVALID, "asc_graph_get_tuning: null argument");
    asc::Tuning d;
    if (g->ws) d = g->ws->tune;
    else if (g->has_tuning) d = g->tuning;
    memset(t, 0, sizeof(*t));
    t->huge_degree = d.huge_degree;
    t->segment_edges = d.segment_edges;
    t->dense_div = d.dense_div;
    t->ctas_per_sm = d.ctas_per_sm;
    t->delta = d.delta;
    t->bu_div = d.bu_div;
    return ASC_OK;
}

asc_status asc_graph_set_tuning(asc_graph *g, const asc_tuning *t) {
    if (!g || !t) return asc::fail(ASC_ERR_INVALID, "asc_graph_set_tuning: null argument");
    asc::Tuning x;
    x.huge_degree = t->huge_degree;
    x.segment_edges = t->segment_edges;
    x.dense_div = t->dense_div;
    x.ctas_per_sm = t->ctas_per_sm;
    x.delta = t->delta;
    x.bu_div = t->bu_div;
    return asc::set_tuning(g, x);
}

asc_status asc_graph_tune(asc_graph *g, asc_algo algo, const uint32_t *sources, uint32_t n, uint32_t flags,
                          asc_tuning *best) {
    using namespace asc;
    if (!g || (!sources && algo != ASC_CC && algo != ASC_PR) || (n == 0 && algo != ASC_CC && algo != ASC_PR))
        return fail(ASC_ERR_INVALID, "asc_graph_tune: graph and sources are required");
    if (algo == ASC_PR) return fail(ASC_ERR_UNSUPPORTED, "tuning runs traversals (BFS, SSSP, CC)");
    const std::string key = tune_key(g, algo);
    Tuning cur;
    if (g->ws) cur = g->ws->tune;
    else if (g->has_tuning) cur = g->tuning;
    if (!(flags & ASC_TUNE_NO_CACHE) && tune_cache_lookup(key, &cur)) {
        ASC_TRY(set_tuning(g, cur));
        if (best) ASC_TRY(asc_graph_get_tuning(g, best));
        if (best) best->ms = -1;  // from the cache
        return ASC_OK;
    }
    asc_params p;
    asc_params_default(&p);
    p.flags = ASC_RUN_NO_OUTPUT;
    const uint32_t runs = std::max<uint32_t>(1, std::min<uint32_t>(n, 4));
    auto measure = [&](const Tuning &t, double *ms) -> asc_status {
        ASC_TRY(set_tuning(g, t));
        double bestms = 1e30;
        for (int pass = 0; pass < 2; pass++) {  // first pass warms up (graph build, caches)
            double sum = 0;
            for (uint32_t i = 0; i < runs; i++) {
                asc_stats st;
                ASC_TRY(run_traversal(g, algo, algo == ASC_CC ? 0 : sources[i], p, nullptr, &st));
                sum += st.ms_total;
            }
            bestms = std::min(bestms, sum);
        }
        *ms = bestms;
        return ASC_OK;
    };
    double cur_ms;
    ASC_TRY(measure(cur, &cur_ms));
    const uint32_t huge_c[] = {128, 256, 512, 1024, 4096};
    const uint32_t seg_c[] = {1024, 2048, 4096, 8192};
    const uint32_t div_c[] = {8, 16, 32, 64, 256, 0};
    const uint32_t delta_c[] = {0, 16, 32, 64, 128, 256};
    const uint32_t bu_c[] = {8, 16, 32, 64, 128, 256, 0};
    for (int round = 0; round < 2; round++) {
        if (algo == ASC_BFS && !g->is_csc)
            for (uint32_t b : bu_c) {
                Tuning t = cur;
                t.bu_div = b;
                if (t.bu_div == cur.bu_div) continue;
                double ms;
                ASC_TRY(measure(t, &ms));
                if (ms < cur_ms) { cur = t; cur_ms = ms; }
            }
        if (algo == ASC_SSSP)
            for (uint32_t dl : delta_c) {
                Tuning t = cur;
                t.delta = dl;
                if (t.delta == cur.delta) continue;
                double ms;
                ASC_TRY(measure(t, &ms));
                if (ms < cur_ms) { cur = t; cur_ms = ms; }
            }
        for (uint32_t d : div_c) {
            Tuning t = cur;
            t.dense_div = d;
            if (t.dense_div == cur.dense_div) continue;
            double ms;
            ASC_TRY(measure(t, &ms));
            if (ms < cur_ms) { cur = t; cur_ms = ms; }
        }
        for (uint32_t h : huge_c) {
            Tuning t = cur;
            t.huge_degree = h;
            if (t.huge_degree == cur.huge_degree) continue;
            double ms;
            ASC_TRY(measure(t, &ms));
            if (ms < cur_ms) { cur = t; cur_ms = ms; }
        }
        for (uint32_t sg : seg_c) {
            Tuning t = cur;
            t.segment_edges = sg;
            if (t.segment_edges == cur.segment_edges) continue;
            double ms;
            ASC_TRY(measure(t, &ms));
            if (ms < cur_ms) { cur = t; cur_ms = ms; }
        }
    }
    ASC_TRY(set_tuning(g, cur));
    if (!(flags & ASC_TUNE_NO_CACHE)) tune_cache_store(key, cur, cur_ms / runs);
    if (best) {
        ASC_TRY(asc_graph_get_tuning(g, best));
        best->ms = cur_ms / runs;
    }
    return ASC_OK;
}

}  // extern "C"

extern "C" asc_status asc_graph_fragment_counts(asc_graph *g, uint64_t *out, uint64_t n, uint64_t *n_out, int reset) {
    using namespace asc;
    if (!g) return fail(ASC_ERR_INVALID, "asc_graph_fragment_counts: graph is NULL");
    const uint64_t nf = fragment_count(g);
    if (n_out) *n_out = nf;
    Workspace *ws = g->ws;
    const uint64_t k = std::min(n, nf);
    if (!ws || !ws->frag_counts) {
        if (out) memset(out, 0, 8 * k);
        return ASC_OK;
    }
    if (out && k) {
        ASC_CUDA(cudaMemcpyAsync(out, ws->frag_counts, 8 * k, cudaMemcpyDeviceToHost, g->stream));
    }
    if (reset) ASC_CUDA(cudaMemsetAsync(ws->frag_counts, 0, 8 * std::max<uint64_t>(1, nf), g->stream));
    ASC_CUDA(cudaStreamSynchronize(g->stream));
    return ASC_OK;
}
