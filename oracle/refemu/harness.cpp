/*
 * Reference emulation harness (TEST INFRASTRUCTURE, builds oracle/_ref/libascref.so).
 *
 * Compiles the reference's own device kernels (gpu_kernels.cuh) and its graph,
 * budget, gather and partition code (GraphMeta.cuh) for the CPU, straight from
 * the reference tree, against the stand-ins in shim/. The kernels run serially
 * (one emulated thread, grid-stride loops over every index); the host iteration
 * loop below restates, step for step, the drivers bfs_opt / cc_opt / sssp_opt /
 * pr_opt of CalculateOpt.cu (whose triple-chevron launches and Thrust calls g++
 * cannot compile). The counts and exclusive scans that CalculateOpt.cu does with
 * thrust::reduce / thrust::exclusive_scan are plain loops here.
 *
 * Its outputs pin the plain-C oracle (oracle/oracle.c): tests/golden/make_golden.py
 * runs both on the same files and stores the reference's results as fixtures.
 *
 * hazard_mode selects what the uninitialised entry staticNodePointer[max_static_node]
 * holds (GraphMeta.cuh:230-233 copies only i < max_static_node):
 *   0: zero, as in the fresh zeroed pages a large new[] gets (the reference's
 *      behaviour on real graphs);
 *   1: the correct offset nodePointers[max_static_node] (the intended semantics,
 *      which the oracle and the CUDA engine implement).
 */
#include <string>
#include <iostream>
#include <vector>
#include <chrono>
#include <fstream>
#include <thread>
#include <cmath>
#include <typeinfo>
#include <iterator>
#include <type_traits>
#include <utility>
#include <fcntl.h>
#include <unistd.h>
#include "cuda_runtime.h"
#include "thrust/device_vector.h"

uint3 threadIdx = {0, 0, 0};
uint3 blockIdx = {0, 0, 0};
dim3 blockDim(1, 1, 1);
dim3 gridDim(1, 1, 1);
size_t asc_emu_avail_bytes = 0;
size_t asc_emu_total_bytes = 0;

// max_static_node is private in GraphMeta; the harness needs it for hazard_mode.
#define private public
#include "GraphMeta.cuh"
#include "gpu_kernels.cuh"
#undef private

namespace {

// The reference prints progress with cout and printf; send both to /dev/null.
struct Silence {
    std::streambuf *old;
    std::ofstream sink;
    int saved_fd;
    Silence() : sink("/dev/null") {
        old = std::cout.rdbuf(sink.rdbuf());
        fflush(stdout);
        saved_fd = dup(1);
        int nul = open("/dev/null", O_WRONLY);
        if (nul >= 0) { dup2(nul, 1); close(nul); }
    }
    ~Silence() {
        fflush(stdout);
        if (saved_fd >= 0) { dup2(saved_fd, 1); close(saved_fd); }
        std::cout.rdbuf(old);
    }
};

// One emulated launch: a 1x1 grid, so every grid-stride loop runs serially.
template <class F, class... A> void launch(F kern, A... args) {
    threadIdx = {0, 0, 0};
    blockIdx = {0, 0, 0};
    blockDim = dim3(1, 1, 1);
    gridDim = dim3(1, 1, 1);
    kern(args...);
}

// gpu_kernels.cu:111-122 (setStaticAndOverloadLabelBool) restated: the .cu file
// also holds host launches that g++ cannot compile.
void split_active(uint n, const bool *act, bool *st, bool *ov, const bool *in_static) {
    for (uint v = 0; v < n; v++)
        if (act[v]) { if (in_static[v]) st[v] = 1; else ov[v] = 1; }
}

uint count_true(const bool *a, uint n) {
    uint s = 0;
    for (uint i = 0; i < n; i++) s += a[i];
    return s;
}

void excl_scan(const bool *a, uint *out, uint n) {
    uint s = 0;
    for (uint i = 0; i < n; i++) { out[i] = s; s += a[i]; }
}

template <class EdgeType> void fix_static_pointer(GraphMeta<EdgeType> &g, int hazard_mode) {
    uint m = g.max_static_node;
    if (m < g.vertexArrSize)
        g.staticNodePointer[m] = hazard_mode == 1 ? (SIZE_TYPE)g.nodePointers[m] : 0;
}

// CalculateOpt.cu:60-124: split the active set, compact the static and overload
// lists, build the 64-bit overload offsets on the host. Returns overload edges.
template <class EdgeType>
EDGE_POINTER_TYPE compact(GraphMeta<EdgeType> &graph, uint &staticNodeNum, uint &overloadNodeNum) {
    uint V = graph.vertexArrSize;
    split_active(V, graph.isActiveD, graph.isStaticActive, graph.isOverloadActive, graph.isInStaticD);
    staticNodeNum = count_true(graph.isStaticActive, V);
    if (staticNodeNum > 0) {
        excl_scan(graph.isStaticActive, graph.prefixSumTemp, V);
        launch(setStaticActiveNodeArray<bool>, V, graph.staticNodeListD, graph.isStaticActive,
               graph.prefixSumTemp);
    }
    overloadNodeNum = count_true(graph.isOverloadActive, V);
    EDGE_POINTER_TYPE overloadEdgeNum = 0;
    if (overloadNodeNum > 0) {
        excl_scan(graph.isOverloadActive, graph.prefixSumTemp, V);
        launch(setOverloadNodePointerSwap<bool, EDGE_POINTER_TYPE>, V, graph.overloadNodeListD,
               graph.activeOverloadDegreeD, graph.isOverloadActive, graph.prefixSumTemp, graph.degreeD);
        memcpy(graph.overloadNodeList, graph.overloadNodeListD, overloadNodeNum * sizeof(uint));
        EDGE_POINTER_TYPE anchor = 0;
        for (uint i = 0; i < overloadNodeNum; ++i) {
            overloadEdgeNum += graph.degree[graph.overloadNodeList[i]];
            if (i > 0) anchor += graph.activeOverloadDegreeD[i - 1];
            graph.activeOverloadNodePointers[i] = anchor;
        }
        memcpy(graph.activeOverloadNodePointersD, graph.activeOverloadNodePointers,
               overloadNodeNum * sizeof(EDGE_POINTER_TYPE));
    }
    return overloadEdgeNum;
}

// The partition planner loops forever when one vertex's list exceeds the
// staging buffer (GraphMeta.cuh:519-559); refuse such inputs instead.
template <class EdgeType> bool planner_safe(GraphMeta<EdgeType> &graph, uint overloadNodeNum) {
    for (uint i = 0; i < overloadNodeNum; i++)
        if (graph.degree[graph.overloadNodeList[i]] > graph.partOverloadSize) return false;
    return true;
}

}  // namespace

extern "C" {

struct asc_ref_stats {
    int32_t iterations;
    uint32_t max_static_node;
    uint64_t static_edges;          // max_partition_size (edges in the static prefix)
    uint64_t staging_edges;         // partOverloadSize
    uint64_t moved_edges;           // sum of overload edges over all iterations ("move overload size" / sizeof)
    uint64_t node_sum;              // sum of active counts (CalculateOpt.cu:190)
    uint64_t parts;                 // number of transferred parts
};

/* algo: 0 BFS (.bcsr), 1 SSSP (.bwcsr), 2 CC (.bcsr), 3 reference PR (.bcsc).
 * avail_bytes is what cudaMemGetInfo reports; advise is --adviseK. out is
 * uint32[V] (0-2) or double[V] (3). Returns 0 on success, 3 when the planner
 * would loop forever, 4 on a bad algorithm. */
int asc_ref_run(int algo, const char *path, uint32_t source, uint64_t avail_bytes, double advise,
                int hazard_mode, void *out, asc_ref_stats *st) {
    Silence quiet;
    asc_emu_avail_bytes = avail_bytes;
    asc_emu_total_bytes = avail_bytes;
    memset(st, 0, sizeof(*st));
    if (algo == 1) {
        GraphMeta<EdgeWithWeight> graph;
        graph.setAlgType(SSSP);
        graph.setSourceNode(source);
        graph.readDataFromFile(path, false);
        graph.setPrestoreRatio(advise, 15);
        graph.initGraphHost();
        fix_static_pointer(graph, hazard_mode);
        graph.initGraphDevice();
        graph.refreshLabelAndValue();
        uint V = graph.vertexArrSize;
        uint active = count_true(graph.isActiveD, V);
        st->node_sum = active;
        while (active) {
            st->iterations++;
            uint sn, on;
            EDGE_POINTER_TYPE oe = compact(graph, sn, on);
            st->moved_edges += oe;
            if (sn > 0) launch(setLabelDefaultOpt<bool>, sn, graph.staticNodeListD, graph.isActiveD);
            if (on > 0) launch(setLabelDefaultOpt<bool>, on, graph.overloadNodeListD, graph.isActiveD);
            launch(sssp_kernel<bool>, sn, graph.staticNodeListD, graph.staticNodePointerD, graph.degreeD,
                   graph.staticEdgeListD, graph.valueD, graph.isActiveD);
            if (on > 0) {
                if (!planner_safe(graph, on)) return 3;
                graph.fillEdgeArrByMultiThread(on);
                graph.caculatePartInfoForEdgeList(on, oe);
                for (auto &p : graph.partEdgeListInfoArr) {
                    st->parts++;
                    memcpy(graph.overloadEdgeListD,
                           graph.overloadEdgeList + graph.activeOverloadNodePointers[p.partStartIndex],
                           p.partEdgeNums * sizeof(EdgeWithWeight));
                    launch(sssp_kernelDynamic<bool, EDGE_POINTER_TYPE>, p.partStartIndex, p.partActiveNodeNums,
                           (const uint *)graph.overloadNodeListD, (const uint *)graph.degreeD, graph.valueD,
                           graph.isActiveD, (const EdgeWithWeight *)graph.overloadEdgeListD,
                           (const EDGE_POINTER_TYPE *)graph.activeOverloadNodePointersD);
                }
            }
            active = count_true(graph.isActiveD, V);
            st->node_sum += active;
        }
        memcpy(out, graph.valueD, sizeof(uint) * V);
        st->max_static_node = graph.max_static_node;
        st->static_edges = graph.max_partition_size;
        st->staging_edges = graph.partOverloadSize;
        return 0;
    }
    if (algo < 0 || algo > 3) return 4;
    GraphMeta<uint> graph;
    graph.setAlgType(algo == 0 ? BFS : (algo == 2 ? CC : PR));
    graph.setSourceNode(source);
    graph.readDataFromFile(path, algo == 3);
    graph.setPrestoreRatio(advise, algo == 3 ? 17 : 13);
    graph.initGraphHost();
    fix_static_pointer(graph, hazard_mode);
    graph.initGraphDevice();
    graph.refreshLabelAndValue();
    uint V = graph.vertexArrSize;
    uint active = count_true(graph.isActiveD, V);
    st->node_sum = active;
    while (active) {
        st->iterations++;
        uint sn, on;
        EDGE_POINTER_TYPE oe = compact(graph, sn, on);
        st->moved_edges += oe;
        if (algo != 3) {
            if (sn > 0) launch(setLabelDefaultOpt<bool>, sn, graph.staticNodeListD, graph.isActiveD);
            if (on > 0) launch(setLabelDefaultOpt<bool>, on, graph.overloadNodeListD, graph.isActiveD);
        }
        if (algo == 0)
            launch(bfs_kernelStatic<bool>, sn, graph.staticNodeListD, graph.staticNodePointerD, graph.degreeD,
                   graph.staticEdgeListD, graph.valueD, graph.isActiveD);
        else if (algo == 2)
            launch(cc_kernelStaticSwap<bool>, sn, graph.staticNodeListD, graph.staticNodePointerD, graph.degreeD,
                   graph.staticEdgeListD, graph.valueD, graph.isActiveD, graph.isInStaticD);
        else
            launch(prSumKernel_static<double>, sn, (const uint *)graph.staticNodeListD,
                   (const uint *)graph.staticNodePointerD, (const uint *)graph.staticEdgeListD,
                   (const uint *)graph.degreeD, (const uint *)graph.outDegreeD, (const double *)graph.valuePrD,
                   graph.sumD);
        if (on > 0) {
            if (!planner_safe(graph, on)) return 3;
            graph.fillEdgeArrByMultiThread(on);
            graph.caculatePartInfoForEdgeList(on, oe);
            for (auto &p : graph.partEdgeListInfoArr) {
                st->parts++;
                memcpy(graph.overloadEdgeListD,
                       graph.overloadEdgeList + graph.activeOverloadNodePointers[p.partStartIndex],
                       p.partEdgeNums * sizeof(uint));
                if (algo == 0)
                    launch(bfs_kernelDynamicPart<bool, EDGE_POINTER_TYPE>, p.partStartIndex, p.partActiveNodeNums,
                           (const uint *)graph.overloadNodeListD, (const uint *)graph.degreeD, graph.valueD,
                           graph.isActiveD, (const uint *)graph.overloadEdgeListD,
                           (const EDGE_POINTER_TYPE *)graph.activeOverloadNodePointersD);
                else if (algo == 2)
                    launch(cc_kernelDynamicSwap<bool, EDGE_POINTER_TYPE>, p.partStartIndex, p.partActiveNodeNums,
                           (const uint *)graph.overloadNodeListD, (const uint *)graph.degreeD, graph.valueD,
                           graph.isActiveD, (const uint *)graph.overloadEdgeListD,
                           (const EDGE_POINTER_TYPE *)graph.activeOverloadNodePointersD);
                else
                    launch(prSumKernel_dynamic<EDGE_POINTER_TYPE, double>, p.partStartIndex, p.partActiveNodeNums,
                           (const uint *)graph.overloadNodeListD,
                           (const EDGE_POINTER_TYPE *)graph.activeOverloadNodePointersD,
                           (const uint *)graph.overloadEdgeListD, (const uint *)graph.degreeD,
                           (const uint *)graph.outDegreeD, (const double *)graph.valuePrD, graph.sumD);
            }
        }
        if (algo == 3) launch(prKernel_Opt<bool, double>, V, graph.valuePrD, graph.sumD, graph.isActiveD);
        active = count_true(graph.isActiveD, V);
        st->node_sum += active;
    }
    if (algo == 3) memcpy(out, graph.valuePrD, sizeof(double) * V);
    else memcpy(out, graph.valueD, sizeof(uint) * V);
    st->max_static_node = graph.max_static_node;
    st->static_edges = graph.max_partition_size;
    st->staging_edges = graph.partOverloadSize;
    return 0;
}

}  // extern "C"
