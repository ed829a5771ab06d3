/* CPU stand-ins for the CUDA builtins that the reference's kernel header
 * (gpu_kernels.cuh) and graph class (GraphMeta.cuh) use, so that those files
 * compile unchanged with g++ and their kernels run serially on one host thread
 * (test infrastructure only). A "launch" sets a 1x1 grid; the reference's
 * grid-stride loops then visit every index in order. */
#ifndef ASC_REFEMU_CUDA_EMU_H
#define ASC_REFEMU_CUDA_EMU_H
#include <cstddef>
#include <cstdint>
#include <climits>
#include <cstring>
#include <cstdlib>
#include <cstdio>

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline

struct dim3 {
    unsigned int x, y, z;
    constexpr dim3(unsigned int a = 1, unsigned int b = 1, unsigned int c = 1) : x(a), y(b), z(c) {}
};
struct uint3 { unsigned int x, y, z; };

extern uint3 threadIdx;
extern uint3 blockIdx;
extern dim3 blockDim;
extern dim3 gridDim;

inline unsigned int atomicMin(unsigned int *p, unsigned int v) {
    unsigned int old = *p;
    if (v < old) *p = v;
    return old;
}
inline int atomicMin(int *p, int v) {
    int old = *p;
    if (v < old) *p = v;
    return old;
}
inline unsigned int atomicAdd(unsigned int *p, unsigned int v) { unsigned int o = *p; *p += v; return o; }
inline int atomicAdd(int *p, int v) { int o = *p; *p += v; return o; }
inline void __syncthreads() {}
#endif
