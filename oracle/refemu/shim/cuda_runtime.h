/* Host-memory stand-in for the CUDA runtime calls made by the reference's
 * GraphMeta.cuh (test infrastructure only): device allocations are malloc,
 * copies are memcpy, and cudaMemGetInfo reports a caller-chosen free size so
 * that the reference's own budget code (getMaxPartitionSize) sizes the static
 * region. */
#ifndef ASC_REFEMU_CUDA_RUNTIME_H
#define ASC_REFEMU_CUDA_RUNTIME_H
#include "cuda_emu.h"

typedef int cudaError_t;
typedef int cudaError;
enum { cudaSuccess = 0 };
enum cudaMemcpyKind { cudaMemcpyHostToHost = 0, cudaMemcpyHostToDevice = 1, cudaMemcpyDeviceToHost = 2,
                      cudaMemcpyDeviceToDevice = 3, cudaMemcpyDefault = 4 };
typedef struct CUstream_st *cudaStream_t;
struct cudaDeviceProp { size_t totalGlobalMem; int multiProcessorCount; };

extern size_t asc_emu_avail_bytes;
extern size_t asc_emu_total_bytes;

template <class T> inline cudaError_t cudaMalloc(T **p, size_t n) {
    *p = (T *)std::calloc(n ? n : 1, 1);
    return *p ? cudaSuccess : 2;
}
inline cudaError_t cudaFree(void *p) { std::free(p); return cudaSuccess; }
inline cudaError_t cudaMemcpy(void *d, const void *s, size_t n, cudaMemcpyKind) {
    if (n) std::memmove(d, s, n);
    return cudaSuccess;
}
inline cudaError_t cudaMemcpyAsync(void *d, const void *s, size_t n, cudaMemcpyKind, cudaStream_t = 0) {
    if (n) std::memmove(d, s, n);
    return cudaSuccess;
}
inline cudaError_t cudaMemset(void *d, int v, size_t n) { std::memset(d, v, n); return cudaSuccess; }
inline cudaError_t cudaStreamCreate(cudaStream_t *s) { *s = 0; return cudaSuccess; }
inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
inline cudaError_t cudaPeekAtLastError() { return cudaSuccess; }
inline cudaError_t cudaGetLastError() { return cudaSuccess; }
inline const char *cudaGetErrorString(cudaError_t) { return "emulated"; }
inline cudaError_t cudaGetDevice(int *d) { *d = 0; return cudaSuccess; }
inline cudaError_t cudaGetDeviceProperties(cudaDeviceProp *p, int) {
    p->totalGlobalMem = asc_emu_total_bytes;
    p->multiProcessorCount = 1;
    return cudaSuccess;
}
inline cudaError_t cudaMemGetInfo(size_t *avail, size_t *total) {
    *avail = asc_emu_avail_bytes;
    *total = asc_emu_total_bytes;
    return cudaSuccess;
}
#endif
