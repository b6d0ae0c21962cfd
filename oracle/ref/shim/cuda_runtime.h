/* Host-only stand-in for the CUDA runtime, used to compile the reference's hot-path
 * sources with g++ for the oracle cross-check (oracle/ref/build_ref.py).  Managed
 * memory becomes calloc, kernels become plain host functions run by a serial loop,
 * events read std::chrono.  Test infrastructure only. */
#pragma once
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#define __host__
#define __device__
#define __global__
#define __forceinline__ inline
#define __constant__
#define __managed__

using std::max;
using std::min;

typedef int cudaError_t;
typedef int cudaError;
enum { cudaSuccess = 0, cudaErrorMemoryAllocation = 2 };
enum cudaMemcpyKind { cudaMemcpyHostToHost, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost,
                      cudaMemcpyDeviceToDevice, cudaMemcpyDefault };
#define cudaMemAttachGlobal 1

struct dim3 {
    unsigned x, y, z;
    dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
extern thread_local dim3 threadIdx, blockIdx, blockDim, gridDim;

struct cudaDeviceProp {
    char name[256];
    int major, minor, memoryClockRate, memoryBusWidth, multiProcessorCount;
    size_t totalGlobalMem;
};

inline cudaError_t cudaMallocManaged(void **p, size_t bytes, unsigned = 1) {
    *p = calloc(1, bytes ? bytes : 1);
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
inline cudaError_t cudaMalloc(void **p, size_t bytes) { return cudaMallocManaged(p, bytes); }
inline cudaError_t cudaFree(void *p) { free(p); return cudaSuccess; }
inline cudaError_t cudaMemcpy(void *d, const void *s, size_t n, cudaMemcpyKind) {
    memcpy(d, s, n);
    return cudaSuccess;
}
inline cudaError_t cudaMemset(void *d, int v, size_t n) { memset(d, v, n); return cudaSuccess; }
inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
inline cudaError_t cudaGetLastError() { return cudaSuccess; }
inline cudaError_t cudaPeekAtLastError() { return cudaSuccess; }
inline const char *cudaGetErrorString(cudaError_t) { return "host-only build"; }
inline cudaError_t cudaDeviceReset() { return cudaSuccess; }
inline cudaError_t cudaSetDevice(int) { return cudaSuccess; }
inline cudaError_t cudaGetDevice(int *d) { *d = 0; return cudaSuccess; }
inline cudaError_t cudaGetDeviceCount(int *c) { *c = 1; return cudaSuccess; }
inline cudaError_t cudaChooseDevice(int *d, const cudaDeviceProp *) { *d = 0; return cudaSuccess; }
inline cudaError_t cudaGetDeviceProperties(cudaDeviceProp *p, int) {
    memset(p, 0, sizeof(*p));
    strcpy(p->name, "host");
    p->major = 1;
    p->totalGlobalMem = (size_t)1 << 40;
    return cudaSuccess;
}
inline cudaError_t cudaMemGetInfo(size_t *free_b, size_t *total_b) {
    *free_b = (size_t)1 << 40;
    *total_b = (size_t)1 << 40;
    return cudaSuccess;
}
template <class F>
inline cudaError_t cudaOccupancyMaxPotentialBlockSize(int *minGrid, int *block, F, size_t = 0, int = 0) {
    *minGrid = 1;
    *block = 64;
    return cudaSuccess;
}

typedef struct bb_shim_event { std::chrono::steady_clock::time_point t; } *cudaEvent_t;
typedef void *cudaStream_t;
inline cudaError_t cudaEventCreate(cudaEvent_t *e) { *e = new bb_shim_event(); return cudaSuccess; }
inline cudaError_t cudaEventDestroy(cudaEvent_t e) { delete e; return cudaSuccess; }
inline cudaError_t cudaEventRecord(cudaEvent_t e, cudaStream_t = 0) {
    e->t = std::chrono::steady_clock::now();
    return cudaSuccess;
}
inline cudaError_t cudaEventSynchronize(cudaEvent_t) { return cudaSuccess; }
inline cudaError_t cudaEventElapsedTime(float *ms, cudaEvent_t a, cudaEvent_t b) {
    *ms = std::chrono::duration<float, std::milli>(b->t - a->t).count();
    return cudaSuccess;
}

/* __constant__ symbols are plain host objects here */
template <class T>
inline cudaError_t cudaMemcpyToSymbol(T &symbol, const void *src, size_t count, size_t offset = 0, int kind = 0) {
    (void)kind;
    memcpy(reinterpret_cast<char *>(&symbol) + offset, src, count);
    return cudaSuccess;
}

