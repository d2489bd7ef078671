/*
 * CPU shim for compiling the reference's CUDA sources as plain host C++ (g++).
 *
 * Test infrastructure only: it lets the oracle recipe build the reference's own
 * kernel.cu / ReadData.cpp / UnitReduce.cpp unmodified into oracle/_ref/, where
 * each __global__ kernel becomes a host function that the driver (ref_driver.cpp)
 * calls once per (block, thread) index.  Nothing in the product links this.
 */
#pragma once
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>

/* execution-space qualifiers vanish on the host; set before CUDA's headers so
 * host_defines.h keeps these empty definitions */
#define __host__
#define __device__
#define __global__
#define __constant__
#define __shared__ thread_local
#define __forceinline__ inline
#define __noinline__

#include <vector_types.h>
#include <vector_functions.h>
#include <driver_types.h>

/* per-OS-thread launch coordinates, set by the driver before each "thread" */
extern thread_local uint3 threadIdx;
extern thread_local uint3 blockIdx;
extern thread_local dim3 blockDim;
extern thread_local dim3 gridDim;

inline void __syncthreads() {}

inline int atomicAdd(int* p, int v) { return __atomic_fetch_add(p, v, __ATOMIC_RELAXED); }

using std::max;
using std::min;

inline const char* cudaGetErrorString(cudaError_t) { return "cpu-shim"; }
inline cudaError_t cudaGetLastError() { return cudaSuccess; }

/* constant memory is ordinary host memory here */
template <class T>
inline cudaError_t cudaMemcpyToSymbol(T& symbol, const void* src, size_t count,
                                      size_t offset = 0,
                                      cudaMemcpyKind kind = cudaMemcpyHostToDevice) {
  (void)kind;
  std::memcpy(reinterpret_cast<char*>(&symbol) + offset, src, count);
  return cudaSuccess;
}

/* device allocations used by the reference's host setup (ReadData.cpp d_Cir) */
inline cudaError_t cudaMalloc(void** p, size_t n) { *p = std::malloc(n ? n : 1); return cudaSuccess; }
template <class T> inline cudaError_t cudaMalloc(T** p, size_t n) { return cudaMalloc((void**)p, n); }
inline cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind) { std::memcpy(d, s, n); return cudaSuccess; }
inline cudaError_t cudaMemset(void* d, int v, size_t n) { std::memset(d, v, n); return cudaSuccess; }
inline cudaError_t cudaFree(void* p) { std::free(p); return cudaSuccess; }
