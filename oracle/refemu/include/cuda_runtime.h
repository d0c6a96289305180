// CPU emulation of the CUDA runtime surface used by the reference's solver sources
// (Velvet/VtClothSolverGPU.cu, Velvet/SpatialHashGPU.cu, Velvet/Common.cuh) — TEST
// INFRASTRUCTURE: it lets those files compile unmodified with g++ so that the oracle can
// be compared with the reference's own kernel code on the CPU.
//
// Execution model: a launch runs its blocks in order and, inside a block, its threads in
// index order; a kernel that calls __syncthreads runs its threads as fibers that all
// reach the barrier before any continues.  So every atomicAdd happens in thread-index
// order, which is one valid serialisation of the reference's unordered atomics.
// Memory is host memory; "device" allocations are malloc'd.
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <cstring>

#define __global__
#define __device__
#define __host__
#define __constant__
#define __shared__
#define __forceinline__ inline

struct uint3 {
    unsigned x, y, z;
};
struct dim3 {
    unsigned x, y, z;
    dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
extern uint3 threadIdx, blockIdx;
extern dim3 blockDim, gridDim;

typedef int cudaError_t;
typedef void* cudaStream_t;
enum { cudaSuccess = 0, cudaErrorMemoryAllocation = 2 };
enum cudaMemcpyKind {
    cudaMemcpyHostToHost = 0,
    cudaMemcpyHostToDevice = 1,
    cudaMemcpyDeviceToHost = 2,
    cudaMemcpyDeviceToDevice = 3,
    cudaMemcpyDefault = 4
};

inline cudaError_t cudaMalloc(void** p, size_t n)
{
    *p = std::calloc(n ? n : 1, 1);
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
inline cudaError_t cudaMallocManaged(void** p, size_t n, unsigned = 1) { return cudaMalloc(p, n); }
inline cudaError_t cudaFree(void* p)
{
    std::free(p);
    return cudaSuccess;
}
inline cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind = cudaMemcpyDefault)
{
    if (n) std::memmove(d, s, n);
    return cudaSuccess;
}
inline cudaError_t cudaMemcpyAsync(void* d, const void* s, size_t n, cudaMemcpyKind k = cudaMemcpyDefault,
                                   cudaStream_t = 0)
{
    return cudaMemcpy(d, s, n, k);
}
inline cudaError_t cudaMemset(void* d, int v, size_t n)
{
    std::memset(d, v, n);
    return cudaSuccess;
}
inline cudaError_t cudaMemsetAsync(void* d, int v, size_t n, cudaStream_t = 0) { return cudaMemset(d, v, n); }
inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
inline cudaError_t cudaGetLastError() { return cudaSuccess; }
inline const char* cudaGetErrorString(cudaError_t) { return "cuda emulation error"; }
template <class T>
inline cudaError_t cudaMemcpyToSymbol(T& symbol, const void* src, size_t n, size_t offset = 0,
                                      cudaMemcpyKind = cudaMemcpyHostToDevice)
{
    std::memcpy(reinterpret_cast<char*>(&symbol) + offset, src, n);
    return cudaSuccess;
}
template <class T>
inline cudaError_t cudaMemcpyToSymbolAsync(T& symbol, const void* src, size_t n, size_t offset = 0,
                                           cudaMemcpyKind k = cudaMemcpyHostToDevice, cudaStream_t = 0)
{
    return cudaMemcpyToSymbol(symbol, src, n, offset, k);
}

// device atomics: read-modify-write in the order the emulator runs the threads
inline float atomicAdd(float* a, float v)
{
    const float old = *a;
    *a = old + v;
    return old;
}
inline int atomicAdd(int* a, int v)
{
    const int old = *a;
    *a = old + v;
    return old;
}
inline unsigned atomicAdd(unsigned* a, unsigned v)
{
    const unsigned old = *a;
    *a = old + v;
    return old;
}

// CUDA's min / max overloads for the argument types the reference passes (fminf / fmaxf
// for float, as CUDA's device overloads)
inline float min(float a, float b) { return std::fmin(a, b); }
inline float max(float a, float b) { return std::fmax(a, b); }
inline unsigned min(unsigned a, unsigned b) { return a < b ? a : b; }
inline unsigned max(unsigned a, unsigned b) { return a > b ? a : b; }
inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }

// block barrier: only valid inside a launch that runs its threads as fibers
void __syncthreads();
