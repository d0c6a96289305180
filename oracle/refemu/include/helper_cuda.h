#pragma once
// CPU emulation of the CUDA samples' checkCudaErrors: abort on a failing call.
#include <cstdio>
#include <cstdlib>

#include <cuda_runtime.h>

inline void vr_check_cuda(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) {
        std::fprintf(stderr, "cuda emulation: %s failed (%d)\n", what, e);
        std::abort();
    }
}
#define checkCudaErrors(call) vr_check_cuda((call), #call)
