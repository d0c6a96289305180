// Force-included (g++ -include) before each of the reference's solver sources when they are
// compiled on the CPU — TEST INFRASTRUCTURE.  It includes the reference's own
// Velvet/Common.cuh, then replaces its launch macros (which expand to CUDA's <<< >>>
// syntax under nvcc and to nothing under g++) with calls into the launch emulator of
// vr_driver.cpp, keeping Common.cuh's grid-size rule (ComputeGridSize).
#pragma once

#include <cstddef>

#include "Common.cuh"

namespace vr {

struct LaunchCfg {
    unsigned blocks, threads;
    bool fibers;  // run the block's threads as fibers (the kernel calls __syncthreads)
};
void run_grid(const LaunchCfg& cfg, void (*body)(void*), void* ctx);

template <class B>
void call_body(void* p)
{
    (*static_cast<B*>(p))();
}

template <class F>
struct Launch {
    LaunchCfg cfg;
    F* f;
    template <class... A>
    void operator()(A... args) const
    {
        auto body = [&]() { f(args...); };
        run_grid(cfg, &call_body<decltype(body)>, &body);
    }
};

template <class F>
Launch<F> make_launch(unsigned blocks, unsigned threads, F* f)
{
    return Launch<F>{{blocks, threads, false}, f};
}
template <class F>
Launch<F> make_launch_v(F* f, unsigned blocks, unsigned threads, size_t /*dynamic shared bytes*/ = 0)
{
    return Launch<F>{{blocks, threads, true}, f};
}

}  // namespace vr

#undef CUDA_CALL
#define CUDA_CALL(func, totalThreads)                                          \
    if (totalThreads == 0) return;                                             \
    uint func##_numBlocks, func##_numThreads;                                  \
    ComputeGridSize(totalThreads, func##_numBlocks, func##_numThreads);        \
    ::vr::make_launch(func##_numBlocks, func##_numThreads, func)
#undef CUDA_CALL_V
#define CUDA_CALL_V(func, ...) ::vr::make_launch_v(func, __VA_ARGS__)

// The reference's bending kernel calls acos (CUDA's device acosf), whose implementation is
// closed; the emulation calls the oracle's arccos instead (vo_acosf, our own series).
// Unqualified lookup inside namespace Velvet finds this overload before std::acos.
extern "C" float vo_acosf(float x);
namespace Velvet {
inline float acos(float x) { return vo_acosf(x); }
}  // namespace Velvet
