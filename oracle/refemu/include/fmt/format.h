#pragma once
// CPU emulation: fmt is included by Common.cuh; the solver kernels print nothing.
namespace fmt {
template <class... A>
inline void print(A&&...)
{
}
}  // namespace fmt
