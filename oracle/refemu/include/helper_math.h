#pragma once
// CPU emulation: the CUDA samples' float3 helpers are not used by the solver kernels.
