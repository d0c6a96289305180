#pragma once
// CPU emulation: thrust is included by Common.cuh but not used by the solver kernels.
