// vt_build.cu — the device grid builder (vt_server_submit_grid): a described grid cloth's
// positions, inverse masses, stretch rest lengths and LRA rests built by one kernel at
// admission instead of by host loops.  Compiled with the exact flags in every build
// variant (no contraction, IEEE division and square root), so a cloth built here has the
// bits of the same cloth registered on the host.
#include "vt_math.cuh"
#include "vt_world.h"

namespace vt {

static constexpr int kBuildBlock = 256;

// VtClothObjectGPU::Start for a grid cloth (Velvet/VtClothObjectGPU.hpp:43-147) without
// host loops: every particle evaluates its vertex, its inverse mass (0 when its distance
// to a slot is 0, AddAttach's rule), its LRA rests |slot - x0_i| and, as generator (a, b),
// the rest lengths of its four stretch constraints from the neighbouring vertices — the
// values grid_rests reads from the host-built constraint list, by the same operations.
__global__ void __launch_bounds__(kBuildBlock)
k_grid_build(float4* __restrict__ x, float4* __restrict__ v, float4* __restrict__ x0,
             float4* __restrict__ grest, float4* __restrict__ glra, GridBuildArgs g)
{
    const int V = g.res + 1;
    const int64_t i = blockIdx.x * (int64_t)kBuildBlock + threadIdx.x;
    if (i >= (int64_t)V * V) return;
    const int a = (int)(i / V), b = (int)(i - (int64_t)a * V), R = g.res;
    const vec3 p = grid_vertex(a, b, R, g.size, g.model);
    float w = 1.0f;
    float r[kGridLraCached] = {0, 0, 0, 0};
#pragma unroll
    for (int s = 0; s < kGridLraCached; ++s)
        if (s < g.ns) {
            const float dist = length(xyz(g.slot[s]) - p);
            if (dist == 0) w = 0;
            r[s] = dist;
        }
    float4 gr = make_float4(0, 0, 0, 0);
    if (b < R) gr.x = length(p - grid_vertex(a, b + 1, R, g.size, g.model));
    if (a < R) gr.y = length(p - grid_vertex(a + 1, b, R, g.size, g.model));
    if (a < R && b < R) {
        gr.z = length(p - grid_vertex(a + 1, b + 1, R, g.size, g.model));
        gr.w = length(grid_vertex(a, b + 1, R, g.size, g.model) - grid_vertex(a + 1, b, R, g.size, g.model));
    }
    x[i] = make_float4(p.x, p.y, p.z, w);
    x0[i] = make_float4(p.x, p.y, p.z, 0.0f);
    v[i] = make_float4(0, 0, 0, 0);
    grest[i] = gr;
    glra[i] = make_float4(r[0], r[1], r[2], r[3]);
}

cudaError_t launch_grid_build(const DeviceArrays& d, int64_t pb, const GridBuildArgs& g, cudaStream_t st)
{
    const int64_t n = (int64_t)(g.res + 1) * (g.res + 1);
    k_grid_build<<<(unsigned)((n + kBuildBlock - 1) / kBuildBlock), kBuildBlock, 0, st>>>(d.x + pb, d.v + pb, d.x0 + pb,
                                                                         d.grest + pb, d.glra + pb, g);
    return cudaGetLastError();
}

}  // namespace vt
