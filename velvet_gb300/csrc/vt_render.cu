// vt_render.cu — headless particle rendering: every particle a shaded sphere impostor
// (the counterpart of Velvet's _InstancedParticle geometry/fragment shaders) splatted
// into a depth|colour buffer with 64-bit atomicMin, then resolved to RGBA8.  One thread
// per particle walks the pixel box of its billboard; the arithmetic is in vt_render.cuh.
#include <cmath>

#include "vt_host.h"
#include "vt_render.cuh"

namespace vt {

static constexpr int kBlock = 256;

__global__ void __launch_bounds__(kBlock) k_render_clear(unsigned long long* __restrict__ z, int64_t npix)
{
    const int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (i < npix) z[i] = ~0ull;
}

__global__ void __launch_bounds__(kBlock)
k_render_splat(const float4* __restrict__ x, int64_t n, vt_render_params rp, unsigned long long* __restrict__ z)
{
    const int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (i >= n) return;
    const SplatFrame f = splat_frame(rp, xyz(x[i]));
    if (!f.visible) return;
    for (int j = f.y0; j <= f.y1; ++j)
        for (int k = f.x0; k <= f.x1; ++k) {
            unsigned long long key;
            if (splat_pixel(rp, f, k, j, key)) atomicMin(&z[(size_t)j * rp.width + k], key);
        }
}

__global__ void __launch_bounds__(kBlock)
k_render_resolve(const unsigned long long* __restrict__ z, int64_t npix, uint32_t background,
                 uint32_t* __restrict__ rgba)
{
    const int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (i >= npix) return;
    const unsigned long long k = z[i];
    rgba[i] = k == ~0ull ? background : (uint32_t)k;
}

cudaError_t launch_render(const float4* x, int64_t n, const vt_render_params& rp, unsigned long long* zbuf,
                          uint32_t* rgba, cudaStream_t st)
{
    const int64_t npix = (int64_t)rp.width * rp.height;
    k_render_clear<<<(unsigned)((npix + kBlock - 1) / kBlock), kBlock, 0, st>>>(zbuf, npix);
    if (n > 0) k_render_splat<<<(unsigned)((n + kBlock - 1) / kBlock), kBlock, 0, st>>>(x, n, rp, zbuf);
    k_render_resolve<<<(unsigned)((npix + kBlock - 1) / kBlock), kBlock, 0, st>>>(zbuf, npix, rp.background, rgba);
    return cudaGetLastError();
}

bool render_params_valid(const vt_render_params& rp)
{
    const auto ok = [](float v) { return std::isfinite(v); };
    return rp.width >= 1 && rp.height >= 1 && (uint64_t)rp.width * rp.height <= (1ull << 28) &&
           ok(rp.z_near) && rp.z_near > 0 && ok(rp.particle_radius) && rp.particle_radius > 0 &&
           ok(rp.projection[0]) && rp.projection[0] > 0 && ok(rp.projection[5]) && rp.projection[5] > 0;
}

// Renders x[0, n) of the device into dst (host or device-addressable), through a
// stream-ordered scratch allocation.
vt_status render_to(const float4* x, int64_t n, const vt_render_params& rp, uint32_t* dst, bool dst_on_device,
                    cudaStream_t st, uint64_t* launches)
{
    const int64_t npix = (int64_t)rp.width * rp.height;
    void* scratch = nullptr;
    cudaError_t e = cudaMallocAsync(&scratch, (size_t)npix * 12, st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMallocAsync(render)");
    unsigned long long* z = static_cast<unsigned long long*>(scratch);
    uint32_t* img = reinterpret_cast<uint32_t*>(z + npix);
    e = launch_render(x, n, rp, z, img, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dst, img, (size_t)npix * 4, dst_on_device ? cudaMemcpyDefault : cudaMemcpyDeviceToHost,
                            st);
    const cudaError_t f = cudaFreeAsync(scratch, st);
    if (e == cudaSuccess) e = f;
    if (e == cudaSuccess && !dst_on_device) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "render");
    if (launches) *launches += n > 0 ? 3 : 2;
    return VT_OK;
}

}  // namespace vt

extern "C" {

vt_status vt_camera_look_at(const float eye[3], const float center[3], const float up[3], float view[16])
{
    if (!eye || !center || !up || !view) {
        vt::set_error("NULL argument");
        return VT_ERR_INVALID_ARGUMENT;
    }
    const vec3 e = mk3(eye[0], eye[1], eye[2]), c = mk3(center[0], center[1], center[2]);
    const vec3 f = normalize(c - e);
    const vec3 s = normalize(cross(f, mk3(up[0], up[1], up[2])));
    const vec3 u = cross(s, f);
    const float m[16] = {s.x, u.x, -f.x, 0, s.y, u.y, -f.y, 0, s.z, u.z, -f.z, 0,
                         -dot(s, e), -dot(u, e), dot(f, e), 1};
    for (int k = 0; k < 16; ++k) {
        if (!std::isfinite(m[k])) {
            vt::set_error("degenerate camera (eye == center or up parallel to the view direction)");
            return VT_ERR_INVALID_ARGUMENT;
        }
        view[k] = m[k];
    }
    return VT_OK;
}

vt_status vt_camera_perspective(float fov_y, float aspect, float z_near, float z_far, float proj[16])
{
    if (!proj || !(fov_y > 0 && fov_y < 3.14159f) || !(aspect > 0) || !(z_near > 0) || !(z_far > z_near)) {
        vt::set_error("invalid perspective");
        return VT_ERR_INVALID_ARGUMENT;
    }
    const float t = std::tan(fov_y / 2.0f);
    for (int k = 0; k < 16; ++k) proj[k] = 0.0f;
    proj[0] = 1.0f / (aspect * t);
    proj[5] = 1.0f / t;
    proj[10] = -(z_far + z_near) / (z_far - z_near);
    proj[11] = -1.0f;
    proj[14] = -(2.0f * z_far * z_near) / (z_far - z_near);
    return VT_OK;
}

vt_status vt_solver_render(vt_solver* s, const vt_render_params* rp, uint32_t* rgba, int32_t dst_on_device,
                           void* stream)
{
    if (!s || !rp || !rgba) {
        vt::set_error("NULL argument");
        return VT_ERR_INVALID_ARGUMENT;
    }
    if (!vt::render_params_valid(*rp)) {
        vt::set_error("invalid render parameters");
        return VT_ERR_INVALID_ARGUMENT;
    }
    if (!s->simulated || !s->on_device) {
        vt::set_error("render after the first simulate");
        return VT_ERR_STATE;
    }
    return vt::render_to(s->world.d.x, (int64_t)s->world.n_particles, *rp, rgba, dst_on_device != 0,
                         (cudaStream_t)stream, &s->world.launches);
}

}  // extern "C"
