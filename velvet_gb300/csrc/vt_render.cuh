// vt_render.cuh — the per-particle, per-pixel arithmetic of the headless sphere-impostor
// renderer, shared by the kernels and host code (same operations on both, so a CPU
// restatement can reproduce every pixel).
#pragma once

#include <string.h>

#include "../../include/velvet_gb300.h"
#include "vt_math.cuh"

namespace vt {

// Where a particle lands: eye-space centre, NDC units per eye unit at its depth, NDC
// centre and the clamped pixel box its billboard covers.
struct SplatFrame {
    vec3 pe;
    float sx, sy, cx, cy;
    int x0, x1, y0, y1;
    bool visible;
};

VT_HD SplatFrame splat_frame(const vt_render_params& rp, vec3 x)
{
    SplatFrame f;
    f.visible = false;
    f.pe = m4v3(rp.view, x, 1.0f);
    f.sx = f.sy = f.cx = f.cy = 0.0f;
    f.x0 = f.x1 = f.y0 = f.y1 = 0;
    if (!(f.pe.z < -rp.z_near)) return f;
    const float inv = 1.0f / (-f.pe.z);
    f.sx = rp.projection[0] * inv;
    f.sy = rp.projection[5] * inv;
    f.cx = f.pe.x * f.sx;
    f.cy = f.pe.y * f.sy;
    const float W = (float)rp.width, H = (float)rp.height;
    const float px = (f.cx * 0.5f + 0.5f) * W, py = (0.5f - f.cy * 0.5f) * H;
    const float rx = rp.particle_radius * f.sx * 0.5f * W, ry = rp.particle_radius * f.sy * 0.5f * H;
    const float lx = px - rx, hx = px + rx, ly = py - ry, hy = py + ry;
    if (!(lx <= W - 1.0f && hx >= 0.0f && ly <= H - 1.0f && hy >= 0.0f)) return f;  // off screen or not finite
    f.x0 = lx > 0.0f ? (int)floorf(lx) : 0;
    f.x1 = hx < W - 1.0f ? (int)ceilf(hx) : (int)rp.width - 1;
    f.y0 = ly > 0.0f ? (int)floorf(ly) : 0;
    f.y1 = hy < H - 1.0f ? (int)ceilf(hy) : (int)rp.height - 1;
    f.visible = true;
    return f;
}

// The sphere surface seen through pixel (i, j): false outside the disc; else the key
// (eye depth bits << 32 | RGBA8) whose minimum over particles is the visible surface.
VT_HD bool splat_pixel(const vt_render_params& rp, const SplatFrame& f, int i, int j, unsigned long long& key)
{
    const float R = rp.particle_radius;
    const float nx = ((float)i + 0.5f) / (float)rp.width * 2.0f - 1.0f;
    const float ny = 1.0f - ((float)j + 0.5f) / (float)rp.height * 2.0f;
    const float u = (nx - f.cx) / (f.sx * R), v = (ny - f.cy) / (f.sy * R);
    const float r2 = u * u + v * v;
    if (!(r2 <= 1.0f)) return false;
    const float nz = sqrtf(1.0f - r2);
    float depth = -(f.pe.z + nz * R);
    if (!(depth > 0.0f)) depth = 0.0f;
    // world-space normal: the transposed rotation of the (rigid) view matrix
    const float* V = rp.view;
    const vec3 nw = mk3((V[0] * u + V[1] * v) + V[2] * nz, (V[4] * u + V[5] * v) + V[6] * nz,
                        (V[8] * u + V[9] * v) + V[10] * nz);
    const float ndl = dot(nw, mk3(rp.light_dir[0], rp.light_dir[1], rp.light_dir[2]));
    const float lit = rp.ambient + (ndl > 0.0f ? ndl : 0.0f);
    uint32_t rgba = 0xff000000u;
    for (int c = 0; c < 3; ++c) {
        float q = rp.tint[c] * lit;
        q = q < 0.0f ? 0.0f : (q > 1.0f ? 1.0f : q);
        rgba |= (uint32_t)(sqrtf(q) * 255.0f + 0.5f) << (8 * c);
    }
    uint32_t bits;
    memcpy(&bits, &depth, 4);
    key = ((unsigned long long)bits << 32) | rgba;
    return true;
}

}  // namespace vt
