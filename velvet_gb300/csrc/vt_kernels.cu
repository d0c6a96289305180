// vt_kernels.cu — XPBD substep kernels for sm_103a.
//
// Same arithmetic as the reference kernels (Velvet/VtClothSolverGPU.cu), different
// packaging:
//   * Jacobi sums are gathers, not atomics.  Each particle adds its constraints'
//     corrections in constraint order, so the sum is the one a sequential run of the
//     reference kernels produces and is identical from run to run.  Grid cloths (the
//     grid builder's topology) use k_grid_iter: implicit topology, a tile of predicted
//     positions in shared memory, every stretch and bending constraint evaluated once
//     per tile.  Other meshes use k_bend + k_solve over CSR lists built at registration:
//     stretch and attachment corrections recomputed by each endpoint (the two endpoints
//     of a stretch constraint get exact negatives of each other's intermediate values,
//     so the recomputation is exact), bending evaluated once per constraint into
//     per-corner slots that the particle gather reads.
//   * ApplyDeltas is fused into the gather that produces the deltas; predicted
//     positions ping-pong between two buffers so every constraint of an iteration sees
//     the positions of the previous iteration, as the reference's launch order implies.
//   * CollideParticles + ApplyDeltas + CollideSDF are one kernel; Finalize and the next
//     substep's PredictPositions are fused into the last iteration's gather; the
//     pre-stabilisation CollideSDF is fused with the first PredictPositions.
//   * float4 particles (w = inverse mass) so each particle is one 16-byte load.
// Also here: read-back packing (k_pack_xyz).  The device grid builder is in vt_build.cu.
#include <utility>

#include <algorithm>

#include "vt_math.cuh"
#include "vt_world.h"

namespace vt {

static constexpr int kBlock = 256;

// 16-byte asynchronous global -> shared copies (cp.async through L2); the zero-fill form
// reads nothing and writes zeros when `valid` is false.  Both addresses 16-byte aligned.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem)
{
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async16_zfill(void* smem, const void* gmem, bool valid)
{
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(valid ? 16 : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

// ------------------------------------------------------------------ TMA + mbarrier
// The tile kernel's bulk tensor loads: one thread arms a shared-memory mbarrier with the
// bytes it expects and issues cp.async.bulk.tensor copies of the halo tile and the other
// per-tile arrays; every thread then waits on the barrier's phase 0 (bounded, see
// mbar_wait).  Coordinates are (component 0, column, row) of a map from tmap_index.
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.b32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(phase)
        : "memory");
    return ok != 0;
}

// Waits for phase `phase` of the barrier; gives up after kMbarTries attempts (each
// attempt may suspend the thread for a short, hardware-chosen time) and returns false.
constexpr int kMbarTries = 1 << 20;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase)
{
    for (int k = 0; k < kMbarTries; ++k)
        if (mbar_try_wait(bar, phase)) return true;
    return false;
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int c0, int c1, int c2,
                                            uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
        : "memory");
}

// ------------------------------------------------------------------ colliders
__device__ __forceinline__ float sgnf(float v) { return (v > 0) ? 1.0f : (v < 0 ? -1.0f : 0.0f); }

// 1 + 2^-20 (exact in FP32): with it RN(RN(r*r) * kFarMargin) >= r^2 (1-2^-24)^2 (1+2^-20)
// > r^2 for r^2 in the normal range, so a squared distance at or above that bound has a
// correctly rounded square root >= r: the distance test `d >= r` can be decided without
// taking the root (the root is monotone and r is a float).
constexpr float kFarMargin = 1.0f + 1.0f / 1048576.0f;

// SDFCollider::ComputeSDF, Velvet/VtClothSolverGPU.cuh:22-89
__device__ vec3 collider_sdf(const ColliderDev& c, vec3 t, float margin)
{
    if (c.type == 1) {  // plane
        float offset = t.y - (c.py + margin);
        if (offset < 0) return mk3(0, -offset, 0);
    } else if (c.type == 0) {  // sphere
        float radius = c.sx + margin;
        vec3 diff = t - mk3(c.px, c.py, c.pz);
        const float q = dot_exact(diff, diff);
        // outside for sure (no square root): q >= RN(RN(r*r) * (1 + 2^-20)) > r^2 gives
        // RN(sqrt(q)) >= r, so offset >= 0, whatever the rounding (r kept in the normal range)
        if (radius > 1e-18f && radius < 1e18f && q >= (radius * radius) * kFarMargin) return mk3(0, 0, 0);
        float distance = sqrt_exact(q);
        float offset = distance - radius;
        if (offset < 0) {
            vec3 direction = diff / distance;
            return direction * (-offset);
        }
    } else if (c.type == 2) {  // cube
        vec3 correction = mk3(0, 0, 0);
        vec3 local = m4v3(c.inv, t, 1.0f);
        vec3 cube = mk3(0.5f + margin / c.sx, 0.5f + margin / c.sy, 0.5f + margin / c.sz);
        vec3 offset = mk3(fabsf(local.x), fabsf(local.y), fabsf(local.z)) - cube;
        float maxv = fmaxf(offset.x, fmaxf(offset.y, offset.z));
        float minv = fminf(offset.x, fminf(offset.y, offset.z));
        float midv = ((offset.x + offset.y) + offset.z - maxv) - minv;
        float scalar = 1.0f;
        if (maxv < 0) {
            const float m = 0.03f;
            if (midv > -m) scalar = 0.2f;
            if (minv > -m) {
                vec3 mask = mk3(offset.x < 0 ? sgnf(local.x) : 0, offset.y < 0 ? sgnf(local.y) : 0,
                                offset.z < 0 ? sgnf(local.z) : 0);
                vec3 vec = offset + mk3(m, m, m);
                float len = length(vec);
                if (len < m) correction = cmul(mask, normalize(vec)) * (m - len);
            } else if (offset.x == maxv) {
                correction = mk3(copysignf(-offset.x, local.x), 0, 0);
            } else if (offset.y == maxv) {
                correction = mk3(0, copysignf(-offset.y, local.y), 0);
            } else if (offset.z == maxv) {
                correction = mk3(0, 0, copysignf(-offset.z, local.z));
            }
        }
        float ms[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) ms[k] = c.cur3[k] * scalar;
        return m3v3(ms, correction);
    }
    return mk3(0, 0, 0);
}

// ComputeFriction, Velvet/VtClothSolverGPU.cu:272-287
__device__ __forceinline__ vec3 friction_of(vec3 corr, vec3 relvel, float friction)
{
    vec3 fr = mk3(0, 0, 0);
    float cl = length(corr);
    if (friction > 0 && cl > 0) {
        vec3 nrm = corr / cl;
        vec3 tan = relvel - nrm * dot(relvel, nrm);
        float tl = length(tan);
        float mt = cl * friction;
        fr = (-tan) * fminf(mt / tl, 1.0f);
    }
    return fr;
}

// CollideSDF_Kernel body, Velvet/VtClothSolverGPU.cu:289-314
__device__ __forceinline__ vec3 collide_sdf(const DomainParams& D, const ColliderDev* __restrict__ cols,
                                            vec3 pred, vec3 pos, float dt)
{
    for (int k = 0; k < D.col_count; ++k) {
        const ColliderDev& c = cols[D.col_begin + k];
        vec3 corr = collider_sdf(c, pred, D.margin);
        pred = pred + corr;
        if (dot(corr, corr) > 0) {
            // VelocityAt, VtClothSolverGPU.cuh:91-96 (last * invCur precomputed)
            vec3 lp = m4v3(c.last_inv, pred, 1.0f);
            vec3 vel = (pred - lp) / c.delta_time;
            vec3 relvel = (pred - pos) - vel * dt;
            pred = pred + friction_of(corr, relvel, D.friction);
        }
    }
    return pred;
}

__device__ __forceinline__ void flag_nonfinite(int32_t* status, const DomainParams& D, int dom, vec3 a)
{
    if (!(isfinite(a.x) && isfinite(a.y) && isfinite(a.z))) {
        atomicOr(&status[0], 1);
        atomicOr(&status[1 + dom], 1);
    }
}

// ------------------------------------------------------------------ pre-stabilisation + predict
// CollideSDF(positions, ..., frameDt) (VtClothSolverGPU.hpp:73) then PredictPositions
// (VtClothSolverGPU.cu:42-53) of substep 0.
// (eight blocks per SM: 32 registers instead of 40, 0.131 -> 0.122 ms per mix frame)
__global__ void __launch_bounds__(kBlock, 8)
k_presdf_predict(const Tile* __restrict__ tiles, const DomainParams* __restrict__ doms,
                 const ColliderDev* __restrict__ cols, float4* __restrict__ x, float4* __restrict__ v,
                 float4* __restrict__ pout)
{
    const Tile tl = tiles[blockIdx.x];
    const int i = tl.begin + (int)threadIdx.x;
    if (i >= tl.end) return;
    const DomainParams& D = doms[tl.dom];
    float4 x4 = x[i];
    vec3 pos = xyz(x4);
    if (D.col_count > 0) {
        pos = collide_sdf(D, cols, pos, pos, D.dt_frame);
        x[i] = make_float4(pos.x, pos.y, pos.z, x4.w);
    }
    const float dt = D.dt_sub;
    vec3 vel = xyz(v[i]);
    vel = vel + mk3(D.gx, D.gy, D.gz) * dt;
    vec3 pred = pos + vel * dt;
    v[i] = make_float4(vel.x, vel.y, vel.z, 0.0f);
    pout[i] = make_float4(pred.x, pred.y, pred.z, x4.w);
}

// ------------------------------------------------------------------ collide particles + SDF
// CollideParticles_Kernel (VtClothSolverGPU.cu:329-373) + ApplyDeltas (:253-264) +
// CollideSDF (:289-314) for one substep.  Thread r of a domain takes the domain's r-th
// particle, whose neighbour list is column r, so a warp reads entry k of 32 lists and
// its own particles' positions as consecutive words.
constexpr int kCollideBatch = 4;  // list entries gathered together (2 / 8 / 16: 1.67 / 1.91 / 2.67 vs 1.66 ms per mix frame)
// at six blocks per SM (40 registers, a few bytes spilled): 1.35 -> 1.06 ms per mix frame
// against four blocks at 64 registers (five blocks: 1.14; six with two entries: 1.22)

// Particle i (the domain's r-th) after its collisions, ApplyDeltas and the SDF: its
// predicted position from pin, the other particles' from pin too (every particle reads the
// positions from before the pass), velocities against x.  Returns (position, inverse mass).
__device__ __forceinline__ float4 collide_particle(const DomainParams& D, const ColliderDev* __restrict__ cols,
                                                   int i, int r, const float4* __restrict__ x,
                                                   const float4* __restrict__ pin, const uint32_t* __restrict__ nbr,
                                                   int32_t* __restrict__ status)
{
    const float4 pi4 = pin[i];
    vec3 pi = xyz(pi4);
    const float wi = pi4.w;
    const vec3 xi = xyz(x[i]);
    if (D.self_collision) {
        vec3 delta = mk3(0, 0, 0);
        int count = 0;
        const vec3 veli = pi - xi;
        const uint32_t* nb = nbr + nbr_offset(D) + r;
        const int stride = D.p_count;
        const float diam = D.diameter;
        const bool far_ok = diam > 1e-18f && diam < 1e18f;
        const float far2 = (diam * diam) * kFarMargin;
        // kCollideBatch list entries and their particles are requested together (loads
        // beyond the list's end read a valid slot and are not used), then taken in list order
        bool done = false;
        for (int k0 = 0; k0 < D.max_nbr && !done; k0 += kCollideBatch) {
            uint32_t jq[kCollideBatch];
            float4 pq[kCollideBatch];
#pragma unroll
            for (int u = 0; u < kCollideBatch; ++u)
                jq[u] = k0 + u < D.max_nbr ? __ldg(nb + (size_t)(k0 + u) * stride) : 0xffffffffu;
#pragma unroll
            for (int u = 0; u < kCollideBatch; ++u)
                pq[u] = pin[jq[u] - (uint32_t)D.p_begin < (uint32_t)D.p_count ? jq[u] : (uint32_t)D.p_begin];
#pragma unroll
            for (int u = 0; u < kCollideBatch; ++u) {
                if (done) break;
                const uint32_t j = jq[u];
                if (j == 0xffffffffu || !VT_IN_RANGE(j, D.p_begin, D.p_begin + D.p_count, status)) {
                    done = true;
                    break;
                }
                const float4 pj4 = pq[u];
                const float denom = wi + pj4.w;
                if (denom <= 0) continue;
                const vec3 pj = xyz(pj4);
                const vec3 diff = pi - pj;
                const float q = dot_exact(diff, diff);
                if (far_ok && q >= far2) continue;  // d >= diam without the square root
                const float d = sqrt_exact(q);
                if (d >= diam) continue;
                const vec3 grad = diff / (d + VT_EPSILON);
                const float lambda = (d - diam) / denom;
                const vec3 common = grad * lambda;
                count++;
                delta = delta - common * wi;
                const vec3 relvel = veli - (pj - xyz(x[j]));
                const vec3 fr = friction_of(common, relvel, D.friction);
                delta = delta + fr * wi;
            }
        }
        if (count > 0) {
            const float c = (float)count;
            pi = pi + (delta / c) * D.relax;
        }
    }
    pi = collide_sdf(D, cols, pi, xi, D.dt_sub);
    return make_float4(pi.x, pi.y, pi.z, wi);
}

__global__ void __launch_bounds__(kBlock, 6)
k_collide(const Tile* __restrict__ tiles, const DomainParams* __restrict__ doms,
          const ColliderDev* __restrict__ cols, const float4* __restrict__ x,
          const float4* __restrict__ pin, float4* __restrict__ pout,
          const uint32_t* __restrict__ nbr, int32_t* __restrict__ status)
{
    const Tile tl = tiles[blockIdx.x];
    const int t = tl.begin + (int)threadIdx.x;
    if (t >= tl.end) return;
    const DomainParams& D = doms[tl.dom];
    pout[t] = collide_particle(D, cols, t, t - D.p_begin, x, pin, nbr, status);
}

// ------------------------------------------------------------------ constraint math
// One dihedral bending constraint, SolveBending_Kernel (VtClothSolverGPU.cu:117-189).
// a0..a3: predicted positions with the inverse mass in w; xpbd = bendCompliance / dt / dt
// (evaluated once per frame on the host, in that order).  Writes the four corrections
// with w = 1 when the constraint fired, all zero when it returned early.
__device__ __forceinline__ void bend_eval(float4 a0, float4 a1, float4 a2, float4 a3, float rest,
                                          float xpbd, float4& c0, float4& c1, float4& c2, float4& c3)
{
    const vec3 p0 = xyz(a0), p1 = xyz(a1), p2 = xyz(a2), p3 = xyz(a3);
    const float w0 = a0.w, w1 = a1.w, w2 = a2.w, w3 = a3.w;
    c0 = make_float4(0, 0, 0, 0);
    c1 = c0;
    c2 = c0;
    c3 = c0;
    const vec3 e = p3 - p2;
    const float elen = length_exact(e);
    if (elen < VT_EPSILON) return;
    const float inv = 1.0f / elen;
    // the angle chain in exact operations (vt_math.cuh: acos near a flat pair)
    vec3 n1 = cross_exact(p2 - p0, p3 - p0);
    n1 = div_exact(n1, dot_exact(n1, n1));
    vec3 n2 = cross_exact(p3 - p1, p2 - p1);
    n2 = div_exact(n2, dot_exact(n2, n2));
    const vec3 d0 = n1 * elen;
    const vec3 d1 = n2 * elen;
    const vec3 d2 = n1 * (dot(p0 - p3, e) * inv) + n2 * (dot(p1 - p3, e) * inv);
    const vec3 d3 = n1 * (dot(p2 - p0, e) * inv) + n2 * (dot(p2 - p1, e) * inv);
    n1 = normalize_exact(n1);
    n2 = normalize_exact(n2);
    const float phi = vt_acosf_exact(gclamp(dot_exact(n1, n2), -1.0f, 1.0f));
    float lambda = w0 * dot(d0, d0) + w1 * dot(d1, d1);
    lambda = lambda + w2 * dot(d2, d2);
    lambda = lambda + w3 * dot(d3, d3);
    if (lambda < VT_EPSILON) return;
    lambda = (phi - rest) / (lambda + xpbd);
    if (dot_exact(cross_exact(n1, n2), e) > 0.0f) lambda = -lambda;
    const vec3 k0 = d0 * (-w0 * lambda), k1 = d1 * (-w1 * lambda);
    const vec3 k2 = d2 * (-w2 * lambda), k3 = d3 * (-w3 * lambda);
    c0 = make_float4(k0.x, k0.y, k0.z, 1.0f);
    c1 = make_float4(k1.x, k1.y, k1.z, 1.0f);
    c2 = make_float4(k2.x, k2.y, k2.z, 1.0f);
    c3 = make_float4(k3.x, k3.y, k3.z, 1.0f);
}

// lambda * gradient of a distance constraint that fires: (diff / (d + eps)) * ((d - rest)
// / denom), the reference's two divisions (VtClothSolverGPU.cu:87-91).  The fast build
// takes one: diff * ((d - rest) / (denom * (d + eps))), within its tolerance.
__device__ __forceinline__ vec3 stretch_scale(vec3 diff, float d, float denom, float rest)
{
#if VT_FAST_DEVICE
    return mul_p(diff, (d - rest) / (denom * (d + VT_EPSILON)));
#else
    const vec3 grad = diff / (d + VT_EPSILON);
    const float lambda = (d - rest) / denom;
    return mul_p(grad, lambda);
#endif
}

// One distance constraint, SolveStretch_Kernel (VtClothSolverGPU.cu:76-98): returns
// whether it fires and `common` = lambda * gradient, gradient taken from pa - pb.  The
// reference adds -w_a * common to a and w_b * common to b.  Evaluated from the other
// endpoint (pa, pb swapped) every intermediate value is the exact negation, so either
// endpoint may evaluate it.
__device__ __forceinline__ bool stretch_common(float4 pa, float4 pb, float rest, vec3& common)
{
    const vec3 diff = sub_p(xyz(pa), xyz(pb));
    const float d = length_exact(diff);
    const float denom = pa.w + pb.w;
    if (!(d != rest && denom > 0)) return false;
    common = stretch_scale(diff, d, denom, rest);
    return true;
}

// One attachment, SolveAttachment_Kernel (VtClothSolverGPU.cu:216-234).
__device__ __forceinline__ void attach_one(vec3 pi, float wi, vec3 slot, float target, vec3& acc, int& cnt)
{
    if (wi == 0 && target > 0) return;
    const vec3 diff = pi - slot;
    const float d = length_exact(diff);
    if (d > target) {
        acc3(acc, (-diff) + (diff / d) * target);
        cnt++;
    }
}

// Filters that let an attachment which cannot fire skip its square roots.  They rest on
// two facts: a correctly rounded sqrt is monotone, so sqrt(q) < t (t a float) gives
// RN(sqrt(q)) <= t and the test d > t fails; and each rounding moves a product by at most
// a factor (1 +- 2^-24).  kAttachMargin = 1 - 2^-20 (exact in FP32) absorbs those factors
// with room to spare; the range guards keep every bound a normal, finite number (no
// underflow, where the relative error of a product is unbounded).  Pairs the filter does
// not drop take the exact path, so results and their order are attach_one's.
constexpr float kAttachMargin = 1.0f - 1.0f / 1048576.0f;

// attach_one for a particle with wi != 0 and a known target t: skips the pair when
// q = |pi - slot|^2 < RN(RN(t*t) * margin) <= t^2 (1+2^-24)^2 (1-2^-20) < t^2.
__device__ __forceinline__ void attach_one_filtered(vec3 pi, float wi, vec3 slot, float target, vec3& acc,
                                                    int& cnt)
{
    if (wi != 0.0f && target > 1e-18f && target < 1e18f) {
        const vec3 diff = pi - slot;
        const float q = dot_exact(diff, diff);
        if (q < (target * target) * kAttachMargin) return;
        const float d = sqrt_exact(q);
        if (d > target) {
            acc3(acc, (-diff) + (diff / d) * target);
            cnt++;
        }
        return;
    }
    attach_one(pi, wi, slot, target, acc, cnt);
}

// An LRA attachment whose rest distance |slot0 - x0i| is recomputed: target =
// RN(RN(sqrt(q0)) * lrs) >= sqrt(q0) lrs (1-2^-24)^2, so with c2 = RN(RN(lrs*lrs) * margin)
// the bound RN(q0 * c2) <= q0 lrs^2 (1+2^-24)^3 (1-2^-20) < target^2 and a pair below it
// needs neither square root.  The guards on q0 and lrs keep lrs^2, q0 * c2 and the target
// within the normal range.
__device__ __forceinline__ void attach_lra_filtered(vec3 pi, float wi, vec3 slot, vec3 slot0, vec3 x0i, float lrs,
                                                    float c2, vec3& acc, int& cnt)
{
    const vec3 r = slot0 - x0i;
    const float q0 = dot_exact(r, r);
    if (wi != 0.0f && q0 > 1e-20f && q0 < 1e20f && lrs > 1e-4f && lrs < 1e4f) {
        const vec3 diff = pi - slot;
        const float q = dot_exact(diff, diff);
        if (q < q0 * c2) return;
    }
    attach_one(pi, wi, slot, sqrt_exact(q0) * lrs, acc, cnt);
}

// Groups of LRA slots (cloths with more slots than the per-particle cache): a whole group
// is skipped when bounds prove that every one of its pairs passes attach_lra_filtered's
// test q < RN(q0 * c2), so that none fires.  Per group, boxes [lo, hi] of the current and
// [lo0, hi0] of the rest slot positions (w of lo = 1 when a coordinate of the group is
// non-finite or beyond 1e9: never skipped).  With u = 2^-24, for every slot s of the group:
//  * D = per-axis max(|p - lo|, |p - hi|) (rounded differences are >= the real ones times
//    1 - u) bounds |p - slot_s| per axis; the computed q_s <= |D|^2 (1+u)^5/(1-u)^5, and
//    qu = RN(RN(|D|^2) * (1 + 2^-18)) is above that;
//  * E = per-axis distance from x0 to the rest box bounds |slot0_s - x0| per axis from
//    below; the computed q0_s >= |E|^2 (1-u)^5/(1+u)^5, and ql = RN(RN(|E|^2) * (1 - 2^-18))
//    is below that;
//  * then RN(RN(ql * c2) * (1 - 2^-18)) <= ql c2 (1+u)^2 (1 - 2^-18) < q0_s c2 (1 - u) <=
//    RN(q0_s * c2), so qu below it gives q_s < RN(q0_s * c2) for the whole group.
// Coordinates below 1e9 keep q0_s < 1e20 and every product finite; |D|^2, |E|^2 > 1e-20
// keep the absolute error of an underflowed component square (<= 2^-149 each) far inside
// the margins; q0_s >= ql > 1e-20 meets attach_lra_filtered's own guard.
constexpr int kLraGroupMin = 16;      // slots per group (more when a cloth has > 1024)
constexpr int kLraGroupsMax = 64;     // groups per cloth: 4 boxes each fill kBlock float4
constexpr int kLraSuper = 4;          // groups per super-group: 16 threads reduce one
static_assert(4 * kLraGroupsMax <= kBlock && kLraGroupsMax * 4 == kBlock, "group boxes fill the LRA rest array");
constexpr float kBoundUp = 1.0f + 1.0f / 262144.0f;
constexpr float kBoundDown = 1.0f - 1.0f / 262144.0f;

__device__ __forceinline__ bool in_bound_range(vec3 v)
{
    return fabsf(v.x) < 1e9f && fabsf(v.y) < 1e9f && fabsf(v.z) < 1e9f;
}

// The four boxes of each group of the domain's ns slots, into box[4 g .. 4 g + 3], and of
// each super-group (kLraSuper consecutive groups) into sup[4 G .. 4 G + 3]; four threads
// per group, sixteen per super-group (all threads of the block take part in the warp
// shuffles).
__device__ __forceinline__ void lra_group_boxes(float4* box, float4* sup, const float4* __restrict__ slots,
                                                const float4* __restrict__ slots0, int ns, int gsize,
                                                int ngroups, int tid)
{
    const int g = tid >> 2, q = tid & 3;
    const float inf = __int_as_float(0x7f800000);
    vec3 lo = mk3(inf, inf, inf), hi = mk3(-inf, -inf, -inf), lo0 = lo, hi0 = hi;
    int bad = 0;
    if (g < ngroups) {
        const int sb = g * gsize, se = min(sb + gsize, ns);
        for (int s = sb + q; s < se; s += 4) {
            const vec3 a = xyz(slots[s]), b = xyz(slots0[s]);
            bad |= (in_bound_range(a) && in_bound_range(b)) ? 0 : 1;
            lo = mk3(fminf(lo.x, a.x), fminf(lo.y, a.y), fminf(lo.z, a.z));
            hi = mk3(fmaxf(hi.x, a.x), fmaxf(hi.y, a.y), fmaxf(hi.z, a.z));
            lo0 = mk3(fminf(lo0.x, b.x), fminf(lo0.y, b.y), fminf(lo0.z, b.z));
            hi0 = mk3(fmaxf(hi0.x, b.x), fmaxf(hi0.y, b.y), fmaxf(hi0.z, b.z));
        }
    }
    auto merge = [&](int m) {
        const unsigned all = 0xffffffffu;
        bad |= __shfl_xor_sync(all, bad, m);
        lo = mk3(fminf(lo.x, __shfl_xor_sync(all, lo.x, m)), fminf(lo.y, __shfl_xor_sync(all, lo.y, m)),
                 fminf(lo.z, __shfl_xor_sync(all, lo.z, m)));
        hi = mk3(fmaxf(hi.x, __shfl_xor_sync(all, hi.x, m)), fmaxf(hi.y, __shfl_xor_sync(all, hi.y, m)),
                 fmaxf(hi.z, __shfl_xor_sync(all, hi.z, m)));
        lo0 = mk3(fminf(lo0.x, __shfl_xor_sync(all, lo0.x, m)), fminf(lo0.y, __shfl_xor_sync(all, lo0.y, m)),
                  fminf(lo0.z, __shfl_xor_sync(all, lo0.z, m)));
        hi0 = mk3(fmaxf(hi0.x, __shfl_xor_sync(all, hi0.x, m)), fmaxf(hi0.y, __shfl_xor_sync(all, hi0.y, m)),
                  fmaxf(hi0.z, __shfl_xor_sync(all, hi0.z, m)));
    };
    auto store = [&](float4* b) {
        b[0] = make_float4(lo.x, lo.y, lo.z, bad ? 1.0f : 0.0f);
        b[1] = make_float4(hi.x, hi.y, hi.z, 0.0f);
        b[2] = make_float4(lo0.x, lo0.y, lo0.z, 0.0f);
        b[3] = make_float4(hi0.x, hi0.y, hi0.z, 0.0f);
    };
    merge(1);
    merge(2);
    if (g < ngroups && q == 0) store(box + 4 * g);
    merge(4);
    merge(8);
    if ((tid & 15) == 0 && g < ngroups) store(sup + 4 * (g / kLraSuper));
}

// True when no pair of the group can fire for the particle at p with rest position x0
// (the caller has checked wi != 0, lrs in (1e-4, 1e4) and p, x0 in range).
__device__ __forceinline__ bool lra_group_quiet(vec3 p, vec3 x0, const float4* box, float c2)
{
    const float4 lo = box[0], hi = box[1], lo0 = box[2], hi0 = box[3];
    if (lo.w != 0.0f) return false;
    const vec3 D = mk3(fmaxf(fabsf(p.x - lo.x), fabsf(p.x - hi.x)), fmaxf(fabsf(p.y - lo.y), fabsf(p.y - hi.y)),
                       fmaxf(fabsf(p.z - lo.z), fabsf(p.z - hi.z)));
    const vec3 E = mk3(fmaxf(fmaxf(lo0.x - x0.x, x0.x - hi0.x), 0.0f), fmaxf(fmaxf(lo0.y - x0.y, x0.y - hi0.y), 0.0f),
                       fmaxf(fmaxf(lo0.z - x0.z, x0.z - hi0.z), 0.0f));
    const float qf = dot(D, D), q0f = dot(E, E);
    if (!(qf > 1e-20f && q0f > 1e-20f)) return false;
    const float qu = qf * kBoundUp, ql = q0f * kBoundDown;
    if (!(ql > 1e-20f)) return false;
    return qu < (ql * c2) * kBoundDown;
}

// ApplyDeltas (VtClothSolverGPU.cu:253-264): the particle moved by the relaxed mean of
// its constraints' corrections.
__device__ __forceinline__ vec3 jacobi_apply(const DomainParams& D, vec3 pi, vec3 acc, int cnt)
{
    if (cnt > 0) {
        const float count = (float)cnt;
        pi = madd_p(acc / count, D.relax, pi);
    }
    return pi;
}

// ApplyDeltas (VtClothSolverGPU.cu:253-264) and, by mode, Finalize (:388-407) and the
// next substep's PredictPositions (:42-53); writes x, v, p_out of particle i.  `xsrc`
// holds x[i] (global memory, or a shared-memory copy staged by the caller).
template <int kMode>
__device__ __forceinline__ void apply_and_finalize(const DomainParams& D, int dom, int i, vec3 pi, float wi,
                                                   vec3 acc, int cnt, const float4* xsrc,
                                                   float4* __restrict__ pout, float4* __restrict__ x,
                                                   float4* __restrict__ v, int32_t* __restrict__ status)
{
    pi = jacobi_apply(D, pi, acc, cnt);
    if (kMode == SOLVE_PLAIN) {
        pout[i] = make_float4(pi.x, pi.y, pi.z, wi);
        return;
    }
    const float dt = D.dt_sub;
    const float4 x4 = *xsrc;
    const vec3 xi = xyz(x4);
    vec3 np = pi;
    vec3 rv = (np - xi) / dt;
    const float rl = length_exact(rv);
    if (rl > D.max_speed) {
        rv = (rv / rl) * D.max_speed;
        np = xi + rv * dt;
    }
    vec3 vn = rv * (1.0f - D.damping * dt);
    flag_nonfinite(status, D, dom, np);
    x[i] = make_float4(np.x, np.y, np.z, x4.w);
    if (kMode == SOLVE_FINALIZE_PREDICT) {
        vn = vn + mk3(D.gx, D.gy, D.gz) * dt;
        pi = np + vn * dt;
    }
    v[i] = make_float4(vn.x, vn.y, vn.z, 0.0f);
    pout[i] = make_float4(pi.x, pi.y, pi.z, x4.w);
}

// ------------------------------------------------------------------ bending (CSR domains)
// SolveBending once per constraint; the four corrections go to per-corner slots.
__global__ void __launch_bounds__(kBlock)
k_bend(const Tile* __restrict__ tiles, const DomainParams* __restrict__ doms,
       const float4* __restrict__ pin, const uint4* __restrict__ bidx,
       const float* __restrict__ brest, float4* __restrict__ bcorr)
{
    const Tile tl = tiles[blockIdx.x];
    const int b = tl.begin + (int)threadIdx.x;
    if (b >= tl.end) return;
    const DomainParams& D = doms[tl.dom];
    const uint4 q = bidx[b];
    float4 c0, c1, c2, c3;
    bend_eval(pin[q.x], pin[q.y], pin[q.z], pin[q.w], brest[b], D.xpbd_bend, c0, c1, c2, c3);
    float4* out = bcorr + 4 * (size_t)b;
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

// ------------------------------------------------------------------ constraint gather (CSR)
// SolveStretch (:65-102) + SolveAttachment (:205-235) + the bending corners written by
// k_bend, summed per particle in constraint order, then ApplyDeltas (:253-264) and, by
// mode, Finalize + the next Predict.  For domains whose topology is arbitrary.
template <int kMode>
__global__ void __launch_bounds__(kBlock)
k_solve(const Tile* __restrict__ tiles, const DomainParams* __restrict__ doms,
        const float4* __restrict__ pin, float4* __restrict__ pout, float4* __restrict__ x,
        float4* __restrict__ v, const float4* __restrict__ x0,
        const int32_t* __restrict__ st_off, const int2* __restrict__ st_ent,
        const int32_t* __restrict__ at_off, const int2* __restrict__ at_ent,
        const LraGroup* __restrict__ lra, const float4* __restrict__ slots,
        const float4* __restrict__ slots0, const int32_t* __restrict__ bd_off,
        const int32_t* __restrict__ bd_ent, const float4* __restrict__ bcorr,
        int32_t* __restrict__ status)
{
    const Tile tl = tiles[blockIdx.x];
    const int i = tl.begin + (int)threadIdx.x;
    if (i >= tl.end) return;
    const DomainParams& D = doms[tl.dom];
    const float4 pi4 = pin[i];
    const vec3 pi = xyz(pi4);
    const float wi = pi4.w;
    vec3 acc = mk3(0, 0, 0);
    int cnt = 0;
    // stretch: each entry is (other particle, rest length); this particle evaluates the
    // constraint as its first endpoint and takes -w_i * common
    // unrolled by four: the entry and position loads of several constraints are in flight
    // at once (the gathers are latency-bound; eight made it slower)
#pragma unroll 4
    for (int e = st_off[i], e1 = st_off[i + 1]; e < e1; ++e) {
        const int2 en = st_ent[e];
        if (!VT_IN_RANGE(en.x, D.p_begin, D.p_begin + D.p_count, status)) continue;
        vec3 common;
        if (stretch_common(pi4, pin[en.x], __int_as_float(en.y), common)) {
            acc3(acc, common * (-wi));
            cnt++;
        }
    }
    // attachments: (slot, distance) or an LRA group (distances recomputed from x0)
    const float lrs = D.lrs;
    for (int e = at_off[i], e1 = at_off[i + 1]; e < e1; ++e) {
        const int2 en = at_ent[e];
        if (en.x >= 0) {
            attach_one(pi, wi, xyz(slots[en.x]), __int_as_float(en.y) * lrs, acc, cnt);
        } else {
            const LraGroup g = lra[-en.x - 1];
            const vec3 x0i = xyz(x0[i]);
            for (int s = g.slot_begin; s < g.slot_begin + g.slot_count; ++s) {
                const float rest = length_exact(xyz(slots0[s]) - x0i);
                attach_one(pi, wi, xyz(slots[s]), rest * lrs, acc, cnt);
            }
        }
    }
    // bending corners
#pragma unroll 4
    for (int e = bd_off[i], e1 = bd_off[i + 1]; e < e1; ++e) {
        const float4 c = bcorr[bd_ent[e]];
        if (c.w != 0.0f) {
            acc3(acc, xyz(c));
            cnt++;
        }
    }
    apply_and_finalize<kMode>(D, tl.dom, i, pi, wi, acc, cnt, x + i, pout, x, v, status);
}

// ------------------------------------------------------------------ grid tile iteration
// One Jacobi iteration of a grid cloth built by the grid constraint builder, with its
// topology implicit: particle (a, b) = a * V + b, stretch constraints of generator (x, y)
// t0 (x,y)-(x,y+1), t1 (x,y)-(x+1,y), t2 (x,y)-(x+1,y+1), t3 (x,y+1)-(x+1,y) in
// constraint order x-major / y / type (VtClothObjectGPU.hpp:75-116), bending of quad
// (x, y) over ((x,y), (x+1,y+1), (x,y+1), (x+1,y)) (:118-132), rest lengths
// |x0_i - x0_j| (the builder's values: registration verifies x == x0 at build time)
// and rest angles 0.  The rest lengths |x0_i - x0_j| of a generator's four constraints
// (grest) and a particle's LRA rest distances (glra, up to kGridLraCached slots) are
// evaluated once at registration with the same FP32 operations instead of every
// iteration: the kernels are bound by instruction issue, HBM is mostly idle.

// stretch_common on a difference diff = pa - pb and its length d computed by the caller.
__device__ __forceinline__ bool stretch_common_d(vec3 diff, float d, float wa, float wb, float rest, vec3& common)
{
    const float denom = wa + wb;
    if (!(d != rest && denom > 0)) return false;
    common = stretch_scale(diff, d, denom, rest);
    return true;
}

// bend_eval for the quad of a grid generator, p0 = (x,y), p1 = (x+1,y+1), p2 = (x,y+1),
// p3 = (x+1,y), given d3 = |p2 - p3|, the length the generator's stretch constraint t3
// already took: the shared edge e = p3 - p2 is its exact negation, so |e| = d3 bit for bit
// and its square root is not taken again.  Every other operation is bend_eval's, in its
// order, so the corrections are bend_eval's bits.
__device__ __forceinline__ void bend_eval_grid(float4 a0, float4 a1, float4 a2, float4 a3, float d3, float rest,
                                               float xpbd, float4& c0, float4& c1, float4& c2, float4& c3)
{
    const vec3 p0 = xyz(a0), p1 = xyz(a1), p2 = xyz(a2), p3 = xyz(a3);
    const float w0 = a0.w, w1 = a1.w, w2 = a2.w, w3 = a3.w;
    c0 = make_float4(0, 0, 0, 0);
    c1 = c0;
    c2 = c0;
    c3 = c0;
    const vec3 e = sub_p(p3, p2);
    const float elen = d3;
    if (elen < VT_EPSILON) return;
    const float inv = 1.0f / elen;
    // the angle chain in exact operations (vt_math.cuh: acos near a flat pair)
    const vec3 p20 = sub_p(p2, p0), p21 = sub_p(p2, p1);
    vec3 n1 = cross_exact(p20, sub_p(p3, p0));
    n1 = div_exact(n1, dot_exact(n1, n1));
    vec3 n2 = cross_exact(sub_p(p3, p1), p21);
    n2 = div_exact(n2, dot_exact(n2, n2));
    const vec3 d0 = mul_p(n1, elen);
    const vec3 d1 = mul_p(n2, elen);
    const vec3 d2 = madd_p(n2, dot(sub_p(p1, p3), e) * inv, mul_p(n1, dot(sub_p(p0, p3), e) * inv));
    const vec3 dd3 = madd_p(n2, dot(p21, e) * inv, mul_p(n1, dot(p20, e) * inv));
    n1 = normalize_exact(n1);
    n2 = normalize_exact(n2);
    const float phi = vt_acosf_exact(gclamp(dot_exact(n1, n2), -1.0f, 1.0f));
    float lambda = w0 * dot(d0, d0) + w1 * dot(d1, d1);
    lambda = lambda + w2 * dot(d2, d2);
    lambda = lambda + w3 * dot(dd3, dd3);
    if (lambda < VT_EPSILON) return;
    lambda = (phi - rest) / (lambda + xpbd);
    if (dot_exact(cross_exact(n1, n2), e) > 0.0f) lambda = -lambda;
    const vec3 k0 = mul_p(d0, -w0 * lambda), k1 = mul_p(d1, -w1 * lambda);
    const vec3 k2 = mul_p(d2, -w2 * lambda), k3 = mul_p(dd3, -w3 * lambda);
    c0 = make_float4(k0.x, k0.y, k0.z, 1.0f);
    c1 = make_float4(k1.x, k1.y, k1.z, 1.0f);
    c2 = make_float4(k2.x, k2.y, k2.z, 1.0f);
    c3 = make_float4(k3.x, k3.y, k3.z, 1.0f);
}

// Generator (X, Y) of a grid cloth of R x R quads: its stretch constraints t0..t3 (rests
// rest.x .. rest.w) and the bend of quad (X, Y), from the predicted position of (X, Y) at
// sp[hx][hy] and of (X,Y+1), (X+1,Y), (X+1,Y+1) beside it.  Each stretch result goes to
// sst[t][gx][gy] (lambda * gradient, w = 1 when it fired) and each bending corner to
// sbd[c][gx][gy]; a generator outside the cloth writes zeros.  The bend reuses t3's
// length (bend_eval_grid).
template <int kHB, int kGA, int kGB>
__device__ __forceinline__ void grid_generator(int X, int Y, int R, const float4 (*sp)[kHB], int hx, int hy,
                                               float4 (*sst)[kGA][kGB], float4 (*sbd)[kGA][kGB], int gx,
                                               int gy, float4 rest, float xpbd)
{
    const float4 zero = make_float4(0, 0, 0, 0);
    const bool gen = X >= 0 && Y >= 0 && X <= R && Y <= R;
    const bool full = gen && X < R && Y < R;
    const float4 pxy = sp[hx][hy];
    vec3 cm;
    float4 r = zero;
    if (gen && Y < R && stretch_common(pxy, sp[hx][hy + 1], rest.x, cm))  // t0: (x,y)-(x,y+1)
        r = make_float4(cm.x, cm.y, cm.z, 1.0f);
    sst[0][gx][gy] = r;
    r = zero;
    if (gen && X < R && stretch_common(pxy, sp[hx + 1][hy], rest.y, cm))  // t1: (x,y)-(x+1,y)
        r = make_float4(cm.x, cm.y, cm.z, 1.0f);
    sst[1][gx][gy] = r;
    r = zero;
    if (full && stretch_common(pxy, sp[hx + 1][hy + 1], rest.z, cm))  // t2: (x,y)-(x+1,y+1)
        r = make_float4(cm.x, cm.y, cm.z, 1.0f);
    sst[2][gx][gy] = r;
    r = zero;
    float d3 = 0.0f;
    if (full) {  // t3: (x,y+1)-(x+1,y); its length is the bend's shared-edge length
        const float4 a01 = sp[hx][hy + 1], a10 = sp[hx + 1][hy];
        const vec3 e3 = xyz(a01) - xyz(a10);
        d3 = length_exact(e3);
        if (stretch_common_d(e3, d3, a01.w, a10.w, rest.w, cm)) r = make_float4(cm.x, cm.y, cm.z, 1.0f);
    }
    sst[3][gx][gy] = r;
    float4 c0 = zero, c1 = zero, c2 = zero, c3 = zero;
    if (full)  // bend of quad (x, y): corners (x,y), (x+1,y+1), (x,y+1), (x+1,y)
        bend_eval_grid(pxy, sp[hx + 1][hy + 1], sp[hx][hy + 1], sp[hx + 1][hy], d3, 0.0f, xpbd, c0, c1, c2, c3);
    sbd[0][gx][gy] = c0;
    sbd[1][gx][gy] = c1;
    sbd[2][gx][gy] = c2;
    sbd[3][gx][gy] = c3;
}

// A stored constraint term s (its correction in xyz, 1 in w when it fired) taken into the
// particle's sums.  Fast build: (x, y) += s.xy * scale and (z, count) += (s.z * scale,
// s.w), two paired FMAs (sm_100 and later), the count summed in FP32 beside z (exact for
// counts this small).  Exact build: (x, y) by a paired product and scalar sums (a paired
// product feeding a paired sum would be fused by the code generator), z by a scalar
// product and sum, and the flag into the integer count — carrying the count in the
// paired sums (with the corners' below) ran slower there (mix 1.552e10 -> 1.538e10
// pit/s), while it took the fast build from 1.806e10 to 1.820e10.
__device__ __forceinline__ void take_term(float2& axy, float2& azc, int& cnt, float4 s, float scale)
{
#if VT_PAIRED && VT_FAST_DEVICE
    axy = __ffma2_rn(make_float2(s.x, s.y), make_float2(scale, scale), axy);
    azc = __ffma2_rn(make_float2(s.z, s.w), make_float2(scale, 1.0f), azc);
#elif VT_PAIRED
    const float2 p = __fmul2_rn(make_float2(s.x, s.y), make_float2(scale, scale));
    axy = make_float2(__fadd_rn(axy.x, p.x), __fadd_rn(axy.y, p.y));
    azc.x = __fadd_rn(azc.x, __fmul_rn(s.z, scale));
    cnt += s.w != 0.0f ? 1 : 0;
#else
    axy = make_float2(axy.x + s.x * scale, axy.y + s.y * scale);
    azc.x = azc.x + s.z * scale;
    cnt += s.w != 0.0f ? 1 : 0;
#endif
}
// A bending corner c (its correction in xyz, 1 in w when it fired): (x, y) += c.xy and,
// in the fast build, (z, count) += c.zw as one paired sum; the exact build adds z alone
// and the flag to the integer count (the paired form ran slower there, mix 1.558e10 ->
// 1.541e10 pit/s).
__device__ __forceinline__ void take_corner(float2& axy, float2& azc, int& cnt, float4 c)
{
#if VT_PAIRED && VT_FAST_DEVICE
    axy = __fadd2_rn(axy, make_float2(c.x, c.y));
    azc = __fadd2_rn(azc, make_float2(c.z, c.w));
#elif VT_PAIRED
    axy = __fadd2_rn(axy, make_float2(c.x, c.y));
    azc.x = __fadd_rn(azc.x, c.z);
    cnt += c.w != 0.0f ? 1 : 0;
#else
    axy = make_float2(axy.x + c.x, axy.y + c.y);
    azc.x = azc.x + c.z;
    cnt += c.w != 0.0f ? 1 : 0;
#endif
}

// The Jacobi sum of grid particle (a, b), i = its index: its eight stretch constraints,
// its LRA attachments in slot order, its four bending corners, all in constraint order.
// Generator (a, b)'s results sit at [gx][gy] of sst / sbd, generator (a-1, b-1)'s at
// [gx-1][gy-1].  gl: the particle's cached LRA rest distances, sslot: the cached slots;
// gbox / gsup: the slot groups' and super-groups' boxes (more slots than the cache holds),
// ngroups of gsize.
template <int kGA, int kGB>
__device__ __forceinline__ void grid_particle_sum(int a, int b, int R, int i, int gx, int gy,
                                                  const float4 (*sst)[kGA][kGB], const float4 (*sbd)[kGA][kGB],
                                                  vec3 pi, float wi, int ns, int s0, const float4* gl,
                                                  const float4* sslot, const float4* gbox, const float4* gsup,
                                                  int gsize, int ngroups,
                                                  const float4* __restrict__ x0, const float4* __restrict__ slots,
                                                  const float4* __restrict__ slots0, float lrs, vec3& acc,
                                                  int& cnt)
{
    const float nw = -wi;
    // Branch-free: a constraint that does not exist (outside the cloth) or did not fire is
    // stored as all zeros, so its term adds +-0, which leaves the sum's bits unchanged (the
    // sum starts at +0 and an exact IEEE sum is never -0).  Its w (1 when it fired, else 0)
    // is summed in FP32 beside z, so a term is two paired operations on (x, y) and
    // (z, count); counts this small are exact in FP32.
    float2 axy = make_float2(acc.x, acc.y), azc = make_float2(acc.z, 0.0f);
    // stretch, constraint order: generators (a-1,b-1) < (a-1,b) < (a,b-1) < (a,b)
    take_term(axy, azc, cnt, sst[2][gx - 1][gy - 1], wi);  // t2, second endpoint
    take_term(axy, azc, cnt, sst[1][gx - 1][gy], wi);      // t1, second endpoint
    take_term(axy, azc, cnt, sst[3][gx - 1][gy], wi);      // t3, second endpoint
    take_term(axy, azc, cnt, sst[0][gx][gy - 1], wi);      // t0, second endpoint
    take_term(axy, azc, cnt, sst[3][gx][gy - 1], nw);      // t3, first endpoint
    take_term(axy, azc, cnt, sst[0][gx][gy], nw);          // t0, first endpoint
    take_term(axy, azc, cnt, sst[1][gx][gy], nw);          // t1, first endpoint
    take_term(axy, azc, cnt, sst[2][gx][gy], nw);          // t2, first endpoint
    acc = mk3(axy.x, axy.y, azc.x);
    // long-range attachments, slot order; pairs that cannot fire skip their square roots
    if (ns) {
        if (ns <= kGridLraCached) {
            const float4 r4 = *gl;
            const float rs[4] = {r4.x, r4.y, r4.z, r4.w};
#pragma unroll
            for (int k = 0; k < kGridLraCached; ++k)
                if (k < ns) attach_one_filtered(pi, wi, xyz(sslot[k]), rs[k] * lrs, acc, cnt);
        } else {
            const vec3 x0i = xyz(x0[i]);
            const float c2 = (lrs * lrs) * kAttachMargin;
            const bool quiet_ok = wi != 0.0f && lrs > 1e-4f && lrs < 1e4f && in_bound_range(pi) && in_bound_range(x0i);
            for (int g0 = 0; g0 < ngroups; g0 += kLraSuper) {
                // a super-group, then each of its groups, skipped when no pair of it fires
                if (quiet_ok && lra_group_quiet(pi, x0i, gsup + 4 * (g0 / kLraSuper), c2)) continue;
                for (int g = g0; g < min(g0 + kLraSuper, ngroups); ++g) {
                    if (quiet_ok && lra_group_quiet(pi, x0i, gbox + 4 * g, c2)) continue;
                    const int sb = s0 + g * gsize, se = min(sb + gsize, s0 + ns);
                    // unrolled: the next slots' loads overlap this pair's arithmetic
#pragma unroll 4
                    for (int s = sb; s < se; ++s)
                        attach_lra_filtered(pi, wi, xyz(slots[s]), xyz(slots0[s]), x0i, lrs, c2, acc, cnt);
                }
            }
        }
    }
    // bending corners, constraint order: quads (a-1,b-1) < (a-1,b) < (a,b-1) < (a,b);
    // branch-free as the stretch terms above
    axy = make_float2(acc.x, acc.y);
    azc.x = acc.z;
    take_corner(axy, azc, cnt, sbd[1][gx - 1][gy - 1]);
    take_corner(axy, azc, cnt, sbd[3][gx - 1][gy]);
    take_corner(axy, azc, cnt, sbd[2][gx][gy - 1]);
    take_corner(axy, azc, cnt, sbd[0][gx][gy]);
    acc = mk3(axy.x, axy.y, azc.x);
    cnt += (int)azc.y;
}

// The tile kernel: a block owns a TA x TB tile; it stages the tile and a one-particle
// halo of predicted positions in shared memory, evaluates each of the (TA+1) x (TB+1)
// generators touching the tile once (one per thread: one bend + four stretch
// constraints), then each particle sums its results in constraint order — the order of
// the CSR kernel and of the oracle.
// The shared memory of one tile (TMA destinations 128-byte aligned); kX = 0 leaves out the
// positions the finalizing modes stage (plain iterations do not use them, and the
// smaller footprint lets five blocks share an SM).
template <int kTA, int kTB, int kX = 1>
struct GridSmem {
    static constexpr int kGHA = kTA + 2, kGHB = kTB + 2;  // halo tile
    static constexpr int kGGA = kTA + 1, kGGB = kTB + 1;  // generators, kGGA * kGGB == kBlock
    __align__(128) float4 sp[kGHA][kGHB];
    __align__(128) float4 sst[4][kGGA][kGGB];  // stretch common + fired flag, per type
    float4 sbd[4][kGGA][kGGB];                 // bending corner corrections + fired flag
    __align__(128) float4 sgl[kBlock];         // the particle's LRA rest distances, or the slot groups' boxes
    __align__(128) float4 sx[kX ? kBlock : 1];  // the particle's position (finalizing modes)
    __align__(16) DomainParams sdom;
    float4 sslot[kGridLraCached];
    float4 ssup[4 * (kLraGroupsMax / kLraSuper)];  // the slot super-groups' boxes
    uint64_t sbar;                                 // TMA completion barrier
};

// One tile's iteration, the body of k_grid_iter (and of each tile step of the cluster
// kernel), on the block's shared tile `S`.  Threads may return before the end; a caller
// that runs several tiles on one block separates them with __syncthreads.
template <int kMode, int kTA, int kTB, int kX>
__device__ __forceinline__ void grid_tile_iteration(GridSmem<kTA, kTB, kX>& S, const GridTile tl,
                                                    const DomainParams* __restrict__ doms,
                                                    const float4* __restrict__ pin, float4* __restrict__ pout,
                                                    float4* __restrict__ x, float4* __restrict__ v,
                                                    const float4* __restrict__ x0, const float4* __restrict__ grest,
                                                    const float4* __restrict__ glra, const float4* __restrict__ slots,
                                                    const float4* __restrict__ slots0, int32_t* __restrict__ status,
                                                    const CUtensorMap* __restrict__ tmaps, int pin_sel)
{
    constexpr int kGHA = kTA + 2, kGHB = kTB + 2;  // halo tile
    constexpr int kGGA = kTA + 1, kGGB = kTB + 1;  // generators, kGGA * kGGB == kBlock
    static_assert(kGGA * kGGB == kBlock, "one generator per thread");
    static_assert(sizeof(DomainParams) % 16 == 0, "DomainParams is staged in 16-byte pieces");
    static_assert(kX || kMode == SOLVE_PLAIN, "the finalizing modes stage positions");
    float4 (*const sp)[kGHB] = S.sp;
    float4 (*const sst)[kGGA][kGGB] = S.sst;
    float4 (*const sbd)[kGGA][kGGB] = S.sbd;
    float4* const sgl = S.sgl;
    float4* const sx = S.sx;
    float4* const sslot = S.sslot;
    float4* const ssup = S.ssup;
    uint64_t& sbar = S.sbar;
    DomainParams& sdom = S.sdom;
    // the generator's four stretch rest lengths are staged in sst[0] at the generator's own
    // slot (gx * kGGB + gy == tid): the thread reads them before it writes that slot
    float4* const sgr = &sst[0][0][0];
    const int tid = (int)threadIdx.x;
    const int R = tl.res, V = R + 1, base = tl.p_begin;
    const int ns = tl.slot_count, s0 = tl.slot_begin;
    const int a0 = tl.a0, b0 = tl.b0;
    const int gx = tid / kGGB, gy = tid - gx * kGGB;  // this thread's generator
    const int ta = tid / kTB, tb = tid - ta * kTB;    // this thread's particle
    const int a = a0 + ta, b = b0 + tb;
    const bool owns = tid < kTA * kTB && a < V && b < V;
    const int i = base + a * V + b;

    // 1. stage the halo tile of predicted positions, each generator's rests and each
    // particle's LRA rests and position: with TMA, four bulk tensor copies (rectangles of
    // the cloth's V x V grid, zero outside it) issued by one thread; otherwise one 16-byte
    // cp.async per element with zero-fill outside the cloth.  Then the LRA slots and the
    // domain's parameters (cp.async), and no registers held across the waits.
    const bool tma = tmaps != nullptr;
    const bool stage_lra = ns >= 1 && ns <= kGridLraCached;
    if (tma) {
        if (tid == 0) {  // the barrier is published to the block by the __syncthreads below
            mbar_init(&sbar, 1);
            const CUtensorMap* m = tmaps + tmap_index(tl.dom, tmap_shape_of(kTA), 0);
            const uint32_t bytes = 16u * (uint32_t)(kGHA * kGHB + kGGA * kGGB + (stage_lra ? kTA * kTB : 0) +
                                                   (kMode != SOLVE_PLAIN ? kTA * kTB : 0));
            mbar_expect_tx(&sbar, bytes);
            tma_load_3d(&sp[0][0], m + (pin_sel ? TMAP_P1 : TMAP_P0), 0, b0 - 1, a0 - 1, &sbar);
            tma_load_3d(sgr, m + TMAP_GREST, 0, b0 - 1, a0 - 1, &sbar);
            if (stage_lra) tma_load_3d(sgl, m + TMAP_GLRA, 0, b0, a0, &sbar);
            if (kMode != SOLVE_PLAIN) tma_load_3d(sx, m + TMAP_X, 0, b0, a0, &sbar);
        }
    } else {
        for (int k = tid; k < kGHA * kGHB; k += kBlock) {
            const int ha = k / kGHB, hb = k - ha * kGHB;
            const int pa = a0 - 1 + ha, pb = b0 - 1 + hb;
            const bool in = pa >= 0 && pa < V && pb >= 0 && pb < V;
            cp_async16_zfill(&sp[ha][hb], pin + (in ? base + pa * V + pb : base), in);
        }
        {
            const int X = a0 - 1 + gx, Y = b0 - 1 + gy;
            const bool gen = X >= 0 && Y >= 0 && X <= R && Y <= R;
            cp_async16_zfill(&sgr[tid], grest + (gen ? base + X * V + Y : base), gen);
        }
        if (owns && stage_lra) cp_async16(&sgl[tid], glra + i);
        if (kMode != SOLVE_PLAIN && owns) cp_async16(&sx[tid], x + i);
    }
    if (tid < ns && tid < kGridLraCached) cp_async16(&sslot[tid], slots + s0 + tid);
    if (tid < (int)(sizeof(DomainParams) / 16))
        cp_async16(reinterpret_cast<float4*>(&sdom) + tid, reinterpret_cast<const float4*>(doms + tl.dom) + tid);
    cp_async_wait_all();
    __syncthreads();
    if (tma && !mbar_wait(&sbar, 0)) {
        // the copies did not arrive in time: report it (the sync calls return
        // VT_ERR_TIMEOUT) and finish the block on whatever the tile holds, without a
        // barrier that the other threads might not reach
        atomicOr(status, VT_STATUS_TIMEOUT);
    }
#if VT_CHECKED
    if (tma) {  // the bounds-checked build compares the staged halo with the global array
        for (int k = tid; k < kGHA * kGHB; k += kBlock) {
            const int ha = k / kGHB, hb = k - ha * kGHB;
            const int pa = a0 - 1 + ha, pb = b0 - 1 + hb;
            const bool in = pa >= 0 && pa < V && pb >= 0 && pb < V;
            const float4 want = in ? pin[base + pa * V + pb] : make_float4(0, 0, 0, 0);
            const float4 got = sp[ha][hb];
            if (__float_as_uint(got.x) != __float_as_uint(want.x) || __float_as_uint(got.y) != __float_as_uint(want.y) ||
                __float_as_uint(got.z) != __float_as_uint(want.z) || __float_as_uint(got.w) != __float_as_uint(want.w))
                atomicOr(status, VT_STATUS_BOUNDS);
        }
    }
#endif
    const DomainParams& D = sdom;

    // 2. the slot groups' boxes when the cloth has more LRA slots than the cache holds
    // (sgl is free then), then the generators (x, y) = (a0 - 1 + gx, b0 - 1 + gy): one per
    // thread (the rests are read before sst[0][gx][gy], the same slot, is written)
    int gsize = 0, ngroups = 0;
    if (ns > kGridLraCached) {
        gsize = max(kLraGroupMin, (ns + kLraGroupsMax - 1) / kLraGroupsMax);
        ngroups = (ns + gsize - 1) / gsize;
        lra_group_boxes(sgl, ssup, slots + s0, slots0 + s0, ns, gsize, ngroups, tid);
    }
    grid_generator<kGHB, kGGA, kGGB>(a0 - 1 + gx, b0 - 1 + gy, R, sp, gx, gy, sst, sbd, gx, gy, sgr[tid],
                                     D.xpbd_bend);
    __syncthreads();

    // 3. particles of the tile
    if (!owns) return;
    if (!VT_IN_RANGE(i, D.p_begin, D.p_begin + D.p_count, status)) return;
    const int hx = ta + 1, hy = tb + 1;  // this particle's generator (a, b) and halo slot
    const float4 pi4 = sp[hx][hy];
    const vec3 pi = xyz(pi4);
    const float wi = pi4.w;
    vec3 acc = mk3(0, 0, 0);
    int cnt = 0;
    grid_particle_sum<kGGA, kGGB>(a, b, R, i, hx, hy, sst, sbd, pi, wi, ns, s0, &sgl[tid], sslot, sgl, ssup,
                                  gsize, ngroups, x0, slots, slots0, D.lrs, acc, cnt);
    apply_and_finalize<kMode>(D, tl.dom, i, pi, wi, acc, cnt, &sx[tid], pout, x, v, status);
}

template <int kMode, int kTA, int kTB, int kMinBlocks>
__global__ void __launch_bounds__(kBlock, kMinBlocks)
k_grid_iter(const GridTile* __restrict__ tiles, const DomainParams* __restrict__ doms,
            const float4* __restrict__ pin, float4* __restrict__ pout, float4* __restrict__ x,
            float4* __restrict__ v, const float4* __restrict__ x0, const float4* __restrict__ grest,
            const float4* __restrict__ glra, const float4* __restrict__ slots,
            const float4* __restrict__ slots0, int32_t* __restrict__ status,
            const CUtensorMap* __restrict__ tmaps, int pin_sel)
{
    constexpr int kX = kMode == SOLVE_PLAIN ? 0 : 1;
    __shared__ GridSmem<kTA, kTB, kX> S;
    grid_tile_iteration<kMode, kTA, kTB, kX>(S, tiles[blockIdx.x], doms, pin, pout, x, v, x0, grest, glra, slots,
                                             slots0, status, tmaps, pin_sel);
}

// ------------------------------------------------------------------ cluster-resident substep
// All Jacobi iterations of one substep of small grid cloths in one launch: a cluster of
// kClusterCtas blocks owns one cloth (tiles [first, end) of the tile table, block r of the
// cluster takes tiles first + r, first + r + kClusterCtas, ...) and runs the iterations
// in order, separated by the cluster's hardware barrier, whose release / acquire makes
// every block's positions of one iteration visible to the whole cluster before the next
// reads them.  No block waits on memory written by another cluster, and the launch's
// blocks of a cluster are co-scheduled by the hardware, so there is no spin-wait.  Each
// tile step is grid_tile_iteration (cp.async staging), so results are k_grid_iter's.
constexpr int kClusterCtas = 16;

__device__ __forceinline__ void cluster_barrier()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_arrive()
{
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_wait()
{
    asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

template <int kTA, int kTB>
__global__ void __launch_bounds__(kBlock, 1)
k_grid_substep_cluster(const GridTile* __restrict__ tiles, const int2* __restrict__ cloth_tiles,
                       const DomainParams* __restrict__ doms, float4* __restrict__ p0, float4* __restrict__ p1,
                       float4* __restrict__ x, float4* __restrict__ v, const float4* __restrict__ x0,
                       const float4* __restrict__ grest, const float4* __restrict__ glra,
                       const float4* __restrict__ slots, const float4* __restrict__ slots0,
                       int32_t* __restrict__ status, int pin0, int iterations, int last_substep)
{
    __shared__ GridSmem<kTA, kTB, 1> S;
    const int2 range = cloth_tiles[blockIdx.x / kClusterCtas];
    const int rank = (int)(blockIdx.x % kClusterCtas);
    int pin = pin0;
    for (int it = 0; it < iterations; ++it) {
        const float4* pi = pin ? p1 : p0;
        float4* po = pin ? p0 : p1;
        for (int t = range.x + rank; t < range.y; t += kClusterCtas) {
            __syncthreads();  // the previous tile step is done with the shared tile
            if (it + 1 < iterations)
                grid_tile_iteration<SOLVE_PLAIN, kTA, kTB, 1>(S, tiles[t], doms, pi, po, x, v, x0, grest, glra, slots,
                                                           slots0, status, nullptr, pin);
            else if (last_substep)
                grid_tile_iteration<SOLVE_FINALIZE, kTA, kTB, 1>(S, tiles[t], doms, pi, po, x, v, x0, grest, glra,
                                                              slots, slots0, status, nullptr, pin);
            else
                grid_tile_iteration<SOLVE_FINALIZE_PREDICT, kTA, kTB, 1>(S, tiles[t], doms, pi, po, x, v, x0, grest,
                                                                      glra, slots, slots0, status, nullptr, pin);
        }
        cluster_barrier();
        pin = 1 - pin;
    }
}

// Cluster-resident substep of a small grid cloth (up to 64 x 64 particles): a cluster of
// 16 blocks, one 16 x 16 tile each, keeps the cloth's predicted positions in shared
// memory for all of a substep's iterations.  Each block holds its tile plus a
// one-particle halo in two buffers (this iteration's and the next's); a particle's new
// position goes to its own block's next buffer and, on a tile edge, into the halo of the
// neighbouring blocks' next buffers through distributed shared memory; the cluster
// barrier (release / acquire) between iterations publishes those stores.  Global memory
// is read once per substep (positions, rests, attachments) and written once (the last
// iteration's finalize).  Generators and particle sums are the tile kernel's functions
// on the same values, so the results are its bits (the fast build included: the
// generator is the tile kernel's grid_generator, whole, so its contracted arithmetic is
// the same).  320 threads: 17 x 17 generators, 16 x 16 particles.
constexpr int kResT = 16;
constexpr int kResThreads = 320;
constexpr int kResHalo = kResT + 2, kResGen = kResT + 1;
static_assert(kResGen * kResGen <= kResThreads && kResT * kResT <= kResThreads, "threads cover the tile");
static_assert(kClusterCtas == 16, "a 4 x 4 grid of tiles");

struct ResidentSmem {
    float4 sp[2][kResHalo][kResHalo];           // positions: this iteration's, the next's
    float4 sst[4][kResGen][kResGen];            // stretch results, per type
    float4 sbd[4][kResGen][kResGen];            // bending corner corrections
    float4 sgr[kResGen * kResGen];              // generators' stretch rests (whole substep)
    float4 sgl[kResT * kResT];                  // LRA rests, or the slot groups' boxes
    float4 sx[kResT * kResT];                   // positions at the substep's start
    float4 sslot[kGridLraCached];
    float4 ssup[4 * (kLraGroupsMax / kLraSuper)];
    __align__(16) DomainParams sdom;
};

__device__ __forceinline__ void st_cluster_f4(const float4* local, uint32_t rank, float4 v)
{
    const uint32_t la = (uint32_t)__cvta_generic_to_shared(local);
    uint32_t ra;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(la), "r"(rank));
    asm volatile("st.shared::cluster.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(ra), "f"(v.x), "f"(v.y), "f"(v.z),
                 "f"(v.w)
                 : "memory");
}

__global__ void __launch_bounds__(kResThreads, 1)
k_grid_substep_resident(const int2* __restrict__ cloth_dom, const DomainParams* __restrict__ doms,
                        float4* __restrict__ p0, float4* __restrict__ p1, float4* __restrict__ x,
                        float4* __restrict__ v, const float4* __restrict__ x0, const float4* __restrict__ grest,
                        const float4* __restrict__ glra, const float4* __restrict__ slots,
                        const float4* __restrict__ slots0, int32_t* __restrict__ status, int pin0,
                        int iterations, int last_substep)
{
    extern __shared__ __align__(128) unsigned char res_smem[];
    ResidentSmem& S = *reinterpret_cast<ResidentSmem*>(res_smem);
    const int dom = cloth_dom[blockIdx.x / kClusterCtas].x;
    const int rank = (int)(blockIdx.x % kClusterCtas);  // the block's rank in its 1-D cluster
    const int tid = (int)threadIdx.x;
    if (tid < (int)(sizeof(DomainParams) / 16))
        cp_async16(reinterpret_cast<float4*>(&S.sdom) + tid, reinterpret_cast<const float4*>(doms + dom) + tid);
    cp_async_wait_all();
    __syncthreads();
    const DomainParams& D = S.sdom;
    const int R = D.grid_res, V = R + 1, base = D.p_begin;
    const int rt = rank >> 2, rc = rank & 3;            // the block's tile in the 4 x 4 grid
    const int a0 = kResT * rt, b0 = kResT * rc;
    const bool active = a0 < V && b0 < V;
    const int ns = D.grid_slot_count, s0 = D.grid_slot_begin;
    // generators (a0 - 1 + gx, b0 - 1 + gy): the 15 x 15 interior ones (no halo position
    // read) first, then the 64 on the border; warps whose generators are all interior
    // compute before waiting for the neighbours' halo stores
    const int g = tid;
    constexpr int kInner = (kResGen - 2) * (kResGen - 2);
    int gx, gy;
    if (g < kInner) {
        gx = 1 + g / (kResGen - 2);
        gy = 1 + g % (kResGen - 2);
    } else {
        const int e = g - kInner;  // row 0, row 16, column 0, column 16
        if (e < kResGen) {
            gx = 0;
            gy = e;
        } else if (e < 2 * kResGen) {
            gx = kResGen - 1;
            gy = e - kResGen;
        } else if (e < 2 * kResGen + (kResGen - 2)) {
            gx = 1 + e - 2 * kResGen;
            gy = 0;
        } else {
            gx = 1 + e - 2 * kResGen - (kResGen - 2);
            gy = kResGen - 1;
        }
    }
    const bool has_gen = g < kResGen * kResGen;
    const bool inner_warp = (tid >> 5) * 32 + 31 < kInner;
    const int ta = tid / kResT, tb = tid - ta * kResT;     // particle (a0 + ta, b0 + tb)
    const int a = a0 + ta, b = b0 + tb;
    const int i = base + a * V + b;
    // a thread never leaves before the end: every thread takes part in the cluster barriers
    const bool owns = active && tid < kResT * kResT && a < V && b < V &&
                      VT_IN_RANGE(i, D.p_begin, D.p_begin + D.p_count, status);
    const float4* pin = pin0 ? p1 : p0;
    const bool stage_lra = ns >= 1 && ns <= kGridLraCached;

    // stage the tile and halo (zero outside the cloth; the next buffer's halo starts at
    // zero and stays so outside the cloth), the rests, the attachments and x
    if (active) {
        for (int k = tid; k < kResHalo * kResHalo; k += kResThreads) {
            const int ha = k / kResHalo, hb = k - ha * kResHalo;
            const int pa = a0 - 1 + ha, pb = b0 - 1 + hb;
            const bool in = pa >= 0 && pa < V && pb >= 0 && pb < V;
            cp_async16_zfill(&S.sp[0][ha][hb], pin + (in ? base + pa * V + pb : base), in);
            S.sp[1][ha][hb] = make_float4(0, 0, 0, 0);
        }
        if (has_gen) {
            const int X = a0 - 1 + gx, Y = b0 - 1 + gy;
            const bool gen = X >= 0 && Y >= 0 && X <= R && Y <= R;
            cp_async16_zfill(&S.sgr[g], grest + (gen ? base + X * V + Y : base), gen);
        }
        if (owns && stage_lra) cp_async16(&S.sgl[tid], glra + i);
        if (owns) cp_async16(&S.sx[tid], x + i);
        if (tid < ns && tid < kGridLraCached) cp_async16(&S.sslot[tid], slots + s0 + tid);
    }
    cp_async_wait_all();
    __syncthreads();
    int gsize = 0, ngroups = 0;
    if (active && ns > kGridLraCached) {
        gsize = max(kLraGroupMin, (ns + kLraGroupsMax - 1) / kLraGroupsMax);
        ngroups = (ns + gsize - 1) / gsize;
        lra_group_boxes(S.sgl, S.ssup, slots + s0, slots0 + s0, ns, gsize, ngroups, tid);
    }
    // every block's next buffer is cleared before any neighbour stores into it
    cluster_barrier();

    int pc = pin0;
    for (int it = 0; it < iterations; ++it) {
        const int cur = it & 1;
        // the previous iteration's halo stores are published by the cluster barrier it
        // arrived at; interior generators read only this block's positions
        if (it > 0 && !inner_warp) cluster_wait();
        if (active && has_gen)
            grid_generator<kResHalo, kResGen, kResGen>(a0 - 1 + gx, b0 - 1 + gy, R, S.sp[cur], gx, gy, S.sst,
                                                       S.sbd, gx, gy, S.sgr[g], D.xpbd_bend);
        if (it > 0 && inner_warp) cluster_wait();
        __syncthreads();
        if (owns) {
            const int hx = ta + 1, hy = tb + 1;
            const float4 pi4 = S.sp[cur][hx][hy];
            const vec3 pi = xyz(pi4);
            const float wi = pi4.w;
            vec3 acc = mk3(0, 0, 0);
            int cnt = 0;
            grid_particle_sum<kResGen, kResGen>(a, b, R, i, hx, hy, S.sst, S.sbd, pi, wi, ns, s0, &S.sgl[tid],
                                                S.sslot, S.sgl, S.ssup, gsize, ngroups, x0, slots, slots0, D.lrs,
                                                acc, cnt);
            if (it + 1 < iterations) {
                const vec3 np = jacobi_apply(D, pi, acc, cnt);
                const float4 q = make_float4(np.x, np.y, np.z, wi);
                const int nx = cur ^ 1;
                S.sp[nx][hx][hy] = q;
                // edge particles into the halos of the neighbouring tiles (which exist:
                // the halo particle a0 - 1 etc. lies in the cloth)
                const bool up = ta == 0 && rt > 0, down = ta == kResT - 1 && rt < 3;
                const bool left = tb == 0 && rc > 0, right = tb == kResT - 1 && rc < 3;
                if (up) st_cluster_f4(&S.sp[nx][kResT + 1][hy], (uint32_t)(rank - 4), q);
                if (down) st_cluster_f4(&S.sp[nx][0][hy], (uint32_t)(rank + 4), q);
                if (left) st_cluster_f4(&S.sp[nx][hx][kResT + 1], (uint32_t)(rank - 1), q);
                if (right) st_cluster_f4(&S.sp[nx][hx][0], (uint32_t)(rank + 1), q);
                if (up && left) st_cluster_f4(&S.sp[nx][kResT + 1][kResT + 1], (uint32_t)(rank - 5), q);
                if (up && right) st_cluster_f4(&S.sp[nx][kResT + 1][0], (uint32_t)(rank - 3), q);
                if (down && left) st_cluster_f4(&S.sp[nx][0][kResT + 1], (uint32_t)(rank + 3), q);
                if (down && right) st_cluster_f4(&S.sp[nx][0][0], (uint32_t)(rank + 5), q);
            } else {
                float4* po = pc ? p0 : p1;  // this iteration's output buffer
                if (last_substep)
                    apply_and_finalize<SOLVE_FINALIZE>(D, dom, i, pi, wi, acc, cnt, &S.sx[tid], po, x, v, status);
                else
                    apply_and_finalize<SOLVE_FINALIZE_PREDICT>(D, dom, i, pi, wi, acc, cnt, &S.sx[tid], po, x, v,
                                                               status);
            }
        }
        if (it + 1 < iterations) {
            cluster_arrive();  // after this thread's halo stores (release)
            __syncthreads();   // the sums have read sst / sbd and written this block's positions
        }
        pc ^= 1;
    }
}

template <int kPredict>
__global__ void __launch_bounds__(kBlock)
k_finalize(const Tile* __restrict__ tiles, const DomainParams* __restrict__ doms,
           float4* __restrict__ p, float4* __restrict__ x, float4* __restrict__ v,
           int32_t* __restrict__ status)
{
    const Tile tl = tiles[blockIdx.x];
    const int i = tl.begin + (int)threadIdx.x;
    if (i >= tl.end) return;
    const DomainParams& D = doms[tl.dom];
    const float dt = D.dt_sub;
    const float4 x4 = x[i];
    const vec3 xi = xyz(x4);
    vec3 pi = xyz(p[i]);
    vec3 np = pi;
    vec3 rv = (np - xi) / dt;
    const float rl = length_exact(rv);
    if (rl > D.max_speed) {
        rv = (rv / rl) * D.max_speed;
        np = xi + rv * dt;
    }
    vec3 vn = rv * (1.0f - D.damping * dt);
    flag_nonfinite(status, D, tl.dom, np);
    x[i] = make_float4(np.x, np.y, np.z, x4.w);
    if (kPredict) {
        vn = vn + mk3(D.gx, D.gy, D.gz) * dt;
        pi = np + vn * dt;
    }
    v[i] = make_float4(vn.x, vn.y, vn.z, 0.0f);
    p[i] = make_float4(pi.x, pi.y, pi.z, x4.w);
}

// ------------------------------------------------------------------ normals
// ComputeTriangleNormals + ComputeVertexNormals (:419-465) as a per-vertex gather over
// incident triangles in triangle order.
__global__ void __launch_bounds__(kBlock)
k_normals(const Tile* __restrict__ tiles, const float4* __restrict__ x,
          const uint4* __restrict__ tri, const int32_t* __restrict__ tn_off,
          const int32_t* __restrict__ tn_ent, float4* __restrict__ nrm)
{
    const Tile tl = tiles[blockIdx.x];
    const int i = tl.begin + (int)threadIdx.x;
    if (i >= tl.end) return;
    vec3 acc = mk3(0, 0, 0);
    const int e0 = tn_off[i], e1 = tn_off[i + 1];
    for (int e = e0; e < e1; ++e) {
        const uint4 t = tri[tn_ent[e]];
        const vec3 p1 = xyz(x[t.x]), p2 = xyz(x[t.y]), p3 = xyz(x[t.z]);
        acc3(acc, cross(p2 - p1, p3 - p1));
    }
    const vec3 n = normalize(acc);
    nrm[i] = make_float4(n.x, n.y, n.z, 0.0f);
}

// Normals of a grid cloth with GenerateClothMesh's triangles, enumerated implicitly:
// quad (x, y) holds triangles 2q = ((x,y), (x+1,y), (x,y+1)) and 2q+1 = ((x,y+1),
// (x+1,y), (x+1,y+1)), q = x*R + y (Velvet/Scene.hpp:153-165).  Vertex (a, b) sums its
// incident triangles in triangle order — (a-1,b-1).1, (a-1,b).0, (a-1,b).1, (a,b-1).0,
// (a,b-1).1, (a,b).0 — as the CSR kernel and the reference's serialised atomics do.
__global__ void __launch_bounds__(kBlock)
k_grid_normals(const Tile* __restrict__ tiles, const DomainParams* __restrict__ doms,
               const float4* __restrict__ x, float4* __restrict__ nrm)
{
    const Tile tl = tiles[blockIdx.x];
    const int i = tl.begin + (int)threadIdx.x;
    if (i >= tl.end) return;
    const DomainParams& D = doms[tl.dom];
    const int R = D.grid_res, V = R + 1, base = D.p_begin;
    const int li = i - base, a = li / V, b = li - a * V;
    auto P = [&](int aa, int bb) { return xyz(x[base + aa * V + bb]); };
    auto tri_n = [&](int a1, int b1, int a2, int b2, int a3, int b3) {
        const vec3 p1 = P(a1, b1), p2 = P(a2, b2), p3 = P(a3, b3);
        return cross(p2 - p1, p3 - p1);
    };
    vec3 acc = mk3(0, 0, 0);
    if (a >= 1 && b >= 1) acc3(acc, tri_n(a - 1, b, a, b - 1, a, b));              // (a-1,b-1).1
    if (a >= 1 && b < R) {
        acc3(acc, tri_n(a - 1, b, a, b, a - 1, b + 1));                               // (a-1,b).0
        acc3(acc, tri_n(a - 1, b + 1, a, b, a, b + 1));                               // (a-1,b).1
    }
    if (a < R && b >= 1) {
        acc3(acc, tri_n(a, b - 1, a + 1, b - 1, a, b));                               // (a,b-1).0
        acc3(acc, tri_n(a, b, a + 1, b - 1, a + 1, b));                               // (a,b-1).1
    }
    if (a < R && b < R) acc3(acc, tri_n(a, b, a + 1, b, a, b + 1));                 // (a,b).0
    const vec3 n = normalize(acc);
    nrm[i] = make_float4(n.x, n.y, n.z, 0.0f);
}

// ------------------------------------------------------------------ read-back packing
__global__ void __launch_bounds__(kBlock) k_pack_xyz(const float4* __restrict__ src, float* __restrict__ dst,
                                                      int64_t n)
{
    const int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x;
    if (i >= n) return;
    const float4 q = src[i];
    dst[3 * i] = q.x;
    dst[3 * i + 1] = q.y;
    dst[3 * i + 2] = q.z;
}

cudaError_t launch_pack_xyz(const float4* src, float* dst, int64_t n, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    k_pack_xyz<<<(unsigned)((n + kBlock - 1) / kBlock), kBlock, 0, st>>>(src, dst, n);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ launchers
cudaError_t launch_presdf_predict(const Launch& L, int pcur)
{
    if (!L.n_ptiles) return cudaSuccess;
    const DeviceArrays& d = *L.d;
    k_presdf_predict<<<L.n_ptiles, kBlock, 0, L.st>>>(d.ptiles, d.dom, d.col, d.x, d.v, d.p[pcur]);
    return cudaGetLastError();
}

cudaError_t launch_collide(const Launch& L, int pin, int pout)
{
    if (!L.n_ptiles) return cudaSuccess;
    const DeviceArrays& d = *L.d;
    k_collide<<<L.n_ptiles, kBlock, 0, L.st>>>(d.ptiles, d.dom, d.col, d.x, d.p[pin], d.p[pout], d.nbr, d.status);
    return cudaGetLastError();
}

cudaError_t launch_bend(const Launch& L, int pin)
{
    if (!L.n_btiles) return cudaSuccess;
    const DeviceArrays& d = *L.d;
    k_bend<<<L.n_btiles, kBlock, 0, L.st>>>(d.btiles, d.dom, d.p[pin], d.bd_idx, d.bd_rest, d.bd_corr);
    return cudaGetLastError();
}

cudaError_t launch_solve(const Launch& L, int pin, int pout, int mode)
{
    if (!L.n_stiles) return cudaSuccess;
    const DeviceArrays& d = *L.d;
#define VT_SOLVE_ARGS                                                                      \
    d.stiles, d.dom, d.p[pin], d.p[pout], d.x, d.v, d.x0, d.st_off, d.st_ent, d.at_off,    \
        d.at_ent, d.lra, d.slots, d.slots0, d.bd_off, d.bd_ent, d.bd_corr, d.status
    if (mode == SOLVE_PLAIN)
        k_solve<SOLVE_PLAIN><<<L.n_stiles, kBlock, 0, L.st>>>(VT_SOLVE_ARGS);
    else if (mode == SOLVE_FINALIZE)
        k_solve<SOLVE_FINALIZE><<<L.n_stiles, kBlock, 0, L.st>>>(VT_SOLVE_ARGS);
    else
        k_solve<SOLVE_FINALIZE_PREDICT><<<L.n_stiles, kBlock, 0, L.st>>>(VT_SOLVE_ARGS);
#undef VT_SOLVE_ARGS
    return cudaGetLastError();
}

template <typename K>
static cudaError_t carveout(K kernel)
{
    return cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
}

// every (mode, occupancy) instance variant v launches
template <int v>
static cudaError_t carveout_variant()
{
    constexpr GridVariant g = kGridVariant[v];
    cudaError_t e = carveout(k_grid_iter<SOLVE_PLAIN, g.ta, g.tb, g.blocks>);
    if (e == cudaSuccess) e = carveout(k_grid_iter<SOLVE_FINALIZE, g.ta, g.tb, 4>);
    if (e == cudaSuccess) e = carveout(k_grid_iter<SOLVE_FINALIZE_PREDICT, g.ta, g.tb, 4>);
    return e;
}

template <int... V>
static cudaError_t carveout_all(std::integer_sequence<int, V...>)
{
    cudaError_t e = cudaSuccess;
    ((e = e == cudaSuccess ? carveout_variant<V>() : e), ...);
    return e;
}

cudaError_t prepare_kernels()
{
    // most shared memory per SM for the tile kernel: more resident tiles per SM
    return carveout_all(std::make_integer_sequence<int, kGridVariants>{});
}

// The plain iterations (nine in ten launches) use the variant's occupancy; the finalizing
// ones always the four-block build.
template <int v>
static void grid_iter_variant(const Launch& L, int pin, int pout, int mode)
{
    constexpr GridVariant g = kGridVariant[v];
    const DeviceArrays& d = *L.d;
    const CUtensorMap* tm = tile_loads_tma() ? d.tmaps : nullptr;
#define VT_GRID_ARGS \
    d.gtiles, d.dom, d.p[pin], d.p[pout], d.x, d.v, d.x0, d.grest, d.glra, d.slots, d.slots0, d.status, tm, pin
    if (mode == SOLVE_PLAIN)
        k_grid_iter<SOLVE_PLAIN, g.ta, g.tb, g.blocks><<<L.n_gtiles, kBlock, 0, L.st>>>(VT_GRID_ARGS);
    else if (mode == SOLVE_FINALIZE)
        k_grid_iter<SOLVE_FINALIZE, g.ta, g.tb, 4><<<L.n_gtiles, kBlock, 0, L.st>>>(VT_GRID_ARGS);
    else
        k_grid_iter<SOLVE_FINALIZE_PREDICT, g.ta, g.tb, 4><<<L.n_gtiles, kBlock, 0, L.st>>>(VT_GRID_ARGS);
#undef VT_GRID_ARGS
}

template <int... V>
static void grid_iter_dispatch(const Launch& L, int pin, int pout, int mode, std::integer_sequence<int, V...>)
{
    ((L.grid_variant == V ? grid_iter_variant<V>(L, pin, pout, mode) : void()), ...);
}

cudaError_t launch_grid_iter(const Launch& L, int pin, int pout, int mode)
{
    if (!L.n_gtiles) return cudaSuccess;
    if (L.grid_variant < 0 || L.grid_variant >= kGridVariants) return cudaErrorInvalidValue;
    grid_iter_dispatch(L, pin, pout, mode, std::make_integer_sequence<int, kGridVariants>{});
    return cudaGetLastError();
}

// The substep's iterations through k_grid_substep_cluster: one cluster per grid cloth,
// cloth_tiles[c] = its tile range in the tile table of the current variant.
template <int v>
static cudaError_t substep_cluster_variant(const Launch& L, const int2* cloth_tiles, int n_cloths, int pin,
                                           int iterations, int last_sub)
{
    constexpr GridVariant g = kGridVariant[v];
    const DeviceArrays& d = *L.d;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)(kClusterCtas * n_cloths));
    cfg.blockDim = dim3(kBlock);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = L.st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = kClusterCtas;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_grid_substep_cluster<g.ta, g.tb>, d.gtiles, cloth_tiles, d.dom, d.p[0],
                              d.p[1], d.x, d.v, d.x0, d.grest, d.glra, d.slots, d.slots0, d.status, pin, iterations,
                              last_sub);
}

template <int... V>
static cudaError_t substep_cluster_dispatch(const Launch& L, const int2* ct, int n, int pin, int its, int last,
                                            std::integer_sequence<int, V...>)
{
    cudaError_t e = cudaErrorInvalidValue;
    ((L.grid_variant == V ? (void)(e = substep_cluster_variant<V>(L, ct, n, pin, its, last)) : void()), ...);
    return e;
}

cudaError_t launch_grid_substep_cluster(const Launch& L, const int2* cloth_tiles, int n_cloths, int pin,
                                        int iterations, int last_sub)
{
    if (!L.n_gtiles || n_cloths <= 0 || iterations <= 0) return cudaSuccess;
    if (L.grid_variant < 0 || L.grid_variant >= kGridVariants) return cudaErrorInvalidValue;
    return substep_cluster_dispatch(L, cloth_tiles, n_cloths, pin, iterations, last_sub,
                                    std::make_integer_sequence<int, kGridVariants>{});
}

// How many clusters of kClusterCtas blocks of the substep kernel this device holds at once
// (0: none; a non-portable size needs the kernel attribute and a GPC with that many free
// SMs).
template <int TA, int TB>
static int cluster_kernel_capacity()
{
    auto k = k_grid_substep_cluster<TA, TB>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) return 0;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(kClusterCtas);
    cfg.blockDim = dim3(kBlock);
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = kClusterCtas;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int n = 0;
    return cudaOccupancyMaxActiveClusters(&n, k, &cfg) == cudaSuccess ? n : 0;
}

int substep_cluster_capacity()
{
    static int cap = -1;
    if (cap < 0) {
        cap = std::min(cluster_kernel_capacity<7, 31>(),
                       std::min(cluster_kernel_capacity<15, 15>(), cluster_kernel_capacity<3, 63>()));
        (void)cudaGetLastError();  // a refused query leaves no sticky error
    }
    return cap;
}

static cudaLaunchConfig_t resident_config(const Launch& L, int n_cloths, cudaLaunchAttribute* at)
{
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)(kClusterCtas * n_cloths));
    cfg.blockDim = dim3(kResThreads);
    cfg.dynamicSmemBytes = sizeof(ResidentSmem);
    cfg.stream = L.st;
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = kClusterCtas;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cfg;
}

cudaError_t launch_grid_substep_resident(const Launch& L, const int2* cloth_dom, int n_cloths, int pin,
                                         int iterations, int last_sub)
{
    if (n_cloths <= 0 || iterations <= 0) return cudaSuccess;
    const DeviceArrays& d = *L.d;
    cudaLaunchAttribute at[1];
    const cudaLaunchConfig_t cfg = resident_config(L, n_cloths, at);
    return cudaLaunchKernelEx(&cfg, k_grid_substep_resident, cloth_dom, (const DomainParams*)d.dom, d.p[0], d.p[1],
                              d.x, d.v, (const float4*)d.x0, (const float4*)d.grest, (const float4*)d.glra,
                              (const float4*)d.slots, (const float4*)d.slots0, d.status, pin, iterations, last_sub);
}

int substep_resident_capacity()
{
    static int cap = -1;
    if (cap < 0) {
        auto k = k_grid_substep_resident;
        int n = 0;
        if (cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess &&
            cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(ResidentSmem)) ==
                cudaSuccess) {
            Launch L{};
            cudaLaunchAttribute at[1];
            const cudaLaunchConfig_t cfg = resident_config(L, 1, at);
            if (cudaOccupancyMaxActiveClusters(&n, k, &cfg) != cudaSuccess) n = 0;
        }
        cap = n;
        (void)cudaGetLastError();  // a refused query leaves no sticky error
    }
    return cap;
}

cudaError_t launch_finalize(const Launch& L, int pcur, int predict_next)
{
    if (!L.n_ptiles) return cudaSuccess;
    const DeviceArrays& d = *L.d;
    if (predict_next)
        k_finalize<1><<<L.n_ptiles, kBlock, 0, L.st>>>(d.ptiles, d.dom, d.p[pcur], d.x, d.v, d.status);
    else
        k_finalize<0><<<L.n_ptiles, kBlock, 0, L.st>>>(d.ptiles, d.dom, d.p[pcur], d.x, d.v, d.status);
    return cudaGetLastError();
}

cudaError_t launch_normals(const Launch& L)
{
    const DeviceArrays& d = *L.d;
    if (L.n_stiles) k_normals<<<L.n_stiles, kBlock, 0, L.st>>>(d.stiles, d.x, d.tri, d.tn_off, d.tn_ent, d.nrm);
    if (L.n_gptiles) k_grid_normals<<<L.n_gptiles, kBlock, 0, L.st>>>(d.gptiles, d.dom, d.x, d.nrm);
    return cudaGetLastError();
}

}  // namespace vt
