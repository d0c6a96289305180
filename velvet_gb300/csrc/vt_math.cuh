// vt_math.cuh — FP32 vector arithmetic of the cloth solver, in the association order of
// glm (the vector library of the reference solver, Velvet/VtClothSolverGPU.cu):
//   dot(a, b)      = (a.x*b.x + a.y*b.y) + a.z*b.z
//   length(v)      = sqrt(dot(v, v))
//   normalize(v)   = v * (1 / sqrt(dot(v, v)))
//   mat4 * vec4    = (c0*x + c1*y) + (c2*z + c3*w)
//   mat3 * vec3    = (c0*x + c1*y) + c2*z
// The exact build compiles the translation units that include this file with
// -fmad=false, so no multiply-add pair is contracted into an FMA: every result is the
// IEEE-rounded value of the operations as written, on the device and in host code alike.
// The fast build (VT_FAST, device code only) divides a vector by one reciprocal and takes
// normalize's reciprocal square root in one step; with its compiler flags (contraction,
// approximate division and square root) its results are within the solver's stated
// tolerance of the exact ones, not equal to them.  Its threshold distances and its
// bending-angle chain keep the exact build's operations (dot_exact ... vt_acosf_exact).
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#define VT_HD __host__ __device__ __forceinline__
#define VT_EPSILON 1e-6f  // EPSILON, Velvet/Common.cuh:12

#if defined(VT_FAST) && defined(__CUDA_ARCH__)
#define VT_FAST_DEVICE 1
#else
#define VT_FAST_DEVICE 0
#endif
// device code for sm_100 and later: paired FP32 arithmetic (sub_p, mul_p, madd_p below)
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
#define VT_PAIRED 1
#else
#define VT_PAIRED 0
#endif

struct vec3 {
    float x, y, z;
};

VT_HD vec3 mk3(float x, float y, float z) { vec3 r; r.x = x; r.y = y; r.z = z; return r; }
VT_HD vec3 xyz(float4 a) { return mk3(a.x, a.y, a.z); }
VT_HD vec3 operator+(vec3 a, vec3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
VT_HD vec3 operator-(vec3 a, vec3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
VT_HD vec3 operator-(vec3 a) { return mk3(-a.x, -a.y, -a.z); }
VT_HD vec3 operator*(vec3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
VT_HD vec3 operator/(vec3 a, float s)
{
#if VT_FAST_DEVICE && VT_PAIRED
    const float r = 1.0f / s;
    const float2 q = __fmul2_rn(make_float2(a.x, a.y), make_float2(r, r));
    return mk3(q.x, q.y, a.z * r);
#elif VT_FAST_DEVICE
    const float r = 1.0f / s;
    return mk3(a.x * r, a.y * r, a.z * r);
#else
    return mk3(a.x / s, a.y / s, a.z / s);
#endif
}
VT_HD vec3 cmul(vec3 a, vec3 b) { return mk3(a.x * b.x, a.y * b.y, a.z * b.z); }
VT_HD float dot(vec3 a, vec3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
VT_HD float length(vec3 a) { return sqrtf(dot(a, a)); }
VT_HD vec3 normalize(vec3 a)
{
#if VT_FAST_DEVICE
    return a * rsqrtf(dot(a, a));
#else
    return a * (1.0f / sqrtf(dot(a, a)));
#endif
}
// The squared distance and distance a threshold decision is taken on (a stretch
// constraint at its rest length, an attachment beyond its target, a contact closer than
// the particle diameter, a particle inside a sphere).  Such a decision changes the count
// the Jacobi update is averaged over, so the fast build takes these values with the exact
// build's operations — IEEE products, sums and square root, no contraction — and fires a
// constraint exactly when the exact build does on the same positions; only the
// corrections themselves use the fast arithmetic.
VT_HD float dot_exact(vec3 a, vec3 b)
{
#if VT_PAIRED
    // the x and y products as one paired multiply, rounded as two
    const float2 xy = __fmul2_rn(make_float2(a.x, a.y), make_float2(b.x, b.y));
    return __fadd_rn(__fadd_rn(xy.x, xy.y), __fmul_rn(a.z, b.z));
#elif VT_FAST_DEVICE
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
#else
    return dot(a, b);
#endif
}
VT_HD float sqrt_exact(float q)
{
#if VT_FAST_DEVICE
    return __fsqrt_rn(q);
#else
    return sqrtf(q);
#endif
}
VT_HD float length_exact(vec3 a) { return sqrt_exact(dot_exact(a, a)); }
VT_HD vec3 cross(vec3 a, vec3 b)
{
    return mk3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
// The dihedral angle of a bending constraint is acos of a dot product of unit normals;
// for a nearly flat pair the dot is within a few ulps of 1, where acos magnifies each ulp
// of it ~1e4-fold.  The fast build therefore takes the whole chain — the two normals, their
// scaling and normalisation, the dot, acos and the sign test — with the exact build's
// operations, so the angle has the exact build's bits on the same positions.
VT_HD vec3 cross_exact(vec3 a, vec3 b)
{
#if VT_FAST_DEVICE
    return mk3(__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(b.y, a.z)), __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(b.z, a.x)),
               __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(b.x, a.y)));
#else
    return cross(a, b);
#endif
}
VT_HD vec3 div_exact(vec3 a, float s)
{
#if VT_FAST_DEVICE
    return mk3(__fdiv_rn(a.x, s), __fdiv_rn(a.y, s), __fdiv_rn(a.z, s));
#else
    return mk3(a.x / s, a.y / s, a.z / s);
#endif
}
VT_HD vec3 normalize_exact(vec3 a)
{
#if VT_FAST_DEVICE
    const float r = __fdiv_rn(1.0f, __fsqrt_rn(dot_exact(a, a)));
    return mk3(__fmul_rn(a.x, r), __fmul_rn(a.y, r), __fmul_rn(a.z, r));
#else
    return a * (1.0f / sqrtf(dot(a, a)));
#endif
}
// glm::clamp: min(max(x, lo), hi) with glm's ternary min / max (NaN passes through)
VT_HD float gclamp(float x, float lo, float hi)
{
    float m = (x < lo) ? lo : x;
    return (hi < m) ? hi : m;
}
VT_HD void acc3(vec3& a, vec3 b)
{
    a.x = a.x + b.x;
    a.y = a.y + b.y;
    a.z = a.z + b.z;
}

// Paired FP32 arithmetic.  sm_100 and later issue the x and y halves of a vector add,
// multiply or fused multiply-add as one instruction (__fadd2_rn, __fmul2_rn, __ffma2_rn),
// each half rounded as the scalar operation is, so a paired form has its scalar form's
// bits.  The hot vector operations of the Jacobi iteration use these forms; host code
// takes the scalar ones.  Where the scalar form is a product followed by a sum, the fast
// build fuses them (__ffma2_rn), as its contraction would; the exact build must round
// both, and a paired product feeding a paired sum is fused into one paired FMA by the
// code generator even without contraction (-fmad=false) and with the PTX .rn forms
// (measured on sm_103a: 43% of uniform random operands differ from the two roundings),
// so its paired product is followed by scalar sums (__fadd_rn, never fused), which keeps
// the bits on every operand tested.
VT_HD vec3 sub_p(vec3 a, vec3 b)  // a - b
{
#if VT_PAIRED
    const float2 r = __fadd2_rn(make_float2(a.x, a.y), make_float2(-b.x, -b.y));
    return mk3(r.x, r.y, a.z - b.z);
#else
    return a - b;
#endif
}
VT_HD vec3 mul_p(vec3 a, float s)  // a * s
{
#if VT_PAIRED
    const float2 r = __fmul2_rn(make_float2(a.x, a.y), make_float2(s, s));
    return mk3(r.x, r.y, a.z * s);
#else
    return a * s;
#endif
}
VT_HD vec3 madd_p(vec3 a, float s, vec3 b)  // a * s + b
{
#if VT_PAIRED && VT_FAST_DEVICE
    const float2 r = __ffma2_rn(make_float2(a.x, a.y), make_float2(s, s), make_float2(b.x, b.y));
    return mk3(r.x, r.y, __fmaf_rn(a.z, s, b.z));
#elif VT_PAIRED
    const float2 p = __fmul2_rn(make_float2(a.x, a.y), make_float2(s, s));
    return mk3(__fadd_rn(p.x, b.x), __fadd_rn(p.y, b.y), __fadd_rn(__fmul_rn(a.z, s), b.z));
#else
    return a * s + b;
#endif
}

// mat4 (column-major) * (v, w), glm association
VT_HD vec3 m4v3(const float* m, vec3 v, float w)
{
    return mk3((m[0] * v.x + m[4] * v.y) + (m[8] * v.z + m[12] * w),
               (m[1] * v.x + m[5] * v.y) + (m[9] * v.z + m[13] * w),
               (m[2] * v.x + m[6] * v.y) + (m[10] * v.z + m[14] * w));
}
// mat3 (column-major) * v
VT_HD vec3 m3v3(const float* m, vec3 v)
{
    return mk3((m[0] * v.x + m[3] * v.y) + m[6] * v.z, (m[1] * v.x + m[4] * v.y) + m[7] * v.z,
               (m[2] * v.x + m[5] * v.y) + m[8] * v.z);
}
// mat4 * mat4, glm: column j = ((A0*B[j][0] + A1*B[j][1]) + A2*B[j][2]) + A3*B[j][3]
VT_HD void m4m4(const float* a, const float* b, float* out)
{
    for (int j = 0; j < 4; ++j)
        for (int r = 0; r < 4; ++r) {
            float s = a[0 + r] * b[4 * j + 0] + a[4 + r] * b[4 * j + 1];
            s = s + a[8 + r] * b[4 * j + 2];
            s = s + a[12 + r] * b[4 * j + 3];
            out[4 * j + r] = s;
        }
}

// arccos for the dihedral angle of the bending constraint.  The reference calls CUDA's
// acosf; this is our own: the Maclaurin series of arcsin,
//   arcsin(t) = t + sum_{n>=1} c_n t^(2n+1),  c_n = (2n)! / (4^n (n!)^2 (2n+1)),
// truncated after n = 11 (|t| <= 1/2: truncation error < 1e-9 relative), with
//   arccos(x) = 2 arcsin(sqrt((1-x)/2))          for x >=  1/2
//             = pi - 2 arcsin(sqrt((1+x)/2))     for x <= -1/2
//             = pi/2 - arcsin(x)                 otherwise.
// Host and device evaluate the same operations, so they agree bit for bit.
VT_HD float vt_asin_series(float t)
{
    const float c1 = 0.16666666666666666f, c2 = 0.075f, c3 = 0.044642857142857144f,
                c4 = 0.030381944444444444f, c5 = 0.022372159090909092f,
                c6 = 0.017352764423076924f, c7 = 0.01396484375f, c8 = 0.011551800896139705f,
                c9 = 0.009761609529194078f, c10 = 0.008390335809616815f,
                c11 = 0.0073125258735988454f;
    float z = t * t;
    float p = c11;
    p = p * z + c10;
    p = p * z + c9;
    p = p * z + c8;
    p = p * z + c7;
    p = p * z + c6;
    p = p * z + c5;
    p = p * z + c4;
    p = p * z + c3;
    p = p * z + c2;
    p = p * z + c1;
    float r = z * p;
    return t + t * r;
}

VT_HD float vt_acosf(float x)
{
    const float pio2_hi = 1.57079637050628662109375f;
    const float pio2_lo = -4.37113900018624283e-8f;
    if (x >= 0.5f) {
        float s = sqrtf((1.0f - x) * 0.5f);
        return 2.0f * vt_asin_series(s);
    }
    if (x <= -0.5f) {
        float s = sqrtf((1.0f + x) * 0.5f);
        return ((pio2_hi - vt_asin_series(s)) + pio2_lo) * 2.0f;
    }
    return (pio2_hi - vt_asin_series(x)) + pio2_lo;
}

// vt_acosf with every operation rounded as written (the fast build's exact angle chain).
VT_HD float vt_acosf_exact(float x)
{
#if VT_FAST_DEVICE
    const float c[11] = {0.16666666666666666f, 0.075f, 0.044642857142857144f, 0.030381944444444444f,
                         0.022372159090909092f, 0.017352764423076924f, 0.01396484375f, 0.011551800896139705f,
                         0.009761609529194078f, 0.008390335809616815f, 0.0073125258735988454f};
    auto series = [&](float t) {
        const float z = __fmul_rn(t, t);
        float p = c[10];
#pragma unroll
        for (int k = 9; k >= 0; --k) p = __fadd_rn(__fmul_rn(p, z), c[k]);
        return __fadd_rn(t, __fmul_rn(t, __fmul_rn(z, p)));
    };
    const float pio2_hi = 1.57079637050628662109375f;
    const float pio2_lo = -4.37113900018624283e-8f;
    if (x >= 0.5f) return __fmul_rn(2.0f, series(__fsqrt_rn(__fmul_rn(__fsub_rn(1.0f, x), 0.5f))));
    if (x <= -0.5f)
        return __fmul_rn(__fadd_rn(__fsub_rn(pio2_hi, series(__fsqrt_rn(__fmul_rn(__fadd_rn(1.0f, x), 0.5f)))),
                                   pio2_lo),
                         2.0f);
    return __fadd_rn(__fsub_rn(pio2_hi, series(x)), pio2_lo);
#else
    return vt_acosf(x);
#endif
}

// Vertex (a, b) of GenerateClothMesh (Velvet/Scene.hpp:131-168) for a cloth of side
// `size`: size * (b / res - 0.5, -(a / res), 0), placed by InitializePositions'
// model * (v, 1) (Velvet/VtClothSolverGPU.cu:30-34).  Host and device evaluate it with
// the same operations, so a cloth built on the device has the bits of one registered
// from host arrays made the same way.
VT_HD vec3 grid_vertex(int a, int b, int res, float size, const float* model)
{
    const float r = (float)res;
    const float fx = (float)b / r - 0.5f;
    const float fy = -((float)a / r);
    return m4v3(model, mk3(size * fx, size * fy, 0.0f), 1.0f);
}

// The dihedral angle SolveBending_Kernel (Velvet/VtClothSolverGPU.cu:117-189) measures for
// corners (p0, p1, p2, p3), shared edge p2-p3, with its operations (each normal divided by
// its squared length, then normalised; acos of the clamped dot): the rest angle that
// makes a registered configuration an equilibrium of the constraint.
VT_HD float bend_angle(vec3 p0, vec3 p1, vec3 p2, vec3 p3)
{
    vec3 n1 = cross(p2 - p0, p3 - p0);
    n1 = n1 / dot(n1, n1);
    vec3 n2 = cross(p3 - p1, p2 - p1);
    n2 = n2 / dot(n2, n2);
    return vt_acosf(gclamp(dot(normalize(n1), normalize(n2)), -1.0f, 1.0f));
}
