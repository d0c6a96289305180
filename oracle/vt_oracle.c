/*
 * vt_oracle.c — CPU ORACLE for the XPBD cloth solver.  TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline leg may load this
 * library, and only as the checker (or the timed CPU stand-in for the reference).  The
 * product (velvet_gb300/) never links, loads or calls it.
 *
 * What it is: a sequential restatement, in plain C, of the reference's GPU solver path
 *   Velvet/VtClothSolverGPU.cu:13-465      kernels (predict, stretch, bending, attachment,
 *                                          apply-deltas, SDF collision + friction,
 *                                          particle collision, finalize, normals)
 *   Velvet/VtClothSolverGPU.cuh:8-97       SDFCollider (plane / sphere / cube, VelocityAt)
 *   Velvet/VtClothSolverGPU.hpp:56-205     Simulate() schedule, AddCloth/AddStretch/
 *                                          AddAttachSlot/AddAttach/AddBend
 *   Velvet/SpatialHashGPU.cu:13-196        hash, stable sort, cell ranges, neighbour cache
 *   Velvet/SpatialHashGPU.hpp:18-52        table sizing, initial positions, HashParams
 *   Velvet/VtClothObjectGPU.hpp:43-147     constraint generation for grid cloths
 *   Velvet/Common.hpp:19-48                parameter defaults
 * Every atomicAdd of the reference becomes a sequential add in constraint-index order
 * (one valid serialisation of the reference's unordered atomics), kernels run in the
 * reference's launch order, and vector arithmetic follows glm's association order
 * (dot = (x*x + y*y) + z*z, mat4*vec4 = (m0*x + m1*y) + (m2*z + m3*w),
 * mat4*mat4 columns left-associated, normalize = v * (1/sqrt(dot))).
 * Build with -ffp-contract=off -fwrapv: no fused multiply-add, wrapping int32 products
 * in the hash (the reference relies on CUDA's wrap-around).
 *
 * acos: the reference calls CUDA's acosf.  This oracle (and the CUDA kernels) use
 * vo_acosf below — the Maclaurin series of arcsin with the half-angle identity — so the
 * two sides agree bit for bit; its distance from the exact arccos is checked in tests.
 *
 * Parity status: PINNED to the reference's own kernel code.  oracle/refemu compiles the
 * reference's Velvet/VtClothSolverGPU.cu and Velvet/SpatialHashGPU.cu unmodified for the
 * CPU (make -C oracle ref -> oracle/_ref/libvr_ref.so, atomics in thread order, acos from
 * vo_acosf below), and this restatement reproduces its outputs bit for bit: the committed
 * fixtures tests/golden/ref_*.npz (every collider kind, the schedule's branches, a row of
 * attachments, two colliding cloths, HashObjects on a cloud) and, where the reference tree
 * is present, the small configuration's 64x64 cloth live (tests/test_ref_pinning.py).  What
 * stays unpinned: glm's own evaluation order (the stand-in glm assumes the orders above)
 * and CUDA's acosf.  Known-answer tests in tests/ check hash keys, single-constraint
 * analytic cases, SDF projections and the acos error bound independently.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/velvet_gb300.h"

#define VO_EPSILON 1e-6f /* EPSILON, Velvet/Common.cuh:12 */

#if defined(_WIN32)
#define VO_API __declspec(dllexport)
#else
#define VO_API __attribute__((visibility("default")))
#endif

/* ------------------------------------------------------------------ vec3 (glm order) */
typedef struct { float x, y, z; } v3;

static inline v3 V(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline v3 vadd(v3 a, v3 b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vneg(v3 a) { return V(-a.x, -a.y, -a.z); }
static inline v3 vmuls(v3 a, float s) { return V(a.x * s, a.y * s, a.z * s); }
static inline v3 vdivs(v3 a, float s) { return V(a.x / s, a.y / s, a.z / s); }
static inline v3 vmul(v3 a, v3 b) { return V(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline float vdot(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline float vlen(v3 a) { return sqrtf(vdot(a, a)); }
static inline v3 vnormalize(v3 a) { return vmuls(a, 1.0f / sqrtf(vdot(a, a))); }
static inline v3 vcross(v3 a, v3 b)
{
    return V(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
/* glm::clamp = min(max(x, lo), hi) with glm's ternary min/max */
static inline float gclamp(float x, float lo, float hi)
{
    float m = (x < lo) ? lo : x;
    return (hi < m) ? hi : m;
}

/* mat4 (column-major) * vec4, glm association: (c0*x + c1*y) + (c2*z + c3*w) */
static void m4v4(const float* m, const float v[4], float out[4])
{
    for (int r = 0; r < 4; ++r) {
        float a0 = m[0 + r] * v[0];
        float a1 = m[4 + r] * v[1];
        float a2 = m[8 + r] * v[2];
        float a3 = m[12 + r] * v[3];
        out[r] = (a0 + a1) + (a2 + a3);
    }
}
/* mat4 * mat4, glm: R[j] = ((A0*B[j][0] + A1*B[j][1]) + A2*B[j][2]) + A3*B[j][3] */
static void m4m4(const float* a, const float* b, float* out)
{
    for (int j = 0; j < 4; ++j)
        for (int r = 0; r < 4; ++r) {
            float s = a[0 + r] * b[4 * j + 0] + a[4 + r] * b[4 * j + 1];
            s = s + a[8 + r] * b[4 * j + 2];
            s = s + a[12 + r] * b[4 * j + 3];
            out[4 * j + r] = s;
        }
}
/* mat3 * vec3, glm: row r = (m[0][r]*x + m[1][r]*y) + m[2][r]*z */
static v3 m3v3(const float* m, v3 v)
{
    return V((m[0] * v.x + m[3] * v.y) + m[6] * v.z,
             (m[1] * v.x + m[4] * v.y) + m[7] * v.z,
             (m[2] * v.x + m[5] * v.y) + m[8] * v.z);
}

/* ------------------------------------------------------------------ acos
 * arcsin(t) = t + sum_{n>=1} c_n t^(2n+1),  c_n = (2n)! / (4^n (n!)^2 (2n+1)),
 * truncated after n = 11 (|t| <= 1/2: truncation < 1e-9 relative); arccos from
 * arccos(x) = 2 arcsin(sqrt((1-x)/2)) for x >= 1/2, pi - 2 arcsin(sqrt((1+x)/2))
 * for x <= -1/2, pi/2 - arcsin(x) otherwise. */
static const float VO_ASIN_C[11] = {
    0.16666666666666666f, 0.075f, 0.044642857142857144f, 0.030381944444444444f,
    0.022372159090909092f, 0.017352764423076924f, 0.01396484375f, 0.011551800896139705f,
    0.009761609529194078f, 0.008390335809616815f, 0.0073125258735988454f};
static const float VO_PIO2_HI = 1.57079637050628662109375f;
static const float VO_PIO2_LO = -4.37113900018624283e-8f;

static inline float vo_asin_series(float t)
{
    float z = t * t;
    float p = VO_ASIN_C[10];
    for (int k = 9; k >= 0; --k) p = p * z + VO_ASIN_C[k];
    float r = z * p;
    return t + t * r;
}

VO_API float vo_acosf(float x)
{
    if (x >= 0.5f) {
        float s = sqrtf((1.0f - x) * 0.5f);
        return 2.0f * vo_asin_series(s);
    }
    if (x <= -0.5f) {
        float s = sqrtf((1.0f + x) * 0.5f);
        return ((VO_PIO2_HI - vo_asin_series(s)) + VO_PIO2_LO) * 2.0f;
    }
    return (VO_PIO2_HI - vo_asin_series(x)) + VO_PIO2_LO;
}

/* ------------------------------------------------------------------ growable arrays */
#define VEC(T) struct { T* d; size_t n, cap; }
#define VPUSH(vec, val)                                                          \
    do {                                                                         \
        if ((vec).n == (vec).cap) {                                              \
            size_t nc = (vec).cap ? (vec).cap * 2 : 64;                          \
            void* nd = realloc((vec).d, nc * sizeof(*(vec).d));                 \
            if (!nd) abort();                                                    \
            (vec).d = nd;                                                        \
            (vec).cap = nc;                                                      \
        }                                                                        \
        (vec).d[(vec).n++] = (val);                                              \
    } while (0)
#define VFREE(vec) free((vec).d)

typedef struct { int32_t offset, count, tri_begin, tri_count; } vo_cloth;

typedef struct vo_solver {
    vt_params P;
    uint32_t n;
    VEC(v3) x;
    VEC(v3) v;
    VEC(v3) p;
    VEC(v3) dl;
    VEC(v3) nrm;
    VEC(v3) x0;
    VEC(float) w;
    VEC(int32_t) cnt;
    VEC(uint32_t) tri;
    VEC(vo_cloth) cloths;
    VEC(int32_t) st_idx;
    VEC(float) st_rest;
    VEC(v3) slots;
    VEC(int32_t) at_pid;
    VEC(int32_t) at_slot;
    VEC(float) at_dist;
    VEC(uint32_t) bd_idx;
    VEC(float) bd_rest;
    vt_sdf_collider* col;
    uint32_t ncol;
    /* 1: the constraint kernels' atomics land in reverse constraint order (another valid
     * order of the reference's unordered atomics), for measuring how much the result
     * depends on that order */
    int reverse_sums;
    /* spatial hash (SpatialHashGPU.hpp:18-29) */
    float cell_spacing;
    int32_t table_size;
    uint32_t *hkey, *hidx, *cstart, *cend, *nbr;
    uint32_t hash_cap_n, hash_cap_t;
    int hashed;
} vo_solver;

VO_API void vo_params_default(vt_params* P)
{
    memset(P, 0, sizeof(*P));
    P->num_substeps = 2;
    P->num_iterations = 4;
    P->max_num_neighbors = 64;
    P->max_speed = 50.0f;
    P->gravity[0] = 0.0f;
    P->gravity[1] = -9.8f;
    P->gravity[2] = 0.0f;
    P->bend_compliance = 0.0f;
    P->damping = 0.25f;
    P->relaxation_factor = 1.0f;
    P->long_range_stretchiness = 1.2f;
    P->collision_margin = 0.06f;
    P->friction = 0.1f;
    P->enable_self_collision = 1;
    P->interleaved_hash = 3;
    P->num_particles = 0;
    P->particle_diameter = 0.0f;
    P->delta_time = 1.0f / 60.0f;
    P->particle_diameter_scalar = 1.5f;
    P->hash_cell_size_scalar = 1.5f;
}

VO_API vo_solver* vo_create(const vt_params* P)
{
    vo_solver* s = (vo_solver*)calloc(1, sizeof(vo_solver));
    if (P) s->P = *P; else vo_params_default(&s->P);
    s->P.num_particles = 0;
    return s;
}

VO_API void vo_destroy(vo_solver* s)
{
    if (!s) return;
    VFREE(s->x); VFREE(s->v); VFREE(s->p); VFREE(s->dl); VFREE(s->nrm); VFREE(s->x0);
    VFREE(s->w); VFREE(s->cnt); VFREE(s->tri); VFREE(s->cloths);
    VFREE(s->st_idx); VFREE(s->st_rest); VFREE(s->slots);
    VFREE(s->at_pid); VFREE(s->at_slot); VFREE(s->at_dist);
    VFREE(s->bd_idx); VFREE(s->bd_rest);
    free(s->col); free(s->hkey); free(s->hidx); free(s->cstart); free(s->cend); free(s->nbr);
    free(s);
}

VO_API void vo_get_params(const vo_solver* s, vt_params* out) { *out = s->P; }
VO_API void vo_set_params(vo_solver* s, const vt_params* P)
{
    uint32_t n = s->P.num_particles;
    s->P = *P;
    s->P.num_particles = n;
}
VO_API uint32_t vo_num_particles(const vo_solver* s) { return s->n; }
/* Sum order of the stretch, attachment and bending corrections: 0 constraint order (the
 * default, the CUDA solver's order), 1 reverse constraint order. */
VO_API void vo_set_sum_order(vo_solver* s, int reversed) { s->reverse_sums = reversed != 0; }
VO_API int32_t vo_table_size(const vo_solver* s) { return s->table_size; }

/* ------------------------------------------------------------------ registration */

/* AddCloth, Velvet/VtClothSolverGPU.hpp:114-156 */
VO_API int32_t vo_cloth_add(vo_solver* s, const float* xyz, uint32_t nv, const uint32_t* idx,
                            uint32_t nidx, const float* model, float diameter)
{
    int32_t prev = (int32_t)s->n;
    s->n += nv;
    s->P.num_particles = s->n;
    s->P.particle_diameter = diameter;
    /* Timer::fixedDeltaTime() is P.delta_time */
    s->P.max_speed = 2.0f * diameter / s->P.delta_time * (float)s->P.num_substeps;

    vo_cloth c = {prev, (int32_t)nv, (int32_t)s->tri.n, (int32_t)nidx};
    VPUSH(s->cloths, c);
    for (uint32_t i = 0; i < nidx; ++i) VPUSH(s->tri, idx[i] + (uint32_t)prev);
    for (uint32_t i = 0; i < nv; ++i) {
        /* InitializePositions_Kernel, VtClothSolverGPU.cu:30-34 */
        float in[4] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], 1.0f}, o[4];
        m4v4(model, in, o);
        VPUSH(s->x, V(o[0], o[1], o[2]));
        VPUSH(s->v, V(0, 0, 0));
        VPUSH(s->p, V(0, 0, 0));
        VPUSH(s->dl, V(0, 0, 0));
        VPUSH(s->nrm, V(0, 0, 0));
        VPUSH(s->cnt, 0);
        VPUSH(s->w, 1.0f);
    }
    /* new SpatialHashGPU(particleDiameter, numParticles) + SetInitialPositions,
     * VtClothSolverGPU.hpp:148-149, SpatialHashGPU.hpp:18-39 */
    s->cell_spacing = diameter * s->P.hash_cell_size_scalar;
    s->table_size = 2 * (int32_t)s->n;
    s->x0.n = 0;
    for (uint32_t i = 0; i < s->n; ++i) VPUSH(s->x0, s->x.d[i]);
    free(s->hkey); free(s->hidx); free(s->cstart); free(s->cend); free(s->nbr);
    uint32_t mn = (uint32_t)s->P.max_num_neighbors;
    s->hkey = (uint32_t*)calloc(s->n, 4);
    s->hidx = (uint32_t*)calloc(s->n, 4);
    s->cstart = (uint32_t*)calloc((size_t)s->table_size + 1, 4);
    s->cend = (uint32_t*)calloc((size_t)s->table_size + 1, 4);
    s->nbr = (uint32_t*)calloc((size_t)s->n * mn, 4);
    s->hashed = 0;
    return prev;
}

VO_API void vo_stretch_add(vo_solver* s, int32_t i, int32_t j, float rest)
{
    VPUSH(s->st_idx, i);
    VPUSH(s->st_idx, j);
    VPUSH(s->st_rest, rest);
}
VO_API int32_t vo_attach_slot_add(vo_solver* s, const float* xyz)
{
    VPUSH(s->slots, V(xyz[0], xyz[1], xyz[2]));
    return (int32_t)s->slots.n - 1;
}
VO_API void vo_attach_add(vo_solver* s, int32_t pid, int32_t slot, float dist)
{
    if (dist == 0) s->w.d[pid] = 0; /* VtClothSolverGPU.hpp:172 */
    VPUSH(s->at_pid, pid);
    VPUSH(s->at_slot, slot);
    VPUSH(s->at_dist, dist);
}
VO_API void vo_bend_add(vo_solver* s, uint32_t i0, uint32_t i1, uint32_t i2, uint32_t i3,
                        float angle)
{
    VPUSH(s->bd_idx, i0); VPUSH(s->bd_idx, i1); VPUSH(s->bd_idx, i2); VPUSH(s->bd_idx, i3);
    VPUSH(s->bd_rest, angle);
}

/* VtClothObjectGPU::Start generation, Velvet/VtClothObjectGPU.hpp:43-147, for the
 * cloth whose first particle is `offset`.  World positions are the solver's positions
 * of that cloth (AddCloth applied the same model matrix with the same arithmetic as
 * ApplyTransform, :67-73).  Slots get solver-global indices. */
VO_API int vo_build_grid_constraints(vo_solver* s, int32_t offset, int32_t res,
                                     const int32_t* attached, uint32_t nat)
{
    const vo_cloth* c = NULL;
    for (size_t k = 0; k < s->cloths.n; ++k)
        if (s->cloths.d[k].offset == offset) c = &s->cloths.d[k];
    if (!c || (int64_t)(res + 1) * (res + 1) != c->count) return -1;
    const v3* pos = s->x.d + offset;
#define VAT(a, b) ((a) * (res + 1) + (b))
    /* GenerateStretch, :75-116 */
    for (int a = 0; a < res + 1; ++a)
        for (int b = 0; b < res + 1; ++b) {
            int i1, i2;
            if (b != res) {
                i1 = VAT(a, b); i2 = VAT(a, b + 1);
                vo_stretch_add(s, offset + i1, offset + i2, vlen(vsub(pos[i1], pos[i2])));
            }
            if (a != res) {
                i1 = VAT(a, b); i2 = VAT(a + 1, b);
                vo_stretch_add(s, offset + i1, offset + i2, vlen(vsub(pos[i1], pos[i2])));
            }
            if (b != res && a != res) {
                i1 = VAT(a, b); i2 = VAT(a + 1, b + 1);
                vo_stretch_add(s, offset + i1, offset + i2, vlen(vsub(pos[i1], pos[i2])));
                i1 = VAT(a, b + 1); i2 = VAT(a + 1, b);
                vo_stretch_add(s, offset + i1, offset + i2, vlen(vsub(pos[i1], pos[i2])));
            }
        }
#undef VAT
    /* GenerateAttach, :134-147 */
    for (uint32_t k = 0; k < nat; ++k) {
        v3 slot = pos[attached[k]];
        float xyz[3] = {slot.x, slot.y, slot.z};
        int32_t sid = vo_attach_slot_add(s, xyz);
        for (int32_t i = 0; i < c->count; ++i)
            vo_attach_add(s, offset + i, sid, vlen(vsub(slot, pos[i])));
    }
    /* GenerateBending, :118-132 (indices i, i+5, i+2, i+1 of each 6-index block) */
    const uint32_t* ind = s->tri.d + c->tri_begin;
    for (int32_t i = 0; i + 5 < c->tri_count; i += 6)
        vo_bend_add(s, ind[i], ind[i + 5], ind[i + 2], ind[i + 1], 0.0f);
    return 0;
}

/* General bending adjacency (vt_cloth_build_bending_adjacency; not in the reference,
 * whose GenerateBending pairs only the two triangles of a grid quad,
 * VtClothObjectGPU.hpp:118-132): one bend per edge shared by exactly two triangles of the
 * cloth, hinges ordered by (first triangle, its corner opposite the edge), corners
 * (first opposite, second opposite, next-next corner, next corner of the first
 * triangle), rest angle = the dihedral angle solve_bending measures at x0. */
typedef struct { uint64_t key; int32_t tri, k; } vo_use;
typedef struct { int32_t tri, k, tri2, k2; } vo_hinge;

static int cmp_use(const void* a, const void* b)
{
    const vo_use *x = (const vo_use*)a, *y = (const vo_use*)b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    if (x->tri != y->tri) return x->tri < y->tri ? -1 : 1;  /* keeps triangle order */
    return x->k < y->k ? -1 : (x->k > y->k);
}

static int cmp_hinge(const void* a, const void* b)
{
    const vo_hinge *x = (const vo_hinge*)a, *y = (const vo_hinge*)b;
    if (x->tri != y->tri) return x->tri < y->tri ? -1 : 1;
    return x->k < y->k ? -1 : (x->k > y->k);
}

static float bend_angle(v3 p0, v3 p1, v3 p2, v3 p3)
{
    v3 n1 = vcross(vsub(p2, p0), vsub(p3, p0));
    n1 = vdivs(n1, vdot(n1, n1));
    v3 n2 = vcross(vsub(p3, p1), vsub(p2, p1));
    n2 = vdivs(n2, vdot(n2, n2));
    return vo_acosf(gclamp(vdot(vnormalize(n1), vnormalize(n2)), -1.0f, 1.0f));
}

VO_API int vo_build_bending_adjacency(vo_solver* s, int32_t offset, uint32_t* out_count)
{
    const vo_cloth* c = NULL;
    for (size_t k = 0; k < s->cloths.n; ++k)
        if (s->cloths.d[k].offset == offset) c = &s->cloths.d[k];
    if (!c) return -1;
    const uint32_t* t = s->tri.d + c->tri_begin;
    const int32_t ntri = c->tri_count / 3;
    vo_use* uses = (vo_use*)malloc(sizeof(vo_use) * (3 * (size_t)ntri + 1));
    vo_hinge* hinges = (vo_hinge*)malloc(sizeof(vo_hinge) * (3 * (size_t)ntri + 1));
    size_t nu = 0, nh = 0;
    for (int32_t q = 0; q < ntri; ++q)
        for (int k = 0; k < 3; ++k) {
            uint32_t u = t[3 * q + (k + 1) % 3], v = t[3 * q + (k + 2) % 3];
            uint32_t lo = u < v ? u : v, hi = u < v ? v : u;
            vo_use e = {((uint64_t)lo << 32) | hi, q, k};
            uses[nu++] = e;
        }
    qsort(uses, nu, sizeof(vo_use), cmp_use);
    for (size_t i = 0; i < nu;) {
        size_t j = i;
        while (j < nu && uses[j].key == uses[i].key) ++j;
        if (j - i == 2) {
            vo_hinge g = {uses[i].tri, uses[i].k, uses[i + 1].tri, uses[i + 1].k};
            hinges[nh++] = g;
        }
        i = j;
    }
    qsort(hinges, nh, sizeof(vo_hinge), cmp_hinge);
    uint32_t added = 0;
    for (size_t h = 0; h < nh; ++h) {
        const vo_hinge g = hinges[h];
        uint32_t i0 = t[3 * g.tri + g.k], i3 = t[3 * g.tri + (g.k + 1) % 3], i2 = t[3 * g.tri + (g.k + 2) % 3];
        uint32_t i1 = t[3 * g.tri2 + g.k2];
        v3 p0 = s->x0.d[i0], p1 = s->x0.d[i1], p2 = s->x0.d[i2], p3 = s->x0.d[i3];
        v3 n1 = vcross(vsub(p2, p0), vsub(p3, p0)), n2 = vcross(vsub(p3, p1), vsub(p2, p1));
        if (vlen(vsub(p3, p2)) < VO_EPSILON || vdot(n1, n1) == 0 || vdot(n2, n2) == 0) continue;
        float rest = bend_angle(p0, p1, p2, p3);
        if (!isfinite(rest)) continue;
        vo_bend_add(s, i0, i1, i2, i3, rest);
        ++added;
    }
    free(uses);
    free(hinges);
    if (out_count) *out_count = added;
    return 0;
}

/* Headless sphere-impostor rendering (vt_solver_render; the library's own feature, the
 * CUDA counterpart of the reference's _InstancedParticle shaders, which need a graphics
 * API): the per-particle pixel box and the per-pixel depth|colour key restated with the
 * same operations, the visible key being the minimum over particles. */
VO_API void vo_render(const float* xyz, uint32_t n, const vt_render_params* rp, uint32_t* rgba)
{
    const size_t npix = (size_t)rp->width * rp->height;
    uint64_t* z = (uint64_t*)malloc(sizeof(uint64_t) * (npix ? npix : 1));
    for (size_t k = 0; k < npix; ++k) z[k] = ~0ull;
    const float W = (float)rp->width, H = (float)rp->height, R = rp->particle_radius;
    const float* Vm = rp->view;
    for (uint32_t i = 0; i < n; ++i) {
        const float xv[4] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], 1.0f};
        float pe4[4];
        m4v4(Vm, xv, pe4);
        const v3 pe = V(pe4[0], pe4[1], pe4[2]);
        if (!(pe.z < -rp->z_near)) continue;
        const float inv = 1.0f / (-pe.z);
        const float sx = rp->projection[0] * inv, sy = rp->projection[5] * inv;
        const float cx = pe.x * sx, cy = pe.y * sy;
        const float px = (cx * 0.5f + 0.5f) * W, py = (0.5f - cy * 0.5f) * H;
        const float rx = R * sx * 0.5f * W, ry = R * sy * 0.5f * H;
        const float lx = px - rx, hx = px + rx, ly = py - ry, hy = py + ry;
        if (!(lx <= W - 1.0f && hx >= 0.0f && ly <= H - 1.0f && hy >= 0.0f)) continue;
        const int x0 = lx > 0.0f ? (int)floorf(lx) : 0;
        const int x1 = hx < W - 1.0f ? (int)ceilf(hx) : (int)rp->width - 1;
        const int y0 = ly > 0.0f ? (int)floorf(ly) : 0;
        const int y1 = hy < H - 1.0f ? (int)ceilf(hy) : (int)rp->height - 1;
        for (int j = y0; j <= y1; ++j)
            for (int k = x0; k <= x1; ++k) {
                const float nx = ((float)k + 0.5f) / W * 2.0f - 1.0f;
                const float ny = 1.0f - ((float)j + 0.5f) / H * 2.0f;
                const float u = (nx - cx) / (sx * R), v = (ny - cy) / (sy * R);
                const float r2 = u * u + v * v;
                if (!(r2 <= 1.0f)) continue;
                const float nz = sqrtf(1.0f - r2);
                float depth = -(pe.z + nz * R);
                if (!(depth > 0.0f)) depth = 0.0f;
                const v3 nw = V((Vm[0] * u + Vm[1] * v) + Vm[2] * nz, (Vm[4] * u + Vm[5] * v) + Vm[6] * nz,
                                (Vm[8] * u + Vm[9] * v) + Vm[10] * nz);
                const float ndl = vdot(nw, V(rp->light_dir[0], rp->light_dir[1], rp->light_dir[2]));
                const float lit = rp->ambient + (ndl > 0.0f ? ndl : 0.0f);
                uint32_t col = 0xff000000u;
                for (int c = 0; c < 3; ++c) {
                    float q = rp->tint[c] * lit;
                    q = q < 0.0f ? 0.0f : (q > 1.0f ? 1.0f : q);
                    col |= (uint32_t)(sqrtf(q) * 255.0f + 0.5f) << (8 * c);
                }
                uint32_t bits;
                memcpy(&bits, &depth, 4);
                const uint64_t key = ((uint64_t)bits << 32) | col;
                uint64_t* zp = &z[(size_t)j * rp->width + k];
                if (key < *zp) *zp = key;
            }
    }
    for (size_t k = 0; k < npix; ++k) rgba[k] = z[k] == ~0ull ? rp->background : (uint32_t)z[k];
    free(z);
}

VO_API void vo_colliders_set(vo_solver* s, const vt_sdf_collider* c, uint32_t n)
{
    free(s->col);
    s->col = (vt_sdf_collider*)malloc(sizeof(vt_sdf_collider) * (n ? n : 1));
    if (n) memcpy(s->col, c, sizeof(vt_sdf_collider) * n);
    s->ncol = n;
}

/* ------------------------------------------------------------------ SDF colliders */
static float sgnf(float v) { return (v > 0) ? 1.0f : (v < 0 ? -1.0f : 0.0f); }

/* SDFCollider::ComputeSDF, VtClothSolverGPU.cuh:22-89 */
static v3 collider_sdf(const vt_sdf_collider* c, v3 t, float margin)
{
    if (c->type == VT_COLLIDER_PLANE) {
        float offset = t.y - (c->position[1] + margin);
        if (offset < 0) return V(0, -offset, 0);
    } else if (c->type == VT_COLLIDER_SPHERE) {
        float radius = c->scale[0] + margin;
        v3 diff = vsub(t, V(c->position[0], c->position[1], c->position[2]));
        float distance = vlen(diff);
        float offset = distance - radius;
        if (offset < 0) {
            v3 direction = vdivs(diff, distance);
            return vmuls(direction, -offset);
        }
    } else if (c->type == VT_COLLIDER_CUBE) {
        v3 correction = V(0, 0, 0);
        float in[4] = {t.x, t.y, t.z, 1.0f}, lp[4];
        m4v4(c->inv_cur_transform, in, lp);
        v3 local = V(lp[0], lp[1], lp[2]);
        v3 cube = V(0.5f + margin / c->scale[0], 0.5f + margin / c->scale[1],
                    0.5f + margin / c->scale[2]);
        v3 offset = vsub(V(fabsf(local.x), fabsf(local.y), fabsf(local.z)), cube);
        float maxv = fmaxf(offset.x, fmaxf(offset.y, offset.z));
        float minv = fminf(offset.x, fminf(offset.y, offset.z));
        float midv = ((offset.x + offset.y) + offset.z - maxv) - minv;
        float scalar = 1.0f;
        if (maxv < 0) {
            const float m = 0.03f;
            if (midv > -m) scalar = 0.2f;
            if (minv > -m) {
                v3 mask = V(offset.x < 0 ? sgnf(local.x) : 0, offset.y < 0 ? sgnf(local.y) : 0,
                            offset.z < 0 ? sgnf(local.z) : 0);
                v3 vec = vadd(offset, V(m, m, m));
                float len = vlen(vec);
                if (len < m) correction = vmuls(vmul(mask, vnormalize(vec)), m - len);
            } else if (offset.x == maxv) {
                correction = V(copysignf(-offset.x, local.x), 0, 0);
            } else if (offset.y == maxv) {
                correction = V(0, copysignf(-offset.y, local.y), 0);
            } else if (offset.z == maxv) {
                correction = V(0, 0, copysignf(-offset.z, local.z));
            }
        }
        float ms[9];
        for (int k = 0; k < 9; ++k) ms[k] = c->cur_transform[k] * scalar;
        return m3v3(ms, correction);
    }
    return V(0, 0, 0);
}

/* SDFCollider::VelocityAt, VtClothSolverGPU.cuh:91-96 */
static v3 collider_velocity(const vt_sdf_collider* c, v3 t)
{
    float m[16];
    m4m4(c->last_transform, c->inv_cur_transform, m);
    float in[4] = {t.x, t.y, t.z, 1.0f}, lp[4];
    m4v4(m, in, lp);
    return vdivs(vsub(t, V(lp[0], lp[1], lp[2])), c->delta_time);
}

/* ComputeFriction, VtClothSolverGPU.cu:272-287 */
static v3 friction_of(v3 corr, v3 relvel, float friction)
{
    v3 fr = V(0, 0, 0);
    float cl = vlen(corr);
    if (friction > 0 && cl > 0) {
        v3 nrm = vdivs(corr, cl);
        v3 tan = vsub(relvel, vmuls(nrm, vdot(relvel, nrm)));
        float tl = vlen(tan);
        float mt = cl * friction;
        fr = vmuls(vneg(tan), fminf(mt / tl, 1.0f));
    }
    return fr;
}

/* ------------------------------------------------------------------ kernels, sequential */

/* CollideSDF_Kernel, VtClothSolverGPU.cu:289-314.  pred and pos may alias (the
 * pre-stabilisation pass runs it on the positions themselves). */
static void collide_sdf(vo_solver* s, v3* pred, const v3* pos, float dt)
{
    if (s->ncol == 0) return;
    for (uint32_t i = 0; i < s->n; ++i) {
        v3 po = pos[i];
        v3 pr = pred[i];
        for (uint32_t k = 0; k < s->ncol; ++k) {
            const vt_sdf_collider* c = &s->col[k];
            v3 corr = collider_sdf(c, pr, s->P.collision_margin);
            pr = vadd(pr, corr);
            if (vdot(corr, corr) > 0) {
                v3 relvel = vsub(vsub(pr, po), vmuls(collider_velocity(c, pr), dt));
                pr = vadd(pr, friction_of(corr, relvel, s->P.friction));
            }
        }
        pred[i] = pr;
    }
}

/* PredictPositions_Kernel, :42-53 */
static void predict(vo_solver* s, float dt)
{
    v3 g = V(s->P.gravity[0], s->P.gravity[1], s->P.gravity[2]);
    for (uint32_t i = 0; i < s->n; ++i) {
        s->v.d[i] = vadd(s->v.d[i], vmuls(g, dt));
        s->p.d[i] = vadd(s->x.d[i], vmuls(s->v.d[i], dt));
    }
}

static inline void add_delta(vo_solver* s, uint32_t i, v3 c)
{
    s->dl.d[i].x = s->dl.d[i].x + c.x;
    s->dl.d[i].y = s->dl.d[i].y + c.y;
    s->dl.d[i].z = s->dl.d[i].z + c.z;
}

/* SolveStretch_Kernel, :65-102 */
static void solve_stretch(vo_solver* s)
{
    const v3* p = s->p.d;
    for (size_t k = 0; k < s->st_rest.n; ++k) {
        const size_t c = s->reverse_sums ? s->st_rest.n - 1 - k : k;
        int i1 = s->st_idx.d[2 * c], i2 = s->st_idx.d[2 * c + 1];
        float rest = s->st_rest.d[c];
        v3 diff = vsub(p[i1], p[i2]);
        float d = vlen(diff);
        float w1 = s->w.d[i1], w2 = s->w.d[i2];
        if (d != rest && w1 + w2 > 0) {
            v3 grad = vdivs(diff, d + VO_EPSILON);
            float denom = w1 + w2;
            float lambda = (d - rest) / denom;
            v3 common = vmuls(grad, lambda);
            add_delta(s, (uint32_t)i1, vmuls(common, -w1));
            add_delta(s, (uint32_t)i2, vmuls(common, w2));
            s->cnt.d[i1]++;
            s->cnt.d[i2]++;
        }
    }
}

/* SolveAttachment_Kernel, :205-235 */
static void solve_attach(vo_solver* s)
{
    for (size_t k = 0; k < s->at_pid.n; ++k) {
        const size_t c = s->reverse_sums ? s->at_pid.n - 1 - k : k;
        uint32_t pid = (uint32_t)s->at_pid.d[c];
        v3 slot = s->slots.d[s->at_slot.d[c]];
        float target = s->at_dist.d[c] * s->P.long_range_stretchiness;
        if (s->w.d[pid] == 0 && target > 0) continue;
        v3 diff = vsub(s->p.d[pid], slot);
        float d = vlen(diff);
        if (d > target) {
            v3 corr = vadd(vneg(diff), vmuls(vdivs(diff, d), target));
            add_delta(s, pid, corr);
            s->cnt.d[pid]++;
        }
    }
}

/* SolveBending_Kernel, :117-189 */
static void solve_bending(vo_solver* s, float dt)
{
    const v3* P = s->p.d;
    for (size_t k = 0; k < s->bd_rest.n; ++k) {
        const size_t c = s->reverse_sums ? s->bd_rest.n - 1 - k : k;
        uint32_t i0 = s->bd_idx.d[4 * c], i1 = s->bd_idx.d[4 * c + 1];
        uint32_t i2 = s->bd_idx.d[4 * c + 2], i3 = s->bd_idx.d[4 * c + 3];
        float rest = s->bd_rest.d[c];
        float w0 = s->w.d[i0], w1 = s->w.d[i1], w2 = s->w.d[i2], w3 = s->w.d[i3];
        v3 p0 = P[i0], p1 = P[i1], p2 = P[i2], p3 = P[i3];
        v3 e = vsub(p3, p2);
        float elen = vlen(e);
        if (elen < VO_EPSILON) continue;
        float inv = 1.0f / elen;
        v3 n1 = vcross(vsub(p2, p0), vsub(p3, p0));
        n1 = vdivs(n1, vdot(n1, n1));
        v3 n2 = vcross(vsub(p3, p1), vsub(p2, p1));
        n2 = vdivs(n2, vdot(n2, n2));
        v3 d0 = vmuls(n1, elen);
        v3 d1 = vmuls(n2, elen);
        v3 d2 = vadd(vmuls(n1, vdot(vsub(p0, p3), e) * inv), vmuls(n2, vdot(vsub(p1, p3), e) * inv));
        v3 d3 = vadd(vmuls(n1, vdot(vsub(p2, p0), e) * inv), vmuls(n2, vdot(vsub(p2, p1), e) * inv));
        n1 = vnormalize(n1);
        n2 = vnormalize(n2);
        float dt_ = gclamp(vdot(n1, n2), -1.0f, 1.0f);
        float phi = vo_acosf(dt_);
        float lambda = w0 * vdot(d0, d0) + w1 * vdot(d1, d1);
        lambda = lambda + w2 * vdot(d2, d2);
        lambda = lambda + w3 * vdot(d3, d3);
        if (lambda < VO_EPSILON) continue;
        float xpbd = s->P.bend_compliance / dt / dt;
        lambda = (phi - rest) / (lambda + xpbd);
        if (vdot(vcross(n1, n2), e) > 0.0f) lambda = -lambda;
        add_delta(s, i0, vmuls(d0, -w0 * lambda));
        add_delta(s, i1, vmuls(d1, -w1 * lambda));
        add_delta(s, i2, vmuls(d2, -w2 * lambda));
        add_delta(s, i3, vmuls(d3, -w3 * lambda));
        s->cnt.d[i0]++;
        s->cnt.d[i1]++;
        s->cnt.d[i2]++;
        s->cnt.d[i3]++;
    }
}

/* ApplyDeltas_Kernel, :253-264 */
static void apply_deltas(vo_solver* s)
{
    for (uint32_t i = 0; i < s->n; ++i) {
        float count = (float)s->cnt.d[i];
        if (count > 0) {
            s->p.d[i] = vadd(s->p.d[i], vmuls(vdivs(s->dl.d[i], count), s->P.relaxation_factor));
            s->dl.d[i] = V(0, 0, 0);
            s->cnt.d[i] = 0;
        }
    }
}

/* CollideParticles_Kernel, :329-373 (writes, not adds, deltas and counts) */
static void collide_particles(vo_solver* s)
{
    const uint32_t N = s->n;
    const uint32_t mn = (uint32_t)s->P.max_num_neighbors;
    const float diam = s->P.particle_diameter;
    for (uint32_t i = 0; i < N; ++i) {
        v3 delta = V(0, 0, 0);
        int count = 0;
        v3 pi = s->p.d[i];
        v3 veli = vsub(pi, s->x.d[i]);
        float wi = s->w.d[i];
        for (uint32_t k = 0; k < mn; ++k) {
            uint32_t j = s->nbr[i + (size_t)k * N];
            if (j > N) break;
            float wj = s->w.d[j];
            float denom = wi + wj;
            if (denom <= 0) continue;
            v3 pj = s->p.d[j];
            v3 diff = vsub(pi, pj);
            float d = vlen(diff);
            if (d >= diam) continue;
            v3 grad = vdivs(diff, d + VO_EPSILON);
            float lambda = (d - diam) / denom;
            v3 common = vmuls(grad, lambda);
            count++;
            delta = vsub(delta, vmuls(common, wi));
            v3 relvel = vsub(veli, vsub(pj, s->x.d[j]));
            v3 fr = friction_of(common, relvel, s->P.friction);
            delta = vadd(delta, vmuls(fr, wi));
        }
        s->dl.d[i] = delta;
        s->cnt.d[i] = count;
    }
}

/* Finalize_Kernel, :388-407 */
static void finalize(vo_solver* s, float dt)
{
    for (uint32_t i = 0; i < s->n; ++i) {
        v3 np = s->p.d[i];
        v3 rv = vdivs(vsub(np, s->x.d[i]), dt);
        float rl = vlen(rv);
        if (rl > s->P.max_speed) {
            rv = vmuls(vdivs(rv, rl), s->P.max_speed);
            np = vadd(s->x.d[i], vmuls(rv, dt));
        }
        s->v.d[i] = vmuls(rv, 1.0f - s->P.damping * dt);
        s->x.d[i] = np;
    }
}

/* ComputeNormal, :419-465 */
static void compute_normals(vo_solver* s)
{
    if (!s->n) return;
    for (uint32_t i = 0; i < s->n; ++i) s->nrm.d[i] = V(0, 0, 0);
    for (size_t t = 0; t + 2 < s->tri.n; t += 3) {
        uint32_t a = s->tri.d[t], b = s->tri.d[t + 1], c = s->tri.d[t + 2];
        v3 p1 = s->x.d[a], p2 = s->x.d[b], p3 = s->x.d[c];
        v3 nn = vcross(vsub(p2, p1), vsub(p3, p1));
        uint32_t ids[3] = {a, b, c};
        for (int k = 0; k < 3; ++k) {
            v3* d = &s->nrm.d[ids[k]];
            d->x = d->x + nn.x;
            d->y = d->y + nn.y;
            d->z = d->z + nn.z;
        }
    }
    for (uint32_t i = 0; i < s->n; ++i) s->nrm.d[i] = vnormalize(s->nrm.d[i]);
}

/* ------------------------------------------------------------------ spatial hash */

/* ComputeIntCoord / HashCoords, SpatialHashGPU.cu:13-22 */
VO_API int32_t vo_int_coord(float v, float spacing) { return (int32_t)floorf(v / spacing); }
VO_API int32_t vo_hash_coords(int32_t x, int32_t y, int32_t z, int32_t table)
{
    int32_t h = (x * 92837111) ^ (y * 689287499) ^ (z * 283923481); /* wraps: -fwrapv */
    return abs(h % table);
}

/* HashObjects, SpatialHashGPU.cu:159-196, on float3 arrays.  The stable radix sort
 * (cub SortPairs) is a stable counting sort by key here: same permutation. */
VO_API void vo_hash_objects(uint32_t* phash, uint32_t* pindex, uint32_t* cstart, uint32_t* cend,
                            uint32_t* nbr, const float* pos, const float* orig,
                            const vt_hash_params* hp)
{
    const uint32_t N = hp->num_objects;
    const int32_t T = hp->table_size;
    const float sp = hp->cell_spacing;
    uint32_t* keys = (uint32_t*)malloc(sizeof(uint32_t) * (N ? N : 1));
    uint32_t* count = (uint32_t*)calloc((size_t)T + 1, sizeof(uint32_t));
    /* ComputeParticleHash_Kernel, :34-42 */
    for (uint32_t i = 0; i < N; ++i) {
        int32_t x = vo_int_coord(pos[3 * i], sp), y = vo_int_coord(pos[3 * i + 1], sp),
                z = vo_int_coord(pos[3 * i + 2], sp);
        keys[i] = (uint32_t)vo_hash_coords(x, y, z, T);
        count[keys[i]]++;
    }
    /* stable sort by key (Sort, :133-157) */
    uint32_t run = 0;
    for (int32_t h = 0; h < T; ++h) {
        uint32_t c = count[h];
        count[h] = run;
        run += c;
    }
    for (uint32_t i = 0; i < N; ++i) {
        uint32_t at = count[keys[i]]++;
        phash[at] = keys[i];
        pindex[at] = i;
    }
    /* cudaMemsetAsync(cellStart, 0xff, 4*(T+1)) + FindCellStart_Kernel, :44-77, 185 */
    for (int32_t h = 0; h <= T; ++h) cstart[h] = 0xffffffffu;
    for (uint32_t t = 0; t < N; ++t) {
        uint32_t h = phash[t];
        if (t == 0 || h != phash[t - 1]) {
            cstart[h] = t;
            if (t > 0) cend[phash[t - 1]] = t;
        }
        if (t == N - 1) cend[h] = t + 1;
    }
    /* CacheNeighbors_Kernel, :79-130 */
    const uint32_t MN = hp->max_num_neighbors;
    const uint64_t limit = (uint64_t)N * MN;
    for (uint32_t t = 0; t < N; ++t) {
        uint32_t id = pindex[t];
        v3 position = V(pos[3 * id], pos[3 * id + 1], pos[3 * id + 2]);
        v3 orig_i = V(orig[3 * id], orig[3 * id + 1], orig[3 * id + 2]);
        int32_t ix = vo_int_coord(position.x, sp), iy = vo_int_coord(position.y, sp),
                iz = vo_int_coord(position.z, sp);
        uint64_t ni = id;
        int full = 0;
        for (int32_t x = ix - 1; x <= ix + 1 && !full; ++x)
            for (int32_t y = iy - 1; y <= iy + 1 && !full; ++y)
                for (int32_t z = iz - 1; z <= iz + 1 && !full; ++z) {
                    int32_t h = vo_hash_coords(x, y, z, T);
                    uint32_t start = cstart[h];
                    if (start == 0xffffffffu) continue;
                    uint32_t end = cend[h];
                    if (start + MN < end) end = start + MN;
                    for (uint32_t k = start; k < end; ++k) {
                        uint32_t nb = pindex[k];
                        v3 pj = V(pos[3 * nb], pos[3 * nb + 1], pos[3 * nb + 2]);
                        v3 oj = V(orig[3 * nb], orig[3 * nb + 1], orig[3 * nb + 2]);
                        v3 d1 = vsub(position, pj), d2 = vsub(orig_i, oj);
                        if (nb != id && vdot(d1, d1) < hp->cell_spacing2 &&
                            vdot(d2, d2) > hp->particle_diameter2) {
                            nbr[ni] = nb;
                            ni += N;
                            if (ni >= limit) { full = 1; break; }
                        }
                    }
                }
        if (!full && ni < limit) nbr[ni] = 0xffffffffu;
    }
    free(keys);
    free(count);
}

/* SpatialHashGPU::Hash, SpatialHashGPU.hpp:41-52 */
static void solver_hash(vo_solver* s)
{
    vt_hash_params hp;
    hp.num_objects = s->n;
    hp.cell_spacing = s->cell_spacing;
    hp.cell_spacing2 = s->cell_spacing * s->cell_spacing;
    hp.table_size = s->table_size;
    hp.max_num_neighbors = (uint32_t)s->P.max_num_neighbors;
    hp.particle_diameter2 = s->P.particle_diameter * s->P.particle_diameter;
    vo_hash_objects(s->hkey, s->hidx, s->cstart, s->cend, s->nbr, (const float*)s->p.d,
                    (const float*)s->x0.d, &hp);
    s->hashed = 1;
}

/* ------------------------------------------------------------------ Simulate */

/* VtClothSolverGPU::Simulate, Velvet/VtClothSolverGPU.hpp:56-111, after the caller's
 * per-frame parameters are written into the parameter block. */
VO_API void vo_simulate(vo_solver* s, float frame_dt, int32_t substeps, int32_t iterations,
                        float relax, float friction, float margin, float diameter)
{
    s->P.num_substeps = substeps;
    s->P.num_iterations = iterations;
    s->P.relaxation_factor = relax;
    s->P.friction = friction;
    s->P.collision_margin = margin;
    s->P.particle_diameter = diameter;
    if (s->n == 0) return;
    float frame = frame_dt;
    float sub = frame_dt / (float)substeps;
    collide_sdf(s, s->x.d, s->x.d, frame);
    for (int st = 0; st < substeps; ++st) {
        predict(s, sub);
        if (s->P.enable_self_collision) {
            if (st % s->P.interleaved_hash == 0) solver_hash(s);
            collide_particles(s);
            apply_deltas(s);
        }
        collide_sdf(s, s->p.d, s->x.d, sub);
        for (int it = 0; it < iterations; ++it) {
            solve_stretch(s);
            solve_attach(s);
            solve_bending(s, sub);
            apply_deltas(s);
        }
        finalize(s, sub);
    }
    compute_normals(s);
}

/* ------------------------------------------------------------------ accessors */
#define VO_GET_POSITIONS 0
#define VO_GET_VELOCITIES 1
#define VO_GET_PREDICTED 2
#define VO_GET_NORMALS 3
#define VO_GET_INV_MASS 4
#define VO_GET_HASH 5
#define VO_GET_INDEX 6
#define VO_GET_CELL_START 7
#define VO_GET_CELL_END 8
#define VO_GET_NEIGHBORS 9
#define VO_GET_INITIAL 10

/* Copies an internal array into dst (sizes as documented in tests/oracle.py). */
VO_API int vo_get(const vo_solver* s, int what, void* dst)
{
    size_t n = s->n;
    switch (what) {
    case VO_GET_POSITIONS: memcpy(dst, s->x.d, n * 12); return 0;
    case VO_GET_VELOCITIES: memcpy(dst, s->v.d, n * 12); return 0;
    case VO_GET_PREDICTED: memcpy(dst, s->p.d, n * 12); return 0;
    case VO_GET_NORMALS: memcpy(dst, s->nrm.d, n * 12); return 0;
    case VO_GET_INV_MASS: memcpy(dst, s->w.d, n * 4); return 0;
    case VO_GET_HASH: memcpy(dst, s->hkey, n * 4); return 0;
    case VO_GET_INDEX: memcpy(dst, s->hidx, n * 4); return 0;
    case VO_GET_CELL_START: memcpy(dst, s->cstart, ((size_t)s->table_size + 1) * 4); return 0;
    case VO_GET_CELL_END: memcpy(dst, s->cend, (size_t)s->table_size * 4); return 0;
    case VO_GET_NEIGHBORS:
        memcpy(dst, s->nbr, n * (size_t)s->P.max_num_neighbors * 4);
        return 0;
    case VO_GET_INITIAL: memcpy(dst, s->x0.d, n * 12); return 0;
    }
    return -1;
}

VO_API void vo_set_positions(vo_solver* s, uint32_t first, uint32_t count, const float* src)
{
    memcpy(s->x.d + first, src, (size_t)count * 12);
}
VO_API void vo_set_velocities(vo_solver* s, uint32_t first, uint32_t count, const float* src)
{
    memcpy(s->v.d + first, src, (size_t)count * 12);
}
VO_API void vo_set_inv_mass(vo_solver* s, uint32_t first, uint32_t count, const float* src)
{
    memcpy(s->w.d + first, src, (size_t)count * 4);
}
VO_API void vo_slot_set(vo_solver* s, int32_t slot, const float* xyz)
{
    s->slots.d[slot] = V(xyz[0], xyz[1], xyz[2]);
}
VO_API uint32_t vo_num_constraints(const vo_solver* s, int kind)
{
    switch (kind) {
    case 0: return (uint32_t)s->st_rest.n;
    case 1: return (uint32_t)s->at_pid.n;
    case 2: return (uint32_t)s->bd_rest.n;
    case 3: return (uint32_t)s->slots.n;
    }
    return 0;
}
/* Constraint arrays, for comparing the builders: kind 0 stretch (2 ints + rest per
 * constraint), 1 attach (pid, slot, dist), 2 bend (4 uints + angle). */
VO_API void vo_get_constraints(const vo_solver* s, int kind, int32_t* ints, float* floats)
{
    if (kind == 0) {
        memcpy(ints, s->st_idx.d, s->st_idx.n * 4);
        memcpy(floats, s->st_rest.d, s->st_rest.n * 4);
    } else if (kind == 1) {
        for (size_t c = 0; c < s->at_pid.n; ++c) {
            ints[2 * c] = s->at_pid.d[c];
            ints[2 * c + 1] = s->at_slot.d[c];
        }
        memcpy(floats, s->at_dist.d, s->at_dist.n * 4);
    } else if (kind == 2) {
        memcpy(ints, s->bd_idx.d, s->bd_idx.n * 4);
        memcpy(floats, s->bd_rest.d, s->bd_rest.n * 4);
    }
}
