/*
 * vt_cpu_solver.c — CPU BASELINE, timing only.  TEST / BENCHMARK INFRASTRUCTURE.
 *
 * A restatement of the reference's CPU cloth solver VtClothSolverCPU
 * (Velvet/VtClothSolverCPU.hpp:17-434) and its spatial hash SpatialHashCPU
 * (Velvet/SpatialHashCPU.hpp:11-124), used by bench.py to report the reference's CPU
 * solver speed on this machine's cores.  It is a different algorithm from the GPU
 * solver (sequential Gauss-Seidel, unilateral stretch, another bending gradient, hard
 * pinned attachments, collisions inside the iteration loop, hash once per frame, no
 * initial-position filter, no speed clamp), so its results are not compared with
 * anything; only its particle-iterations per second are reported.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/velvet_gb300.h"

#if defined(_WIN32)
#define VC_API __declspec(dllexport)
#else
#define VC_API __attribute__((visibility("default")))
#endif

typedef struct { float x, y, z; } v3;
static inline v3 V(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline v3 add(v3 a, v3 b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub(v3 a, v3 b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 mul(v3 a, float s) { return V(a.x * s, a.y * s, a.z * s); }
static inline v3 dv(v3 a, float s) { return V(a.x / s, a.y / s, a.z / s); }
static inline float dot(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline float len(v3 a) { return sqrtf(dot(a, a)); }
static inline v3 nrmz(v3 a) { return mul(a, 1.0f / sqrtf(dot(a, a))); }
static inline v3 crs(v3 a, v3 b) { return V(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y); }

typedef struct { int i, j; float rest; } vc_stretch;
typedef struct { int i; v3 pos; } vc_attach;
typedef struct { int i1, i2, i3, i4; float angle; } vc_bend;

typedef struct vc_solver {
    int n, res;
    v3 *x, *p, *v, *nrm;
    float* w;
    uint32_t* tri;
    int ntri;
    vc_stretch* st;
    int nst;
    vc_attach* at;
    int nat;
    vc_bend* bd;
    int nbd;
    float diameter;
    vt_params P;
    vt_sdf_collider* col;
    int ncol;
    /* SpatialHashCPU */
    float spacing;
    int T;
    int *cell_start, *entries;
    int **nb;
    int *nb_n, *nb_cap;
} vc_solver;

/* VtClothSolverCPU::Initialize + Generate* (:42-176) for a grid mesh from
 * Scene::GenerateClothMesh with the given model matrix. */
VC_API vc_solver* vc_create(const float* xyz, int n, const uint32_t* tri, int ntri_idx, const float* m,
                            int res, const int* attached, int nattached, const vt_params* P)
{
    vc_solver* s = (vc_solver*)calloc(1, sizeof(vc_solver));
    s->n = n;
    s->res = res;
    s->P = *P;
    s->x = (v3*)malloc(sizeof(v3) * n);
    s->p = (v3*)calloc(n, sizeof(v3));
    s->v = (v3*)calloc(n, sizeof(v3));
    s->nrm = (v3*)calloc(n, sizeof(v3));
    s->w = (float*)malloc(sizeof(float) * n);
    for (int i = 0; i < n; ++i) {
        float a = xyz[3 * i], b = xyz[3 * i + 1], c = xyz[3 * i + 2];
        s->x[i] = V((m[0] * a + m[4] * b) + (m[8] * c + m[12]), (m[1] * a + m[5] * b) + (m[9] * c + m[13]),
                    (m[2] * a + m[6] * b) + (m[10] * c + m[14]));
        s->w[i] = 1.0f;
    }
    s->tri = (uint32_t*)malloc(sizeof(uint32_t) * (ntri_idx ? ntri_idx : 1));
    memcpy(s->tri, tri, sizeof(uint32_t) * ntri_idx);
    s->ntri = ntri_idx;
    s->diameter = len(sub(s->x[0], s->x[res + 1]));  /* :61 */
    s->spacing = s->diameter;
    s->T = 2 * n;
    s->cell_start = (int*)calloc(s->T + 1, sizeof(int));
    s->entries = (int*)calloc(n, sizeof(int));
    s->nb = (int**)calloc(n, sizeof(int*));
    s->nb_n = (int*)calloc(n, sizeof(int));
    s->nb_cap = (int*)calloc(n, sizeof(int));
    /* GenerateStretch :109-151 */
    int V1 = res + 1;
    s->st = (vc_stretch*)malloc(sizeof(vc_stretch) * (4 * V1 * V1 + 4));
#define AT(a, b) ((a) * V1 + (b))
#define ADD_ST(A, B) do { s->st[s->nst].i = (A); s->st[s->nst].j = (B); \
        s->st[s->nst].rest = len(sub(s->x[(A)], s->x[(B)])); s->nst++; } while (0)
    for (int a = 0; a < V1; ++a)
        for (int b = 0; b < V1; ++b) {
            if (b != res) ADD_ST(AT(a, b), AT(a, b + 1));
            if (a != res) ADD_ST(AT(a, b), AT(a + 1, b));
            if (b != res && a != res) {
                ADD_ST(AT(a, b), AT(a + 1, b + 1));
                ADD_ST(AT(a, b + 1), AT(a + 1, b));
            }
        }
    /* GenerateAttachment :153-160 */
    s->at = (vc_attach*)malloc(sizeof(vc_attach) * (nattached ? nattached : 1));
    for (int k = 0; k < nattached; ++k) {
        s->at[k].i = attached[k];
        s->at[k].pos = s->x[attached[k]];
        s->w[attached[k]] = 0;
    }
    s->nat = nattached;
    /* GenerateBending :162-176 */
    s->bd = (vc_bend*)malloc(sizeof(vc_bend) * (ntri_idx / 6 + 1));
    for (int i = 0; i + 5 < ntri_idx; i += 6) {
        vc_bend b = {(int)tri[i], (int)tri[i + 1], (int)tri[i + 2], (int)tri[i + 5], 0.0f};
        s->bd[s->nbd++] = b;
    }
    return s;
}

VC_API void vc_destroy(vc_solver* s)
{
    if (!s) return;
    for (int i = 0; i < s->n; ++i) free(s->nb[i]);
    free(s->nb); free(s->nb_n); free(s->nb_cap); free(s->cell_start); free(s->entries);
    free(s->x); free(s->p); free(s->v); free(s->nrm); free(s->w); free(s->tri);
    free(s->st); free(s->at); free(s->bd); free(s->col);
    free(s);
}

VC_API void vc_colliders_set(vc_solver* s, const vt_sdf_collider* c, int n)
{
    free(s->col);
    s->col = (vt_sdf_collider*)malloc(sizeof(vt_sdf_collider) * (n ? n : 1));
    memcpy(s->col, c, sizeof(vt_sdf_collider) * n);
    s->ncol = n;
}

/* SpatialHashCPU (:14-124) */
static int ic(float v, float sp) { return (int)floorf(v / sp); }
static int hc(int x, int y, int z, int T)
{
    int h = (x * 92837111) ^ (y * 689287499) ^ (z * 283923481);
    return abs(h % T);
}
static void push_nb(vc_solver* s, int i, int j)
{
    if (s->nb_n[i] == s->nb_cap[i]) {
        s->nb_cap[i] = s->nb_cap[i] ? 2 * s->nb_cap[i] : 32;
        s->nb[i] = (int*)realloc(s->nb[i], sizeof(int) * s->nb_cap[i]);
    }
    s->nb[i][s->nb_n[i]++] = j;
}
static void hash_objects(vc_solver* s, const v3* pos)
{
    int T = s->T;
    memset(s->cell_start, 0, sizeof(int) * (T + 1));
    for (int i = 0; i < s->n; ++i) s->cell_start[hc(ic(pos[i].x, s->spacing), ic(pos[i].y, s->spacing), ic(pos[i].z, s->spacing), T)]++;
    int start = 0;
    for (int h = 0; h < T; ++h) { start += s->cell_start[h]; s->cell_start[h] = start; }
    s->cell_start[T] = start;
    for (int i = 0; i < s->n; ++i) {
        int h = hc(ic(pos[i].x, s->spacing), ic(pos[i].y, s->spacing), ic(pos[i].z, s->spacing), T);
        s->cell_start[h]--;
        s->entries[s->cell_start[h]] = i;
    }
    for (int i = 0; i < s->n; ++i) {
        s->nb_n[i] = 0;
        int x0 = ic(pos[i].x, s->spacing), y0 = ic(pos[i].y, s->spacing), z0 = ic(pos[i].z, s->spacing);
        for (int x = x0 - 1; x <= x0 + 1; ++x)
            for (int y = y0 - 1; y <= y0 + 1; ++y)
                for (int z = z0 - 1; z <= z0 + 1; ++z) {
                    int h = hc(x, y, z, T);
                    for (int k = s->cell_start[h]; k < s->cell_start[h + 1]; ++k) push_nb(s, i, s->entries[k]);
                }
    }
}

/* Collider::ComputeSDF (Velvet/Collider.hpp:43-77): plane at margin, sphere */
static v3 sdf(const vc_solver* s, const vt_sdf_collider* c, v3 p)
{
    float m = s->P.collision_margin;
    if (c->type == VT_COLLIDER_PLANE) {
        if (p.y < m) return V(0, m - p.y, 0);
    } else if (c->type == VT_COLLIDER_SPHERE) {
        v3 ctr = V(c->position[0], c->position[1], c->position[2]);
        float r = c->scale[0] + m;
        v3 d = sub(p, ctr);
        float dist = len(d);
        if (dist < r) return mul(dv(d, dist), r - dist);
    }
    return V(0, 0, 0);
}
static v3 friction(const vc_solver* s, v3 corr, v3 rel)
{
    v3 f = V(0, 0, 0);
    float cl = len(corr);
    if (s->P.friction > 0 && cl > 0) {
        v3 nn = dv(corr, cl);
        v3 t = sub(rel, mul(nn, dot(rel, nn)));
        float tl = len(t);
        float mt = cl * s->P.friction;
        f = mul(V(-t.x, -t.y, -t.z), fminf(mt / tl, 1.0f));
    }
    return f;
}
static void collide_sdf(vc_solver* s, v3* pos)
{
    for (int i = 0; i < s->n; ++i)
        for (int k = 0; k < s->ncol; ++k) {
            v3 corr = sdf(s, &s->col[k], pos[i]);
            pos[i] = add(pos[i], corr);
            v3 rel = sub(pos[i], s->x[i]);
            pos[i] = add(pos[i], friction(s, corr, rel));
        }
}
static void predict(vc_solver* s, float dt)
{
    v3 g = V(s->P.gravity[0], s->P.gravity[1], s->P.gravity[2]);
    for (int i = 0; i < s->n; ++i) {
        s->v[i] = add(s->v[i], mul(g, dt));
        s->p[i] = add(s->x[i], mul(s->v[i], dt));
    }
}

/* VtClothSolverCPU::Simulate (:69-100) for one frame */
VC_API void vc_simulate(vc_solver* s, float frame_dt, int substeps, int iterations)
{
    const float eps = 1e-6f;
    float sub_dt = frame_dt / (float)substeps;
    collide_sdf(s, s->x);
    predict(s, frame_dt);
    hash_objects(s, s->p);
    for (int st = 0; st < substeps; ++st) {
        predict(s, sub_dt);
        for (int it = 0; it < iterations; ++it) {
            for (int c = 0; c < s->nst; ++c) { /* SolveStretch :194-219, unilateral */
                int i = s->st[c].i, j = s->st[c].j;
                v3 d = sub(s->p[i], s->p[j]);
                float dist = len(d);
                float wi = s->w[i], wj = s->w[j];
                if (dist > s->st[c].rest && wi + wj > 0) {
                    v3 g = dv(d, dist + eps);
                    float lam = (dist - s->st[c].rest) / (wi + wj);
                    s->p[i] = sub(s->p[i], mul(g, wi * lam));
                    s->p[j] = add(s->p[j], mul(g, wj * lam));
                }
            }
            float xpbd = s->P.bend_compliance / sub_dt / sub_dt;
            for (int c = 0; c < s->nbd; ++c) { /* SolveBending :221-272 */
                int i1 = s->bd[c].i3, i2 = s->bd[c].i2, i3 = s->bd[c].i1, i4 = s->bd[c].i4;
                float w1 = s->w[i1], w2 = s->w[i2], w3 = s->w[i3], w4 = s->w[i4];
                v3 p1 = s->p[i1], p2 = sub(s->p[i2], p1), p3 = sub(s->p[i3], p1), p4 = sub(s->p[i4], p1);
                v3 n1 = nrmz(crs(p2, p3)), n2 = nrmz(crs(p2, p4));
                float d = dot(n1, n2);
                d = d < 0 ? 0 : (d > 1 ? 1 : d);
                float ang = acosf(d);
                if (ang < eps || isnan(d)) continue;
                float l23 = len(crs(p2, p3)) + eps, l24 = len(crs(p2, p4)) + eps;
                v3 q3 = dv(add(crs(p2, n2), mul(crs(n1, p2), d)), l23);
                v3 q4 = dv(add(crs(p2, n1), mul(crs(n2, p2), d)), l24);
                v3 q2 = sub(mul(dv(add(crs(p3, n2), mul(crs(n1, p3), d)), l23), -1.0f),
                            dv(add(crs(p4, n1), mul(crs(n2, p4), d)), l24));
                v3 q1 = sub(sub(mul(q2, -1.0f), q3), q4);
                float den = xpbd + (((w1 * dot(q1, q1) + w2 * dot(q2, q2)) + w3 * dot(q3, q3)) + w4 * dot(q4, q4));
                if (den < eps) continue;
                float lam = sqrtf(1.0f - d * d) * (ang - s->bd[c].angle) / den;
                s->p[i1] = add(s->p[i1], mul(q1, w1 * lam));
                s->p[i2] = add(s->p[i2], mul(q2, w2 * lam));
                s->p[i3] = add(s->p[i3], mul(q3, w3 * lam));
                s->p[i4] = add(s->p[i4], mul(q4, w4 * lam));
            }
            for (int i = 0; i < s->n; ++i) /* CollideParticles :316-349 */
                for (int k = 0; k < s->nb_n[i]; ++k) {
                    int j = s->nb[i][k];
                    if (i >= j) continue;
                    v3 d = sub(s->p[i], s->p[j]);
                    float dist = len(d);
                    float wi = s->w[i], wj = s->w[j];
                    if (dist < s->diameter && wi + wj > 0) {
                        v3 g = dv(d, dist + eps);
                        v3 common = mul(g, (dist - s->diameter) / (wi + wj));
                        s->p[i] = sub(s->p[i], mul(common, wi));
                        s->p[j] = add(s->p[j], mul(common, wj));
                        v3 rel = sub(sub(s->p[i], s->x[i]), sub(s->p[j], s->x[j]));
                        v3 f = friction(s, common, rel);
                        s->p[i] = add(s->p[i], mul(f, wi));
                        s->p[j] = sub(s->p[j], mul(f, wj));
                    }
                }
            collide_sdf(s, s->p);
            for (int k = 0; k < s->nat; ++k) s->p[s->at[k].i] = s->at[k].pos; /* SolveAttachment */
        }
        float damp = 1.0f - s->P.damping * sub_dt; /* Finalize :351-361 */
        for (int i = 0; i < s->n; ++i) {
            s->v[i] = mul(dv(sub(s->p[i], s->x[i]), sub_dt), damp);
            s->x[i] = s->p[i];
        }
    }
    for (int i = 0; i < s->n; ++i) s->nrm[i] = V(0, 0, 0); /* ComputeNormals :382-405 */
    for (int t = 0; t + 2 < s->ntri; t += 3) {
        uint32_t a = s->tri[t], b = s->tri[t + 1], c = s->tri[t + 2];
        v3 nn = crs(sub(s->x[b], s->x[a]), sub(s->x[c], s->x[a]));
        s->nrm[a] = add(s->nrm[a], nn);
        s->nrm[b] = add(s->nrm[b], nn);
        s->nrm[c] = add(s->nrm[c], nn);
    }
    for (int i = 0; i < s->n; ++i) s->nrm[i] = nrmz(s->nrm[i]);
}

VC_API void vc_positions(const vc_solver* s, float* out) { memcpy(out, s->x, sizeof(v3) * s->n); }
