// vt_capi.cu — extern "C" entry points of the plain solver and the spatial hash
// (declared in include/velvet_gb300.h).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "vt_host.h"
#include "vt_math.cuh"

namespace vt {
const std::string& last_error();
}

using vt::AttachOp;
using vt::ClothRec;
using vt::HostSolver;


#define VT_CHECK(cond, code, msg)   \
    do {                            \
        if (!(cond)) {              \
            vt::set_error(msg);     \
            return code;            \
        }                           \
    } while (0)

#define VT_TRY_CUDA(call, what)                                  \
    do {                                                         \
        cudaError_t e_ = (call);                                 \
        if (e_ != cudaSuccess) return vt::cuda_fail(e_, what);   \
    } while (0)

#define VT_GUARD_BEGIN try {
#define VT_GUARD_END                                                          \
    }                                                                         \
    catch (const std::bad_alloc&) {                                           \
        vt::set_error("host allocation failed");                              \
        return VT_ERR_OUT_OF_MEMORY;                                          \
    }                                                                         \
    catch (...) {                                                             \
        vt::set_error("unexpected host exception");                           \
        return VT_ERR_STATE;                                                  \
    }

// Copies the device's dynamic state (x, v, inverse mass) back into the host staging so
// that registration can extend it.
vt_status vt::pull_state(vt::SolverImpl* s)
{
    if (!s->on_device || !s->world.built()) return VT_OK;
    const size_t n = s->h.n();
    if (n) {
        VT_TRY_CUDA(cudaStreamSynchronize(s->stream), "sync");
        VT_TRY_CUDA(cudaMemcpy2D(s->h.x.data(), 12, s->world.d.x, 16, 12, n, cudaMemcpyDeviceToHost), "pull x");
        VT_TRY_CUDA(cudaMemcpy2D(s->h.v.data(), 12, s->world.d.v, 16, 12, n, cudaMemcpyDeviceToHost), "pull v");
        VT_TRY_CUDA(cudaMemcpy2D(s->h.w.data(), 4, &s->world.d.x->w, 16, 4, n, cudaMemcpyDeviceToHost), "pull w");
    }
    s->on_device = false;
    return VT_OK;
}

static vt_status make_topology_change(vt_solver* s)
{
    vt_status st = vt::pull_state(s);
    if (st != VT_OK) return st;
    s->topo_dirty = true;
    return VT_OK;
}

extern "C" {

void vt_params_default(vt_params* P)
{
    if (!P) return;
    std::memset(P, 0, sizeof(*P));
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

const char* vt_status_string(vt_status s)
{
    switch (s) {
    case VT_OK: return "VT_OK";
    case VT_ERR_INVALID_ARGUMENT: return "VT_ERR_INVALID_ARGUMENT";
    case VT_ERR_OUT_OF_MEMORY: return "VT_ERR_OUT_OF_MEMORY";
    case VT_ERR_CUDA: return "VT_ERR_CUDA";
    case VT_ERR_NOT_FOUND: return "VT_ERR_NOT_FOUND";
    case VT_ERR_STATE: return "VT_ERR_STATE";
    case VT_ERR_CAPACITY: return "VT_ERR_CAPACITY";
    case VT_ERR_NUMERIC: return "VT_ERR_NUMERIC";
    case VT_ERR_TIMEOUT: return "VT_ERR_TIMEOUT";
    }
    return "VT_ERR_UNKNOWN";
}

const char* vt_last_error(void) { return vt::last_error().c_str(); }

int32_t vt_abi_version(void) { return VT_ABI_VERSION; }

static bool params_valid(const vt_params* p)
{
    return p->num_substeps >= 1 && p->num_iterations >= 0 && p->max_num_neighbors >= 1 &&
           p->max_num_neighbors <= 64 && p->interleaved_hash >= 1 && p->delta_time > 0;
}

vt_status vt_solver_create(const vt_params* params, vt_solver** out)
{
    VT_CHECK(out, VT_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    VT_GUARD_BEGIN
    vt_params P;
    if (params) P = *params;
    else vt_params_default(&P);
    VT_CHECK(params_valid(&P), VT_ERR_INVALID_ARGUMENT, "invalid parameter block");
    vt_solver* s = new vt_solver();
    s->h.P = P;
    s->h.P.num_particles = 0;
    *out = s;
    return VT_OK;
    VT_GUARD_END
}

vt_status vt_solver_destroy(vt_solver* s)
{
    if (!s) return VT_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    delete s;
    return VT_OK;
}

vt_status vt_solver_get_params(const vt_solver* s, vt_params* out)
{
    VT_CHECK(s && out, VT_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = s->h.P;
    return VT_OK;
}

vt_status vt_solver_set_params(vt_solver* s, const vt_params* p)
{
    VT_CHECK(s && p, VT_ERR_INVALID_ARGUMENT, "NULL argument");
    VT_CHECK(params_valid(p), VT_ERR_INVALID_ARGUMENT, "invalid parameter block");
    const uint32_t n = s->h.P.num_particles;
    const int32_t old_mn = s->h.P.max_num_neighbors;
    s->h.P = *p;
    s->h.P.num_particles = n;
    if (p->max_num_neighbors != old_mn) return make_topology_change(s);
    return VT_OK;
}

vt_status vt_cloth_add(vt_solver* s, const float* xyz, uint32_t nv, const uint32_t* indices,
                       uint32_t nidx, const float model[16], float diameter, int32_t* out_offset)
{
    VT_CHECK(s && model, VT_ERR_INVALID_ARGUMENT, "NULL argument");
    VT_CHECK(nv == 0 || xyz, VT_ERR_INVALID_ARGUMENT, "xyz is NULL");
    VT_CHECK(nidx == 0 || indices, VT_ERR_INVALID_ARGUMENT, "indices is NULL");
    VT_CHECK(nidx % 3 == 0, VT_ERR_INVALID_ARGUMENT, "index count is not a multiple of 3");
    VT_CHECK((uint64_t)s->h.n() + nv < (1u << 29), VT_ERR_CAPACITY, "too many particles");
    for (uint32_t i = 0; i < nidx; ++i)
        VT_CHECK(indices[i] < nv, VT_ERR_INVALID_ARGUMENT, "triangle index out of range");
    VT_GUARD_BEGIN
    vt_status st = make_topology_change(s);
    if (st != VT_OK) return st;
    HostSolver& h = s->h;
    h.grid_res = -1;
    const int32_t prev = (int32_t)h.n();
    ClothRec c{prev, (int32_t)nv, (int32_t)(h.tri.size() / 3), (int32_t)(nidx / 3)};
    h.cloths.push_back(c);
    for (uint32_t i = 0; i < nidx; ++i) h.tri.push_back(indices[i] + (uint32_t)prev);
    for (uint32_t i = 0; i < nv; ++i) {
        // InitializePositions_Kernel (VtClothSolverGPU.cu:30-34): model * (x, 1)
        const vec3 p = m4v3(model, mk3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]), 1.0f);
        h.x.push_back(p.x); h.x.push_back(p.y); h.x.push_back(p.z);
        h.v.push_back(0); h.v.push_back(0); h.v.push_back(0);
        h.w.push_back(1.0f);
    }
    // AddCloth, VtClothSolverGPU.hpp:118-125, 148-149
    h.P.num_particles = h.n();
    h.P.particle_diameter = diameter;
    h.P.max_speed = 2.0f * diameter / h.P.delta_time * (float)h.P.num_substeps;
    h.cell_spacing = diameter * h.P.hash_cell_size_scalar;
    h.table_size = 2 * (int32_t)h.n();
    h.x0 = h.x;  // SpatialHashGPU::SetInitialPositions
    if (out_offset) *out_offset = prev;
    return VT_OK;
    VT_GUARD_END
}

vt_status vt_stretch_add(vt_solver* s, const int32_t* pairs, const float* rest, uint32_t count)
{
    VT_CHECK(s, VT_ERR_INVALID_ARGUMENT, "NULL solver");
    VT_CHECK(count == 0 || (pairs && rest), VT_ERR_INVALID_ARGUMENT, "NULL array");
    const int64_t n = s->h.n();
    for (uint32_t c = 0; c < 2 * count; ++c)
        VT_CHECK(pairs[c] >= 0 && pairs[c] < n, VT_ERR_INVALID_ARGUMENT, "stretch index out of range");
    VT_GUARD_BEGIN
    vt_status st = make_topology_change(s);
    if (st != VT_OK) return st;
    s->h.grid_res = -1;
    s->h.st_idx.insert(s->h.st_idx.end(), pairs, pairs + 2 * (size_t)count);
    s->h.st_rest.insert(s->h.st_rest.end(), rest, rest + count);
    return VT_OK;
    VT_GUARD_END
}

vt_status vt_attach_slot_add(vt_solver* s, const float xyz[3], int32_t* out_slot)
{
    VT_CHECK(s && xyz, VT_ERR_INVALID_ARGUMENT, "NULL argument");
    VT_GUARD_BEGIN
    vt_status st = make_topology_change(s);
    if (st != VT_OK) return st;
    for (int k = 0; k < 3; ++k) {
        s->h.slots.push_back(xyz[k]);
        s->h.slots0.push_back(xyz[k]);
    }
    if (out_slot) *out_slot = (int32_t)s->h.nslots() - 1;
    return VT_OK;
    VT_GUARD_END
}

vt_status vt_attach_add(vt_solver* s, const int32_t* particles, const int32_t* slots,
                        const float* distances, uint32_t count)
{
    VT_CHECK(s, VT_ERR_INVALID_ARGUMENT, "NULL solver");
    VT_CHECK(count == 0 || (particles && slots && distances), VT_ERR_INVALID_ARGUMENT, "NULL array");
    const int64_t n = s->h.n(), ns = s->h.nslots();
    for (uint32_t c = 0; c < count; ++c) {
        VT_CHECK(particles[c] >= 0 && particles[c] < n, VT_ERR_INVALID_ARGUMENT, "attach particle out of range");
        VT_CHECK(slots[c] >= 0 && slots[c] < ns, VT_ERR_INVALID_ARGUMENT, "attach slot out of range");
    }
    VT_GUARD_BEGIN
    vt_status st = make_topology_change(s);
    if (st != VT_OK) return st;
    s->h.grid_res = -1;
    for (uint32_t c = 0; c < count; ++c) {
        if (distances[c] == 0) s->h.w[particles[c]] = 0;  // VtClothSolverGPU.hpp:172
        AttachOp a{};
        a.kind = 0;
        a.pid = particles[c];
        a.slot = slots[c];
        a.dist = distances[c];
        s->h.at_ops.push_back(a);
    }
    return VT_OK;
    VT_GUARD_END
}

vt_status vt_attach_generate_lra(vt_solver* s, int32_t first_slot, uint32_t num_slots,
                                 int32_t particle_begin, uint32_t particle_count)
{
    VT_CHECK(s, VT_ERR_INVALID_ARGUMENT, "NULL solver");
    const int64_t n = s->h.n(), ns = s->h.nslots();
    VT_CHECK(first_slot >= 0 && first_slot + (int64_t)num_slots <= ns, VT_ERR_INVALID_ARGUMENT,
             "slot range out of range");
    VT_CHECK(particle_begin >= 0 && particle_begin + (int64_t)particle_count <= n,
             VT_ERR_INVALID_ARGUMENT, "particle range out of range");
    if (num_slots == 0 || particle_count == 0) return VT_OK;
    VT_GUARD_BEGIN
    vt_status st = make_topology_change(s);
    if (st != VT_OK) return st;
    HostSolver& h = s->h;
    h.grid_res = -1;
    // The device recomputes |slot0 - x0_i|; that equals the distance the reference
    // stores only while the particles still sit at their initial positions.
    bool at_rest = true;
    for (uint32_t i = 0; i < 3 * particle_count && at_rest; ++i)
        at_rest = h.x[3 * (size_t)particle_begin + i] == h.x0[3 * (size_t)particle_begin + i];
    for (uint32_t k = 0; k < num_slots; ++k)
        for (int j = 0; j < 3; ++j)
            h.slots0[3 * (size_t)(first_slot + k) + j] = h.slots[3 * (size_t)(first_slot + k) + j];
    // GenerateAttach (VtClothObjectGPU.hpp:134-147) + AddAttach's zero-distance rule
    for (uint32_t k = 0; k < num_slots; ++k) {
        const float* sp = &h.slots[3 * (size_t)(first_slot + k)];
        const vec3 slot = mk3(sp[0], sp[1], sp[2]);
        for (uint32_t i = 0; i < particle_count; ++i) {
            const size_t q = (size_t)particle_begin + i;
            const vec3 xi = mk3(h.x[3 * q], h.x[3 * q + 1], h.x[3 * q + 2]);
            const float dist = length(slot - xi);
            if (dist == 0) h.w[q] = 0;
            if (!at_rest) {
                AttachOp a{};
                a.kind = 0;
                a.pid = (int32_t)q;
                a.slot = first_slot + (int32_t)k;
                a.dist = dist;
                h.at_ops.push_back(a);
            }
        }
    }
    if (at_rest) {
        AttachOp a{};
        a.kind = 1;
        a.slot_begin = first_slot;
        a.slot_count = (int32_t)num_slots;
        a.p_begin = particle_begin;
        a.p_count = (int32_t)particle_count;
        h.at_ops.push_back(a);
    }
    return VT_OK;
    VT_GUARD_END
}

vt_status vt_bend_add(vt_solver* s, const uint32_t* quads, const float* rest_angles, uint32_t count)
{
    VT_CHECK(s, VT_ERR_INVALID_ARGUMENT, "NULL solver");
    VT_CHECK(count == 0 || (quads && rest_angles), VT_ERR_INVALID_ARGUMENT, "NULL array");
    const uint64_t n = s->h.n();
    for (uint32_t c = 0; c < 4 * count; ++c)
        VT_CHECK(quads[c] < n, VT_ERR_INVALID_ARGUMENT, "bend index out of range");
    VT_GUARD_BEGIN
    vt_status st = make_topology_change(s);
    if (st != VT_OK) return st;
    s->h.grid_res = -1;
    s->h.bd_idx.insert(s->h.bd_idx.end(), quads, quads + 4 * (size_t)count);
    s->h.bd_rest.insert(s->h.bd_rest.end(), rest_angles, rest_angles + count);
    return VT_OK;
    VT_GUARD_END
}

vt_status vt_cloth_build_grid_constraints(vt_solver* s, int32_t offset, int32_t res,
                                          const int32_t* attached, uint32_t nat)
{
    VT_CHECK(s, VT_ERR_INVALID_ARGUMENT, "NULL solver");
    VT_CHECK(nat == 0 || attached, VT_ERR_INVALID_ARGUMENT, "attached is NULL");
    VT_CHECK(res >= 1, VT_ERR_INVALID_ARGUMENT, "resolution must be >= 1");
    const ClothRec* c = nullptr;
    for (const ClothRec& r : s->h.cloths)
        if (r.offset == offset) c = &r;
    VT_CHECK(c, VT_ERR_NOT_FOUND, "no cloth starts at this offset");
    VT_CHECK((int64_t)(res + 1) * (res + 1) == c->count, VT_ERR_INVALID_ARGUMENT,
             "resolution does not match the cloth's vertex count");
    for (uint32_t k = 0; k < nat; ++k)
        VT_CHECK(attached[k] >= 0 && attached[k] < c->count, VT_ERR_INVALID_ARGUMENT,
                 "attached vertex out of range");
    VT_GUARD_BEGIN
    const ClothRec cl = *c;
    vt_status st = make_topology_change(s);
    if (st != VT_OK) return st;
    HostSolver& h = s->h;
    // The implicit-topology kernel applies when this is the solver's only cloth, nothing
    // else is registered, and the positions are still the initial ones (its rest lengths
    // are recomputed from the initial positions).
    const bool grid_candidate = h.cloths.size() == 1 && cl.offset == 0 && h.st_rest.empty() &&
                                h.at_ops.empty() && h.bd_rest.empty() && h.x == h.x0;
    const int32_t first_slot = (int32_t)h.nslots();
    auto P = [&](int i) { const size_t q = 3 * (size_t)(cl.offset + i); return mk3(h.x[q], h.x[q + 1], h.x[q + 2]); };
    auto VAT = [res](int a, int b) { return a * (res + 1) + b; };
    auto add = [&](int i1, int i2) {
        h.st_idx.push_back(cl.offset + i1);
        h.st_idx.push_back(cl.offset + i2);
        h.st_rest.push_back(length(P(i1) - P(i2)));
    };
    // GenerateStretch, VtClothObjectGPU.hpp:75-116
    for (int a = 0; a < res + 1; ++a)
        for (int b = 0; b < res + 1; ++b) {
            if (b != res) add(VAT(a, b), VAT(a, b + 1));
            if (a != res) add(VAT(a, b), VAT(a + 1, b));
            if (b != res && a != res) {
                add(VAT(a, b), VAT(a + 1, b + 1));
                add(VAT(a, b + 1), VAT(a + 1, b));
            }
        }
    // GenerateAttach, :134-147
    if (nat) {
        const int32_t first = (int32_t)h.nslots();
        for (uint32_t k = 0; k < nat; ++k) {
            const vec3 p = P(attached[k]);
            h.slots.push_back(p.x); h.slots.push_back(p.y); h.slots.push_back(p.z);
            h.slots0.push_back(p.x); h.slots0.push_back(p.y); h.slots0.push_back(p.z);
        }
        st = vt_attach_generate_lra(s, first, nat, cl.offset, (uint32_t)cl.count);
        if (st != VT_OK) return st;
    }
    // GenerateBending, :118-132
    const uint32_t* ind = h.tri.data() + 3 * (size_t)cl.tri_begin;
    const int32_t ni = 3 * cl.tri_count;
    for (int32_t i = 0; i + 5 < ni; i += 6) {
        h.bd_idx.push_back(ind[i]);
        h.bd_idx.push_back(ind[i + 5]);
        h.bd_idx.push_back(ind[i + 2]);
        h.bd_idx.push_back(ind[i + 1]);
        h.bd_rest.push_back(0.0f);
    }
    h.grid_res = -1;
    if (grid_candidate) {
        // bending must be one constraint per quad (x, y), in x-major order, over
        // ((x,y), (x+1,y+1), (x,y+1), (x+1,y)): true for GenerateClothMesh's triangles
        bool ok = (int64_t)h.nbend() == (int64_t)res * res && (int64_t)ni == 6ll * res * res;
        // triangles must be GenerateClothMesh's (Velvet/Scene.hpp:153-165): the normals
        // kernel of grid domains enumerates them implicitly
        for (int32_t xq = 0; ok && xq < res; ++xq)
            for (int32_t yq = 0; ok && yq < res; ++yq) {
                const uint32_t* t = ind + 6 * ((size_t)xq * res + yq);
                ok = t[0] == (uint32_t)VAT(xq, yq) && t[1] == (uint32_t)VAT(xq + 1, yq) &&
                     t[2] == (uint32_t)VAT(xq, yq + 1) && t[3] == (uint32_t)VAT(xq, yq + 1) &&
                     t[4] == (uint32_t)VAT(xq + 1, yq) && t[5] == (uint32_t)VAT(xq + 1, yq + 1);
            }
        for (int32_t xq = 0; ok && xq < res; ++xq)
            for (int32_t yq = 0; ok && yq < res; ++yq) {
                const uint32_t* q = &h.bd_idx[4 * ((size_t)xq * res + yq)];
                ok = q[0] == (uint32_t)VAT(xq, yq) && q[1] == (uint32_t)VAT(xq + 1, yq + 1) &&
                     q[2] == (uint32_t)VAT(xq, yq + 1) && q[3] == (uint32_t)VAT(xq + 1, yq);
            }
        // attachments: nothing, or one LRA group of the whole cloth over the new slots
        if (ok && nat) {
            ok = h.at_ops.size() == 1 && h.at_ops[0].kind == 1 && h.at_ops[0].slot_begin == first_slot &&
                 h.at_ops[0].slot_count == (int32_t)nat && h.at_ops[0].p_begin == 0 &&
                 h.at_ops[0].p_count == cl.count;
        } else if (ok) {
            ok = h.at_ops.empty();
        }
        if (ok) {
            h.grid_res = res;
            h.grid_slot_begin = first_slot;
            h.grid_slot_count = (int32_t)nat;
        }
    }
    return VT_OK;
    VT_GUARD_END
}

vt_status vt_cloth_build_bending_adjacency(vt_solver* s, int32_t offset, uint32_t* out_count)
{
    VT_CHECK(s, VT_ERR_INVALID_ARGUMENT, "NULL solver");
    const ClothRec* c = nullptr;
    for (const ClothRec& r : s->h.cloths)
        if (r.offset == offset) c = &r;
    VT_CHECK(c, VT_ERR_NOT_FOUND, "no cloth starts at this offset");
    VT_GUARD_BEGIN
    const ClothRec cl = *c;
    vt_status st = make_topology_change(s);
    if (st != VT_OK) return st;
    HostSolver& h = s->h;
    const uint32_t* t = h.tri.data() + 3 * (size_t)cl.tri_begin;
    // every edge (key = the smaller and larger vertex) with the triangles and corners
    // that contain it, in triangle order; an edge of exactly two triangles is a hinge
    struct Use {
        uint64_t key;
        int32_t tri, k;  // opposite corner k of triangle tri
    };
    std::vector<Use> uses;
    uses.reserve(3 * (size_t)cl.tri_count);
    for (int32_t q = 0; q < cl.tri_count; ++q)
        for (int k = 0; k < 3; ++k) {
            const uint32_t u = t[3 * q + (k + 1) % 3], v = t[3 * q + (k + 2) % 3];
            uses.push_back({((uint64_t)std::min(u, v) << 32) | std::max(u, v), q, k});
        }
    std::stable_sort(uses.begin(), uses.end(), [](const Use& a, const Use& b) { return a.key < b.key; });
    struct Hinge {
        int32_t tri, k, tri2, k2;
    };
    std::vector<Hinge> hinges;
    for (size_t i = 0; i < uses.size();) {
        size_t j = i;
        while (j < uses.size() && uses[j].key == uses[i].key) ++j;
        if (j - i == 2) hinges.push_back({uses[i].tri, uses[i].k, uses[i + 1].tri, uses[i + 1].k});
        i = j;
    }
    std::sort(hinges.begin(), hinges.end(),
              [](const Hinge& a, const Hinge& b) { return a.tri != b.tri ? a.tri < b.tri : a.k < b.k; });
    auto X0 = [&](uint32_t i) { const size_t q = 3 * (size_t)i; return mk3(h.x0[q], h.x0[q + 1], h.x0[q + 2]); };
    uint32_t added = 0;
    for (const Hinge& g : hinges) {
        // corners as GenerateBending orders a quad: p0 the first triangle's opposite
        // vertex, p1 the second's, p2-p3 the shared edge with p3 the first triangle's next
        // corner after p0 (VtClothObjectGPU.hpp:118-132 for a grid quad)
        const uint32_t i0 = t[3 * g.tri + g.k], i3 = t[3 * g.tri + (g.k + 1) % 3], i2 = t[3 * g.tri + (g.k + 2) % 3];
        const uint32_t i1 = t[3 * g.tri2 + g.k2];
        const vec3 p0 = X0(i0), p1 = X0(i1), p2 = X0(i2), p3 = X0(i3);
        const vec3 n1 = cross(p2 - p0, p3 - p0), n2 = cross(p3 - p1, p2 - p1);
        if (length(p3 - p2) < VT_EPSILON || dot(n1, n1) == 0 || dot(n2, n2) == 0) continue;  // degenerate
        const float rest = bend_angle(p0, p1, p2, p3);
        if (!std::isfinite(rest)) continue;
        h.bd_idx.insert(h.bd_idx.end(), {i0, i1, i2, i3});
        h.bd_rest.push_back(rest);
        ++added;
    }
    h.grid_res = -1;
    if (out_count) *out_count = added;
    return VT_OK;
    VT_GUARD_END
}

vt_status vt_colliders_set(vt_solver* s, const vt_sdf_collider* colliders, uint32_t count)
{
    VT_CHECK(s, VT_ERR_INVALID_ARGUMENT, "NULL solver");
    VT_CHECK(count == 0 || colliders, VT_ERR_INVALID_ARGUMENT, "colliders is NULL");
    for (uint32_t k = 0; k < count; ++k)
        VT_CHECK(colliders[k].type >= 0 && colliders[k].type <= 2, VT_ERR_INVALID_ARGUMENT,
                 "unknown collider type");
    VT_GUARD_BEGIN
    const bool same_count = count == s->h.colliders.size();
    s->h.colliders.assign(colliders, colliders + count);
    if (s->world.built() && !s->topo_dirty && same_count)
        return s->world.set_colliders(0, s->h.colliders);
    return make_topology_change(s);
    VT_GUARD_END
}

vt_status vt_simulate(vt_solver* s, float frame_dt, int32_t substeps, int32_t iterations,
                      float relaxation, float friction, float collision_margin,
                      float particle_diameter, void* stream)
{
    VT_CHECK(s, VT_ERR_INVALID_ARGUMENT, "NULL solver");
    VT_CHECK(substeps >= 1 && iterations >= 0 && frame_dt > 0, VT_ERR_INVALID_ARGUMENT,
             "substeps must be >= 1, iterations >= 0, frame_dt > 0");
    VT_GUARD_BEGIN
    HostSolver& h = s->h;
    h.P.num_substeps = substeps;
    h.P.num_iterations = iterations;
    h.P.relaxation_factor = relaxation;
    h.P.friction = friction;
    h.P.collision_margin = collision_margin;
    h.P.particle_diameter = particle_diameter;
    cudaStream_t st = (cudaStream_t)stream;
    if (s->topo_dirty) {
        if (s->stream) VT_TRY_CUDA(cudaStreamSynchronize(s->stream), "sync");
        std::vector<const HostSolver*> doms{&h};
        s->launches_before += s->world.launches;
        vt_status r = s->world.build(doms);
        if (r != VT_OK) return r;
        s->topo_dirty = false;
        s->on_device = true;
    }
    s->stream = st;
    vt::FrameArgs a{frame_dt, substeps, iterations, relaxation, friction, collision_margin, particle_diameter};
    s->world.set_frame(0, h, a);
    vt_status r = s->world.simulate(a, h.P.interleaved_hash, h.P.enable_self_collision != 0, st,
                                    s->use_graph);
    if (r == VT_OK) s->simulated = true;
    return r;
    VT_GUARD_END
}

vt_status vt_solver_sync(vt_solver* s)
{
    VT_CHECK(s, VT_ERR_INVALID_ARGUMENT, "NULL solver");
    VT_GUARD_BEGIN
    VT_TRY_CUDA(cudaStreamSynchronize(s->stream), "sync");
    if (!s->world.built()) return VT_OK;
    std::vector<int32_t> flags;
    vt_status r = s->world.read_status(flags, s->stream);
    if (r != VT_OK) return r;
    if (flags[0]) {
        s->world.clear_status(s->stream);
        VT_TRY_CUDA(cudaStreamSynchronize(s->stream), "sync");
        if (flags[0] & vt::VT_STATUS_BOUNDS) {
            vt::set_error("a device-side bounds check failed (bounds-checked build)");
            return VT_ERR_STATE;
        }
        if (flags[0] & vt::VT_STATUS_TIMEOUT) {
            vt::set_error("a device-side bounded wait gave up (tile loads did not arrive)");
            return VT_ERR_TIMEOUT;
        }
        vt::set_error("non-finite particle state detected on the device");
        return VT_ERR_NUMERIC;
    }
    return VT_OK;
    VT_GUARD_END
}

vt_status vt_solver_num_particles(const vt_solver* s, uint32_t* out)
{
    VT_CHECK(s && out, VT_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = s->h.n();
    return VT_OK;
}

// float4 device array <-> float3 caller buffer
static vt_status get3(vt_solver* s, const float4* dev, const std::vector<float>& host, uint32_t first,
                      uint32_t count, float* dst, int32_t on_dev, void* stream)
{
    VT_CHECK(s && (count == 0 || dst), VT_ERR_INVALID_ARGUMENT, "NULL argument");
    VT_CHECK((uint64_t)first + count <= s->h.n(), VT_ERR_INVALID_ARGUMENT, "range out of bounds");
    if (!count) return VT_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (dev) {
        float* pk = s->world.d.packed + 3 * (size_t)first;
        VT_TRY_CUDA(vt::launch_pack_xyz(dev + first, pk, (int64_t)count, st), "pack");
        s->world.launches += 1;
        VT_TRY_CUDA(cudaMemcpyAsync(dst, pk, 12 * (size_t)count, on_dev ? cudaMemcpyDefault : cudaMemcpyDeviceToHost,
                                    st),
                    "copy out");
        if (!on_dev) VT_TRY_CUDA(cudaStreamSynchronize(st), "sync");
        return VT_OK;
    }
    if (on_dev) {
        VT_TRY_CUDA(cudaMemcpyAsync(dst, host.data() + 3 * (size_t)first, 12 * (size_t)count,
                                    cudaMemcpyHostToDevice, st), "copy out");
        VT_TRY_CUDA(cudaStreamSynchronize(st), "sync");
    } else {
        std::memcpy(dst, host.data() + 3 * (size_t)first, 12 * (size_t)count);
    }
    return VT_OK;
}

vt_status vt_positions_get(vt_solver* s, uint32_t first, uint32_t count, float* dst,
                           int32_t dst_on_device, void* stream)
{
    VT_CHECK(s, VT_ERR_INVALID_ARGUMENT, "NULL solver");
    return get3(s, s->on_device ? s->world.d.x : nullptr, s->h.x, first, count, dst, dst_on_device, stream);
}

vt_status vt_velocities_get(vt_solver* s, uint32_t first, uint32_t count, float* dst,
                            int32_t dst_on_device, void* stream)
{
    VT_CHECK(s, VT_ERR_INVALID_ARGUMENT, "NULL solver");
    return get3(s, s->on_device ? s->world.d.v : nullptr, s->h.v, first, count, dst, dst_on_device, stream);
}

vt_status vt_normals_get(vt_solver* s, uint32_t first, uint32_t count, float* dst,
                         int32_t dst_on_device, void* stream)
{
    VT_CHECK(s, VT_ERR_INVALID_ARGUMENT, "NULL solver");
    VT_CHECK(s->simulated && s->on_device, VT_ERR_STATE, "normals exist after the first simulate");
    return get3(s, s->world.d.nrm, s->h.x, first, count, dst, dst_on_device, stream);
}

static vt_status set3(vt_solver* s, float4* dev, std::vector<float>& host, uint32_t first,
                      uint32_t count, const float* src, int32_t on_dev, void* stream)
{
    VT_CHECK(s && (count == 0 || src), VT_ERR_INVALID_ARGUMENT, "NULL argument");
    VT_CHECK((uint64_t)first + count <= s->h.n(), VT_ERR_INVALID_ARGUMENT, "range out of bounds");
    if (!count) return VT_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (dev) {
        VT_TRY_CUDA(cudaMemcpy2DAsync(dev + first, 16, src, 12, 12, count,
                                      on_dev ? cudaMemcpyDefault : cudaMemcpyHostToDevice, st),
                    "copy in");
        if (!on_dev) VT_TRY_CUDA(cudaStreamSynchronize(st), "sync");
        return VT_OK;
    }
    if (on_dev) {
        VT_TRY_CUDA(cudaMemcpy(host.data() + 3 * (size_t)first, src, 12 * (size_t)count,
                               cudaMemcpyDeviceToHost), "copy in");
    } else {
        std::memcpy(host.data() + 3 * (size_t)first, src, 12 * (size_t)count);
    }
    return VT_OK;
}

vt_status vt_positions_set(vt_solver* s, uint32_t first, uint32_t count, const float* src,
                           int32_t src_on_device, void* stream)
{
    VT_CHECK(s, VT_ERR_INVALID_ARGUMENT, "NULL solver");
    return set3(s, s->on_device ? s->world.d.x : nullptr, s->h.x, first, count, src, src_on_device, stream);
}

vt_status vt_velocities_set(vt_solver* s, uint32_t first, uint32_t count, const float* src,
                            int32_t src_on_device, void* stream)
{
    VT_CHECK(s, VT_ERR_INVALID_ARGUMENT, "NULL solver");
    return set3(s, s->on_device ? s->world.d.v : nullptr, s->h.v, first, count, src, src_on_device, stream);
}

vt_status vt_inv_mass_get(vt_solver* s, uint32_t first, uint32_t count, float* dst)
{
    VT_CHECK(s && (count == 0 || dst), VT_ERR_INVALID_ARGUMENT, "NULL argument");
    VT_CHECK((uint64_t)first + count <= s->h.n(), VT_ERR_INVALID_ARGUMENT, "range out of bounds");
    if (!count) return VT_OK;
    if (s->on_device) {
        VT_TRY_CUDA(cudaStreamSynchronize(s->stream), "sync");
        VT_TRY_CUDA(cudaMemcpy2D(dst, 4, &s->world.d.x[first].w, 16, 4, count, cudaMemcpyDeviceToHost),
                    "copy inverse mass");
    } else {
        std::memcpy(dst, s->h.w.data() + first, 4 * (size_t)count);
    }
    return VT_OK;
}

vt_status vt_inv_mass_set(vt_solver* s, uint32_t first, uint32_t count, const float* src)
{
    VT_CHECK(s && (count == 0 || src), VT_ERR_INVALID_ARGUMENT, "NULL argument");
    VT_CHECK((uint64_t)first + count <= s->h.n(), VT_ERR_INVALID_ARGUMENT, "range out of bounds");
    if (!count) return VT_OK;
    std::memcpy(s->h.w.data() + first, src, 4 * (size_t)count);
    if (s->on_device) {
        VT_TRY_CUDA(cudaStreamSynchronize(s->stream), "sync");
        VT_TRY_CUDA(cudaMemcpy2D(&s->world.d.x[first].w, 16, src, 4, 4, count, cudaMemcpyHostToDevice),
                    "copy inverse mass");
    }
    return VT_OK;
}

vt_status vt_attach_slot_set(vt_solver* s, int32_t slot, const float xyz[3])
{
    VT_CHECK(s && xyz, VT_ERR_INVALID_ARGUMENT, "NULL argument");
    VT_CHECK(slot >= 0 && slot < (int32_t)s->h.nslots(), VT_ERR_INVALID_ARGUMENT, "slot out of range");
    for (int k = 0; k < 3; ++k) s->h.slots[3 * (size_t)slot + k] = xyz[k];
    if (s->world.built() && !s->topo_dirty) return s->world.set_slot(0, slot, xyz);
    return VT_OK;
}

// ------------------------------------------------------------------ checkpoint / resume
namespace {
struct StateHeader {
    uint32_t magic, version, n, nslots;
};
constexpr uint32_t kStateMagic = 0x4b435456u;  // "VTCK"
uint64_t state_bytes(uint64_t n, uint64_t ns) { return sizeof(StateHeader) + 4 * (7 * n + 3 * ns); }
}  // namespace

vt_status vt_solver_state_size(const vt_solver* s, uint64_t* bytes)
{
    VT_CHECK(s && bytes, VT_ERR_INVALID_ARGUMENT, "NULL argument");
    *bytes = state_bytes(s->h.n(), s->h.nslots());
    return VT_OK;
}

vt_status vt_solver_state_save(vt_solver* s, void* dst, uint64_t bytes)
{
    VT_CHECK(s && dst, VT_ERR_INVALID_ARGUMENT, "NULL argument");
    const uint32_t n = s->h.n(), ns = s->h.nslots();
    VT_CHECK(bytes >= state_bytes(n, ns), VT_ERR_INVALID_ARGUMENT, "buffer smaller than vt_solver_state_size");
    VT_GUARD_BEGIN
    const StateHeader hd{kStateMagic, 1u, n, ns};
    std::memcpy(dst, &hd, sizeof(hd));
    float* f = reinterpret_cast<float*>(static_cast<char*>(dst) + sizeof(hd));
    vt_status st = vt_positions_get(s, 0, n, f, 0, s->stream);
    if (st == VT_OK) st = vt_velocities_get(s, 0, n, f + 3 * (size_t)n, 0, s->stream);
    if (st == VT_OK) st = vt_inv_mass_get(s, 0, n, f + 6 * (size_t)n);
    if (st != VT_OK) return st;
    if (ns) std::memcpy(f + 7 * (size_t)n, s->h.slots.data(), 12 * (size_t)ns);
    return VT_OK;
    VT_GUARD_END
}

vt_status vt_solver_state_load(vt_solver* s, const void* src, uint64_t bytes)
{
    VT_CHECK(s && src, VT_ERR_INVALID_ARGUMENT, "NULL argument");
    VT_CHECK(bytes >= sizeof(StateHeader), VT_ERR_INVALID_ARGUMENT, "buffer too small");
    StateHeader hd;
    std::memcpy(&hd, src, sizeof(hd));
    VT_CHECK(hd.magic == kStateMagic && hd.version == 1, VT_ERR_INVALID_ARGUMENT, "not a solver state");
    VT_CHECK(hd.n == s->h.n() && hd.nslots == s->h.nslots(), VT_ERR_INVALID_ARGUMENT,
             "state of a solver with other particle or slot counts");
    VT_CHECK(bytes >= state_bytes(hd.n, hd.nslots), VT_ERR_INVALID_ARGUMENT, "truncated state");
    VT_GUARD_BEGIN
    const float* f = reinterpret_cast<const float*>(static_cast<const char*>(src) + sizeof(hd));
    const uint32_t n = hd.n;
    vt_status st = vt_positions_set(s, 0, n, f, 0, s->stream);
    if (st == VT_OK) st = vt_velocities_set(s, 0, n, f + 3 * (size_t)n, 0, s->stream);
    if (st == VT_OK) st = vt_inv_mass_set(s, 0, n, f + 6 * (size_t)n);
    for (uint32_t k = 0; st == VT_OK && k < hd.nslots; ++k) st = vt_attach_slot_set(s, (int32_t)k, f + 7 * (size_t)n + 3 * k);
    return st;
    VT_GUARD_END
}

vt_status vt_solver_debug_get(vt_solver* s, int32_t what, void* dst, uint64_t bytes)
{
    VT_CHECK(s && dst, VT_ERR_INVALID_ARGUMENT, "NULL argument");
    const uint64_t n = s->h.n();
    if (what == VT_DEBUG_TABLE_SIZE) {
        VT_CHECK(bytes >= 4, VT_ERR_INVALID_ARGUMENT, "buffer too small");
        std::memcpy(dst, &s->h.table_size, 4);
        return VT_OK;
    }
    VT_CHECK(s->simulated && s->on_device, VT_ERR_STATE, "debug views exist after the first simulate");
    const vt::DeviceArrays& d = s->world.d;
    const uint64_t T = (uint64_t)s->h.table_size;
    const void* src = nullptr;
    uint64_t need = 0;
    switch (what) {
    case VT_DEBUG_PARTICLE_HASH: src = d.keys; need = 4 * n; break;
    case VT_DEBUG_PARTICLE_INDEX: src = d.vals; need = 4 * n; break;
    case VT_DEBUG_CELL_START: need = 4 * (T + 1); break;
    case VT_DEBUG_CELL_END: need = 4 * T; break;
    // the lists are kept in the reference's layout (particle id's list in column id)
    case VT_DEBUG_NEIGHBORS: src = d.nbr; need = 4 * n * (uint64_t)s->h.P.max_num_neighbors; break;
    case VT_DEBUG_PREDICTED: need = 12 * n; break;
    default: vt::set_error("unknown debug view"); return VT_ERR_INVALID_ARGUMENT;
    }
    VT_CHECK(bytes >= need, VT_ERR_INVALID_ARGUMENT, "buffer too small");
    VT_TRY_CUDA(cudaStreamSynchronize(s->stream), "sync");
    if (what == VT_DEBUG_PREDICTED) {
        if (n) VT_TRY_CUDA(cudaMemcpy2D(dst, 12, d.p[s->world.pcur], 16, 12, n, cudaMemcpyDeviceToHost), "copy");
        return VT_OK;
    }
    if (what == VT_DEBUG_CELL_START || what == VT_DEBUG_CELL_END) {
        // the device keeps (start, end) pairs; each view is one column of them
        const char* col = reinterpret_cast<const char*>(d.cells) + (what == VT_DEBUG_CELL_END ? 4 : 0);
        const uint64_t rows = what == VT_DEBUG_CELL_END ? T : T + 1;
        if (rows) VT_TRY_CUDA(cudaMemcpy2D(dst, 4, col, 8, 4, rows, cudaMemcpyDeviceToHost), "copy");
        return VT_OK;
    }
    if (need) VT_TRY_CUDA(cudaMemcpy(dst, src, need, cudaMemcpyDeviceToHost), "copy");
    return VT_OK;
}

vt_status vt_solver_launch_count(const vt_solver* s, uint64_t* out)
{
    VT_CHECK(s && out, VT_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = s->world.launches + s->launches_before;
    return VT_OK;
}

vt_status vt_solver_use_graphs(vt_solver* s, int32_t on)
{
    VT_CHECK(s, VT_ERR_INVALID_ARGUMENT, "NULL solver");
    s->use_graph = on != 0;
    return VT_OK;
}

vt_status vt_solver_use_grid_kernel(vt_solver* s, int32_t on)
{
    VT_CHECK(s, VT_ERR_INVALID_ARGUMENT, "NULL solver");
    VT_GUARD_BEGIN
    if (s->h.use_grid_kernel == (on != 0)) return VT_OK;
    vt_status st = make_topology_change(s);  // the device world is rebuilt at the next simulate
    if (st != VT_OK) return st;
    s->h.use_grid_kernel = on != 0;
    return VT_OK;
    VT_GUARD_END
}

vt_status vt_tuning_set_grid_tile(int32_t variant) { return vt::tuning_force(variant); }
vt_status vt_tuning_set_tile_loads(int32_t tma) { return vt::set_tile_loads_tma(tma != 0); }
vt_status vt_tuning_set_substep_clusters(int32_t mode) { return vt::set_substep_clusters(mode); }

vt_status vt_solver_grid_tile(const vt_solver* s, int32_t* variant)
{
    VT_CHECK(s && variant, VT_ERR_INVALID_ARGUMENT, "NULL argument");
    *variant = s->world.grid_variant;
    return VT_OK;
}

vt_status vt_profiler_enable(int32_t on) { return vt::profiler_enable(on != 0); }
vt_status vt_profiler_reset(void) { return vt::profiler_reset(); }
vt_status vt_profiler_read(vt_stage_time* out, uint32_t capacity, uint32_t* count)
{
    return vt::profiler_read(out, capacity, count);
}

// ------------------------------------------------------------------ HashObjects
namespace {
struct HashScratch {
    uint32_t* buf = nullptr;
    size_t words = 0;
};
std::mutex g_hash_mu;
HashScratch g_hash_scratch[64];  // per device ordinal
}  // namespace

vt_status vt_hash_objects(uint32_t* particle_hash, uint32_t* particle_index, uint32_t* cell_start,
                          uint32_t* cell_end, uint32_t* neighbors, const float* positions,
                          const float* original_positions, const vt_hash_params* hp, void* stream)
{
    VT_CHECK(hp, VT_ERR_INVALID_ARGUMENT, "params is NULL");
    VT_CHECK(cell_start, VT_ERR_INVALID_ARGUMENT, "cell_start is NULL");
    VT_CHECK(hp->table_size >= 1, VT_ERR_INVALID_ARGUMENT, "table_size must be >= 1");
    VT_CHECK(hp->max_num_neighbors >= 1 && hp->max_num_neighbors <= 64, VT_ERR_INVALID_ARGUMENT,
             "max_num_neighbors must be in [1, 64]");
    VT_CHECK(hp->num_objects < (1u << 30), VT_ERR_CAPACITY, "too many objects");
    VT_CHECK((uint64_t)hp->num_objects * hp->max_num_neighbors < (1ull << 32), VT_ERR_CAPACITY,
             "neighbour table exceeds 32-bit indexing");
    if (hp->num_objects)
        VT_CHECK(particle_hash && particle_index && cell_end && neighbors && positions &&
                     original_positions, VT_ERR_INVALID_ARGUMENT, "NULL buffer");
    VT_GUARD_BEGIN
    int dev = 0;
    VT_TRY_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    VT_CHECK(dev >= 0 && dev < 64, VT_ERR_STATE, "device ordinal beyond 64");
    const int32_t n = (int32_t)hp->num_objects;
    const size_t need = 2 * (size_t)(n > 0 ? n : 1) + vt::radix_hist_words(n);
    std::lock_guard<std::mutex> lock(g_hash_mu);
    HashScratch& S = g_hash_scratch[dev];
    if (S.words < need) {
        if (S.buf) VT_TRY_CUDA(cudaFree(S.buf), "cudaFree(hash scratch)");
        S.buf = nullptr;
        S.words = 0;
        VT_TRY_CUDA(cudaMalloc(&S.buf, need * 4), "cudaMalloc(hash scratch)");
        S.words = need;
    }
    uint32_t* kt = S.buf;
    uint32_t* vt_ = kt + (n > 0 ? n : 1);
    uint32_t* hist = vt_ + (n > 0 ? n : 1);
    VT_TRY_CUDA(vt::hash_objects_f3(particle_hash, particle_index, cell_start, cell_end, neighbors,
                                    positions, original_positions, *hp, kt, vt_, hist,
                                    (cudaStream_t)stream),
                "hash_objects");
    return VT_OK;
    VT_GUARD_END
}

}  // extern "C"
