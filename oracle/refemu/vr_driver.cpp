// vr_driver.cpp — the reference's own GPU solver kernels, run on the CPU.  TEST
// INFRASTRUCTURE ONLY (built into oracle/_ref/libvr_ref.so from the sources in the
// reference tree; never part of the product).
//
// Velvet/VtClothSolverGPU.cu, Velvet/SpatialHashGPU.cu and the headers they include
// (Velvet/VtClothSolverGPU.cuh, Velvet/SpatialHashGPU.cuh, Velvet/Common.cuh) are compiled
// unmodified with g++ against the stand-in headers in oracle/refemu/include (the CUDA
// runtime, glm, cub's radix sort, and Common.hpp / Timer.hpp / VtBuffer.hpp, see each
// file), with the launch emulator below.  This file restates only the host code that
// drives those kernels, whose own files need the engine, the mesh and OpenGL:
//   VtClothSolverGPU::Simulate        Velvet/VtClothSolverGPU.hpp:56-111
//   AddCloth / AddStretch / AddAttachSlot / AddAttach / AddBend   :114-185
//   UpdateColliders                   :187-205 (the caller passes the inverse transform)
//   SpatialHashGPU (table, Hash)      Velvet/SpatialHashGPU.hpp:18-52
//   VtClothObjectGPU::Start + Generate*  Velvet/VtClothObjectGPU.hpp:43-147
// It exports the oracle's C surface (vr_* for vo_*), so a test drives both the same way.
// Differences from running the reference on a GPU, all deliberate: atomics land in
// thread-index order (one valid order of the reference's unordered atomics); acos is the
// oracle's (CUDA's acosf is closed); cellStart gets T + 1 entries (the reference allocates
// T and clears T + 1); attach slots are solver-global in the oracle but cloth-local here,
// as in the reference (they agree for one cloth with slots, or when only the first
// registered cloth has slots).
#include <ucontext.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include <velvet_gb300.h>
#include "SpatialHashGPU.cuh"
#include "VtClothSolverGPU.cuh"

// ------------------------------------------------------------------ launch emulator
uint3 threadIdx, blockIdx;
dim3 blockDim, gridDim;
unsigned int sharedHash[1025];  // FindCellStart_Kernel's dynamic shared memory (256 + 1 used)

namespace {

constexpr size_t kFiberStack = 64 * 1024;
enum FiberState { kReady, kWaiting, kDone };
ucontext_t g_sched;
std::vector<ucontext_t> g_ctx;
std::vector<int> g_state;
std::vector<char> g_stacks;
unsigned g_cur = 0;
bool g_in_fibers = false;
void (*g_body)(void*) = nullptr;
void* g_body_ctx = nullptr;

void fiber_main()
{
    g_body(g_body_ctx);
    g_state[g_cur] = kDone;  // returns to g_sched through uc_link
}

}  // namespace

void __syncthreads()
{
    if (!g_in_fibers) {
        std::fprintf(stderr, "refemu: __syncthreads outside a fiber launch\n");
        std::abort();
    }
    g_state[g_cur] = kWaiting;
    swapcontext(&g_ctx[g_cur], &g_sched);
}

void vr::run_grid(const LaunchCfg& cfg, void (*body)(void*), void* ctx)
{
    gridDim = dim3(cfg.blocks);
    blockDim = dim3(cfg.threads);
    threadIdx.y = threadIdx.z = blockIdx.y = blockIdx.z = 0;
    if (!cfg.fibers) {
        for (unsigned b = 0; b < cfg.blocks; ++b) {
            blockIdx.x = b;
            for (unsigned t = 0; t < cfg.threads; ++t) {
                threadIdx.x = t;
                body(ctx);
            }
        }
        return;
    }
    if (cfg.threads * sizeof(unsigned) > sizeof(sharedHash)) std::abort();
    const unsigned nt = cfg.threads;
    g_ctx.resize(nt);
    g_state.assign(nt, kReady);
    if (g_stacks.size() < nt * kFiberStack) g_stacks.resize(nt * kFiberStack);
    g_body = body;
    g_body_ctx = ctx;
    g_in_fibers = true;
    for (unsigned b = 0; b < cfg.blocks; ++b) {
        blockIdx.x = b;
        for (unsigned t = 0; t < nt; ++t) {
            getcontext(&g_ctx[t]);
            g_ctx[t].uc_stack.ss_sp = g_stacks.data() + t * kFiberStack;
            g_ctx[t].uc_stack.ss_size = kFiberStack;
            g_ctx[t].uc_link = &g_sched;
            makecontext(&g_ctx[t], fiber_main, 0);
            g_state[t] = kReady;
        }
        // rounds: every live thread runs to its next barrier (or its end) before any
        // thread passes that barrier
        for (unsigned live = nt; live > 0;) {
            for (unsigned t = 0; t < nt; ++t) {
                if (g_state[t] == kDone) continue;
                g_cur = t;
                threadIdx.x = t;
                g_state[t] = kReady;
                swapcontext(&g_sched, &g_ctx[t]);
                if (g_state[t] == kDone) --live;
            }
        }
    }
    g_in_fibers = false;
}

// ------------------------------------------------------------------ solver driver
using Velvet::HashParams;
using Velvet::SDFCollider;

namespace {

struct Cloth {
    int32_t offset, count;
    std::vector<glm::vec3> mesh;      // the mesh's own (untransformed) vertices
    std::vector<uint32_t> indices;    // the mesh's own indices
    glm::mat4 model;
};

struct Solver {
    VtSimParams P;
    std::vector<Cloth> cloths;
    std::vector<glm::vec3> positions, normals, velocities, predicted, deltas;
    std::vector<int> deltaCounts;
    std::vector<float> invMasses;
    std::vector<uint32_t> indices;
    std::vector<int> stretchIndices;
    std::vector<float> stretchLengths;
    std::vector<uint32_t> bendIndices;
    std::vector<float> bendAngles;
    std::vector<int> attachParticleIDs, attachSlotIDs;
    std::vector<float> attachDistances;
    std::vector<glm::vec3> attachSlotPositions;
    std::vector<SDFCollider> colliders;
    // SpatialHashGPU (Velvet/SpatialHashGPU.hpp:18-52)
    float spacing = 0;
    int tableSize = 0;
    std::vector<uint32_t> neighbors, particleHash, particleIndex, cellStart, cellEnd;
    std::vector<glm::vec3> initialPositions;
};

template <class T>
T* ptr(std::vector<T>& v)
{
    return v.empty() ? nullptr : v.data();
}

void hash(Solver& s)
{
    HashParams hp;
    hp.numObjects = (uint32_t)s.predicted.size();
    hp.cellSpacing = s.spacing;
    hp.cellSpacing2 = s.spacing * s.spacing;
    hp.tableSize = s.tableSize;
    hp.maxNumNeighbors = (uint32_t)s.P.maxNumNeighbors;
    hp.particleDiameter2 = s.P.particleDiameter * s.P.particleDiameter;
    Velvet::HashObjects(ptr(s.particleHash), ptr(s.particleIndex), ptr(s.cellStart), ptr(s.cellEnd),
                        ptr(s.neighbors), ptr(s.predicted), ptr(s.initialPositions), hp);
}

glm::mat4 mat4_of(const float* m)
{
    glm::mat4 r;
    for (int j = 0; j < 4; ++j) r.c[j] = glm::vec4(m[4 * j], m[4 * j + 1], m[4 * j + 2], m[4 * j + 3]);
    return r;
}

}  // namespace

extern "C" {

__attribute__((visibility("default"))) void* vr_create(const vt_params* p)
{
    Solver* s = new Solver();
    VtSimParams& P = s->P;
    P.numSubsteps = p->num_substeps;
    P.numIterations = p->num_iterations;
    P.maxNumNeighbors = p->max_num_neighbors;
    P.maxSpeed = p->max_speed;
    P.gravity = glm::vec3(p->gravity[0], p->gravity[1], p->gravity[2]);
    P.bendCompliance = p->bend_compliance;
    P.damping = p->damping;
    P.relaxationFactor = p->relaxation_factor;
    P.longRangeStretchiness = p->long_range_stretchiness;
    P.collisionMargin = p->collision_margin;
    P.friction = p->friction;
    P.enableSelfCollision = p->enable_self_collision != 0;
    P.interleavedHash = p->interleaved_hash;
    P.numParticles = 0;
    P.particleDiameter = p->particle_diameter;
    P.deltaTime = p->delta_time;
    P.particleDiameterScalar = p->particle_diameter_scalar;
    P.hashCellSizeScalar = p->hash_cell_size_scalar;
    return s;
}

__attribute__((visibility("default"))) void vr_destroy(void* h) { delete static_cast<Solver*>(h); }

__attribute__((visibility("default"))) uint32_t vr_num_particles(void* h)
{
    return (uint32_t)static_cast<Solver*>(h)->positions.size();
}
__attribute__((visibility("default"))) int32_t vr_table_size(void* h) { return static_cast<Solver*>(h)->tableSize; }

// AddCloth, Velvet/VtClothSolverGPU.hpp:114-156 (Timer::fixedDeltaTime() = P.deltaTime)
__attribute__((visibility("default"))) int32_t vr_cloth_add(void* h, const float* xyz, uint32_t nv,
                                                            const uint32_t* idx, uint32_t nidx,
                                                            const float* model, float diameter)
{
    Solver& s = *static_cast<Solver*>(h);
    const int32_t prev = (int32_t)s.P.numParticles;
    s.P.numParticles += nv;
    s.P.particleDiameter = diameter;
    s.P.maxSpeed = 2 * diameter / s.P.deltaTime * s.P.numSubsteps;
    Cloth c;
    c.offset = prev;
    c.count = (int32_t)nv;
    c.model = mat4_of(model);
    for (uint32_t i = 0; i < nv; ++i) c.mesh.push_back(glm::vec3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]));
    c.indices.assign(idx, idx + nidx);
    s.positions.insert(s.positions.end(), c.mesh.begin(), c.mesh.end());
    s.normals.resize(s.positions.size(), glm::vec3(0));
    for (uint32_t i = 0; i < nidx; ++i) s.indices.push_back(idx[i] + (uint32_t)prev);
    s.velocities.resize(s.positions.size(), glm::vec3(0));
    s.predicted.resize(s.positions.size(), glm::vec3(0));
    s.deltas.resize(s.positions.size(), glm::vec3(0));
    s.deltaCounts.resize(s.positions.size(), 0);
    s.invMasses.resize(s.positions.size(), 1.0f);
    Velvet::InitializePositions(s.positions.data(), prev, (int)nv, c.model);
    // m_spatialHash = make_shared<SpatialHashGPU>(particleDiameter, numParticles) and
    // SetInitialPositions(positions)
    const int n = (int)s.P.numParticles;
    s.spacing = diameter * s.P.hashCellSizeScalar;
    s.tableSize = 2 * n;
    s.neighbors.assign((size_t)n * s.P.maxNumNeighbors, 0);
    s.particleHash.assign(n, 0);
    s.particleIndex.assign(n, 0);
    s.cellStart.assign((size_t)s.tableSize + 1, 0);
    s.cellEnd.assign((size_t)s.tableSize + 1, 0);
    s.initialPositions = s.positions;
    s.cloths.push_back(c);
    return prev;
}

// VtClothObjectGPU::Start after AddCloth, Velvet/VtClothObjectGPU.hpp:55-62, for the cloth
// registered at `offset` with `res` quads per side: ApplyTransform (:67-73), GenerateStretch
// (:75-116), GenerateAttach (:134-147; slot indices local to the cloth, AddAttach
// zeroing the inverse mass at distance 0), GenerateBending (:118-132).
__attribute__((visibility("default"))) int vr_build_grid_constraints(void* h, int32_t offset, int32_t res,
                                                                     const int32_t* attached, uint32_t nat)
{
    Solver& s = *static_cast<Solver*>(h);
    const Cloth* c = nullptr;
    for (const Cloth& k : s.cloths)
        if (k.offset == offset) c = &k;
    if (!c || (int64_t)(res + 1) * (res + 1) != c->count) return -1;
    std::vector<glm::vec3> positions = c->mesh;
    for (auto& p : positions) p = c->model * glm::vec4(p, 1.0);
    auto vertexAt = [res](int x, int y) { return x * (res + 1) + y; };
    auto distanceBetween = [&positions](int a, int b) { return glm::length(positions[a] - positions[b]); };
    auto addStretch = [&s](int a, int b, float d) {
        s.stretchIndices.push_back(a);
        s.stretchIndices.push_back(b);
        s.stretchLengths.push_back(d);
    };
    for (int x = 0; x < res + 1; x++)
        for (int y = 0; y < res + 1; y++) {
            int a, b;
            if (y != res) {
                a = vertexAt(x, y);
                b = vertexAt(x, y + 1);
                addStretch(offset + a, offset + b, distanceBetween(a, b));
            }
            if (x != res) {
                a = vertexAt(x, y);
                b = vertexAt(x + 1, y);
                addStretch(offset + a, offset + b, distanceBetween(a, b));
            }
            if (y != res && x != res) {
                a = vertexAt(x, y);
                b = vertexAt(x + 1, y + 1);
                addStretch(offset + a, offset + b, distanceBetween(a, b));
                a = vertexAt(x, y + 1);
                b = vertexAt(x + 1, y);
                addStretch(offset + a, offset + b, distanceBetween(a, b));
            }
        }
    for (uint32_t slot = 0; slot < nat; ++slot) {
        const glm::vec3 slotPos = positions[attached[slot]];
        s.attachSlotPositions.push_back(slotPos);
        for (size_t i = 0; i < positions.size(); i++) {
            const float rest = glm::length(slotPos - positions[i]);
            if (rest == 0) s.invMasses[offset + i] = 0;
            s.attachParticleIDs.push_back(offset + (int)i);
            s.attachSlotIDs.push_back((int)slot);
            s.attachDistances.push_back(rest);
        }
    }
    for (size_t i = 0; i + 5 < c->indices.size(); i += 6) {
        s.bendIndices.push_back(offset + c->indices[i]);
        s.bendIndices.push_back(offset + c->indices[i + 5]);
        s.bendIndices.push_back(offset + c->indices[i + 2]);
        s.bendIndices.push_back(offset + c->indices[i + 1]);
        s.bendAngles.push_back(0.0f);
    }
    return 0;
}

// UpdateColliders, Velvet/VtClothSolverGPU.hpp:187-205
__attribute__((visibility("default"))) void vr_colliders_set(void* h, const vt_sdf_collider* c, uint32_t n)
{
    Solver& s = *static_cast<Solver*>(h);
    s.colliders.resize(n);
    for (uint32_t i = 0; i < n; ++i) {
        SDFCollider& d = s.colliders[i];
        d.type = (ColliderType)c[i].type;
        d.position = glm::vec3(c[i].position[0], c[i].position[1], c[i].position[2]);
        d.scale = glm::vec3(c[i].scale[0], c[i].scale[1], c[i].scale[2]);
        d.deltaTime = c[i].delta_time;
        for (int j = 0; j < 3; ++j)
            d.curTransform.c[j] = glm::vec3(c[i].cur_transform[3 * j], c[i].cur_transform[3 * j + 1],
                                            c[i].cur_transform[3 * j + 2]);
        d.invCurTransform = mat4_of(c[i].inv_cur_transform);
        d.lastTransform = mat4_of(c[i].last_transform);
    }
}

// VtClothSolverGPU::Simulate, Velvet/VtClothSolverGPU.hpp:56-111, with the per-frame
// parameters the caller sets in Global::simParams
__attribute__((visibility("default"))) void vr_simulate(void* h, float frame_dt, int32_t substeps,
                                                        int32_t iterations, float relax, float friction,
                                                        float margin, float diameter)
{
    Solver& s = *static_cast<Solver*>(h);
    VtSimParams& P = s.P;
    P.numSubsteps = substeps;
    P.numIterations = iterations;
    P.relaxationFactor = relax;
    P.friction = friction;
    P.collisionMargin = margin;
    P.particleDiameter = diameter;
    if (P.numParticles == 0) return;
    const float frameTime = frame_dt;
    const float substepTime = frame_dt / P.numSubsteps;
    const uint32_t ncol = (uint32_t)s.colliders.size();
    Velvet::SetSimulationParams(&P);
    Velvet::CollideSDF(ptr(s.positions), ptr(s.colliders), ptr(s.positions), ncol, frameTime);
    for (int substep = 0; substep < P.numSubsteps; substep++) {
        Velvet::PredictPositions(ptr(s.predicted), ptr(s.velocities), ptr(s.positions), substepTime);
        if (P.enableSelfCollision) {
            if (substep % P.interleavedHash == 0) hash(s);
            Velvet::CollideParticles(ptr(s.deltas), ptr(s.deltaCounts), ptr(s.predicted), ptr(s.invMasses),
                                     ptr(s.neighbors), ptr(s.positions));
        }
        Velvet::CollideSDF(ptr(s.predicted), ptr(s.colliders), ptr(s.positions), ncol, substepTime);
        for (int iteration = 0; iteration < P.numIterations; iteration++) {
            Velvet::SolveStretch(ptr(s.predicted), ptr(s.deltas), ptr(s.deltaCounts), ptr(s.stretchIndices),
                                 ptr(s.stretchLengths), ptr(s.invMasses), (uint32_t)s.stretchLengths.size());
            Velvet::SolveAttachment(ptr(s.predicted), ptr(s.deltas), ptr(s.deltaCounts), ptr(s.invMasses),
                                    ptr(s.attachParticleIDs), ptr(s.attachSlotIDs), ptr(s.attachSlotPositions),
                                    ptr(s.attachDistances), (int)s.attachParticleIDs.size());
            Velvet::SolveBending(ptr(s.predicted), ptr(s.deltas), ptr(s.deltaCounts), ptr(s.bendIndices),
                                 ptr(s.bendAngles), ptr(s.invMasses), (uint32_t)s.bendAngles.size(), substepTime);
            Velvet::ApplyDeltas(ptr(s.predicted), ptr(s.deltas), ptr(s.deltaCounts));
        }
        Velvet::Finalize(ptr(s.velocities), ptr(s.positions), ptr(s.predicted), substepTime);
    }
    Velvet::ComputeNormal(ptr(s.normals), ptr(s.positions), ptr(s.indices), (uint32_t)(s.indices.size() / 3));
}

// the oracle's vo_get codes: 0 positions, 1 velocities, 2 predicted, 3 normals, 4 inverse
// masses, 5 hash keys, 6 sorted indices, 7 cell start (T + 1), 8 cell end (T),
// 9 neighbours (N x maxNumNeighbors), 10 initial positions
__attribute__((visibility("default"))) int vr_get(void* h, int what, void* dst)
{
    Solver& s = *static_cast<Solver*>(h);
    const size_t n = s.positions.size();
    switch (what) {
    case 0: std::memcpy(dst, s.positions.data(), n * 12); return 0;
    case 1: std::memcpy(dst, s.velocities.data(), n * 12); return 0;
    case 2: std::memcpy(dst, s.predicted.data(), n * 12); return 0;
    case 3: std::memcpy(dst, s.normals.data(), n * 12); return 0;
    case 4: std::memcpy(dst, s.invMasses.data(), n * 4); return 0;
    case 5: std::memcpy(dst, s.particleHash.data(), n * 4); return 0;
    case 6: std::memcpy(dst, s.particleIndex.data(), n * 4); return 0;
    case 7: std::memcpy(dst, s.cellStart.data(), ((size_t)s.tableSize + 1) * 4); return 0;
    case 8: std::memcpy(dst, s.cellEnd.data(), (size_t)s.tableSize * 4); return 0;
    case 9: std::memcpy(dst, s.neighbors.data(), s.neighbors.size() * 4); return 0;
    case 10: std::memcpy(dst, s.initialPositions.data(), n * 12); return 0;
    }
    return -1;
}

__attribute__((visibility("default"))) void vr_set_positions(void* h, uint32_t first, uint32_t count,
                                                             const float* src)
{
    std::memcpy(static_cast<Solver*>(h)->positions.data() + first, src, (size_t)count * 12);
}
__attribute__((visibility("default"))) void vr_set_velocities(void* h, uint32_t first, uint32_t count,
                                                              const float* src)
{
    std::memcpy(static_cast<Solver*>(h)->velocities.data() + first, src, (size_t)count * 12);
}

// HashObjects on caller buffers (cellStart needs T + 1 entries)
__attribute__((visibility("default"))) void vr_hash_objects(uint32_t* phash, uint32_t* pindex, uint32_t* cstart,
                                                            uint32_t* cend, uint32_t* nbr, const float* pos,
                                                            const float* orig, const vt_hash_params* p)
{
    HashParams hp;
    hp.numObjects = p->num_objects;
    hp.maxNumNeighbors = p->max_num_neighbors;
    hp.cellSpacing = p->cell_spacing;
    hp.cellSpacing2 = p->cell_spacing2;
    hp.tableSize = p->table_size;
    hp.particleDiameter2 = p->particle_diameter2;
    Velvet::HashObjects(phash, pindex, cstart, cend, nbr, reinterpret_cast<const glm::vec3*>(pos),
                        reinterpret_cast<const glm::vec3*>(orig), hp);
}

}  // extern "C"
