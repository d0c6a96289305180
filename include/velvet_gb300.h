/*
 * velvet_gb300.h — C ABI of the GB300 XPBD cloth solver.
 *
 * The surface follows the GPU cloth solver of Velvet (vitalight/Velvet):
 *   - the class API of VtClothSolverGPU (Velvet/VtClothSolverGPU.hpp:114-205):
 *     AddCloth / AddStretch / AddAttachSlot / AddAttach / AddBend /
 *     UpdateColliders / Simulate, plus the public buffers callers mutate
 *     (positions, normals, invMasses, attachSlotPositions);
 *   - the constraint builder VtClothObjectGPU::Start (Velvet/VtClothObjectGPU.hpp:43-147);
 *   - the spatial-hash launch function HashObjects (Velvet/SpatialHashGPU.cuh:17-24).
 *
 * Conventions (differences from the reference are deliberate and listed):
 *   - every entry point returns a vt_status; nothing calls exit() (the reference's
 *     checkCudaErrors does) and no C++ exception crosses the ABI;
 *   - vector data crosses the ABI as float triples (x, y, z), the memory layout of
 *     glm::vec3 arrays; matrices are 16 floats, column-major (glm::mat4 layout);
 *   - `stream` arguments are cudaStream_t passed as void* (NULL = legacy default
 *     stream); work is enqueued asynchronously, getters that write host memory
 *     synchronise the stream first;
 *   - one handle must not be used from two host threads at once; separate handles
 *     are independent (the reference keeps its parameters in a process-wide
 *     __constant__ block and a global singleton, so it is not re-entrant at all).
 *
 * Arithmetic is FP32 with IEEE division and square root and no fused multiply-add,
 * and every Jacobi sum is accumulated per particle in constraint order, so results do
 * not depend on thread scheduling: two runs on the same inputs give identical bits.
 */
#ifndef VELVET_GB300_H
#define VELVET_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VT_ABI_VERSION 1

/* ------------------------------------------------------------------ status codes */
typedef int32_t vt_status;
#define VT_OK                    0
#define VT_ERR_INVALID_ARGUMENT (-1)  /* null pointer, index out of range, bad size  */
#define VT_ERR_OUT_OF_MEMORY    (-2)  /* device or host allocation failed           */
#define VT_ERR_CUDA             (-3)  /* a CUDA runtime call failed (see vt_last_error) */
#define VT_ERR_NOT_FOUND        (-4)  /* unknown request / cloth id                  */
#define VT_ERR_STATE            (-5)  /* call not valid in the handle's current state */
#define VT_ERR_CAPACITY         (-6)  /* a fixed limit or budget would be exceeded    */
#define VT_ERR_NUMERIC          (-7)  /* a device-side check found NaN/Inf state      */
#define VT_ERR_TIMEOUT          (-8)  /* a bounded wait gave up                       */

/* Collider kinds, in the order of Velvet's ColliderType (Velvet/Common.hpp:67-72). */
#define VT_COLLIDER_SPHERE 0
#define VT_COLLIDER_PLANE  1
#define VT_COLLIDER_CUBE   2

/* Simulation parameters: VtSimParams (Velvet/Common.hpp:19-48), same fields, same
 * defaults (vt_params_default).  Fields marked "runtime" are maintained by the solver
 * (AddCloth writes them, Velvet/VtClothSolverGPU.hpp:122-125). */
typedef struct vt_params {
    int32_t  num_substeps;             /* 2                                        */
    int32_t  num_iterations;           /* 4                                        */
    int32_t  max_num_neighbors;        /* 64 (1..64)                               */
    float    max_speed;                /* 50; AddCloth sets 2*d/dt*substeps        */
    float    gravity[3];               /* (0, -9.8, 0)                             */
    float    bend_compliance;          /* 0                                        */
    float    damping;                  /* 0.25                                     */
    float    relaxation_factor;        /* 1                                        */
    float    long_range_stretchiness;  /* 1.2                                      */
    float    collision_margin;         /* 0.06                                     */
    float    friction;                 /* 0.1                                      */
    int32_t  enable_self_collision;    /* 1                                        */
    int32_t  interleaved_hash;         /* 3: hash every n-th substep               */
    uint32_t num_particles;            /* runtime                                  */
    float    particle_diameter;        /* runtime: the last cloth's diameter       */
    float    delta_time;               /* fixed frame time, 1/60                   */
    float    particle_diameter_scalar; /* 1.5                                      */
    float    hash_cell_size_scalar;    /* 1.5                                      */
} vt_params;

/* One SDF collider: SDFCollider (Velvet/VtClothSolverGPU.cuh:8-18).  The caller fills
 * it the way VtClothSolverGPU::UpdateColliders does (Velvet/VtClothSolverGPU.hpp:187-205):
 * cur_transform is the upper-left 3x3 of the current model matrix, inv_cur_transform
 * its 4x4 inverse, last_transform the previous frame's model matrix, delta_time the
 * fixed frame time.  Planes use position.y, spheres position and scale.x (radius),
 * cubes the matrices and scale. */
typedef struct vt_sdf_collider {
    int32_t type;                  /* VT_COLLIDER_*                   */
    float   position[3];
    float   scale[3];
    float   delta_time;
    float   cur_transform[9];      /* mat3, column-major              */
    float   inv_cur_transform[16]; /* mat4, column-major              */
    float   last_transform[16];    /* mat4, column-major              */
} vt_sdf_collider;

/* Parameters of one spatial-hash build: HashParams (Velvet/SpatialHashGPU.cuh:7-15). */
typedef struct vt_hash_params {
    uint32_t num_objects;
    uint32_t max_num_neighbors;
    float    cell_spacing;
    float    cell_spacing2;
    int32_t  table_size;
    float    particle_diameter2;
} vt_hash_params;

typedef struct vt_solver vt_solver;

/* ------------------------------------------------------------------ library */

/* Fills *p with VtSimParams' defaults (Velvet/Common.hpp:21-46). */
void vt_params_default(vt_params* p);

/* Human-readable name of a status code. */
const char* vt_status_string(vt_status s);

/* Message of the last failure on the calling host thread ("" if none). */
const char* vt_last_error(void);

/* ABI version of the loaded library (VT_ABI_VERSION it was built with). */
int32_t vt_abi_version(void);

/* ------------------------------------------------------------------ plain solver */

/* Creates an empty solver; replaces `new VtClothSolverGPU` + Start()
 * (Velvet/VtClothSolverGPU.hpp:27-33).  params may be NULL (defaults). */
vt_status vt_solver_create(const vt_params* params, vt_solver** out);

/* Frees every device and host buffer of the solver (OnDestroy, :50-54). */
vt_status vt_solver_destroy(vt_solver* s);

/* Reads / replaces the solver's parameter block (Global::simParams). */
vt_status vt_solver_get_params(const vt_solver* s, vt_params* out);
vt_status vt_solver_set_params(vt_solver* s, const vt_params* p);

/* AddCloth (Velvet/VtClothSolverGPU.hpp:114-156): appends num_vertices particles at
 * model * (x, y, z, 1), the triangle indices offset by the previous particle count,
 * zero velocity, inverse mass 1; sets particle_diameter and max_speed in the params,
 * resizes the hash table to twice the particle count and snapshots the current
 * positions as the initial positions of the self-collision filter.
 * *out_offset receives the index of the cloth's first particle. */
vt_status vt_cloth_add(vt_solver* s, const float* xyz, uint32_t num_vertices,
                       const uint32_t* indices, uint32_t num_indices,
                       const float model[16], float particle_diameter,
                       int32_t* out_offset);

/* AddStretch (:158-163), in bulk: pairs[2*k], pairs[2*k+1], rest[k]. */
vt_status vt_stretch_add(vt_solver* s, const int32_t* pairs, const float* rest,
                         uint32_t count);

/* AddAttachSlot (:165-168): appends a slot; *out_slot gets its index (may be NULL). */
vt_status vt_attach_slot_add(vt_solver* s, const float xyz[3], int32_t* out_slot);

/* AddAttach (:170-176), in bulk: particle, slot, rest distance.  A distance of exactly
 * 0 sets that particle's inverse mass to 0, as the reference does. */
vt_status vt_attach_add(vt_solver* s, const int32_t* particles, const int32_t* slots,
                        const float* distances, uint32_t count);

/* Long-range attachments in compact form: the constraint set VtClothObjectGPU::
 * GenerateAttach (Velvet/VtClothObjectGPU.hpp:134-147) appends, i.e. for each slot k in
 * [first_slot, first_slot + num_slots), in that order, one attachment of every particle
 * in [particle_begin, particle_begin + particle_count) with rest distance
 * |slot_k - x_i| taken from the slot position at this call and the particles' current
 * positions.  The distances are recomputed on the device instead of stored (S x N of
 * them), with the same FP32 arithmetic, so the results equal those of the expanded
 * list; inverse masses of particles at distance 0 are set to 0. */
vt_status vt_attach_generate_lra(vt_solver* s, int32_t first_slot, uint32_t num_slots,
                                 int32_t particle_begin, uint32_t particle_count);

/* AddBend (:178-185), in bulk: quads[4*k .. 4*k+3], rest_angles[k]. */
vt_status vt_bend_add(vt_solver* s, const uint32_t* quads, const float* rest_angles,
                      uint32_t count);

/* VtClothObjectGPU::Start's constraint generation (Velvet/VtClothObjectGPU.hpp:43-58,
 * 75-147) for a (resolution+1)^2 grid cloth registered at `offset` with the triangle
 * order of Scene::GenerateClothMesh (Velvet/Scene.hpp:131-168): stretch constraints on
 * grid edges and both diagonals with rest lengths from the current positions, one
 * attach slot per entry of `attached` (cloth-local vertex indices) with long-range
 * attachments of every particle of the cloth, and one bend constraint per quad with
 * rest angle 0.  Slots get solver-global indices (the reference reuses 0..n-1 for each
 * cloth, which points a second cloth at the first cloth's slots; not reproduced). */
vt_status vt_cloth_build_grid_constraints(vt_solver* s, int32_t offset, int32_t resolution,
                                          const int32_t* attached, uint32_t num_attached);

/* General bending adjacency (no reference counterpart: GenerateBending pairs only the two
 * triangles of each grid quad, Velvet/VtClothObjectGPU.hpp:118-132).  For the cloth at
 * `offset`, every edge shared by exactly two of its triangles gets one bend constraint
 * over (first triangle's opposite vertex, second triangle's opposite vertex, shared
 * edge), hinges in order of their first triangle and corner, with the rest angle the
 * bending kernel measures at the initial positions (so the registered shape is at rest);
 * degenerate hinges are skipped.  Any triangle mesh; appended to the cloth's bends and
 * solved by the general (CSR) kernels.  *out_count (may be NULL) = constraints added. */
vt_status vt_cloth_build_bending_adjacency(vt_solver* s, int32_t offset, uint32_t* out_count);

/* UpdateColliders (:187-205): replaces the collider list (applied in list order). */
vt_status vt_colliders_set(vt_solver* s, const vt_sdf_collider* colliders, uint32_t count);

/* Simulate (:56-111) for one frame of length frame_dt, after setting substeps,
 * iterations, relaxation factor, friction, collision margin and particle diameter in
 * the parameter block (the reference reads them from Global::simParams).  Enqueued on
 * `stream`; returns without waiting.  Normals are recomputed at the end of the frame. */
vt_status vt_simulate(vt_solver* s, float frame_dt, int32_t substeps, int32_t iterations,
                      float relaxation, float friction, float collision_margin,
                      float particle_diameter, void* stream);

/* Blocks until all work enqueued on the solver has finished; reports a device-side
 * numeric fault (VT_ERR_NUMERIC) if one was flagged. */
vt_status vt_solver_sync(vt_solver* s);

/* Number of particles registered so far. */
vt_status vt_solver_num_particles(const vt_solver* s, uint32_t* out);

/* State access: `count` particles from `first`, as (x, y, z) triples.  With
 * *_on_device = 0 the buffer is ordinary host memory and the call returns after the
 * copy; with 1 it is any memory the device can address (device memory, or pinned /
 * registered host memory) and the copy is only enqueued on `stream`.  The public
 * buffers positions / normals / velocities of VtClothSolverGPU (:209-217). */
vt_status vt_positions_get(vt_solver* s, uint32_t first, uint32_t count, float* dst,
                           int32_t dst_on_device, void* stream);
vt_status vt_normals_get(vt_solver* s, uint32_t first, uint32_t count, float* dst,
                         int32_t dst_on_device, void* stream);
vt_status vt_velocities_get(vt_solver* s, uint32_t first, uint32_t count, float* dst,
                            int32_t dst_on_device, void* stream);
vt_status vt_positions_set(vt_solver* s, uint32_t first, uint32_t count, const float* src,
                           int32_t src_on_device, void* stream);
vt_status vt_velocities_set(vt_solver* s, uint32_t first, uint32_t count, const float* src,
                            int32_t src_on_device, void* stream);

/* invMasses (:217), mutated by MouseGrabber (Velvet/MouseGrabber.hpp:45-60). */
vt_status vt_inv_mass_get(vt_solver* s, uint32_t first, uint32_t count, float* dst);
vt_status vt_inv_mass_set(vt_solver* s, uint32_t first, uint32_t count, const float* src);

/* attachSlotPositions (:229), moved by scenes (Velvet/main.cpp:326-331). */
vt_status vt_attach_slot_set(vt_solver* s, int32_t slot, const float xyz[3]);

/* Debug views of the solver's spatial hash after the last hash build, in the
 * reference's layouts: VT_DEBUG_PARTICLE_HASH / _PARTICLE_INDEX (sorted keys and
 * particle ids, num_particles uint32 each), _CELL_START (table_size + 1), _CELL_END
 * (table_size), _NEIGHBORS (max_num_neighbors * num_particles, column-major
 * neighbors[id + k * num_particles], terminated by 0xffffffff), _PREDICTED (float3
 * per particle).  `bytes` is the size of dst; the call fails if it is too small. */
#define VT_DEBUG_PARTICLE_HASH  0
#define VT_DEBUG_PARTICLE_INDEX 1
#define VT_DEBUG_CELL_START     2
#define VT_DEBUG_CELL_END       3
#define VT_DEBUG_NEIGHBORS      4
#define VT_DEBUG_PREDICTED      5
#define VT_DEBUG_TABLE_SIZE     6   /* one int32 */
vt_status vt_solver_debug_get(vt_solver* s, int32_t what, void* dst, uint64_t bytes);

/* Kernel launches this solver has enqueued since it was created (every CUDA kernel of
 * this library counts; memsets and copies do not). */
vt_status vt_solver_launch_count(const vt_solver* s, uint64_t* out);

/* Replay each frame's launches as one CUDA graph (default 1); 0 launches every kernel
 * directly, as the reference does. */
vt_status vt_solver_use_graphs(vt_solver* s, int32_t on);

/* 1 (default): a cloth built by vt_cloth_build_grid_constraints is solved by the
 * implicit-topology tile kernel; 0: by the general CSR kernels, from the constraint lists
 * the builder generated.  Results are identical either way (a cross-check of the two
 * kernels); the next simulate rebuilds the device state. */
vt_status vt_solver_use_grid_kernel(vt_solver* s, int32_t on);

/* ------------------------------------------------------------------ checkpoint / resume
 * The simulation state of a solver as one flat binary (no reference counterpart; a reset
 * there re-runs the scene): a 16-byte header (magic "VTCK", version 1, particle count,
 * slot count), then positions (3 floats each), velocities (3), inverse masses (1) and
 * attach slot positions (3).  Loading it into a solver registered the same way (same
 * particle and slot counts) and continuing gives the bits the saved solver would have
 * produced: everything else a frame reads is rebuilt from these. */
vt_status vt_solver_state_size(const vt_solver* s, uint64_t* bytes);
vt_status vt_solver_state_save(vt_solver* s, void* dst, uint64_t bytes);
vt_status vt_solver_state_load(vt_solver* s, const void* src, uint64_t bytes);

/* ------------------------------------------------------------------ batched solver
 * Many independent cloths advanced together.  Each cloth is registered on its own
 * vt_solver (the plain API above), then copied into the batch, where it keeps its own
 * parameter block, spatial hash, colliders and attach slots: a cloth's result in the
 * batch is bit-identical to the same vt_solver simulated alone.  (The reference has no
 * isolated batching: several cloths added to one VtClothSolverGPU share one hash and
 * collide with each other, Velvet/main.cpp:243-279; that form is the plain solver.)
 * One frame of the whole batch is one CUDA graph launch of multi-cloth kernels. */
typedef struct vt_batch vt_batch;

vt_status vt_batch_create(vt_batch** out);
vt_status vt_batch_destroy(vt_batch* b);

/* Copies everything `cloth` has registered (particles, constraints, colliders, slots,
 * parameters, current state) into the batch; *out_index receives its index.  The
 * source solver may be destroyed afterwards. */
vt_status vt_batch_add(vt_batch* b, vt_solver* cloth, int32_t* out_index);

vt_status vt_batch_size(const vt_batch* b, int32_t* num_cloths, uint64_t* num_particles);

/* Replaces the colliders of cloth `index` (same count as when it was added). */
vt_status vt_batch_colliders_set(vt_batch* b, int32_t index, const vt_sdf_collider* colliders,
                                 uint32_t count);

/* Moves attach slot `slot` (cloth-local index) of cloth `index`. */
vt_status vt_batch_attach_slot_set(vt_batch* b, int32_t index, int32_t slot, const float xyz[3]);

/* One frame of every cloth, with the same frame arguments as vt_simulate.
 * particle_diameters: one per cloth, or NULL to use each cloth's registered diameter. */
vt_status vt_batch_simulate(vt_batch* b, float frame_dt, int32_t substeps, int32_t iterations,
                            float relaxation, float friction, float collision_margin,
                            const float* particle_diameters, void* stream);

vt_status vt_batch_sync(vt_batch* b);

/* Positions / normals / velocities of cloth `index` (all its particles), with the
 * dst_on_device convention of vt_positions_get. */
vt_status vt_batch_positions_get(vt_batch* b, int32_t index, float* dst, int32_t dst_on_device,
                                 void* stream);
vt_status vt_batch_normals_get(vt_batch* b, int32_t index, float* dst, int32_t dst_on_device,
                               void* stream);
vt_status vt_batch_velocities_get(vt_batch* b, int32_t index, float* dst, int32_t dst_on_device,
                                  void* stream);
/* Every cloth's state at once, cloth after cloth in index order: what = 0 positions,
 * 1 normals, 2 velocities. */
vt_status vt_batch_all_get(vt_batch* b, int32_t what, float* dst, int32_t dst_on_device, void* stream);

/* Pipelined read-back of every particle (what as vt_batch_all_get): packs on the
 * stream of the last vt_batch_simulate into one of two device buffers used in turn, then
 * copies into dst (pinned host or device memory) on copy_stream; returns at once.  The
 * next frames may be enqueued while the copy runs; dst is complete when copy_stream has
 * passed this call.  A buffer is reused only after its previous copy ended. */
vt_status vt_batch_all_get_async(vt_batch* b, int32_t what, float* dst, void* copy_stream);

/* Kernels enqueued by this batch so far (graph replays count their kernel nodes). */
vt_status vt_batch_launch_count(const vt_batch* b, uint64_t* out);

/* Use CUDA graphs for frames (default 1); 0 launches every kernel directly. */
vt_status vt_batch_use_graphs(vt_batch* b, int32_t on);

/* ------------------------------------------------------------------ served solver
 * Continuous batching of cloth-simulation requests (no reference counterpart).  A
 * request is one grid cloth registered on a vt_solver with
 * vt_cloth_build_grid_constraints, plus a number of frames.  Requests wait in a FIFO
 * queue; each vt_server_tick first retires finished requests (their final positions are
 * kept for vt_server_result), then admits queued requests while the device-memory
 * budget, the slot table and the active-particle cap allow, then advances every active
 * request by one frame with one set of multi-cloth launches.  Admitted state stays
 * resident on the device until retirement; admission and retirement never move other
 * requests' state.  A request's results are bit-identical to the same cloth simulated
 * alone on a vt_solver with the server's frame arguments. */
typedef struct vt_server vt_server;

typedef struct vt_server_config {
    uint64_t hbm_budget_bytes;     /* device memory the arena may use (admission budget)   */
    uint32_t max_cloths;           /* active request slots                                  */
    uint32_t max_active_particles; /* admission stops above this (0: no cap); bounds a tick */
    float    frame_dt;             /* frame arguments shared by all requests                */
    int32_t  substeps, iterations;
    float    relaxation, friction, collision_margin;
} vt_server_config;

#define VT_REQ_QUEUED 0
#define VT_REQ_ACTIVE 1
#define VT_REQ_DONE   2
#define VT_REQ_FAILED 3  /* its state became NaN / Inf: evicted, no result (VT_ERR_NUMERIC) */
#define VT_REQ_CANCELLED 4  /* cancelled by the client: dropped or evicted, no result */

typedef struct vt_server_tick_info {
    int32_t  admitted, retired, active, queued;
    uint64_t active_particles;
    double   frame_ms;             /* GPU time of the frame completed in this tick (the
                                      previous tick's frame; CUDA events), 0 if none      */
} vt_server_tick_info;

typedef struct vt_server_stats {
    uint64_t ticks, frames_done, requests_done;
    double   particle_iterations;  /* sum over ticks of active particles * substeps * iterations */
    double   gpu_ms;               /* sum of frame_ms                                        */
    double   p50_frame_ms, p99_frame_ms;  /* over all (request, frame) pairs                 */
    uint64_t bytes_in_use, bytes_budget;
    uint64_t requests_failed;      /* evicted after a NaN / Inf fault, the others unaffected */
    uint64_t requests_cancelled;   /* vt_server_cancel of a queued or active request         */
} vt_server_stats;

vt_status vt_server_create(const vt_server_config* cfg, vt_server** out);
vt_status vt_server_destroy(vt_server* s);

/* Queues `cloth` (copied; the solver may be destroyed afterwards) for `frames` frames.
 * VT_ERR_CAPACITY if the request could never be admitted (larger than the budget). */
vt_status vt_server_submit(vt_server* s, vt_solver* cloth, int32_t frames, int64_t* request_id);

/* A grid cloth described instead of registered (no reference counterpart; the device
 * form of GenerateClothMesh + AddCloth + VtClothObjectGPU::Start, Velvet/Scene.hpp:131-168,
 * Velvet/VtClothSolverGPU.hpp:114-156, Velvet/VtClothObjectGPU.hpp:43-147): vertex (a, b),
 * a, b in [0, resolution], at cloth_size * (b / resolution - 0.5, -(a / resolution), 0)
 * placed by `model`; the grid builder's stretch, bending and LRA attachments to the
 * `attached` vertices.  Admission builds positions, inverse masses and rest lengths on
 * the device: no per-particle work on the host.  The result equals registering the same
 * mesh with vt_cloth_add + vt_cloth_build_grid_constraints and vt_server_submit. */
typedef struct vt_grid_cloth {
    int32_t        resolution;
    float          cloth_size;
    float          model[16];          /* column-major, as vt_cloth_add */
    float          particle_diameter;  /* AddCloth's diameter, > 0 */
    const int32_t* attached;           /* at most 4 vertex indices */
    uint32_t       n_attached;
} vt_grid_cloth;

/* Queues a described grid cloth; params NULL = vt_params_default. */
vt_status vt_server_submit_grid(vt_server* s, const vt_grid_cloth* cloth, const vt_params* params,
                                const vt_sdf_collider* colliders, uint32_t n_colliders, int32_t frames,
                                int64_t* request_id);

/* Retire requests whose frames are all enqueued, admit queued ones, enqueue one frame
 * for every active request, then wait for the PREVIOUS tick's frame: the host work of a
 * tick overlaps the GPU work of the one before.  `active` counts admitted requests whose
 * result is not yet available; a request reaches VT_REQ_DONE one or two ticks after its
 * last frame was enqueued.  Use one stream per server (a change of stream synchronises
 * the old one first). */
vt_status vt_server_tick(vt_server* s, void* stream, vt_server_tick_info* info);

/* State (VT_REQ_*) and frames completed.  A request whose state turns NaN / Inf raises
 * its slot's fault flag; the tick that sees the flag evicts it at the next tick
 * (VT_REQ_FAILED, counted in requests_failed) and no other request is affected. */
vt_status vt_server_poll(vt_server* s, int64_t request_id, int32_t* state, int32_t* frames_done);

/* Cancels a request (a client that went away): a queued one leaves the queue at once; an
 * active one is evicted at the next tick, its range and slot returned as for a fault,
 * the requests beside it unaffected.  Either way it ends as VT_REQ_CANCELLED with no
 * result.  VT_ERR_STATE once its last frame is enqueued (it finishes normally) or it has
 * ended. */
vt_status vt_server_cancel(vt_server* s, int64_t request_id);

/* Final positions of a finished request (count = its particle count) into host memory;
 * VT_ERR_NUMERIC for an evicted request. */
vt_status vt_server_result(vt_server* s, int64_t request_id, float* dst, uint32_t count);

vt_status vt_server_stats_get(vt_server* s, vt_server_stats* out);

/* ------------------------------------------------------------------ headless rendering
 * The particles drawn as shaded spheres into an RGBA8 image by CUDA kernels, the
 * counterpart of Velvet's ParticleGeometryRenderer + _InstancedParticle shaders
 * (Velvet/ParticleGeometryRenderer.hpp, Velvet/Assets/Shader/_InstancedParticle.*):
 * each particle is a screen-space sphere impostor of radius particle_radius (the
 * reference draws diameter / 2), eye-space normal (u, v, sqrt(1 - u^2 - v^2)) over the
 * billboard, nearest surface wins, lit by ambient + max(0, N . light_dir) times tint,
 * gamma 2 (no graphics API exists on the target machines; no shadow map).
 * view / projection are column-major (glm::lookAt / glm::perspective: a symmetric
 * frustum); row 0 of the image is the top; pixels no particle covers get `background`. */
typedef struct vt_render_params {
    uint32_t width, height;
    float    view[16], projection[16];
    float    z_near;                /* particles nearer than this are not drawn */
    float    particle_radius;       /* world units */
    float    light_dir[3];          /* world space, towards the light, unit length */
    float    tint[3];               /* 0.2, 0.3, 0.6 in the reference */
    float    ambient;               /* 0.3 in the reference */
    uint32_t background;            /* RGBA8, red in the low byte */
} vt_render_params;

/* glm::lookAt (right-handed) and glm::perspective (depth -1..1) into column-major arrays. */
vt_status vt_camera_look_at(const float eye[3], const float center[3], const float up[3], float view[16]);
vt_status vt_camera_perspective(float fov_y_radians, float aspect, float z_near, float z_far, float proj[16]);

/* Renders the current positions of a solver (after its first simulate) or of every cloth
 * of a batch into rgba[width * height] (host or device-addressable memory). */
vt_status vt_solver_render(vt_solver* s, const vt_render_params* rp, uint32_t* rgba, int32_t dst_on_device,
                           void* stream);
vt_status vt_batch_render(vt_batch* b, const vt_render_params* rp, uint32_t* rgba, int32_t dst_on_device,
                          void* stream);

/* ------------------------------------------------------------------ tuning
 * The grid-cloth kernel has several variants; on its first frame a solver, batch or
 * server times them on its own cloths and keeps the fastest (decisions are cached per
 * size signature for the process).  The variant never changes a result.  This forces one
 * for all handles created or tuned afterwards: 0 = 7x31, 1 = 15x15, 2 = 3x63 tiles at
 * four resident blocks per SM, 3-5 the same shapes at five; -1 returns to autotuning. */
vt_status vt_tuning_set_grid_tile(int32_t variant);
/* How the grid-cloth kernel stages its tiles in shared memory: 1 with TMA bulk tensor
 * copies (one thread issues them, an mbarrier signals their arrival: ~5% fewer
 * instructions, but the block waits on one thread's copies), 0 (default, measured ~2%
 * faster) with one 16-byte cp.async per element by every thread.  Same results either
 * way; applies to frames enqueued (and CUDA graphs captured) afterwards.  No counterpart
 * in the reference (its kernels read global memory directly). */
vt_status vt_tuning_set_tile_loads(int32_t tma);
/* Small grid cloths run all Jacobi iterations of a substep in one launch of thread-block
 * clusters, one cluster of 16 blocks per cloth, with the cluster's hardware barrier
 * between iterations, when the solver's or batch's clusters all fit on the device at once
 * (else one launch per iteration is faster).  mode 1 (the default): when every cloth of a
 * solver or batch is within 64 x 64 particles, each block keeps one 16 x 16 tile of predicted positions in
 * shared memory for the whole substep and passes its edges to the neighbouring blocks
 * through distributed shared memory; otherwise, when every cloth is within 16 tiles of
 * the grid kernel, the blocks step through those tiles, reading positions from global
 * memory each iteration.  mode 2: the latter form only.  mode 0: one launch per
 * iteration.  Same results in every mode; applies to frames enqueued, and CUDA graphs
 * captured, afterwards (a solver or batch that already captured its frame graph keeps
 * it).  VT_ERR_INVALID_ARGUMENT for another mode.  The reference launches each constraint
 * kernel once per iteration (Velvet/VtClothSolverGPU.hpp:90-96). */
vt_status vt_tuning_set_substep_clusters(int32_t mode);
/* The shape in use by a solver / batch (after its first frame). */
vt_status vt_solver_grid_tile(const vt_solver* s, int32_t* variant);
vt_status vt_batch_grid_tile(const vt_batch* b, int32_t* variant);

/* ------------------------------------------------------------------ profiler
 * Per-stage GPU timing, the counterpart of the reference's ScopedTimerGPU labels
 * (Velvet/Timer.hpp:95-151, 242-260): while enabled, every stage launch of every
 * handle is bracketed by a pair of CUDA events on its stream.  vt_profiler_read waits
 * for the recorded events and reports, per stage, the launches and the summed event
 * time.  Process-wide; off by default. */
typedef struct vt_stage_time {
    char     name[32];
    uint64_t launches;
    double   total_ms;
} vt_stage_time;

vt_status vt_profiler_enable(int32_t on);
vt_status vt_profiler_reset(void);
/* Writes up to `capacity` entries; *count receives the number of stages with data. */
vt_status vt_profiler_read(vt_stage_time* out, uint32_t capacity, uint32_t* count);

/* ------------------------------------------------------------------ spatial hash */

/* HashObjects (Velvet/SpatialHashGPU.cu:159-196) on caller-owned device buffers:
 * hashes positions[num_objects] (float3) into cells of cell_spacing, sorts
 * (key, index) pairs stably by key, fills cell_start[table_size + 1] (0xffffffff for
 * empty cells) and cell_end[table_size] for occupied cells, and writes the column-major
 * neighbour lists with the initial-position filter.  Sort scratch space is allocated
 * on first use per device and kept until the library is unloaded (the reference keeps
 * a static cub buffer), so cudaDeviceReset after the first call on a device is not
 * supported.  Enqueued on `stream`. */
vt_status vt_hash_objects(uint32_t* particle_hash, uint32_t* particle_index,
                          uint32_t* cell_start, uint32_t* cell_end, uint32_t* neighbors,
                          const float* positions, const float* original_positions,
                          const vt_hash_params* params, void* stream);

/* HashObjects without any device allocation.  No counterpart in the reference: it
 * exists for callers that cannot call cudaMalloc — an engine that hands out all device
 * memory once at start-up and forbids allocation afterwards, a host that owns every
 * device allocation, or a real-time frame loop where cudaMalloc / cudaFree would
 * synchronise the device and stall the frame.  vt_hash_objects allocates its sort
 * scratch on first use; this variant uses a fixed scratch array compiled into the
 * library instead (about 2.4 MB, held on every GPU that loads the library until the
 * process exits), so it accepts at most VT_HASH_NOALLOC_MAX_OBJECTS objects and returns
 * VT_ERR_CAPACITY above that.  Same arguments, same outputs as vt_hash_objects.
 *   - The first call on each device looks up the scratch array's device address (a
 *     one-time set-up, no allocation); make that first call before any stream capture.
 *   - All calls share the one array: calls whose work overlaps on the GPU (different
 *     streams, or different host threads) race and corrupt each other's results;
 *     serialise them on one stream.
 *   - Nothing in the scratch needs to start at zero, so a previous call's contents do
 *     not affect the result.
 *   - The array's device address is kept for the life of the process: calling
 *     cudaDeviceReset on a device after its first call is not supported. */
#define VT_HASH_NOALLOC_MAX_OBJECTS 262144
vt_status vt_hash_objects_noalloc(uint32_t* particle_hash, uint32_t* particle_index,
                                  uint32_t* cell_start, uint32_t* cell_end, uint32_t* neighbors,
                                  const float* positions, const float* original_positions,
                                  const vt_hash_params* params, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* VELVET_GB300_H */
