// vt_host.h — host-side staging of one solver domain and the device world built from
// one or more of them.
#pragma once

#include <nvtx3/nvToolsExt.h>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/velvet_gb300.h"
#include "vt_world.h"

namespace vt {

// Last error message of the calling thread (vt_last_error).
void set_error(const std::string& msg);
vt_status cuda_fail(cudaError_t e, const char* what);

struct ClothRec {
    int32_t offset, count, tri_begin, tri_count;
};

// One entry of the attachment list, in constraint order: a single attachment
// (AddAttach) or a compact long-range-attachment group (GenerateAttach's S x N loop).
struct AttachOp {
    int32_t kind;  // 0 single, 1 group
    int32_t pid, slot;
    float dist;
    int32_t slot_begin, slot_count, p_begin, p_count;
};

// Everything a VtClothSolverGPU owns, staged on the host (Velvet/VtClothSolverGPU.hpp:
// 207-237).  Indices are solver-local.
struct HostSolver {
    vt_params P{};
    std::vector<float> x, v, x0;  // 3 floats per particle
    std::vector<float> w;         // inverse mass
    std::vector<uint32_t> tri;
    std::vector<ClothRec> cloths;
    std::vector<int32_t> st_idx;
    std::vector<float> st_rest;
    std::vector<float> slots, slots0;  // current / generation-time slot positions
    std::vector<AttachOp> at_ops;
    std::vector<uint32_t> bd_idx;
    std::vector<float> bd_rest;
    std::vector<vt_sdf_collider> colliders;
    float cell_spacing = 0.0f;
    int32_t table_size = 0;
    // Set when the solver holds exactly one grid cloth whose constraints are exactly what
    // vt_cloth_build_grid_constraints generates (verified element by element), so the
    // implicit-topology kernel computes the same sums as the CSR kernels: the grid
    // resolution, and the LRA slot range (local slot indices).
    int32_t grid_res = -1;
    int32_t grid_slot_begin = 0, grid_slot_count = 0;
    bool use_grid_kernel = true;

    uint32_t n() const { return (uint32_t)(x.size() / 3); }
    uint32_t nbend() const { return (uint32_t)bd_rest.size(); }
    uint32_t nslots() const { return (uint32_t)(slots.size() / 3); }
    // bytes of device memory World::build uses for this solver as one domain
    uint64_t device_bytes() const;
};

// An NVTX range over a host scope (frame submission, server tick, stage launches):
// visible in a timeline tool when one is attached, a no-op otherwise (header-only NVTX).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// Per-stage GPU timing (vt_profiler_*): event pairs around stage launches.
enum Stage {
    ST_PRESDF_PREDICT, ST_HASH_KEYS, ST_RADIX_SORT, ST_CELL_RANGES, ST_CACHE_NEIGHBORS,
    ST_COLLIDE, ST_BEND, ST_SOLVE, ST_FINALIZE, ST_NORMALS, ST_GRID_ITER, ST_COUNT
};
const char* stage_name(int stage);
bool profiler_on();
vt_status profiler_enable(bool on);
vt_status profiler_reset();
vt_status profiler_read(vt_stage_time* out, uint32_t cap, uint32_t* count);
struct StageScope {
    StageScope(int stage, cudaStream_t st);
    ~StageScope();
    int stage;
    cudaStream_t st;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
};

// Per-frame arguments of Simulate.
struct FrameArgs {
    float frame_dt;
    int32_t substeps, iterations;
    float relax, friction, margin, diameter;
};

// Device state of a list of domains and the launch schedule of one frame.
class World {
public:
    World() = default;
    ~World();
    World(const World&) = delete;
    World& operator=(const World&) = delete;

    // Allocates and uploads everything; each host solver becomes one domain.
    vt_status build(const std::vector<const HostSolver*>& doms);
    void release();
    bool built() const { return built_; }

    // Writes the per-frame parameters of domain k (host copy; uploaded by simulate).
    void set_frame(int k, const HostSolver& h, const FrameArgs& a);
    // Replaces domain k's colliders / slot positions (host copy; uploaded by simulate).
    vt_status set_colliders(int k, const std::vector<vt_sdf_collider>& c);
    vt_status set_slot(int k, int32_t slot, const float xyz[3]);
    // Enqueues one frame for all domains on `st`: the per-frame uploads (parameters,
    // colliders, slots), then the kernels, either launched directly or as one CUDA graph
    // captured on first use for this (substeps, iterations, hash interval, self) key.
    vt_status simulate(const FrameArgs& a, int32_t interleaved_hash, bool any_self, cudaStream_t st,
                       bool use_graph = false);
    // kernels of one frame only (no uploads)
    vt_status enqueue_frame(const FrameArgs& a, int32_t interleaved_hash, bool any_self, cudaStream_t st);
    vt_status upload_frame(cudaStream_t st);
    // Reads back status flags (after the stream finished); bit 0 = non-finite state.
    vt_status read_status(std::vector<int32_t>& flags, cudaStream_t st);
    vt_status clear_status(cudaStream_t st);

    DeviceArrays d;
    std::vector<DomainParams> hdom;
    std::vector<ColliderDev> hcol;
    std::vector<float4> hslots;
    int32_t n_domains = 0, n_particles = 0, n_bends = 0, n_slots = 0, n_cols = 0;
    int32_t total_keys = 0, n_ptiles = 0, n_btiles = 0, nbr_words = 0;
    int32_t n_stiles = 0, n_gtiles = 0, n_gptiles = 0;
    int32_t grid_variant = 0;  // grid kernel variant (kGridVariant index)
    // Times every grid kernel variant on this world's cloths (one Jacobi iteration each,
    // from the current positions, into scratch buffers) and keeps the fastest; decisions
    // are cached per size signature for the process.  A cached or forced variant applies
    // at once; timing waits for may_time (a frame simulated), the default variant runs
    // until then.  Never changes a result.
    vt_status autotune(cudaStream_t st, bool may_time);
    vt_status set_grid_variant(int variant);
    int32_t pcur = 0;  // which of p[0], p[1] holds the latest predicted positions
    uint64_t bytes = 0;
    uint64_t launches = 0;  // kernels enqueued so far

private:
    bool built_ = false;
    void* arena_ = nullptr;
    void* staging_ = nullptr;  // pinned: DomainParams + ColliderDev + slots
    size_t staging_bytes_ = 0;
    cudaEvent_t staged_ = nullptr;
    bool cols_dirty_ = true, slots_dirty_ = true;
    bool tuned_ = false;
    int64_t frames_ = 0;  // frames simulated since the last build
    std::vector<std::pair<int32_t, int32_t>> grid_doms_;  // (domain, resolution) of grid domains
    int32_t gtiles_cap_ = 0;
    // cluster-resident substeps (small grid cloths): per grid cloth its tile range
    int2* cloth_tiles_dev_ = nullptr;
    int32_t n_cluster_cloths_ = 0;
    bool cluster_ok_ = false;
    // the resident form (every cloth within kResidentMaxSide): per cloth (domain, 0)
    int2* cloth_doms_dev_ = nullptr;
    int32_t n_resident_cloths_ = 0;
    bool resident_ok_ = false;
    vt_status update_cluster_plan();
    // frame graph
    cudaStream_t cap_ = nullptr;
    cudaGraphExec_t gexec_ = nullptr;
    int32_t gkey_[4] = {-1, -1, -1, -1};
    uint64_t glaunches_ = 0;
    int32_t gpcur_ = 0;
};

// The plain solver handle (vt_solver in the C ABI).
struct SolverImpl {
    HostSolver h;
    World world;
    bool topo_dirty = true;  // particles or constraints changed: rebuild the device world
    bool on_device = false;  // the device holds the authoritative x, v, inverse mass
    bool simulated = false;  // normals / hash views exist
    bool use_graph = true;
    cudaStream_t stream = nullptr;
    uint64_t launches_before = 0;  // launches of worlds replaced by rebuilds
};
// Copies x, v and inverse mass from the device back into the host staging.
vt_status pull_state(SolverImpl* s);

// Headless rendering (vt_render.cu): parameter check, and x[0, n) rendered into dst.
bool render_params_valid(const vt_render_params& rp);
vt_status render_to(const float4* x, int64_t n, const vt_render_params& rp, uint32_t* dst, bool dst_on_device,
                    cudaStream_t st, uint64_t* launches);

ColliderDev collider_to_device(const vt_sdf_collider& c);

// Grid kernel variant to use: the forced one (vt_tuning_set), else `tuned`.
int grid_variant_for(int tuned);
// Forces a grid kernel variant for every world (-1: autotune again).
vt_status tuning_force(int32_t variant);

// Per-frame fields of a domain's parameter block from its vt_params and frame arguments.
void fill_frame_params(DomainParams& D, const vt_params& P, const FrameArgs& a);
// Grid domains: per-generator stretch rest lengths (from the constraint list) and
// per-particle LRA rest distances, one float4 per particle each.
void grid_rests(const HostSolver& h, float4* grest, float4* glra);

}  // namespace vt

struct vt_solver : vt::SolverImpl {};
