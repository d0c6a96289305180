// vt_world.cu — builds the device state of one or more solver domains (grid rests and
// tiles for grid cloths, CSR adjacency for other meshes, hash buffers), autotunes the
// grid kernel's tile variant, and enqueues (or replays as a CUDA graph) one frame.
//
// Schedule of one frame (Velvet/VtClothSolverGPU.hpp:56-111, with the fusions listed
// in vt_kernels.cu):
//   presdf_predict                           CollideSDF(x, frameDt) + Predict(substep 0)
//   for each substep s:
//     if self-collision and s % interleavedHash == 0:
//        fill the cell ranges 0xff, hash_keys, radix sort, cell_ranges_gather
//        (+ sorted copies of the positions), cache_neighbors
//     collide                                CollideParticles + ApplyDeltas + CollideSDF
//     for each iteration:                    Stretch + Attach + Bending + ApplyDeltas
//       grid_iter (grid domains) and bend + solve (CSR domains); the last iteration
//       also runs Finalize and, except after the last substep, the next Predict
//   normals
#include <cudaTypedefs.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <mutex>
#include <string>

#include "vt_host.h"
#include "vt_math.cuh"

namespace vt {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }
const std::string& last_error() { return g_last_error; }

vt_status cuda_fail(cudaError_t e, const char* what)
{
    set_error(std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
    return e == cudaErrorMemoryAllocation ? VT_ERR_OUT_OF_MEMORY : VT_ERR_CUDA;
}

#define VT_CUDA(call, what)                                 \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_fail(e_, what);  \
    } while (0)

static constexpr int kTile = 256;

// ------------------------------------------------------------------ profiler
namespace {
struct Pending {
    int stage;
    cudaEvent_t e0, e1;
};
struct ProfilerState {
    std::mutex mu;
    bool on = false;
    std::vector<cudaEvent_t> pool;
    std::vector<Pending> pending;
    uint64_t launches[ST_COUNT] = {};
    double ms[ST_COUNT] = {};
};
ProfilerState& prof()
{
    static ProfilerState* p = new ProfilerState();  // never destroyed: outlives static teardown
    return *p;
}
cudaEvent_t take_event(ProfilerState& P)
{
    if (!P.pool.empty()) {
        cudaEvent_t e = P.pool.back();
        P.pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}
// Folds finished event pairs into the totals; with `wait`, waits for all of them.
void drain(ProfilerState& P, bool wait)
{
    std::vector<Pending> keep;
    for (const Pending& q : P.pending) {
        if (!wait && cudaEventQuery(q.e1) == cudaErrorNotReady) {
            keep.push_back(q);
            continue;
        }
        if (wait) cudaEventSynchronize(q.e1);
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, q.e0, q.e1) == cudaSuccess) {
            P.ms[q.stage] += ms;
            P.launches[q.stage] += 1;
        }
        P.pool.push_back(q.e0);
        P.pool.push_back(q.e1);
    }
    cudaGetLastError();  // clear a not-ready status left by cudaEventQuery
    P.pending.swap(keep);
}
}  // namespace

const char* stage_name(int s)
{
    static const char* names[ST_COUNT] = {"presdf_predict", "hash_keys", "radix_sort", "cell_ranges",
                                          "cache_neighbors", "collide", "bend", "solve", "finalize",
                                          "normals", "grid_iter"};
    return (s >= 0 && s < ST_COUNT) ? names[s] : "?";
}

bool profiler_on() { return prof().on; }

StageScope::StageScope(int stage_, cudaStream_t st_) : stage(stage_), st(st_)
{
    nvtxRangePushA(stage_name(stage_));
    ProfilerState& P = prof();
    if (!P.on) return;
    std::lock_guard<std::mutex> lock(P.mu);
    e0 = take_event(P);
    e1 = take_event(P);
    cudaEventRecord(e0, st);
}

StageScope::~StageScope()
{
    nvtxRangePop();
    if (!e0) return;
    ProfilerState& P = prof();
    std::lock_guard<std::mutex> lock(P.mu);
    cudaEventRecord(e1, st);
    P.pending.push_back(Pending{stage, e0, e1});
    if (P.pending.size() > 4096) drain(P, false);
}

vt_status profiler_enable(bool on)
{
    ProfilerState& P = prof();
    std::lock_guard<std::mutex> lock(P.mu);
    P.on = on;
    return VT_OK;
}

vt_status profiler_reset()
{
    ProfilerState& P = prof();
    std::lock_guard<std::mutex> lock(P.mu);
    drain(P, true);
    for (int s = 0; s < ST_COUNT; ++s) {
        P.ms[s] = 0;
        P.launches[s] = 0;
    }
    return VT_OK;
}

vt_status profiler_read(vt_stage_time* out, uint32_t cap, uint32_t* count)
{
    ProfilerState& P = prof();
    std::lock_guard<std::mutex> lock(P.mu);
    drain(P, true);
    uint32_t n = 0;
    for (int s = 0; s < ST_COUNT; ++s) {
        if (!P.launches[s]) continue;
        if (out && n < cap) {
            std::memset(&out[n], 0, sizeof(vt_stage_time));
            std::strncpy(out[n].name, stage_name(s), sizeof(out[n].name) - 1);
            out[n].launches = P.launches[s];
            out[n].total_ms = P.ms[s];
        }
        ++n;
    }
    if (count) *count = n;
    return VT_OK;
}

// ------------------------------------------------------------------ tuning state
namespace {
std::mutex g_tune_mu;
int g_forced_variant = -1;
std::vector<std::pair<std::vector<int64_t>, int>> g_tune_cache;  // signature -> variant
}  // namespace

int grid_variant_for(int tuned)
{
    std::lock_guard<std::mutex> lock(g_tune_mu);
    return g_forced_variant >= 0 ? g_forced_variant : tuned;
}

// ------------------------------------------------------------------ tensor maps
namespace {
std::atomic<bool> g_tile_tma{false};  // per-thread cp.async measured faster (see vt_tuning_set_tile_loads)

PFN_cuTensorMapEncodeTiled_v12000 tmap_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// A V x V grid of float4 at base as a 3-D FP32 tensor (xyzw, column, row) with a box of
// bw columns by bh rows.
bool encode_one(CUtensorMap* m, const float4* base, int V, int bw, int bh)
{
    PFN_cuTensorMapEncodeTiled_v12000 enc = tmap_encoder();
    if (!enc) {
        set_error("cuTensorMapEncodeTiled is not available from the driver");
        return false;
    }
    const cuuint64_t dims[3] = {4, (cuuint64_t)V, (cuuint64_t)V};
    const cuuint64_t strides[2] = {16, (cuuint64_t)V * 16};  // bytes, dims 1 and 2
    const cuuint32_t box[3] = {4, (cuuint32_t)bw, (cuuint32_t)bh};
    const cuuint32_t es[3] = {1, 1, 1};
    const CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float4*>(base), dims, strides, box, es,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
        return false;
    }
    return true;
}
}  // namespace

bool encode_grid_tmaps(CUtensorMap* dst, const float4* p0, const float4* p1, const float4* grest,
                       const float4* glra, const float4* x, int64_t p_begin, int V)
{
    static_assert(sizeof(CUtensorMap) == 128, "tensor map size");
    const int shapes[kTmapShapes][2] = {{7, 31}, {15, 15}, {3, 63}};
    for (int sh = 0; sh < kTmapShapes; ++sh) {
        const int ta = shapes[sh][0], tb = shapes[sh][1];
        CUtensorMap* m = dst + tmap_index(0, sh, 0);
        if (!encode_one(m + TMAP_P0, p0 + p_begin, V, tb + 2, ta + 2) ||
            !encode_one(m + TMAP_P1, p1 + p_begin, V, tb + 2, ta + 2) ||
            !encode_one(m + TMAP_GREST, grest + p_begin, V, tb + 1, ta + 1) ||
            !encode_one(m + TMAP_GLRA, glra + p_begin, V, tb, ta) || !encode_one(m + TMAP_X, x + p_begin, V, tb, ta))
            return false;
    }
    return true;
}

bool tile_loads_tma() { return g_tile_tma.load(); }

namespace {
std::atomic<int> g_substep_clusters{1};
}
int substep_clusters_mode() { return g_substep_clusters.load(); }
vt_status set_substep_clusters(int mode)
{
    if (mode < 0 || mode > 2) {
        set_error("substep cluster mode must be 0, 1 or 2");
        return VT_ERR_INVALID_ARGUMENT;
    }
    g_substep_clusters.store(mode);
    return VT_OK;
}
vt_status set_tile_loads_tma(bool on)
{
    g_tile_tma.store(on);
    return VT_OK;
}

vt_status tuning_force(int32_t variant)
{
    if (variant < -1 || variant >= kGridVariants) {
        set_error("grid tile variant out of range");
        return VT_ERR_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_forced_variant = variant;
    return VT_OK;
}

ColliderDev collider_to_device(const vt_sdf_collider& c)
{
    ColliderDev d{};
    d.type = c.type;
    d.px = c.position[0]; d.py = c.position[1]; d.pz = c.position[2];
    d.sx = c.scale[0]; d.sy = c.scale[1]; d.sz = c.scale[2];
    d.delta_time = c.delta_time;
    std::memcpy(d.cur3, c.cur_transform, sizeof(d.cur3));
    std::memcpy(d.inv, c.inv_cur_transform, sizeof(d.inv));
    // VelocityAt: lastTransform * invCurTransform (glm mat4 product order)
    m4m4(c.last_transform, c.inv_cur_transform, d.last_inv);
    return d;
}

uint64_t HostSolver::device_bytes() const
{
    const uint64_t N = n(), B = nbend(), T = (uint64_t)table_size + 1;
    uint64_t at = 0;
    for (const AttachOp& a : at_ops) at += a.kind == 0 ? 1 : (uint64_t)a.p_count;
    const uint64_t mn = (uint64_t)P.max_num_neighbors;
    uint64_t b = 0;
    b += N * 16 * 6;                       // x, v, x0, p[2], nrm
    b += (N + 1) * 4 * 4;                  // st/at/bd/tn offsets
    b += st_rest.size() * 2 * 8;           // stretch entries
    b += at * 8;                           // attach entries
    b += B * (16 + 4 + 64) + B * 4 * 4;    // bend idx, rest, corners, entries
    b += tri.size() / 3 * (16 + 12);       // triangles + entries
    b += N * 4 * 4 + (N / 4096 + 2) * 256 * 4;  // keys, vals, tmp, hist
    b += T * 8 + mn * N * 4;               // cells, neighbours
    b += (uint64_t)nslots() * 32 + colliders.size() * sizeof(ColliderDev);
    return b + 64 * 256;                   // alignment slack
}

World::~World() { release(); }

void World::release()
{
    if (gexec_) cudaGraphExecDestroy(gexec_);
    if (cap_) cudaStreamDestroy(cap_);
    if (arena_) cudaFree(arena_);
    if (staging_) cudaFreeHost(staging_);
    if (staged_) cudaEventDestroy(staged_);
    gexec_ = nullptr;
    cap_ = nullptr;
    gkey_[0] = gkey_[1] = gkey_[2] = gkey_[3] = -1;
    arena_ = nullptr;
    staging_ = nullptr;
    staged_ = nullptr;
    d = DeviceArrays{};
    hdom.clear();
    hcol.clear();
    hslots.clear();
    grid_doms_.clear();
    built_ = false;
    tuned_ = false;
    frames_ = 0;
    bytes = 0;
}

vt_status World::set_grid_variant(int variant)
{
    std::vector<GridTile> gt;
    for (auto& gd : grid_doms_) grid_tiles_for(gt, gd.first, hdom[gd.first], variant);
    if ((int32_t)gt.size() > gtiles_cap_) {
        set_error("grid tile table capacity exceeded");
        return VT_ERR_STATE;
    }
    if (!gt.empty())
        VT_CUDA(cudaMemcpy(d.gtiles, gt.data(), gt.size() * sizeof(GridTile), cudaMemcpyHostToDevice),
                "upload gtiles");
    n_gtiles = (int32_t)gt.size();
    grid_variant = variant;
    {
        const vt_status r = update_cluster_plan();
        if (r != VT_OK) return r;
    }
    if (gexec_) {  // a captured frame bakes in the tile count
        cudaGraphExecDestroy(gexec_);
        gexec_ = nullptr;
        gkey_[0] = -1;
    }
    return VT_OK;
}

// Tile ranges of the grid cloths for the cluster-resident substep kernel, and whether this
// world can use it: every domain solved by the tile kernel (no CSR domain has launches of
// its own inside the iterations) and every cloth within kClusterMaxTiles tiles.
vt_status World::update_cluster_plan()
{
    cluster_ok_ = false;
    resident_ok_ = false;
    n_cluster_cloths_ = 0;
    if (grid_doms_.empty() || n_stiles || n_btiles || (int32_t)grid_doms_.size() != n_domains) return VT_OK;
    {
        // the resident form: every cloth within 4 x 4 tiles of 16 x 16 particles
        std::vector<int2> doms;
        for (auto& gd : grid_doms_) {
            if (hdom[gd.first].grid_res + 1 > kResidentMaxSide) {
                doms.clear();
                break;
            }
            doms.push_back(make_int2(gd.first, 0));
        }
        if (!doms.empty() && (int64_t)doms.size() <= substep_resident_capacity()) {
            VT_CUDA(cudaMemcpy(cloth_doms_dev_, doms.data(), doms.size() * sizeof(int2), cudaMemcpyHostToDevice),
                    "upload resident cloth list");
            n_resident_cloths_ = (int32_t)doms.size();
            resident_ok_ = true;
        }
    }
    std::vector<int2> ranges;
    int32_t t0 = 0;
    for (auto& gd : grid_doms_) {
        std::vector<GridTile> tmp;
        grid_tiles_for(tmp, gd.first, hdom[gd.first], grid_variant);
        if ((int32_t)tmp.size() > kClusterMaxTiles) return VT_OK;
        ranges.push_back(make_int2(t0, t0 + (int32_t)tmp.size()));
        t0 += (int32_t)tmp.size();
    }
    if (t0 != n_gtiles || (int64_t)ranges.size() > substep_cluster_capacity()) return VT_OK;
    VT_CUDA(cudaMemcpy(cloth_tiles_dev_, ranges.data(), ranges.size() * sizeof(int2), cudaMemcpyHostToDevice),
            "upload cloth tile ranges");
    n_cluster_cloths_ = (int32_t)ranges.size();
    cluster_ok_ = true;
    return VT_OK;
}

vt_status World::autotune(cudaStream_t st, bool may_time)
{
    if (grid_doms_.empty()) {
        tuned_ = true;
        return VT_OK;
    }
    int forced = -1;
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        forced = g_forced_variant;
    }
    if (forced >= 0) {
        tuned_ = true;
        return forced == grid_variant ? VT_OK : set_grid_variant(forced);
    }
    // signature: cloth count and total particles (log2 buckets), mean side
    int64_t parts = 0;
    for (auto& gd : grid_doms_) parts += (int64_t)(gd.second + 1) * (gd.second + 1);
    auto lg = [](int64_t v) { int b = 0; while ((1ll << b) < v) ++b; return (int64_t)b; };
    const std::vector<int64_t> sig{lg((int64_t)grid_doms_.size()), lg(parts),
                                   lg(parts / (int64_t)grid_doms_.size())};
    int best = -1;
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        for (auto& e : g_tune_cache)
            if (e.first == sig) best = e.second;
    }
    if (best < 0 && !may_time) return VT_OK;  // the default variant until a frame has moved the cloths
    tuned_ = true;
    if (best < 0) {
        // time one Jacobi iteration per variant from the current positions (x -> p[0] ->
        // p[1]), once a frame has been simulated: at the registered rest state (x == x0)
        // every stretch constraint has d == rest and returns early, which is not the cost
        // of a frame
        VT_CUDA(cudaMemcpyAsync(d.p[0], d.x, 16 * (size_t)n_particles, cudaMemcpyDeviceToDevice, st), "tune copy");
        cudaEvent_t e0, e1;
        VT_CUDA(cudaEventCreate(&e0), "event");
        VT_CUDA(cudaEventCreate(&e1), "event");
        // three interleaved rounds over the variants (a warm-up and three timed launches
        // each), the lowest total kept: variants within a percent of each other are ranked
        // under the same drift of clocks and caches
        constexpr int kRounds = 3;
        float total[kGridVariants] = {};
        for (int round = 0; round < kRounds; ++round)
            for (int v = 0; v < kGridVariants; ++v) {
                vt_status r = set_grid_variant(v);
                if (r != VT_OK) return r;
                Launch L{&d, n_ptiles, n_btiles, n_particles, st, n_stiles, n_gtiles, n_gptiles, grid_variant};
                VT_CUDA(launch_grid_iter(L, 0, 1, SOLVE_PLAIN), "tune warm-up");
                VT_CUDA(cudaEventRecord(e0, st), "event");
                for (int k = 0; k < 3; ++k) VT_CUDA(launch_grid_iter(L, 0, 1, SOLVE_PLAIN), "tune");
                VT_CUDA(cudaEventRecord(e1, st), "event");
                VT_CUDA(cudaEventSynchronize(e1), "tune sync");
                float ms = 0;
                VT_CUDA(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
                launches += 4;
                total[v] += ms;
            }
        for (int v = 0; v < kGridVariants; ++v)
            if (best < 0 || total[v] < total[best]) best = v;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tune_cache.push_back({sig, best});
    }
    return best == grid_variant ? VT_OK : set_grid_variant(best);
}

namespace {
struct Arena {
    size_t off = 0;
    template <typename T>
    size_t take(size_t count)
    {
        const size_t at = off;
        off += (count * sizeof(T) + 255) & ~size_t(255);
        return at;
    }
};

void tiles_for(std::vector<Tile>& out, int dom, int begin, int count)
{
    for (int b = begin; b < begin + count; b += kTile) {
        Tile t;
        t.dom = dom;
        t.begin = b;
        t.end = std::min(begin + count, b + kTile);
        t.pad_ = 0;
        out.push_back(t);
    }
}

// counting-sort style CSR: `rows` entries per row in the order items are pushed
template <typename E>
struct Csr {
    std::vector<int32_t> off;
    std::vector<E> ent;
    std::vector<int32_t> cur;
    void init(size_t rows) { off.assign(rows + 1, 0); }
    void count(int32_t r) { off[r + 1]++; }
    void finish_counts()
    {
        for (size_t r = 1; r < off.size(); ++r) off[r] += off[r - 1];
        ent.resize(off.back());
        cur.assign(off.begin(), off.end() - 1);
    }
    void put(int32_t r, const E& e) { ent[cur[r]++] = e; }
};
}  // namespace

vt_status World::build(const std::vector<const HostSolver*>& S)
{
    release();
    n_domains = (int32_t)S.size();
    // domains solved by the implicit-topology grid kernel (their CSR rows stay empty)
    std::vector<char> grid(S.size());
    for (size_t k = 0; k < S.size(); ++k) grid[k] = S[k]->grid_res >= 1 && S[k]->use_grid_kernel;
    int64_t N = 0, B = 0, SL = 0, C = 0, G = 0, TR = 0, TK = 0, NW = 0;
    for (size_t k = 0; k < S.size(); ++k) {
        const HostSolver* h = S[k];
        N += h->n();
        B += grid[k] ? 0 : h->nbend();
        SL += h->nslots();
        C += (int64_t)h->colliders.size();
        TR += (int64_t)h->tri.size() / 3;
        TK += (int64_t)h->table_size + 1;
        NW += (int64_t)h->P.max_num_neighbors * h->n();
        for (const AttachOp& a : h->at_ops) G += a.kind == 1;
    }
    if (N > INT32_MAX / 2 || TK > INT32_MAX / 2 || NW > INT32_MAX) {
        set_error("world too large for 32-bit indices");
        return VT_ERR_CAPACITY;
    }
    n_particles = (int32_t)N;
    n_bends = (int32_t)B;
    n_slots = (int32_t)SL;
    n_cols = (int32_t)C;
    total_keys = (int32_t)TK;
    nbr_words = (int32_t)NW;

    // ---- host images
    std::vector<float4> hx(N), hv(N), hx0(N), hp(N);
    std::vector<float4> hslot(SL), hslot0(SL);
    std::vector<LraGroup> hlra;
    std::vector<uint4> hbd(B);
    std::vector<float> hbr(B);
    std::vector<uint4> htri(TR);
    Csr<int2> st;
    Csr<int2> at;
    Csr<int32_t> bd;
    Csr<int32_t> tn;
    st.init(N);
    at.init(N);
    bd.init(N);
    tn.init(N);
    std::vector<Tile> pt, st_tiles, bt, gpt;
    std::vector<GridTile> gt;
    std::vector<float4> hgrest(N, make_float4(0, 0, 0, 0)), hglra(N, make_float4(0, 0, 0, 0));
    hdom.assign(n_domains, DomainParams{});
    hcol.clear();

    int32_t pb = 0, bb = 0, sb = 0, tb = 0, tkb = 0, nwb = 0, gb = 0, cb = 0;
    // pass 1: counts
    {
        int32_t p0 = 0;
        for (size_t k = 0; k < S.size(); ++k) {
            const HostSolver* h = S[k];
            if (grid[k]) {
                p0 += (int32_t)h->n();
                continue;
            }
            for (size_t q = 0; q < h->tri.size() / 3 * 3; ++q) tn.count(p0 + (int32_t)h->tri[q]);
            for (size_t c = 0; c < h->st_rest.size(); ++c) {
                st.count(p0 + h->st_idx[2 * c]);
                st.count(p0 + h->st_idx[2 * c + 1]);
            }
            for (const AttachOp& a : h->at_ops) {
                if (a.kind == 0) at.count(p0 + a.pid);
                else
                    for (int32_t i = 0; i < a.p_count; ++i) at.count(p0 + a.p_begin + i);
            }
            for (size_t q = 0; q < h->bd_idx.size(); ++q) bd.count(p0 + (int32_t)h->bd_idx[q]);
            p0 += (int32_t)h->n();
        }
    }
    st.finish_counts();
    at.finish_counts();
    bd.finish_counts();
    tn.finish_counts();

    // pass 2: fill
    for (int32_t k = 0; k < n_domains; ++k) {
        const HostSolver& h = *S[k];
        const int32_t n = (int32_t)h.n();
        for (int32_t i = 0; i < n; ++i) {
            const float w = h.w[i];
            hx[pb + i] = make_float4(h.x[3 * i], h.x[3 * i + 1], h.x[3 * i + 2], w);
            hv[pb + i] = make_float4(h.v[3 * i], h.v[3 * i + 1], h.v[3 * i + 2], 0.0f);
            hx0[pb + i] = make_float4(h.x0[3 * i], h.x0[3 * i + 1], h.x0[3 * i + 2], 0.0f);
            hp[pb + i] = make_float4(0, 0, 0, w);
        }
        for (uint32_t s = 0; s < h.nslots(); ++s) {
            hslot[sb + s] = make_float4(h.slots[3 * s], h.slots[3 * s + 1], h.slots[3 * s + 2], 0.0f);
            hslot0[sb + s] = make_float4(h.slots0[3 * s], h.slots0[3 * s + 1], h.slots0[3 * s + 2], 0.0f);
        }
        const bool g = grid[k] != 0;
        for (size_t c = 0; !g && c < h.st_rest.size(); ++c) {
            const int32_t a = pb + h.st_idx[2 * c], b = pb + h.st_idx[2 * c + 1];
            int32_t rb;
            std::memcpy(&rb, &h.st_rest[c], 4);
            st.put(a, make_int2(b, rb));
            st.put(b, make_int2(a, rb));
        }
        for (const AttachOp& a : h.at_ops) {
            if (g) break;
            if (a.kind == 0) {
                int32_t db;
                std::memcpy(&db, &a.dist, 4);
                at.put(pb + a.pid, make_int2(sb + a.slot, db));
            } else {
                LraGroup g;
                g.slot_begin = sb + a.slot_begin;
                g.slot_count = a.slot_count;
                g.p_begin = pb + a.p_begin;
                g.p_count = a.p_count;
                hlra.push_back(g);
                const int32_t gid = gb++;
                for (int32_t i = 0; i < a.p_count; ++i) at.put(pb + a.p_begin + i, make_int2(-(gid + 1), 0));
            }
        }
        for (uint32_t c = 0; !g && c < h.nbend(); ++c) {
            const uint32_t* q = &h.bd_idx[4 * c];
            hbd[bb + c] = make_uint4(pb + q[0], pb + q[1], pb + q[2], pb + q[3]);
            hbr[bb + c] = h.bd_rest[c];
            for (int j = 0; j < 4; ++j) bd.put(pb + (int32_t)q[j], 4 * (bb + (int32_t)c) + j);
        }
        const int32_t ntri = (int32_t)(h.tri.size() / 3);
        for (int32_t t = 0; t < ntri; ++t) {
            const uint32_t* q = &h.tri[3 * t];
            htri[tb + t] = make_uint4(pb + q[0], pb + q[1], pb + q[2], 0);
            for (int j = 0; !g && j < 3; ++j) tn.put(pb + (int32_t)q[j], tb + t);
        }
        for (const vt_sdf_collider& c : h.colliders) hcol.push_back(collider_to_device(c));

        DomainParams& D = hdom[k];
        D.p_begin = pb;
        D.p_count = n;
        D.col_begin = cb;
        D.col_count = (int32_t)h.colliders.size();
        D.table_base = tkb;
        D.table_size = h.table_size;
        vt::set_nbr_offset(D, nwb);
        D.max_nbr = h.P.max_num_neighbors;
        D.cell_spacing = h.cell_spacing;
        D.cell_spacing2 = h.cell_spacing * h.cell_spacing;
        set_table_magic(D);
        tiles_for(pt, k, pb, n);
        if (g) {
            D.grid_res = h.grid_res;
            D.grid_slot_begin = sb + h.grid_slot_begin;
            D.grid_slot_count = h.grid_slot_count;
            grid_rests(h, hgrest.data() + pb, hglra.data() + pb);
            grid_doms_.push_back({k, h.grid_res});
            tiles_for(gpt, k, pb, n);
        } else {
            D.grid_res = 0;
            tiles_for(st_tiles, k, pb, n);
            tiles_for(bt, k, bb, (int32_t)h.nbend());
            bb += (int32_t)h.nbend();
        }

        pb += n;
        sb += (int32_t)h.nslots();
        tb += ntri;
        tkb += h.table_size + 1;
        nwb += h.P.max_num_neighbors * n;
        cb += (int32_t)h.colliders.size();
    }
    // grid tiles of the variant to start with; capacity for the variant with the most
    gtiles_cap_ = 0;
    for (int v = 0; v < kGridVariants; ++v) {
        std::vector<GridTile> tmp;
        for (auto& gd : grid_doms_) grid_tiles_for(tmp, gd.first, hdom[gd.first], v);
        gtiles_cap_ = std::max(gtiles_cap_, (int32_t)tmp.size());
    }
    grid_variant = grid_variant_for(kGridDefaultVariant);
    for (auto& gd : grid_doms_) grid_tiles_for(gt, gd.first, hdom[gd.first], grid_variant);
    n_ptiles = (int32_t)pt.size();
    n_btiles = (int32_t)bt.size();
    n_stiles = (int32_t)st_tiles.size();
    n_gtiles = (int32_t)gt.size();
    n_gptiles = (int32_t)gpt.size();
    hslots = hslot;

    // ---- device arena
    Arena A;
    const size_t o_x = A.take<float4>(N), o_v = A.take<float4>(N), o_x0 = A.take<float4>(N);
    const size_t o_p0 = A.take<float4>(N), o_p1 = A.take<float4>(N), o_nrm = A.take<float4>(N);
    const size_t o_sto = A.take<int32_t>(N + 1), o_ste = A.take<int2>(st.ent.size());
    const size_t o_ato = A.take<int32_t>(N + 1), o_ate = A.take<int2>(at.ent.size());
    const size_t o_lra = A.take<LraGroup>(hlra.size());
    const size_t o_sl = A.take<float4>(SL), o_sl0 = A.take<float4>(SL);
    const size_t o_bdi = A.take<uint4>(B), o_bdr = A.take<float>(B), o_bdc = A.take<float4>(4 * B);
    const size_t o_bdo = A.take<int32_t>(N + 1), o_bde = A.take<int32_t>(bd.ent.size());
    const size_t o_tri = A.take<uint4>(TR), o_tno = A.take<int32_t>(N + 1), o_tne = A.take<int32_t>(tn.ent.size());
    const size_t o_k = A.take<uint32_t>(N), o_vl = A.take<uint32_t>(N);
    const size_t o_kt = A.take<uint32_t>(N), o_vt = A.take<uint32_t>(N);
    const size_t o_h = A.take<uint32_t>(radix_hist_words(N));
    const size_t o_cs = A.take<uint2>(TK), o_nb = A.take<uint32_t>(NW);
    const size_t o_dom = A.take<DomainParams>(n_domains), o_col = A.take<ColliderDev>(C);
    const size_t o_pt = A.take<Tile>(pt.size()), o_bt = A.take<Tile>(bt.size());
    const size_t o_stt = A.take<Tile>(st_tiles.size()), o_gt = A.take<GridTile>(gtiles_cap_);
    const size_t o_gpt = A.take<Tile>(gpt.size());
    const bool any_grid = !gt.empty();
    const size_t o_grest = A.take<float4>(any_grid ? N : 0), o_glra = A.take<float4>(any_grid ? N : 0);
    const size_t o_st = A.take<int32_t>(1 + n_domains), o_pk = A.take<float>(3 * (size_t)N);
    const size_t o_ps = A.take<float4>(N), o_x0s = A.take<float4>(N);
    const size_t o_tm = A.take<CUtensorMap>(any_grid ? (size_t)kTmapsPerDomain * n_domains : 0);
    const size_t o_ctl = A.take<int2>(n_domains), o_cdl = A.take<int2>(n_domains);
    bytes = A.off;
    VT_CUDA(cudaMalloc(&arena_, A.off), "cudaMalloc(world)");
    char* base = (char*)arena_;
#define AT(T, o) reinterpret_cast<T*>(base + (o))
    d.x = AT(float4, o_x); d.v = AT(float4, o_v); d.x0 = AT(float4, o_x0);
    d.p[0] = AT(float4, o_p0); d.p[1] = AT(float4, o_p1); d.nrm = AT(float4, o_nrm);
    d.st_off = AT(int32_t, o_sto); d.st_ent = AT(int2, o_ste);
    d.at_off = AT(int32_t, o_ato); d.at_ent = AT(int2, o_ate); d.lra = AT(LraGroup, o_lra);
    d.slots = AT(float4, o_sl); d.slots0 = AT(float4, o_sl0);
    d.bd_idx = AT(uint4, o_bdi); d.bd_rest = AT(float, o_bdr); d.bd_corr = AT(float4, o_bdc);
    d.bd_off = AT(int32_t, o_bdo); d.bd_ent = AT(int32_t, o_bde);
    d.tri = AT(uint4, o_tri); d.tn_off = AT(int32_t, o_tno); d.tn_ent = AT(int32_t, o_tne);
    d.keys = AT(uint32_t, o_k); d.vals = AT(uint32_t, o_vl);
    d.keys_tmp = AT(uint32_t, o_kt); d.vals_tmp = AT(uint32_t, o_vt);
    d.hist = AT(uint32_t, o_h);
    d.cells = AT(uint2, o_cs); d.nbr = AT(uint32_t, o_nb);
    d.dom = AT(DomainParams, o_dom); d.col = AT(ColliderDev, o_col);
    d.ptiles = AT(Tile, o_pt); d.btiles = AT(Tile, o_bt); d.status = AT(int32_t, o_st);
    d.stiles = AT(Tile, o_stt); d.gtiles = AT(GridTile, o_gt); d.gptiles = AT(Tile, o_gpt);
    d.grest = AT(float4, o_grest); d.glra = AT(float4, o_glra); d.packed = AT(float, o_pk);
    d.ps = AT(float4, o_ps); d.x0s = AT(float4, o_x0s);
    CUtensorMap* tmaps_dev = any_grid ? AT(CUtensorMap, o_tm) : nullptr;
    cloth_tiles_dev_ = AT(int2, o_ctl);
    cloth_doms_dev_ = AT(int2, o_cdl);
#undef AT
    auto up = [](void* dst, const void* src, size_t bytes_) -> cudaError_t {
        return bytes_ ? cudaMemcpy(dst, src, bytes_, cudaMemcpyHostToDevice) : cudaSuccess;
    };
    VT_CUDA(up(d.x, hx.data(), N * 16), "upload x");
    VT_CUDA(up(d.v, hv.data(), N * 16), "upload v");
    VT_CUDA(up(d.x0, hx0.data(), N * 16), "upload x0");
    VT_CUDA(up(d.p[0], hp.data(), N * 16), "upload p");
    VT_CUDA(up(d.p[1], hp.data(), N * 16), "upload p");
    VT_CUDA(cudaMemset(d.nrm, 0, N * 16), "memset nrm");
    VT_CUDA(up(d.st_off, st.off.data(), (N + 1) * 4), "upload st_off");
    VT_CUDA(up(d.st_ent, st.ent.data(), st.ent.size() * 8), "upload st_ent");
    VT_CUDA(up(d.at_off, at.off.data(), (N + 1) * 4), "upload at_off");
    VT_CUDA(up(d.at_ent, at.ent.data(), at.ent.size() * 8), "upload at_ent");
    VT_CUDA(up(d.lra, hlra.data(), hlra.size() * sizeof(LraGroup)), "upload lra");
    VT_CUDA(up(d.slots, hslot.data(), SL * 16), "upload slots");
    VT_CUDA(up(d.slots0, hslot0.data(), SL * 16), "upload slots0");
    VT_CUDA(up(d.bd_idx, hbd.data(), B * 16), "upload bd_idx");
    VT_CUDA(up(d.bd_rest, hbr.data(), B * 4), "upload bd_rest");
    VT_CUDA(up(d.bd_off, bd.off.data(), (N + 1) * 4), "upload bd_off");
    VT_CUDA(up(d.bd_ent, bd.ent.data(), bd.ent.size() * 4), "upload bd_ent");
    VT_CUDA(up(d.tri, htri.data(), TR * 16), "upload tri");
    VT_CUDA(up(d.tn_off, tn.off.data(), (N + 1) * 4), "upload tn_off");
    VT_CUDA(up(d.tn_ent, tn.ent.data(), tn.ent.size() * 4), "upload tn_ent");
    VT_CUDA(cudaMemset(d.cells, 0xff, (size_t)TK * sizeof(uint2)), "memset cells");
    VT_CUDA(cudaMemset(d.nbr, 0xff, (size_t)NW * 4), "memset nbr");
    VT_CUDA(up(d.ptiles, pt.data(), pt.size() * sizeof(Tile)), "upload ptiles");
    VT_CUDA(up(d.btiles, bt.data(), bt.size() * sizeof(Tile)), "upload btiles");
    VT_CUDA(up(d.stiles, st_tiles.data(), st_tiles.size() * sizeof(Tile)), "upload stiles");
    VT_CUDA(up(d.gtiles, gt.data(), gt.size() * sizeof(GridTile)), "upload gtiles");
    VT_CUDA(up(d.gptiles, gpt.data(), gpt.size() * sizeof(Tile)), "upload gptiles");
    if (any_grid) {
        VT_CUDA(up(d.grest, hgrest.data(), N * 16), "upload grest");
        VT_CUDA(up(d.glra, hglra.data(), N * 16), "upload glra");
        // the tile kernel's tensor maps (zeroed for domains the CSR kernels solve)
        std::vector<CUtensorMap> htm((size_t)kTmapsPerDomain * n_domains);
        std::memset(htm.data(), 0, htm.size() * sizeof(CUtensorMap));
        for (auto& gd : grid_doms_) {
            const DomainParams& D = hdom[gd.first];
            if (!encode_grid_tmaps(htm.data() + tmap_index(gd.first, 0, 0), d.p[0], d.p[1], d.grest, d.glra, d.x,
                                   D.p_begin, D.grid_res + 1))
                return VT_ERR_CUDA;
        }
        VT_CUDA(up(tmaps_dev, htm.data(), htm.size() * sizeof(CUtensorMap)), "upload tensor maps");
        d.tmaps = tmaps_dev;
    }
    VT_CUDA(prepare_kernels(), "kernel attributes");
    {
        const vt_status r = update_cluster_plan();
        if (r != VT_OK) return r;
    }
    tuned_ = false;
    frames_ = 0;
    VT_CUDA(cudaMemset(d.status, 0, (1 + n_domains) * 4), "memset status");

    staging_bytes_ = sizeof(DomainParams) * n_domains + sizeof(ColliderDev) * C + 16 * SL + 64;
    VT_CUDA(cudaMallocHost(&staging_, staging_bytes_), "cudaMallocHost(staging)");
    VT_CUDA(cudaEventCreateWithFlags(&staged_, cudaEventDisableTiming), "cudaEventCreate");
    VT_CUDA(cudaDeviceSynchronize(), "world upload");
    cols_dirty_ = true;
    slots_dirty_ = true;
    pcur = 0;
    built_ = true;
    return VT_OK;
}

void grid_rests(const HostSolver& h, float4* grest, float4* glra)
{
    const int32_t R = h.grid_res, V = R + 1, n = (int32_t)h.n();
    size_t c = 0;  // rest lengths per generator, read from the constraint list in its order
    for (int32_t X = 0; X <= R; ++X)
        for (int32_t Y = 0; Y <= R; ++Y) {
            float r[4] = {0, 0, 0, 0};
            if (Y != R) r[0] = h.st_rest[c++];
            if (X != R) r[1] = h.st_rest[c++];
            if (X != R && Y != R) {
                r[2] = h.st_rest[c++];
                r[3] = h.st_rest[c++];
            }
            grest[X * V + Y] = make_float4(r[0], r[1], r[2], r[3]);
        }
    const int32_t ns = std::min(h.grid_slot_count, kGridLraCached);  // |slot0 - x0_i|
    for (int32_t i = 0; i < n; ++i) {
        float r[4] = {0, 0, 0, 0};
        const vec3 xi = mk3(h.x0[3 * i], h.x0[3 * i + 1], h.x0[3 * i + 2]);
        for (int32_t s = 0; s < ns; ++s) {
            const float* q = &h.slots0[3 * (size_t)(h.grid_slot_begin + s)];
            r[s] = length(mk3(q[0], q[1], q[2]) - xi);
        }
        glra[i] = make_float4(r[0], r[1], r[2], r[3]);
    }
}

void World::set_frame(int k, const HostSolver& h, const FrameArgs& a) { fill_frame_params(hdom[k], h.P, a); }

void fill_frame_params(DomainParams& D, const vt_params& P, const FrameArgs& a)
{
    D.diameter = a.diameter;
    D.diameter2 = a.diameter * a.diameter;
    D.gx = P.gravity[0];
    D.gy = P.gravity[1];
    D.gz = P.gravity[2];
    D.dt_frame = a.frame_dt;
    D.dt_sub = a.frame_dt / (float)a.substeps;
    D.relax = a.relax;
    D.friction = a.friction;
    D.margin = a.margin;
    D.max_speed = P.max_speed;
    D.damping = P.damping;
    D.lrs = P.long_range_stretchiness;
    D.bend_compliance = P.bend_compliance;
    D.xpbd_bend = P.bend_compliance / D.dt_sub / D.dt_sub;  // SolveBending_Kernel's xpbd_bend
    D.self_collision = P.enable_self_collision ? 1 : 0;
}

vt_status World::set_colliders(int k, const std::vector<vt_sdf_collider>& c)
{
    DomainParams& D = hdom[k];
    if ((int32_t)c.size() != D.col_count) {
        set_error("collider count of a built world cannot change; rebuild");
        return VT_ERR_STATE;
    }
    for (size_t j = 0; j < c.size(); ++j) hcol[D.col_begin + j] = collider_to_device(c[j]);
    cols_dirty_ = true;
    return VT_OK;
}

vt_status World::set_slot(int k, int32_t slot, const float xyz[3])
{
    (void)k;
    if (slot < 0 || slot >= n_slots) return VT_ERR_INVALID_ARGUMENT;
    hslots[slot] = make_float4(xyz[0], xyz[1], xyz[2], 0.0f);
    slots_dirty_ = true;
    return VT_OK;
}

vt_status World::simulate(const FrameArgs& a, int32_t ih, bool any_self, cudaStream_t st,
                          bool use_graph)
{
    if (!built_) return VT_ERR_STATE;
    if (n_particles == 0) return VT_OK;
    NvtxRange range("vt frame");
    vt_status r = upload_frame(st);
    if (r != VT_OK) return r;
    if (!tuned_) {
        r = autotune(st, frames_ > 0);
        if (r != VT_OK) return r;
    }
    ++frames_;
    if (!use_graph || profiler_on()) return enqueue_frame(a, ih, any_self, st);
    const int32_t key[4] = {a.substeps, a.iterations, ih, any_self ? 1 : 0};
    if (!gexec_ || std::memcmp(key, gkey_, sizeof(key)) != 0) {
        if (gexec_) {
            VT_CUDA(cudaGraphExecDestroy(gexec_), "cudaGraphExecDestroy");
            gexec_ = nullptr;
        }
        if (!cap_) VT_CUDA(cudaStreamCreateWithFlags(&cap_, cudaStreamNonBlocking), "cudaStreamCreate");
        const uint64_t before = launches;
        VT_CUDA(cudaStreamBeginCapture(cap_, cudaStreamCaptureModeThreadLocal), "begin capture");
        vt_status er = enqueue_frame(a, ih, any_self, cap_);
        cudaGraph_t g = nullptr;
        cudaError_t ce = cudaStreamEndCapture(cap_, &g);
        if (er != VT_OK) {
            if (g) cudaGraphDestroy(g);
            return er;
        }
        if (ce != cudaSuccess) return cuda_fail(ce, "end capture");
        ce = cudaGraphInstantiate(&gexec_, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) {
            gexec_ = nullptr;
            return cuda_fail(ce, "cudaGraphInstantiate");
        }
        glaunches_ = launches - before;
        launches = before;
        gpcur_ = pcur;
        std::memcpy(gkey_, key, sizeof(key));
    }
    VT_CUDA(cudaGraphLaunch(gexec_, st), "cudaGraphLaunch");
    launches += glaunches_;
    pcur = gpcur_;
    return VT_OK;
}

vt_status World::upload_frame(cudaStream_t st)
{
    // stage small per-frame uploads (guarded: the previous copy must have left staging)
    VT_CUDA(cudaEventSynchronize(staged_), "staging event");
    char* s = (char*)staging_;
    const size_t dom_b = sizeof(DomainParams) * n_domains;
    std::memcpy(s, hdom.data(), dom_b);
    VT_CUDA(cudaMemcpyAsync(d.dom, s, dom_b, cudaMemcpyHostToDevice, st), "upload params");
    size_t off = dom_b;
    if (cols_dirty_ && n_cols) {
        const size_t cb = sizeof(ColliderDev) * n_cols;
        std::memcpy(s + off, hcol.data(), cb);
        VT_CUDA(cudaMemcpyAsync(d.col, s + off, cb, cudaMemcpyHostToDevice, st), "upload colliders");
        off += cb;
    }
    if (slots_dirty_ && n_slots) {
        const size_t sb = 16 * (size_t)n_slots;
        std::memcpy(s + off, hslots.data(), sb);
        VT_CUDA(cudaMemcpyAsync(d.slots, s + off, sb, cudaMemcpyHostToDevice, st), "upload slots");
    }
    VT_CUDA(cudaEventRecord(staged_, st), "staging record");
    cols_dirty_ = slots_dirty_ = false;
    return VT_OK;
}

vt_status World::enqueue_frame(const FrameArgs& a, int32_t ih, bool any_self, cudaStream_t st)
{
    Launch L{&d, n_ptiles, n_btiles, n_particles, st, n_stiles, n_gtiles, n_gptiles, grid_variant};
    int pc = 0;
    int bits = 0;
    while ((1ll << bits) < (int64_t)total_keys) ++bits;
    const bool sort_odd = radix_passes(n_particles, bits) % 2;  // keys go to the temporaries
    const uint64_t pk = n_ptiles ? 1 : 0, bk = n_btiles ? 1 : 0;
#define VT_STAGE(stage, call, what, count)          \
    do {                                            \
        StageScope scope_(stage, st);               \
        VT_CUDA(call, what);                        \
        launches += (count);                        \
    } while (0)
    VT_STAGE(ST_PRESDF_PREDICT, launch_presdf_predict(L, pc), "presdf_predict", pk);
    for (int sub = 0; sub < a.substeps; ++sub) {
        if (any_self && sub % ih == 0) {
            if (hash_one_tile(n_particles, total_keys)) {
                VT_STAGE(ST_HASH_KEYS, launch_hash_one_tile(L, pc, bits, total_keys), "hash_one_tile", 1);
            } else {
                VT_CUDA(cudaMemsetAsync(d.cells, 0xff, (size_t)total_keys * sizeof(uint2), st), "memset cells");
                VT_STAGE(ST_HASH_KEYS, launch_hash_keys(L, pc, sort_odd), "hash_keys", pk);
                VT_STAGE(ST_RADIX_SORT,
                         radix_sort_pairs(d.keys, d.vals, d.keys_tmp, d.vals_tmp, d.hist, n_particles,
                                          bits, st, d.status),
                         "radix_sort", (uint64_t)radix_launches(n_particles, bits));
                VT_STAGE(ST_CELL_RANGES, launch_cell_ranges_gather(d, pc, n_particles, st), "cell_ranges", 1);
            }
            VT_STAGE(ST_CACHE_NEIGHBORS, launch_cache_neighbors(L, pc), "cache_neighbors", pk);
        }
        VT_STAGE(ST_COLLIDE, launch_collide(L, pc, 1 - pc), "collide", pk);
        pc = 1 - pc;
        const bool last_sub = sub == a.substeps - 1;
        const int cmode = substep_clusters_mode();
        if (resident_ok_ && a.iterations > 0 && cmode == 1) {
            // small grid cloths: the substep's iterations in one launch, positions resident
            // in the clusters' shared memory (the collision pass stays k_collide: folded into
            // this kernel it compiled with other register limits, and the fast build's
            // contracted arithmetic then differed from a batch's k_collide)
            VT_STAGE(ST_GRID_ITER,
                     launch_grid_substep_resident(L, cloth_doms_dev_, n_resident_cloths_, pc, a.iterations,
                                                  last_sub ? 1 : 0),
                     "grid_iter", 1);
            if (a.iterations % 2) pc = 1 - pc;
        } else if (cluster_ok_ && a.iterations > 0 && cmode != 0) {
            // small grid cloths: the substep's iterations in one launch of clusters
            VT_STAGE(ST_GRID_ITER,
                     launch_grid_substep_cluster(L, cloth_tiles_dev_, n_cluster_cloths_, pc, a.iterations,
                                                 last_sub ? 1 : 0),
                     "grid_iter", 1);
            if (a.iterations % 2) pc = 1 - pc;
        } else
        for (int it = 0; it < a.iterations; ++it) {
            if (n_btiles) VT_STAGE(ST_BEND, launch_bend(L, pc), "bend", bk);
            const int mode = it < a.iterations - 1 ? SOLVE_PLAIN
                                                   : (last_sub ? SOLVE_FINALIZE : SOLVE_FINALIZE_PREDICT);
            if (n_stiles) VT_STAGE(ST_SOLVE, launch_solve(L, pc, 1 - pc, mode), "solve", 1);
            if (n_gtiles) VT_STAGE(ST_GRID_ITER, launch_grid_iter(L, pc, 1 - pc, mode), "grid_iter", 1);
            pc = 1 - pc;
        }
        if (a.iterations == 0)
            VT_STAGE(ST_FINALIZE, launch_finalize(L, pc, last_sub ? 0 : 1), "finalize", pk);
    }
    VT_STAGE(ST_NORMALS, launch_normals(L), "normals", pk);
#undef VT_STAGE
    pcur = pc;
    return VT_OK;
}

vt_status World::read_status(std::vector<int32_t>& flags, cudaStream_t st)
{
    flags.assign(1 + n_domains, 0);
    if (!built_) return VT_OK;
    VT_CUDA(cudaMemcpyAsync(flags.data(), d.status, flags.size() * 4, cudaMemcpyDeviceToHost, st),
            "read status");
    VT_CUDA(cudaStreamSynchronize(st), "sync status");
    return VT_OK;
}

vt_status World::clear_status(cudaStream_t st)
{
    if (!built_) return VT_OK;
    VT_CUDA(cudaMemsetAsync(d.status, 0, (1 + n_domains) * 4, st), "clear status");
    return VT_OK;
}

}  // namespace vt
