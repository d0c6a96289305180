// vt_server.cu — the served form: continuous batching of cloth requests in a resident
// particle arena.
//
// Device memory is one arena sized by the HBM budget.  An admitted request gets a
// particle range [pb, pb + n) from a first-fit allocator; every other per-request array
// is addressed from it (hash cells [3 pb, 3 pb + 2n + 1), neighbour lists
// [64 pb, 64 (pb + n)), attach slots and colliders at fixed per-slot offsets), so
// admitting or retiring a request touches nothing of the others.  A per-particle domain
// id marks live particles; the spatial hash sorts the whole arena prefix with free slots
// keyed last (launch_hash_arena).  One tick = retire finished requests, admit queued ones
// in FIFO order while the budget, the slot table and the active-particle cap allow,
// rebuild the tile tables if the active set changed, then one frame for every active
// request with the same kernels as the batched form.
//
// Ticks are pipelined: a tick enqueues its frame and then waits only for the previous
// tick's frame, so the host's retire / admit / table work of tick t runs while frame t-1
// is on the GPU.  Everything a tick enqueues goes on one stream after the previous frame,
// so a range released by a request that finished in frame t-1 can be handed to a new
// request in tick t: the new request's uploads are ordered after the old one's result
// copy.  Uploads and result copies go through two pinned rings each, alternating by
// tick parity; ring t%2 is free again once frame t-1 has completed.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <new>
#include <vector>

#include "vt_host.h"
#include "vt_math.cuh"

namespace {

constexpr int kSlotsPerCloth = vt::kGridLraCached;  // attach slots a request may use
constexpr int kCollidersPerCloth = 8;
constexpr int kMaxNbr = 64;
// device bytes per arena particle: x v x0 p0 p1 nrm grest glra ps x0s (float4), domain id,
// keys vals + sort temporaries, neighbour lists, cell start/end (3 cells per particle),
// packed read-back xyz
constexpr uint64_t kBytesPerParticle = 10 * 16 + 4 + 4 * 4 + kMaxNbr * 4 + 3 * 2 * 4 + 12;

struct Request {
    int64_t id = 0;
    int32_t frames = 0, state = VT_REQ_QUEUED;
    int32_t enq = 0;   // frames enqueued
    int32_t done = 0;  // frames completed on the GPU
    vt::HostSolver h;
    int32_t sid = -1;
    int64_t pb = -1;
    uint32_t n = 0;
    const float* res_pin = nullptr;  // result in a pinned ring (copied out when complete)
    std::vector<float> result;
    bool failed = false;  // a frame produced NaN / Inf state: evicted, reported, no result
    bool cancelled = false;  // vt_server_cancel while active: evicted at the next tick
    // described grid cloth (vt_server_submit_grid): built on the device at admission,
    // h holds its parameters, slots and colliders but no particle arrays
    bool described = false;
    vt::GridBuildArgs grid{};
};

// Bump allocator over one pinned host buffer, reset once the copies it fed completed.
struct PinnedRing {
    char* base = nullptr;
    size_t cap = 0, used = 0;
    void* take(size_t bytes)
    {
        const size_t b = (bytes + 255) & ~size_t(255);
        if (!base || used + b > cap) return nullptr;
        void* p = base + used;
        used += b;
        return p;
    }
};
constexpr size_t kUploadRingBytes = 64u << 20;  // 80 B per admitted particle
constexpr size_t kResultRingBytes = 32u << 20;  // 12 B per finished particle

// First-fit allocator of [begin, end) ranges in [0, cap).
struct RangeAlloc {
    std::map<int64_t, int64_t> free_;  // begin -> end
    int64_t cap = 0;
    void init(int64_t c)
    {
        cap = c;
        free_.clear();
        if (c > 0) free_[0] = c;
    }
    int64_t alloc(int64_t n)
    {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second - it->first < n) continue;
            const int64_t b = it->first, e = it->second;
            free_.erase(it);
            if (b + n < e) free_[b + n] = e;
            return b;
        }
        return -1;
    }
    void release(int64_t b, int64_t n)
    {
        int64_t e = b + n;
        auto next = free_.lower_bound(b);
        if (next != free_.end() && next->first == e) {
            e = next->second;
            free_.erase(next);
        }
        auto prev = free_.lower_bound(b);
        if (prev != free_.begin()) {
            --prev;
            if (prev->second == b) {
                b = prev->first;
                free_.erase(prev);
            }
        }
        free_[b] = e;
    }
    // end of the last allocated range
    int64_t high_water() const
    {
        if (free_.empty()) return cap;
        const auto last = std::prev(free_.end());
        return last->second == cap ? last->first : cap;
    }
};

__global__ void k_fill_i32(int32_t* p, int64_t n, int32_t v)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

}  // namespace

struct vt_server {
    vt_server_config cfg{};
    int64_t cap_p = 0;
    int32_t cap_ptiles = 0, cap_gtiles = 0;
    void* arena = nullptr;
    vt::DeviceArrays d;
    int32_t* pdom = nullptr;
    void* staging = nullptr;  // pinned: params, colliders, slots, tile tables
    size_t staging_bytes = 0;
    cudaEvent_t staged = nullptr;
    cudaEvent_t ev0[2] = {nullptr, nullptr}, ev1[2] = {nullptr, nullptr};  // frame of tick parity
    PinnedRing up[2], res[2];
    std::vector<std::pair<Request*, int32_t>> members[2];  // (request, slot) in the frame of parity k
    int32_t* status_pin[2] = {nullptr, nullptr};  // per-slot fault flags read after each frame
    std::vector<Request*> finishing[2];  // result copies enqueued in the tick of parity k
    uint64_t frame_particles[2] = {0, 0};
    bool inflight[2] = {false, false};
    uint64_t tick_no = 0;
    cudaStream_t last_stream = nullptr;
    bool stream_set = false;
    int32_t n_finishing = 0;
    RangeAlloc alloc;
    std::deque<Request*> queue;
    std::vector<Request*> slot;  // per slot id, nullptr when free
    std::map<int64_t, std::unique_ptr<Request>> reqs;
    int64_t next_id = 1;
    uint64_t active_particles = 0;
    int32_t n_active = 0;
    int32_t interleaved_hash = 3;
    bool tables_dirty = true;
    std::vector<vt::DomainParams> hdom;
    std::vector<vt::ColliderDev> hcol;
    std::vector<float4> hslots, hslots0;
    CUtensorMap* tmaps = nullptr;          // device: kTmapsPerDomain per slot id
    std::vector<CUtensorMap> htmaps;       // host copy, encoded at admission
    int32_t n_ptiles = 0, n_gtiles = 0, grid_variant = 0;
    std::vector<std::pair<double, int32_t>> frame_log;  // (frame ms, active requests)
    vt_server_stats stats{};
    uint64_t launches = 0;

    ~vt_server()
    {
        if (arena) cudaFree(arena);
        if (staging) cudaFreeHost(staging);
        if (staged) cudaEventDestroy(staged);
        for (int k = 0; k < 2; ++k) {
            if (ev0[k]) cudaEventDestroy(ev0[k]);
            if (ev1[k]) cudaEventDestroy(ev1[k]);
            if (up[k].base) cudaFreeHost(up[k].base);
            if (status_pin[k]) cudaFreeHost(status_pin[k]);
            if (res[k].base) cudaFreeHost(res[k].base);
        }
    }
};

#define VT_CHECK(cond, code, msg) \
    do {                          \
        if (!(cond)) {            \
            vt::set_error(msg);   \
            return code;          \
        }                         \
    } while (0)

#define VT_TRY_CUDA(call, what)                                \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) return vt::cuda_fail(e_, what); \
    } while (0)

#define VT_GUARD_BEGIN try {
#define VT_GUARD_END                                \
    }                                               \
    catch (const std::bad_alloc&) {                 \
        vt::set_error("host allocation failed");    \
        return VT_ERR_OUT_OF_MEMORY;                \
    }                                               \
    catch (...) {                                   \
        vt::set_error("unexpected host exception"); \
        return VT_ERR_STATE;                        \
    }

namespace {

vt::FrameArgs frame_args(const vt_server* s, const vt::HostSolver& h)
{
    const vt_server_config& c = s->cfg;
    return vt::FrameArgs{c.frame_dt, c.substeps, c.iterations, c.relaxation, c.friction, c.collision_margin,
                         h.P.particle_diameter};
}

// The request's parameter block, colliders and attach slots in its slot of the host
// tables (uploaded with the tile tables).
vt_status fill_slot_tables(vt_server* s, const Request* r)
{
    const vt::HostSolver& h = r->h;
    const size_t n = r->n, pb = (size_t)r->pb;
    const int sid = r->sid;
    vt::DomainParams D{};
    D.p_begin = (int32_t)pb;
    D.p_count = (int32_t)n;
    D.col_begin = sid * kCollidersPerCloth;
    D.col_count = (int32_t)h.colliders.size();
    D.table_base = (int32_t)(3 * pb);
    D.table_size = h.table_size;
    vt::set_nbr_offset(D, (int64_t)kMaxNbr * pb);
    D.max_nbr = h.P.max_num_neighbors;
    D.cell_spacing = h.cell_spacing;
    D.cell_spacing2 = h.cell_spacing * h.cell_spacing;
    vt::set_table_magic(D);
    D.grid_res = h.grid_res;
    D.grid_slot_begin = sid * kSlotsPerCloth;
    D.grid_slot_count = h.grid_slot_count;
    vt::fill_frame_params(D, h.P, frame_args(s, h));
    s->hdom[sid] = D;
    // the tile kernel's tensor maps for this request's range of the arena
    if (!vt::encode_grid_tmaps(&s->htmaps[vt::tmap_index(sid, 0, 0)], s->d.p[0], s->d.p[1], s->d.grest, s->d.glra,
                               s->d.x, (int64_t)pb, h.grid_res + 1))
        return VT_ERR_CUDA;
    for (size_t k = 0; k < h.colliders.size(); ++k)
        s->hcol[sid * kCollidersPerCloth + k] = vt::collider_to_device(h.colliders[k]);
    for (int32_t k = 0; k < h.grid_slot_count; ++k) {
        const float* q = &h.slots[3 * (size_t)(h.grid_slot_begin + k)];
        const float* q0 = &h.slots0[3 * (size_t)(h.grid_slot_begin + k)];
        s->hslots[sid * kSlotsPerCloth + k] = make_float4(q[0], q[1], q[2], 0.0f);
        s->hslots0[sid * kSlotsPerCloth + k] = make_float4(q0[0], q0[1], q0[2], 0.0f);
    }
    return VT_OK;
}

// Uploads a request's state into its arena range and fills its parameter slot (a
// described grid cloth is built there by a kernel instead).  The upload images are built
// in `ring` (pinned; reused once this tick's frame completed);
// a request larger than a whole ring is uploaded from pageable memory and waited for.
// Returns VT_ERR_CAPACITY, with nothing done, when the ring has no room left this tick.
vt_status place(vt_server* s, Request* r, cudaStream_t st, PinnedRing& ring)
{
    const vt::HostSolver& h = r->h;
    const size_t n = r->n, pb = (size_t)r->pb;
    if (r->described) {
        VT_TRY_CUDA(vt::launch_grid_build(s->d, (int64_t)pb, r->grid, st), "grid build");
        k_fill_i32<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(s->pdom + pb, (int64_t)n, r->sid);
        VT_TRY_CUDA(cudaGetLastError(), "fill domain ids");
        s->launches += 2;
        return fill_slot_tables(s, r);
    }
    std::vector<float4> own;
    float4* buf = static_cast<float4*>(ring.take(5 * 16 * n));
    if (!buf) {
        if (5 * 16 * n + 256 <= ring.cap) return VT_ERR_CAPACITY;  // fits an emptier ring
        own.resize(5 * n);
        buf = own.data();
    }
    float4 *x = buf, *v = buf + n, *x0 = buf + 2 * n, *grest = buf + 3 * n, *glra = buf + 4 * n;
    for (size_t i = 0; i < n; ++i) {
        x[i] = make_float4(h.x[3 * i], h.x[3 * i + 1], h.x[3 * i + 2], h.w[i]);
        v[i] = make_float4(h.v[3 * i], h.v[3 * i + 1], h.v[3 * i + 2], 0.0f);
        x0[i] = make_float4(h.x0[3 * i], h.x0[3 * i + 1], h.x0[3 * i + 2], 0.0f);
    }
    vt::grid_rests(h, grest, glra);
    VT_TRY_CUDA(cudaMemcpyAsync(s->d.x + pb, x, 16 * n, cudaMemcpyHostToDevice, st), "upload x");
    VT_TRY_CUDA(cudaMemcpyAsync(s->d.v + pb, v, 16 * n, cudaMemcpyHostToDevice, st), "upload v");
    VT_TRY_CUDA(cudaMemcpyAsync(s->d.x0 + pb, x0, 16 * n, cudaMemcpyHostToDevice, st), "upload x0");
    VT_TRY_CUDA(cudaMemcpyAsync(s->d.grest + pb, grest, 16 * n, cudaMemcpyHostToDevice, st), "upload grest");
    VT_TRY_CUDA(cudaMemcpyAsync(s->d.glra + pb, glra, 16 * n, cudaMemcpyHostToDevice, st), "upload glra");
    k_fill_i32<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(s->pdom + pb, (int64_t)n, r->sid);
    VT_TRY_CUDA(cudaGetLastError(), "fill domain ids");
    if (!own.empty()) VT_TRY_CUDA(cudaStreamSynchronize(st), "upload");  // pageable images go out of scope
    s->launches += 1;

    return fill_slot_tables(s, r);
}

// Tile tables of the active requests + parameter / collider / slot tables -> device.
vt_status upload_tables(vt_server* s, cudaStream_t st)
{
    std::vector<vt::Tile> pt, gpt;
    std::vector<vt::GridTile> gt;
    // the tile shape the batched mix tunes to (15x15, four blocks per SM), or the one
    // vt_tuning_set_grid_tile forces: never the last shape some other solver tuned to
    s->grid_variant = vt::grid_variant_for(vt::kGridDefaultVariant);
    for (int32_t sid = 0; sid < (int32_t)s->slot.size(); ++sid) {
        const Request* r = s->slot[sid];
        if (!r) continue;
        const int32_t pb = (int32_t)r->pb, n = (int32_t)r->n;
        for (int32_t b = pb; b < pb + n; b += 256) pt.push_back(vt::Tile{sid, b, std::min(pb + n, b + 256), 0});
        vt::grid_tiles_for(gt, sid, s->hdom[sid], s->grid_variant);
    }
    gpt = pt;
    if ((int32_t)pt.size() > s->cap_ptiles || (int32_t)gt.size() > s->cap_gtiles) {
        vt::set_error("tile table capacity exceeded");
        return VT_ERR_CAPACITY;
    }
    VT_TRY_CUDA(cudaEventSynchronize(s->staged), "staging event");
    char* p = (char*)s->staging;
    auto put = [&](void* dst, const void* src, size_t bytes) -> cudaError_t {
        if (!bytes) return cudaSuccess;
        std::memcpy(p, src, bytes);
        cudaError_t e = cudaMemcpyAsync(dst, p, bytes, cudaMemcpyHostToDevice, st);
        p += (bytes + 255) & ~size_t(255);
        return e;
    };
    VT_TRY_CUDA(put(s->d.dom, s->hdom.data(), sizeof(vt::DomainParams) * s->hdom.size()), "upload params");
    int32_t used = 0;  // slot ids below the highest active one
    for (int32_t sid = 0; sid < (int32_t)s->slot.size(); ++sid)
        if (s->slot[sid]) used = sid + 1;
    VT_TRY_CUDA(put(s->tmaps, s->htmaps.data(), sizeof(CUtensorMap) * vt::kTmapsPerDomain * (size_t)used),
                "upload tensor maps");
    VT_TRY_CUDA(put(s->d.col, s->hcol.data(), sizeof(vt::ColliderDev) * s->hcol.size()), "upload colliders");
    VT_TRY_CUDA(put(s->d.slots, s->hslots.data(), 16 * s->hslots.size()), "upload slots");
    VT_TRY_CUDA(put(s->d.slots0, s->hslots0.data(), 16 * s->hslots0.size()), "upload slots0");
    VT_TRY_CUDA(put(s->d.ptiles, pt.data(), sizeof(vt::Tile) * pt.size()), "upload tiles");
    VT_TRY_CUDA(put(s->d.gptiles, gpt.data(), sizeof(vt::Tile) * gpt.size()), "upload tiles");
    VT_TRY_CUDA(put(s->d.gtiles, gt.data(), sizeof(vt::GridTile) * gt.size()), "upload tiles");
    VT_TRY_CUDA(cudaEventRecord(s->staged, st), "staging record");
    s->n_ptiles = (int32_t)pt.size();
    s->n_gtiles = (int32_t)gt.size();
    s->tables_dirty = false;
    return VT_OK;
}

// One frame of every active request.
vt_status run_frame(vt_server* s, cudaStream_t st)
{
    vt::Launch L{&s->d, s->n_ptiles, 0, 0, st, 0, s->n_gtiles, s->n_ptiles, s->grid_variant};
    const vt_server_config& c = s->cfg;
    const int64_t hw = s->alloc.high_water();
    const uint32_t sentinel = (uint32_t)(3 * hw);
    int bits = 0;
    while ((1ll << bits) < (int64_t)sentinel + 1) ++bits;
    int pc = 0;
    VT_TRY_CUDA(vt::launch_presdf_predict(L, pc), "presdf_predict");
    s->launches += 1;
    for (int sub = 0; sub < c.substeps; ++sub) {
        if (sub % s->interleaved_hash == 0)
            VT_TRY_CUDA(vt::launch_hash_arena(L, s->pdom, pc, (int32_t)hw, (int32_t)s->active_particles,
                                              sentinel, bits, &s->launches),
                        "hash");
        VT_TRY_CUDA(vt::launch_collide(L, pc, 1 - pc), "collide");
        s->launches += 1;
        pc = 1 - pc;
        const bool last = sub == c.substeps - 1;
        for (int it = 0; it < c.iterations; ++it) {
            const int mode = it < c.iterations - 1 ? vt::SOLVE_PLAIN
                                                   : (last ? vt::SOLVE_FINALIZE : vt::SOLVE_FINALIZE_PREDICT);
            VT_TRY_CUDA(vt::launch_grid_iter(L, pc, 1 - pc, mode), "grid_iter");
            s->launches += 1;
            pc = 1 - pc;
        }
        if (c.iterations == 0) {
            VT_TRY_CUDA(vt::launch_finalize(L, pc, last ? 0 : 1), "finalize");
            s->launches += 1;
        }
    }
    VT_TRY_CUDA(vt::launch_normals(L), "normals");
    s->launches += 1;
    return VT_OK;
}

double weighted_percentile(std::vector<std::pair<double, int32_t>> v, double q)
{
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    double total = 0;
    for (auto& e : v) total += e.second;
    double run = 0;
    for (auto& e : v) {
        run += e.second;
        if (run >= q * total) return e.first;
    }
    return v.back().first;
}

}  // namespace

extern "C" {

vt_status vt_server_create(const vt_server_config* cfg, vt_server** out)
{
    VT_CHECK(cfg && out, VT_ERR_INVALID_ARGUMENT, "NULL argument");
    VT_CHECK(cfg->max_cloths >= 1 && cfg->max_cloths <= (1u << 20), VT_ERR_INVALID_ARGUMENT, "max_cloths out of range");
    VT_CHECK(cfg->substeps >= 1 && cfg->iterations >= 0 && cfg->frame_dt > 0, VT_ERR_INVALID_ARGUMENT,
             "invalid frame arguments");
    *out = nullptr;
    VT_GUARD_BEGIN
    std::unique_ptr<vt_server> s(new vt_server());
    s->cfg = *cfg;
    const uint64_t M = cfg->max_cloths;
    const uint64_t fixed = M * (sizeof(vt::DomainParams) + kCollidersPerCloth * sizeof(vt::ColliderDev) +
                                2 * 16 * kSlotsPerCloth + 4) + (1 << 20);
    VT_CHECK(cfg->hbm_budget_bytes > fixed + 1024 * kBytesPerParticle, VT_ERR_CAPACITY, "budget too small");
    int64_t cap = (int64_t)((cfg->hbm_budget_bytes - fixed) / kBytesPerParticle);
    // particle indices, sorted slots and cell keys (3 cells per arena particle) are 32-bit;
    // neighbour-list offsets are 64-bit (nbr_offset)
    cap = std::min<int64_t>(cap, ((int64_t)INT32_MAX - 16) / 3);
    // tile tables: sides up to sqrt(cap); generators per tile 217 particles
    const int64_t cap_pt = cap / 256 + M + 1;
    // grid tiles of the shape with the most tiles (3 x 63: ~V^2/189 + V/3 per cloth)
    const int64_t cap_gt = cap / 189 + (int64_t)(0.4 * std::sqrt((double)cap * M)) + 2 * M + 16;
    // the arena
    auto tiles_bytes = [&](int64_t nt, size_t sz) { return ((nt * sz + 255) & ~size_t(255)); };
    const size_t a16 = ((size_t)cap * 16 + 255) & ~size_t(255), a4 = ((size_t)cap * 4 + 255) & ~size_t(255);
    const size_t hist = (vt::radix_hist_words(cap) * 4 + 255) & ~size_t(255);
    const size_t cells = ((size_t)cap * 3 * 4 + 255) & ~size_t(255), nbr = (size_t)cap * kMaxNbr * 4;
    const size_t small = M * (sizeof(vt::DomainParams) + kCollidersPerCloth * sizeof(vt::ColliderDev) +
                              2 * 16 * kSlotsPerCloth) + 4 * (M + 1) + 4 * M + 4096 * 4 +
                         M * vt::kTmapsPerDomain * sizeof(CUtensorMap) + 256;
    const size_t a12 = ((size_t)cap * 12 + 255) & ~size_t(255);
    const size_t total = 10 * a16 + 5 * a4 + a12 + hist + 2 * cells + nbr + small +
                         tiles_bytes(cap_pt, sizeof(vt::Tile)) * 2 + tiles_bytes(cap_gt, sizeof(vt::GridTile)) +
                         64 * 256;
    VT_TRY_CUDA(cudaMalloc(&s->arena, total), "cudaMalloc(server arena)");
    char* b = (char*)s->arena;
    auto take = [&](size_t bytes) { char* p = b; b += (bytes + 255) & ~size_t(255); return (void*)p; };
    s->d.x = (float4*)take(a16); s->d.v = (float4*)take(a16); s->d.x0 = (float4*)take(a16);
    s->d.p[0] = (float4*)take(a16); s->d.p[1] = (float4*)take(a16); s->d.nrm = (float4*)take(a16);
    s->d.grest = (float4*)take(a16); s->d.glra = (float4*)take(a16);
    s->d.ps = (float4*)take(a16); s->d.x0s = (float4*)take(a16);
    s->pdom = (int32_t*)take(a4);
    s->d.keys = (uint32_t*)take(a4); s->d.vals = (uint32_t*)take(a4);
    s->d.keys_tmp = (uint32_t*)take(a4); s->d.vals_tmp = (uint32_t*)take(a4);
    s->d.hist = (uint32_t*)take(hist);
    s->d.cells = (uint2*)take(2 * cells);
    s->d.nbr = (uint32_t*)take(nbr);
    s->d.packed = (float*)take(a12);
    s->d.dom = (vt::DomainParams*)take(M * sizeof(vt::DomainParams));
    s->d.col = (vt::ColliderDev*)take(M * kCollidersPerCloth * sizeof(vt::ColliderDev));
    s->d.slots = (float4*)take(M * kSlotsPerCloth * 16);
    s->d.slots0 = (float4*)take(M * kSlotsPerCloth * 16);
    s->d.status = (int32_t*)take(4 * (M + 1));
    s->d.dslot = (int32_t*)take(4 * M);
    s->tmaps = (CUtensorMap*)take(M * vt::kTmapsPerDomain * sizeof(CUtensorMap));
    s->d.tmaps = s->tmaps;
    s->htmaps.assign(M * vt::kTmapsPerDomain, CUtensorMap{});
    s->d.ptiles = (vt::Tile*)take(cap_pt * sizeof(vt::Tile));
    s->d.gptiles = (vt::Tile*)take(cap_pt * sizeof(vt::Tile));
    s->d.gtiles = (vt::GridTile*)take(cap_gt * sizeof(vt::GridTile));
    VT_CHECK((size_t)(b - (char*)s->arena) <= total, VT_ERR_STATE, "arena layout overflow");
    s->cap_p = cap;
    s->cap_ptiles = (int32_t)cap_pt;
    s->cap_gtiles = (int32_t)cap_gt;
    VT_TRY_CUDA(cudaMemset(s->pdom, 0xff, (size_t)cap * 4), "init domain ids");
    VT_TRY_CUDA(cudaMemset(s->d.status, 0, 4 * (M + 1)), "init status");
    VT_TRY_CUDA(cudaMemset(s->d.nbr, 0xff, nbr), "init neighbours");
    s->staging_bytes = M * (sizeof(vt::DomainParams) + kCollidersPerCloth * sizeof(vt::ColliderDev) +
                            2 * 16 * kSlotsPerCloth + vt::kTmapsPerDomain * sizeof(CUtensorMap)) +
                      cap_pt * 2 * sizeof(vt::Tile) + cap_gt * sizeof(vt::GridTile) + 16 * 256;
    VT_TRY_CUDA(cudaMallocHost(&s->staging, s->staging_bytes), "cudaMallocHost(server staging)");
    VT_TRY_CUDA(cudaEventCreateWithFlags(&s->staged, cudaEventDisableTiming), "event");
    for (int k = 0; k < 2; ++k) {
        VT_TRY_CUDA(cudaEventCreate(&s->ev0[k]), "event");
        VT_TRY_CUDA(cudaEventCreate(&s->ev1[k]), "event");
        VT_TRY_CUDA(cudaMallocHost((void**)&s->up[k].base, kUploadRingBytes), "cudaMallocHost(upload ring)");
        s->up[k].cap = kUploadRingBytes;
        VT_TRY_CUDA(cudaMallocHost((void**)&s->status_pin[k], 4 * (M + 1)), "cudaMallocHost(fault flags)");
        VT_TRY_CUDA(cudaMallocHost((void**)&s->res[k].base, kResultRingBytes), "cudaMallocHost(result ring)");
        s->res[k].cap = kResultRingBytes;
    }
    VT_TRY_CUDA(vt::prepare_kernels(), "kernel attributes");
    s->alloc.init(cap);
    s->slot.assign(M, nullptr);
    s->hdom.assign(M, vt::DomainParams{});
    s->hcol.assign(M * kCollidersPerCloth, vt::ColliderDev{});
    s->hslots.assign(M * kSlotsPerCloth, make_float4(0, 0, 0, 0));
    s->hslots0 = s->hslots;
    s->stats.bytes_budget = cfg->hbm_budget_bytes;
    *out = s.release();
    return VT_OK;
    VT_GUARD_END
}

vt_status vt_server_destroy(vt_server* s)
{
    if (!s) return VT_OK;
    cudaDeviceSynchronize();
    delete s;
    return VT_OK;
}

vt_status vt_server_submit(vt_server* s, vt_solver* cloth, int32_t frames, int64_t* request_id)
{
    VT_CHECK(s && cloth, VT_ERR_INVALID_ARGUMENT, "NULL argument");
    VT_CHECK(frames >= 1, VT_ERR_INVALID_ARGUMENT, "frames must be >= 1");
    VT_GUARD_BEGIN
    vt_status st = vt::pull_state(cloth);
    if (st != VT_OK) return st;
    const vt::HostSolver& h = cloth->h;
    VT_CHECK(h.grid_res >= 1, VT_ERR_INVALID_ARGUMENT,
             "the server takes one grid cloth registered with vt_cloth_build_grid_constraints");
    VT_CHECK(h.grid_slot_count <= kSlotsPerCloth, VT_ERR_CAPACITY, "more than 4 attach slots");
    VT_CHECK(h.colliders.size() <= (size_t)kCollidersPerCloth, VT_ERR_CAPACITY, "more than 8 colliders");
    VT_CHECK(h.P.max_num_neighbors <= kMaxNbr, VT_ERR_INVALID_ARGUMENT, "max_num_neighbors above 64");
    VT_CHECK((int64_t)h.n() <= s->cap_p, VT_ERR_CAPACITY, "request larger than the device-memory budget");
    if (s->reqs.empty() && s->queue.empty()) s->interleaved_hash = h.P.interleaved_hash;
    VT_CHECK(h.P.interleaved_hash == s->interleaved_hash, VT_ERR_INVALID_ARGUMENT,
             "all requests of a server share interleaved_hash");
    std::unique_ptr<Request> r(new Request());
    r->id = s->next_id++;
    r->frames = frames;
    r->h = h;
    r->n = h.n();
    s->queue.push_back(r.get());
    if (request_id) *request_id = r->id;
    s->reqs[r->id] = std::move(r);
    return VT_OK;
    VT_GUARD_END
}

vt_status vt_server_submit_grid(vt_server* s, const vt_grid_cloth* c, const vt_params* params,
                                const vt_sdf_collider* colliders, uint32_t n_colliders, int32_t frames,
                                int64_t* request_id)
{
    VT_CHECK(s && c, VT_ERR_INVALID_ARGUMENT, "NULL argument");
    VT_CHECK(frames >= 1, VT_ERR_INVALID_ARGUMENT, "frames must be >= 1");
    VT_CHECK(c->resolution >= 1 && c->resolution <= 46340, VT_ERR_INVALID_ARGUMENT, "resolution out of range");
    VT_CHECK(c->particle_diameter > 0, VT_ERR_INVALID_ARGUMENT, "particle_diameter must be > 0");
    VT_CHECK(c->n_attached <= (uint32_t)kSlotsPerCloth, VT_ERR_CAPACITY, "more than 4 attach slots");
    VT_CHECK(c->n_attached == 0 || c->attached, VT_ERR_INVALID_ARGUMENT, "attached is NULL");
    VT_CHECK(n_colliders <= (uint32_t)kCollidersPerCloth, VT_ERR_CAPACITY, "more than 8 colliders");
    VT_CHECK(n_colliders == 0 || colliders, VT_ERR_INVALID_ARGUMENT, "colliders is NULL");
    const int32_t V = c->resolution + 1;
    const int64_t n = (int64_t)V * V;
    VT_CHECK(n <= s->cap_p, VT_ERR_CAPACITY, "request larger than the device-memory budget");
    for (uint32_t k = 0; k < c->n_attached; ++k)
        VT_CHECK(c->attached[k] >= 0 && c->attached[k] < n, VT_ERR_INVALID_ARGUMENT, "attached vertex out of range");
    for (uint32_t k = 0; k < n_colliders; ++k)
        VT_CHECK(colliders[k].type >= 0 && colliders[k].type <= 2, VT_ERR_INVALID_ARGUMENT, "unknown collider type");
    vt_params P;
    if (params) {
        P = *params;
    } else {
        vt_params_default(&P);
    }
    VT_CHECK(P.num_substeps >= 1 && P.num_iterations >= 0 && P.max_num_neighbors >= 1 &&
                 P.max_num_neighbors <= kMaxNbr && P.interleaved_hash >= 1 && P.delta_time > 0,
             VT_ERR_INVALID_ARGUMENT, "invalid parameters");
    VT_GUARD_BEGIN
    if (s->reqs.empty() && s->queue.empty()) s->interleaved_hash = P.interleaved_hash;
    VT_CHECK(P.interleaved_hash == s->interleaved_hash, VT_ERR_INVALID_ARGUMENT,
             "all requests of a server share interleaved_hash");
    std::unique_ptr<Request> r(new Request());
    vt::HostSolver& h = r->h;
    h.P = P;
    // AddCloth's parameter updates (Velvet/VtClothSolverGPU.hpp:118-125, 148-149)
    const float d = c->particle_diameter;
    h.P.num_particles = (uint32_t)n;
    h.P.particle_diameter = d;
    h.P.max_speed = 2.0f * d / h.P.delta_time * (float)h.P.num_substeps;
    h.cell_spacing = d * h.P.hash_cell_size_scalar;
    h.table_size = 2 * (int32_t)n;
    h.grid_res = c->resolution;
    h.grid_slot_begin = 0;
    h.grid_slot_count = (int32_t)c->n_attached;
    h.colliders.assign(colliders, colliders + n_colliders);
    r->grid.res = c->resolution;
    r->grid.size = c->cloth_size;
    std::memcpy(r->grid.model, c->model, sizeof(r->grid.model));
    r->grid.ns = (int32_t)c->n_attached;
    for (uint32_t k = 0; k < c->n_attached; ++k) {  // GenerateAttach's slots: the attached vertices
        const vec3 q = grid_vertex(c->attached[k] / V, c->attached[k] % V, c->resolution, c->cloth_size,
                                           c->model);
        h.slots.insert(h.slots.end(), {q.x, q.y, q.z});
        r->grid.slot[k] = make_float4(q.x, q.y, q.z, 0.0f);
    }
    h.slots0 = h.slots;
    r->described = true;
    r->id = s->next_id++;
    r->frames = frames;
    r->n = (uint32_t)n;
    s->queue.push_back(r.get());
    if (request_id) *request_id = r->id;
    s->reqs[r->id] = std::move(r);
    return VT_OK;
    VT_GUARD_END
}

vt_status vt_server_tick(vt_server* s, void* stream, vt_server_tick_info* info)
{
    VT_CHECK(s, VT_ERR_INVALID_ARGUMENT, "NULL server");
    VT_GUARD_BEGIN
    cudaStream_t st = (cudaStream_t)stream;
    vt::NvtxRange range("vt server tick");
    if (s->stream_set && st != s->last_stream)  // the pipeline is ordered by one stream
        VT_TRY_CUDA(cudaStreamSynchronize(s->last_stream), "previous stream");
    s->last_stream = st;
    s->stream_set = true;
    const int par = (int)(s->tick_no & 1), prev = 1 - par;
    vt_server_tick_info ti{};
    // 1. retire: requests whose last frame is enqueued; their result copy is ordered after
    // that frame on the stream, so their range and slot are free for this tick's admissions
    for (int32_t sid = 0; sid < (int32_t)s->slot.size(); ++sid) {
        Request* r = s->slot[sid];
        if (!r || (r->enq < r->frames && !r->failed && !r->cancelled)) continue;
        // the slot's fault flag is cleared before a new request can take the slot
        VT_TRY_CUDA(cudaMemsetAsync(s->d.status + 1 + sid, 0, 4, st), "clear fault flag");
        if (r->failed || r->cancelled) {  // evicted: no result, the range and slot return at once
            k_fill_i32<<<(unsigned)((r->n + 255) / 256), 256, 0, st>>>(s->pdom + r->pb, (int64_t)r->n, -1);
            VT_TRY_CUDA(cudaGetLastError(), "clear domain ids");
            s->launches += 1;
            s->alloc.release(r->pb, r->n);
            s->active_particles -= r->n;
            s->n_active -= 1;
            s->slot[sid] = nullptr;
            r->sid = -1;
            r->state = r->failed ? VT_REQ_FAILED : VT_REQ_CANCELLED;
            r->h = vt::HostSolver{};
            if (r->failed)
                s->stats.requests_failed += 1;
            else
                s->stats.requests_cancelled += 1;
            s->tables_dirty = true;
            ti.retired += 1;
            continue;
        }
        float* pk = s->d.packed + 3 * r->pb;
        VT_TRY_CUDA(vt::launch_pack_xyz(s->d.x + r->pb, pk, (int64_t)r->n, st), "pack result");
        s->launches += 1;
        float* dst = static_cast<float*>(s->res[par].take(12 * (size_t)r->n));
        if (dst) {
            VT_TRY_CUDA(cudaMemcpyAsync(dst, pk, 12 * (size_t)r->n, cudaMemcpyDeviceToHost, st), "read result");
            r->res_pin = dst;
        } else {  // larger than the ring: straight into the request, waited for
            r->result.resize(3 * (size_t)r->n);
            VT_TRY_CUDA(cudaMemcpyAsync(r->result.data(), pk, 12 * (size_t)r->n, cudaMemcpyDeviceToHost, st),
                        "read result");
            VT_TRY_CUDA(cudaStreamSynchronize(st), "read result");
            r->res_pin = nullptr;
        }
        k_fill_i32<<<(unsigned)((r->n + 255) / 256), 256, 0, st>>>(s->pdom + r->pb, (int64_t)r->n, -1);
        VT_TRY_CUDA(cudaGetLastError(), "clear domain ids");
        s->launches += 1;
        s->alloc.release(r->pb, r->n);
        s->active_particles -= r->n;
        s->n_active -= 1;
        s->slot[sid] = nullptr;
        r->sid = -1;
        s->finishing[par].push_back(r);
        s->n_finishing += 1;
        s->tables_dirty = true;
        ti.retired += 1;
    }
    // 2. admit, FIFO
    while (!s->queue.empty()) {
        Request* r = s->queue.front();
        const uint32_t cap = s->cfg.max_active_particles;
        if (cap && s->n_active > 0 && s->active_particles + r->n > cap) break;
        int32_t sid = -1;
        for (int32_t k = 0; k < (int32_t)s->slot.size(); ++k)
            if (!s->slot[k]) { sid = k; break; }
        if (sid < 0) break;
        const int64_t pb = s->alloc.alloc(r->n);
        if (pb < 0) break;
        r->sid = sid;
        r->pb = pb;
        const vt_status pr = place(s, r, st, s->up[par]);
        if (pr != VT_OK) {
            s->alloc.release(pb, r->n);
            r->sid = -1;
            r->pb = -1;
            if (pr == VT_ERR_CAPACITY) break;  // upload ring full: next tick
            return pr;
        }
        s->slot[sid] = r;
        r->state = VT_REQ_ACTIVE;
        s->active_particles += r->n;
        s->n_active += 1;
        s->queue.pop_front();
        s->tables_dirty = true;
        ti.admitted += 1;
    }
    // 3. tables, 4. enqueue one frame for every active request
    if (s->tables_dirty) {
        const vt_status ur = upload_tables(s, st);
        if (ur != VT_OK) return ur;
    }
    s->members[par].clear();
    if (s->n_active > 0) {
        VT_TRY_CUDA(cudaEventRecord(s->ev0[par], st), "event");
        const vt_status fr = run_frame(s, st);
        if (fr != VT_OK) return fr;
        VT_TRY_CUDA(cudaMemcpyAsync(s->status_pin[par], s->d.status, 4 * (s->slot.size() + 1),
                                    cudaMemcpyDeviceToHost, st),
                    "read fault flags");
        VT_TRY_CUDA(cudaEventRecord(s->ev1[par], st), "event");
        for (int32_t sid = 0; sid < (int32_t)s->slot.size(); ++sid)
            if (Request* r = s->slot[sid]) {
                r->enq += 1;
                s->members[par].push_back({r, sid});
            }
        s->frame_particles[par] = s->active_particles;
        s->inflight[par] = true;
    }
    // 5. complete the previous tick's frame; its uploads and result copies preceded it
    if (s->inflight[prev]) {
        VT_TRY_CUDA(cudaEventSynchronize(s->ev1[prev]), "frame");
        float ms = 0;
        VT_TRY_CUDA(cudaEventElapsedTime(&ms, s->ev0[prev], s->ev1[prev]), "elapsed");
        ti.frame_ms = ms;
        if (s->status_pin[prev][0] & vt::VT_STATUS_BOUNDS) {
            vt::set_error("a device-side bounds check failed (bounds-checked build)");
            return VT_ERR_STATE;
        }
        if (s->status_pin[prev][0] & vt::VT_STATUS_TIMEOUT) {
            vt::set_error("a device-side bounded wait gave up (tile loads did not arrive)");
            return VT_ERR_TIMEOUT;
        }
        for (const auto& m : s->members[prev]) {
            m.first->done += 1;
            if (s->status_pin[prev][1 + m.second] != 0) m.first->failed = true;  // evicted next tick
        }
        const int32_t m = (int32_t)s->members[prev].size();
        s->frame_log.emplace_back(ms, m);
        s->stats.ticks += 1;
        s->stats.frames_done += (uint64_t)m;
        s->stats.particle_iterations +=
            (double)s->frame_particles[prev] * (double)s->cfg.substeps * (double)s->cfg.iterations;
        s->stats.gpu_ms += ms;
        s->inflight[prev] = false;
    } else if (!s->finishing[prev].empty()) {
        VT_TRY_CUDA(cudaStreamSynchronize(st), "result copies");
    }
    for (Request* r : s->finishing[prev]) {
        if (r->res_pin && !r->failed) r->result.assign(r->res_pin, r->res_pin + 3 * (size_t)r->n);
        r->res_pin = nullptr;
        r->state = r->failed ? VT_REQ_FAILED : VT_REQ_DONE;  // a fault in the last frame
        r->h = vt::HostSolver{};  // release the staging copy
        if (r->failed)
            s->stats.requests_failed += 1;
        else
            s->stats.requests_done += 1;
        s->n_finishing -= 1;
    }
    s->finishing[prev].clear();
    s->res[prev].used = 0;
    s->up[prev].used = 0;
    s->tick_no += 1;
    ti.active = s->n_active + s->n_finishing;
    ti.queued = (int32_t)s->queue.size();
    ti.active_particles = s->active_particles;
    if (info) *info = ti;
    return VT_OK;
    VT_GUARD_END
}

vt_status vt_server_poll(vt_server* s, int64_t id, int32_t* state, int32_t* frames_done)
{
    VT_CHECK(s, VT_ERR_INVALID_ARGUMENT, "NULL server");
    auto it = s->reqs.find(id);
    VT_CHECK(it != s->reqs.end(), VT_ERR_NOT_FOUND, "unknown request");
    if (state) *state = it->second->state;
    if (frames_done) *frames_done = it->second->done;
    return VT_OK;
}

vt_status vt_server_cancel(vt_server* s, int64_t id)
{
    VT_CHECK(s, VT_ERR_INVALID_ARGUMENT, "NULL server");
    auto it = s->reqs.find(id);
    VT_CHECK(it != s->reqs.end(), VT_ERR_NOT_FOUND, "unknown request");
    Request* r = it->second.get();
    if (r->state == VT_REQ_QUEUED) {
        for (auto q = s->queue.begin(); q != s->queue.end(); ++q)
            if (*q == r) {
                s->queue.erase(q);
                break;
            }
        r->state = VT_REQ_CANCELLED;
        r->h = vt::HostSolver{};
        s->stats.requests_cancelled += 1;
        return VT_OK;
    }
    VT_CHECK(!(r->state == VT_REQ_ACTIVE && r->failed), VT_ERR_STATE,
             "the request's state became NaN / Inf; it ends as failed and is evicted at the next tick");
    VT_CHECK(r->state == VT_REQ_ACTIVE && r->sid >= 0 && r->enq < r->frames, VT_ERR_STATE,
             "the request has its last frame enqueued or has ended");
    r->cancelled = true;  // evicted by the next tick's retire step
    return VT_OK;
}

vt_status vt_server_result(vt_server* s, int64_t id, float* dst, uint32_t count)
{
    VT_CHECK(s && dst, VT_ERR_INVALID_ARGUMENT, "NULL argument");
    auto it = s->reqs.find(id);
    VT_CHECK(it != s->reqs.end(), VT_ERR_NOT_FOUND, "unknown request");
    const Request& r = *it->second;
    VT_CHECK(r.state != VT_REQ_FAILED, VT_ERR_NUMERIC, "the request's state became NaN / Inf; it was evicted");
    VT_CHECK(r.state != VT_REQ_CANCELLED, VT_ERR_STATE, "the request was cancelled");
    VT_CHECK(r.state == VT_REQ_DONE, VT_ERR_STATE, "request not finished");
    VT_CHECK(count == r.n, VT_ERR_INVALID_ARGUMENT, "count must equal the request's particle count");
    std::memcpy(dst, r.result.data(), 12 * (size_t)count);
    return VT_OK;
}

vt_status vt_server_stats_get(vt_server* s, vt_server_stats* out)
{
    VT_CHECK(s && out, VT_ERR_INVALID_ARGUMENT, "NULL argument");
    VT_GUARD_BEGIN
    vt_server_stats st = s->stats;
    st.p50_frame_ms = weighted_percentile(s->frame_log, 0.50);
    st.p99_frame_ms = weighted_percentile(s->frame_log, 0.99);
    st.bytes_in_use = s->active_particles * kBytesPerParticle;
    *out = st;
    return VT_OK;
    VT_GUARD_END
}

}  // extern "C"
