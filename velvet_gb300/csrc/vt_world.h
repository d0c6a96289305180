// vt_world.h — device-side layout of one or more independent cloth-solver domains.
//
// A domain is everything one VtClothSolverGPU instance owns (Velvet/VtClothSolverGPU.hpp:
// 207-237): a particle range, its constraints, colliders, attach slots, parameter block
// and spatial hash.  The plain solver is one domain holding all of its cloths (merged,
// as the reference merges them: one hash, one diameter, cloths collide with each
// other).  The batched and served forms hold many domains, one per independent cloth,
// and advance them all with the same launches: every kernel reads a tile table that
// maps each thread block to (domain, first item, end item), so a block never spans two
// domains and per-domain parameters are loaded once per block.
//
// HBM layout (all arrays concatenated over domains, in domain order):
//   particles   x, v, x0      float4 (xyz, w = inverse mass for x; 0 otherwise)
//               p[2]          float4 ping-pong predicted positions (w = inverse mass)
//               nrm           float4 normals
//   stretch     st_off[N+1]   CSR offsets per particle, st_ent int2 (other, rest bits),
//                             each particle's entries in constraint order
//   attach      at_off[N+1]   CSR offsets, at_ent int2 (slot | -(group+1), dist bits)
//   bending     bd_idx uint4, bd_rest float per constraint; bd_corr float4 per
//               (constraint, corner): correction + fired flag; bd_off/bd_ent CSR of
//               corner slots per particle in constraint order
//   normals     tn_off/tn_ent CSR of triangles per vertex; tri uint4 per triangle
//   hash        keys/vals (sorted pairs), cells (start, end) per bucket (sum of (T_d + 1)),
//               neighbours (max_nbr * n_d per domain, column-major inside a domain: the
//               list of the domain's r-th particle is column r, the reference's
//               neighbors[id + k N], read by the collision pass in particle order)
#pragma once

#include <cstdint>
#include <vector>
#include <cuda.h>  // CUtensorMap (the type only; maps are encoded through the runtime's driver entry point)
#include <cuda_runtime.h>

#include "../../include/velvet_gb300.h"

namespace vt {

// Bounds-checked builds (-DVT_CHECKED=1: libvelvet_gb300_checked.so, made by build()
// beside the production library): data-dependent indices — neighbour and constraint
// entries, sorted-slot ranges, scatter positions — are range-checked before use; a
// failure sets VT_STATUS_BOUNDS in the status word (vt_solver_sync, vt_batch_sync and
// vt_server_tick then return VT_ERR_STATE) and the access is skipped.  The production
// build compiles the checks away.  (Stands in for a sanitizer, which is not available.)
#ifndef VT_CHECKED
#define VT_CHECKED 0
#endif
constexpr int32_t VT_STATUS_NONFINITE = 1, VT_STATUS_BOUNDS = 2, VT_STATUS_TIMEOUT = 4;
#if VT_CHECKED
__device__ __forceinline__ bool vt_in_range(long long v, long long lo, long long hi, int32_t* status)
{
    if (v >= lo && v < hi) return true;
    if (status) atomicOr(status, VT_STATUS_BOUNDS);
    return false;
}
#define VT_IN_RANGE(v, lo, hi, status) vt_in_range((long long)(v), (long long)(lo), (long long)(hi), (status))
#else
#define VT_IN_RANGE(v, lo, hi, status) true
#endif

// Per-domain parameters, rewritten on the device before every frame.
struct DomainParams {
    int32_t p_begin, p_count;      // particle range
    int32_t col_begin, col_count;  // colliders
    int32_t table_base, table_size; // hash cells [table_base, table_base + table_size)
    uint32_t nbr_base_lo;          // neighbour block of this domain (low 32 bits; nbr_offset)
    int32_t max_nbr;
    float cell_spacing, cell_spacing2, diameter, diameter2;
    float gx, gy, gz;
    float dt_frame, dt_sub;
    float relax, friction, margin, max_speed, damping, lrs, bend_compliance;
    int32_t self_collision;
    int32_t grid_res;        // >= 1: one grid cloth of (grid_res+1)^2 particles, implicit topology
    int32_t grid_slot_begin, grid_slot_count;  // its LRA slots (global slot indices)
    float xpbd_bend;         // bend_compliance / dt_sub / dt_sub, evaluated in that order
    uint32_t tmod_lo, tmod_hi;  // floor((2^64 - 1) / table_size) + 1, for the cell-key remainder
    uint32_t nbr_base_hi;       // high 32 bits of the neighbour block offset (128 bytes:
                                // kernels stage the block in 16-byte copies)
};
static_assert(sizeof(DomainParams) == 128, "DomainParams layout");

// Offset of a domain's neighbour block in 32-bit words: 64-bit, since the served form's
// arena can hold more than 2^31 list words (64 per particle).
__host__ __device__ __forceinline__ int64_t nbr_offset(const DomainParams& D)
{
    return (int64_t)(((uint64_t)D.nbr_base_hi << 32) | (uint64_t)D.nbr_base_lo);
}
inline void set_nbr_offset(DomainParams& D, int64_t words)
{
    D.nbr_base_lo = (uint32_t)(uint64_t)words;
    D.nbr_base_hi = (uint32_t)((uint64_t)words >> 32);
}

// The 64-bit reciprocal of a hash table size used by the direct-remainder modulo.
inline void set_table_magic(DomainParams& D)
{
    const uint64_t M = ~0ull / (uint64_t)(D.table_size > 0 ? D.table_size : 1) + 1ull;
    D.tmod_lo = (uint32_t)M;
    D.tmod_hi = (uint32_t)(M >> 32);
}

// Most LRA slots per grid cloth whose rest distances are precomputed per particle.
constexpr int kGridLraCached = 4;

// Grid tile: a TA x TB block of one grid cloth's particles, rows a in [a0, a0+TA),
// columns b in [b0, b0+TB) of VertexAt(a, b) = p_begin + a * (res+1) + b.  The fields a
// block needs to address its loads are copied from the domain so that they arrive with
// the tile's own load.
struct GridTile {
    int32_t dom, a0, b0, res;
    int32_t p_begin, slot_begin, slot_count, pad_;
};
// Variants of the tile kernel: a tile shape, every one with (TA+1) x (TB+1) = 256
// generators (one per thread), and the resident blocks per SM its plain Jacobi
// iterations are compiled for (four: 64 registers; five: 48, the shared-memory
// footprint allows five).  The variant changes which block computes what, never a result.
struct GridVariant {
    int ta, tb, blocks;
};
constexpr int kGridVariants = 6;
constexpr int kGridDefaultVariant = 1;  // 15x15 at four blocks: the variant used before tuning
constexpr GridVariant kGridVariant[kGridVariants] = {{7, 31, 4}, {15, 15, 4}, {3, 63, 4},
                                                     {7, 31, 5}, {15, 15, 5}, {3, 63, 5}};
// Tiles of variant `variant` covering the (grid_res+1)^2 grid cloth of domain `dom`.
inline void grid_tiles_for(std::vector<GridTile>& out, int dom, const DomainParams& D, int variant)
{
    const GridVariant g = kGridVariant[variant];
    const int V = D.grid_res + 1;
    for (int a = 0; a < V; a += g.ta)
        for (int b = 0; b < V; b += g.tb)
            out.push_back(GridTile{dom, a, b, D.grid_res, D.p_begin, D.grid_slot_begin, D.grid_slot_count, 0});
}

// Tensor maps for the tile kernel's TMA loads.  Per grid domain and tile shape (7x31,
// 15x15, 3x63: the variants' shapes in order), one 3-D map (float xyzw, column b, row a)
// of each array the kernel stages: the two predicted-position buffers, the generators'
// rest lengths, the particles' LRA rests and positions, with the box of that shape
// (halo tile, generator tile, particle tile).  Out-of-range boxes are filled with zeros,
// as the cp.async path's zero-fill does.
constexpr int kTmapShapes = 3;
constexpr int kTmapKinds = 5;  // p[0], p[1], grest, glra, x
constexpr int kTmapsPerDomain = kTmapShapes * kTmapKinds;
enum TmapKind { TMAP_P0 = 0, TMAP_P1 = 1, TMAP_GREST = 2, TMAP_GLRA = 3, TMAP_X = 4 };
__host__ __device__ constexpr int tmap_shape_of(int ta) { return ta == 7 ? 0 : (ta == 15 ? 1 : 2); }
__host__ __device__ constexpr int tmap_index(int dom, int shape, int kind)
{
    return (dom * kTmapShapes + shape) * kTmapKinds + kind;
}
// Encodes the kTmapsPerDomain maps of the V x V grid cloth whose first particle is p_begin
// into dst.  Returns false (with the error set) if the driver refuses a map.
bool encode_grid_tmaps(CUtensorMap* dst, const float4* p0, const float4* p1, const float4* grest,
                       const float4* glra, const float4* x, int64_t p_begin, int V);
// Whether the tile kernel stages its tiles with TMA or with per-thread cp.async (default).
bool tile_loads_tma();
vt_status set_tile_loads_tma(bool on);

// One collider on the device: the reference's SDFCollider with VelocityAt's matrix
// product lastTransform * invCurTransform precomputed (same arithmetic, once per frame).
struct ColliderDev {
    int32_t type;
    float px, py, pz;
    float sx, sy, sz;
    float delta_time;
    float cur3[9];
    float inv[16];
    float last_inv[16];
    float pad_[1];
};

// LRA group: every particle of [p_begin, p_begin + p_count) attached to each slot of
// [slot_begin, slot_begin + slot_count), rest distance |slot0 - x0| recomputed.
struct LraGroup {
    int32_t slot_begin, slot_count, p_begin, p_count;
};

// Block tile: (domain, begin, end) of the items one thread block processes.
struct Tile {
    int32_t dom, begin, end, pad_;
};

struct DeviceArrays {
    // particles
    float4 *x = nullptr, *v = nullptr, *x0 = nullptr, *p[2] = {nullptr, nullptr}, *nrm = nullptr;
    // constraints
    int32_t *st_off = nullptr; int2* st_ent = nullptr;
    int32_t *at_off = nullptr; int2* at_ent = nullptr;
    LraGroup* lra = nullptr;
    float4 *slots = nullptr, *slots0 = nullptr;
    uint4* bd_idx = nullptr; float* bd_rest = nullptr; float4* bd_corr = nullptr;
    int32_t *bd_off = nullptr, *bd_ent = nullptr;
    uint4* tri = nullptr; int32_t *tn_off = nullptr, *tn_ent = nullptr;
    // grid domains: rest lengths of the four stretch constraints generator (a, b) owns
    // (t0..t3, |x0_i - x0_j|), and the LRA rest distances of up to four slots
    float4 *grest = nullptr, *glra = nullptr;
    // hash
    uint32_t *keys = nullptr, *vals = nullptr, *keys_tmp = nullptr, *vals_tmp = nullptr;
    uint32_t* hist = nullptr;  // radix-sort scratch, radix_hist_words(n) words
    // cell ranges of the solver's hash: cells[h] = (start, end) of bucket h, start
    // 0xffffffff when empty, so one 8-byte load answers a bucket probe
    uint2* cells = nullptr;
    uint32_t* nbr = nullptr;
    // tables
    DomainParams* dom = nullptr;
    ColliderDev* col = nullptr;
    // ptiles: every domain's particles (per-particle kernels); stiles / btiles: particles
    // and bends of the domains solved by the CSR kernels; gtiles: 2-D tiles of the grid
    // domains solved by the implicit-topology kernel
    Tile *ptiles = nullptr, *stiles = nullptr, *btiles = nullptr;
    Tile* gptiles = nullptr;  // particles of the grid domains (normals)
    GridTile* gtiles = nullptr;
    int32_t* status = nullptr;  // device-side fault flag
    float* packed = nullptr;    // 3 floats per particle: read-back staging (contiguous xyz)
    // predicted and initial positions in sorted-slot order, rebuilt with every hash
    float4 *ps = nullptr, *x0s = nullptr;
    // tensor maps of the grid domains' arrays for the tile kernel's TMA loads:
    // kTmapsPerDomain per domain (tmap_index); nullptr: the kernel stages with cp.async
    const CUtensorMap* tmaps = nullptr;
    // served form only: the first sorted slot of each domain, rebuilt with every hash (a
    // domain's particles fill consecutive sorted slots; with free arena ranges between
    // requests they do not start at p_begin).  nullptr elsewhere: slots = particle range.
    int32_t* dslot = nullptr;
};

// ------------------------------------------------------------------ kernel launchers
// (vt_kernels.cu).  All enqueue on `st` and return the launch error, if any.
struct Launch {
    const DeviceArrays* d;
    int32_t n_ptiles, n_btiles;
    int32_t n_particles;
    cudaStream_t st;
    int32_t n_stiles = 0, n_gtiles = 0, n_gptiles = 0;
    int32_t grid_variant = 0;  // grid kernel variant of the gtiles (kGridVariant index)
};

// One grid cloth built on the device: GenerateClothMesh + AddCloth (positions, inverse
// masses with AddAttach's zero-distance rule) + the grid builder's rest lengths and LRA
// rests, written at particle offset pb of x, v, x0, grest, glra.
struct GridBuildArgs {
    int32_t res;
    float size;
    float model[16];
    float4 slot[kGridLraCached];  // LRA slot positions (xyz)
    int32_t ns;                   // <= kGridLraCached
};
cudaError_t launch_grid_build(const DeviceArrays& d, int64_t pb, const GridBuildArgs& g, cudaStream_t st);

// Splats x[0, n) into rgba (vt_render.cu); zbuf: width * height 64-bit depth|colour keys.
cudaError_t launch_render(const float4* x, int64_t n, const vt_render_params& rp, unsigned long long* zbuf,
                          uint32_t* rgba, cudaStream_t st);

// xyz of src[0, n) into dst as 3 n contiguous floats, so that a read-back is one
// contiguous copy instead of a copy of 12-byte rows out of 16-byte ones.
// Cell start/end of the sorted keys plus ps / x0s (positions in sorted-slot order).
cudaError_t launch_cell_ranges_gather(const DeviceArrays& d, int pin, int32_t n, cudaStream_t st);
// A world of at most kHashOneTileMaxParticles particles hashes in one launch
// (k_hash_one_tile: table clear, keys, sort, cell ranges, sorted copies on one block) when
// its cell table has at most kHashOneTileMaxKeys buckets.  One block does the work of the
// four launches' many: a 32x32 cloth's frame 0.231 -> 0.220 ms, a 64x64 one's 0.243 ->
// 0.264 ms, so larger worlds keep the four launches.
constexpr int32_t kHashOneTileMaxParticles = 2048;
constexpr int32_t kHashOneTileMaxKeys = 1 << 16;
bool hash_one_tile(int32_t n, int32_t total_keys);
cudaError_t launch_hash_one_tile(const Launch& L, int pin, int32_t bits, int32_t total_keys);
cudaError_t launch_pack_xyz(const float4* src, float* dst, int64_t n, cudaStream_t st);

// One Jacobi iteration of the grid domains (stretch + attach + bending + ApplyDeltas,
// optionally Finalize / Predict) with implicit topology and shared-memory tiles.
cudaError_t launch_grid_iter(const Launch& L, int pin, int pout, int final_mode);
// One-time kernel attributes (call outside any stream capture).
cudaError_t prepare_kernels();
// All iterations of one substep of every grid cloth in one launch of clusters (one
// cluster per cloth, cloth_tiles[c] its tile range); see k_grid_substep_cluster.
cudaError_t launch_grid_substep_cluster(const Launch& L, const int2* cloth_tiles, int n_cloths, int pin,
                                        int iterations, int last_sub);
// Clusters of the substep kernels this device holds at once (0: none).  A world takes a
// cluster form only when one cluster per cloth fits at once: with more cloths the clusters
// run in waves, each paying a substep's whole chain of iterations, and one launch per
// iteration is faster (a batch of 32 cloths of sides 24-48: 0.45 ms per frame per
// iteration, 0.68 resident, 0.83 re-staging).
int substep_cluster_capacity();
// Grid cloths of at most this many tiles (of the variant in use) take the cluster kernel:
// one tile per block, a single round per iteration.  (With two rounds — a 64x64 cloth's 25
// tiles of 15x15 on 16 blocks — each iteration pays the tile's dependent-latency chain
// twice and the frame took 0.62 ms against 0.48 ms with one launch per iteration.)
constexpr int kClusterMaxTiles = 16;
// How small-cloth worlds run a substep's iterations: 0 one launch per iteration; 1 (the
// default) one launch of cluster-resident tiles when every cloth is within
// kResidentMaxSide particles a side, else one launch of clusters stepping through the
// tile kernel's tiles when every cloth is within kClusterMaxTiles tiles; 2 the latter
// only.
constexpr int kResidentMaxSide = 64;
int substep_clusters_mode();
vt_status set_substep_clusters(int mode);
cudaError_t launch_grid_substep_resident(const Launch& L, const int2* cloth_dom, int n_cloths, int pin,
                                         int iterations, int last_sub);
int substep_resident_capacity();

cudaError_t launch_presdf_predict(const Launch& L, int pcur);
cudaError_t launch_collide(const Launch& L, int pin, int pout);
cudaError_t launch_bend(const Launch& L, int pin);
cudaError_t launch_solve(const Launch& L, int pin, int pout, int final_mode);
cudaError_t launch_finalize(const Launch& L, int pcur, int predict_next);
cudaError_t launch_normals(const Launch& L);

// final_mode of launch_solve / predict_next of launch_finalize
enum { SOLVE_PLAIN = 0, SOLVE_FINALIZE = 1, SOLVE_FINALIZE_PREDICT = 2 };

// Spatial hash (vt_hash.cu)
// Keys of the solver's particles into (keys, vals), or into (keys_tmp, vals_tmp) when
// to_tmp (an odd number of sort passes; see radix_sort_pairs).
cudaError_t launch_hash_keys(const Launch& L, int pin, bool to_tmp);
// Stable LSD radix sort of (key, val) pairs by the low `bits` bits of the keys, in
// radix_passes(n, bits) passes of up to 8 bits that move the pairs between (keys, vals)
// and (keys_tmp, vals_tmp).  The input is read from keys / vals when the number of passes
// is even and from keys_tmp / vals_tmp when it is odd; the result always lands in
// keys / vals.  Scratch: hist, radix_hist_words(n) words, needing no initial contents.
// radix_launches(n, bits) kernels are launched.
cudaError_t radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t* keys_tmp,
                             uint32_t* vals_tmp, uint32_t* hist, int32_t n, int32_t bits,
                             cudaStream_t st, int32_t* status = nullptr);
int radix_passes(int32_t n, int32_t bits);
int radix_launches(int32_t n, int32_t bits);
constexpr int32_t kRadixTileItems = 4096;  // pairs per sort tile
constexpr size_t kRadixScratchHead = 1280;  // digit counts and tile counters of 4 passes
// size of `hist` for n items: the head plus a look-back word per (pass, tile, digit)
constexpr size_t radix_hist_words(int64_t n)
{
    return kRadixScratchHead + (size_t)4 * 256 * (size_t)(n > kRadixTileItems ? (n + kRadixTileItems - 1) / kRadixTileItems : 1);
}
cudaError_t launch_cell_ranges(const uint32_t* keys, int32_t n, uint32_t* cell_start,
                               uint32_t* cell_end, cudaStream_t st);
// The neighbour walk: a warp per particle in worlds of up to kWarpWalkMaxParticles
// particles (latency-bound: too few particles to hide a thread's serial chain of probes
// and candidates), else a thread per particle (half the instructions).  Frame of one
// cloth, warp / thread form: 64x64 0.241 / 0.342 ms, 128x128 0.355 / 0.446, 181x181
// 0.419 / 0.475, 256x256 0.576 / 0.559.
constexpr int32_t kWarpWalkMaxParticles = 49152;
cudaError_t launch_cache_neighbors(const Launch& L, int pin);
// Spatial hash of a sparse particle arena (the served form): particles [0, hw) with
// per-particle domain ids pdom (< 0: free); cells [0, sentinel); n_active live particles.
cudaError_t launch_hash_arena(const Launch& L, const int32_t* pdom, int pin, int32_t hw,
                              int32_t n_active, uint32_t sentinel, int32_t bits, uint64_t* launches);
// HashObjects on float3 caller buffers (vt_hash_objects); scratch supplied by the caller:
// keys_tmp / vals_tmp num_objects words each, hist radix_hist_words(num_objects).
cudaError_t hash_objects_f3(uint32_t* phash, uint32_t* pindex, uint32_t* cell_start,
                            uint32_t* cell_end, uint32_t* neighbors, const float* positions,
                            const float* original, const vt_hash_params& hp,
                            uint32_t* keys_tmp, uint32_t* vals_tmp, uint32_t* hist, cudaStream_t st);

}  // namespace vt
