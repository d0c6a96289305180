// vt_hash.cu — spatial hash for self-collision: cell keys, a stable LSD radix sort of
// (key, particle) pairs, cell start/end ranges and cached neighbour lists.
//
// Follows Velvet/SpatialHashGPU.cu:13-196:
//   key   = abs(((ix*92837111) ^ (iy*689287499) ^ (iz*283923481)) % T),
//           ix = (int)floor(x / cellSpacing) with IEEE division (no reciprocal),
//           int32 products wrapping;
//   sort  = stable by key (the reference uses cub::DeviceRadixSort::SortPairs; here a
//           hand-written LSD radix sort in the single-sweep form: one count of every
//           pass's digits, then per pass one kernel whose tiles rank their pairs with
//           warp match-any + per-warp counters, so equal digits keep index order, and
//           find their output offsets by a decoupled look-back over earlier tiles);
//   cells = cellStart[h] / cellEnd[h] of every occupied bucket, 0xffffffff elsewhere;
//   lists = 27 buckets in x, y, z loop order, at most maxNumNeighbors entries read per
//           bucket, pairs kept if |p_i - p_j|^2 < cellSpacing^2 and the initial
//           positions are more than one diameter apart, column-major
//           neighbors[id + k * N], 0xffffffff-terminated unless full.  Two of the 27
//           cells that hash to the same bucket are visited twice, as in the reference.
// In the multi-domain form each domain hashes into its own bucket range
// [table_base, table_base + T) so one sort serves all domains and each domain's order
// equals the order it would have alone.  The solver's walk runs one thread per sorted
// slot over copies of the positions in sorted order (made with the cell ranges), so a
// warp's threads share buckets and each candidate is one contiguous 16-byte load (in
// worlds of up to 49,152 particles a warp per particle, lane per bucket; up to 2,048
// particles the keys, sort and cell ranges run on one block); the caller-buffer form
// (HashObjects) walks the caller's float3 arrays directly.
#include "vt_math.cuh"
#include "vt_world.h"

namespace vt {

static constexpr int kBlock = 256;

__device__ __forceinline__ int32_t int_coord(float v, float spacing)
{
    return (int32_t)floorf(v / spacing);
}

__device__ __forceinline__ uint32_t hash_coords(int32_t x, int32_t y, int32_t z, int32_t table)
{
    const uint32_t h = ((uint32_t)x * 92837111u) ^ ((uint32_t)y * 689287499u) ^
                       ((uint32_t)z * 283923481u);
    const int32_t r = ((int32_t)h) % table;
    return (uint32_t)(r < 0 ? -r : r);
}

// abs(h % T) for the int32 h whose bits are `h`, via |h| mod T (C's remainder truncates
// toward zero, so |h % T| = |h| mod T), with the remainder computed directly from a
// precomputed 64-bit reciprocal M = floor((2^64 - 1) / T) + 1: n mod T =
// mulhi64((M * n) mod 2^64, T), exact for every 32-bit n and T (Lemire, Kaser, Kurz,
// "Faster remainder by direct computation", 2019).
__device__ __forceinline__ uint32_t abs_mod(uint32_t h, uint64_t M, uint32_t T)
{
    const uint32_t n = ((int32_t)h < 0) ? 0u - h : h;
    const uint64_t low = M * (uint64_t)n;
    return (uint32_t)__umul64hi(low, (uint64_t)T);
}

// ------------------------------------------------------------------ keys
__global__ void __launch_bounds__(kBlock)
k_hash_keys(const Tile* __restrict__ tiles, const DomainParams* __restrict__ doms,
            const float4* __restrict__ p, uint32_t* __restrict__ keys, uint32_t* __restrict__ vals)
{
    const Tile tl = tiles[blockIdx.x];
    const int i = tl.begin + (int)threadIdx.x;
    if (i >= tl.end) return;
    const DomainParams& D = doms[tl.dom];
    const float4 q = p[i];
    const float sp = D.cell_spacing;
    keys[i] = (uint32_t)D.table_base +
              hash_coords(int_coord(q.x, sp), int_coord(q.y, sp), int_coord(q.z, sp), D.table_size);
    vals[i] = (uint32_t)i;
}

// float3 input, one domain (the HashObjects entry point)
__global__ void __launch_bounds__(kBlock)
k_hash_keys_f3(const float* __restrict__ pos, int32_t n, float sp, int32_t table,
               uint32_t* __restrict__ keys, uint32_t* __restrict__ vals)
{
    const int i = blockIdx.x * kBlock + (int)threadIdx.x;
    if (i >= n) return;
    keys[i] = hash_coords(int_coord(pos[3 * i], sp), int_coord(pos[3 * i + 1], sp),
                          int_coord(pos[3 * i + 2], sp), table);
    vals[i] = (uint32_t)i;
}

// ------------------------------------------------------------------ radix sort
// A stable LSD radix sort in the single-sweep form (chained scan with decoupled look-back,
// Merrill and Garland 2016; its radix-sort use, Adinets and Merrill 2022): one kernel
// counts the digits of every pass over all keys at once, then one kernel per pass ranks
// each 4096-pair tile in shared memory and learns where its digits start from the
// tiles before it through per-(tile, digit) words published in global memory, so no
// per-tile histogram and no separate scan pass is needed.  Tiles take their ids from an
// atomic counter in the order their blocks start, so a tile only ever waits on tiles
// whose blocks are already running, and every wait is bounded.
static constexpr int kRsItems = 16;
static constexpr int kRsWarps = kBlock / 32;
static constexpr int kRsTile = kBlock * kRsItems;  // 4096 pairs per tile
static_assert(kRsTile == kRadixTileItems, "tile size shared with the scratch-size formula");
static constexpr int kRsMaxPasses = 4;             // 32-bit keys in 8-bit digits
// hist layout (words): digit counts of pass p at [256 p, 256 p + 256); the tile counter of
// pass p at kRsCounters + p; the look-back word of (pass p, tile i, digit d) at
// kRsLookBase + (p * ntiles + i) * 256 + d.
static constexpr size_t kRsCounters = (size_t)kRsMaxPasses * 256, kRsLookBase = kRsCounters + 256;
// look-back word: flag in the top two bits, a count below (counts stay under 2^30)
static constexpr uint32_t kRsAggregate = 1u << 30, kRsPrefix = 2u << 30, kRsCountMask = (1u << 30) - 1;
static constexpr int kRsLookTries = 1 << 21;

static_assert(kRsLookBase == kRadixScratchHead, "scratch head shared with the scratch-size formula");

int radix_passes(int32_t n, int32_t bits) { return (n > 1 && bits > 0) ? (bits + 7) / 8 : 0; }

int radix_launches(int32_t n, int32_t bits)
{
    const int passes = radix_passes(n, bits);
    if (!passes) return 0;
    return n <= kRadixTileItems ? 1 : 1 + passes;
}

__device__ __forceinline__ uint32_t ld_relaxed_gpu(const uint32_t* a)
{
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(a) : "memory");
    return v;
}

__device__ __forceinline__ void st_relaxed_gpu(uint32_t* a, uint32_t v)
{
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(a), "r"(v) : "memory");
}

// Digit counts of all passes in one read of the keys.
__global__ void __launch_bounds__(kBlock)
k_rs_count(const uint32_t* __restrict__ keys, int32_t n, int passes, int per, int bits,
           uint32_t* __restrict__ hist)
{
    __shared__ uint32_t h[kRsMaxPasses][256];
    for (int k = threadIdx.x; k < kRsMaxPasses * 256; k += kBlock) (&h[0][0])[k] = 0;
    __syncthreads();
    const int stride = gridDim.x * kBlock;
#pragma unroll 4
    for (int idx = blockIdx.x * kBlock + (int)threadIdx.x; idx < n; idx += stride) {
        const uint32_t key = keys[idx];
        for (int p = 0; p < passes; ++p) {
            const int shift = p * per, nb = min(per, bits - shift);
            atomicAdd(&h[p][(key >> shift) & ((1u << nb) - 1u)], 1u);
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < passes * 256; k += kBlock) {
        const uint32_t c = (&h[0][0])[k];
        if (c) atomicAdd(&hist[k], c);
    }
}

// Block-wide exclusive scan of one value per thread (kBlock threads); returns the
// exclusive prefix, *total gets the block sum.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total)
{
    __shared__ uint32_t warp_sums[kRsWarps];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    uint32_t wpre = 0, tot = 0;
#pragma unroll
    for (int w = 0; w < kRsWarps; ++w) {
        const uint32_t s = warp_sums[w];
        if (w < warp) wpre += s;
        tot += s;
    }
    __syncthreads();
    *total = tot;
    return wpre + incl - v;
}

// One pass: rank a tile's pairs by digit (stable), find each digit's output start from
// the global digit counts and the look-back over earlier tiles, and scatter.
// (four blocks per SM: 64 registers instead of 80, 0.396 -> 0.385 ms of sorting per mix frame)
__global__ void __launch_bounds__(kBlock, 4)
k_rs_onesweep(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
              uint32_t* __restrict__ kout, uint32_t* __restrict__ vout, int32_t n, int pass, int shift,
              int nbits, uint32_t* __restrict__ hist, int32_t ntiles, int32_t* __restrict__ status)
{
    __shared__ uint32_t off[256];   // the tile's first output position per digit
    __shared__ uint32_t lofs[256];  // the digit's first slot in the tile's sorted copy
    __shared__ uint32_t wcnt[kRsWarps][256];
    __shared__ uint32_t sk[kRsTile], sv[kRsTile];  // the tile's pairs in output order
    __shared__ int32_t tile_s;
    const int ndig = 1 << nbits;
    const uint32_t mask = (uint32_t)ndig - 1;
    if (threadIdx.x == 0) tile_s = (int32_t)atomicAdd(&hist[kRsCounters + pass], 1u);
    for (int k = threadIdx.x; k < kRsWarps * 256; k += kBlock) (&wcnt[0][0])[k] = 0;
    __syncthreads();
    const int tile = tile_s;
    if (tile >= ntiles) return;  // not reached: the grid has ntiles blocks

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t lt = (1u << lane) - 1u;
    const int wbase = tile * kRsTile + warp * (32 * kRsItems);
    uint32_t mk[kRsItems], mv[kRsItems], mr[kRsItems];
#pragma unroll
    for (int j = 0; j < kRsItems; ++j) {
        const int idx = wbase + j * 32 + lane;
        const bool valid = idx < n;
        const uint32_t key = valid ? kin[idx] : 0u;
        const uint32_t val = valid ? vin[idx] : 0u;
        const uint32_t d = valid ? ((key >> shift) & mask) : 0x100u;  // 0x100: not a digit
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        uint32_t rank = 0;
        if (valid) rank = wcnt[warp][d] + __popc(peers & lt);
        __syncwarp();
        if (valid && lane == __ffs(peers) - 1) wcnt[warp][d] += __popc(peers);
        __syncwarp();
        mk[j] = key;
        mv[j] = val;
        mr[j] = rank;
    }
    __syncthreads();
    uint32_t run = 0;  // the tile's count of digit threadIdx.x
    if ((int)threadIdx.x < ndig) {
#pragma unroll
        for (int w = 0; w < kRsWarps; ++w) {
            const uint32_t c = wcnt[w][threadIdx.x];
            wcnt[w][threadIdx.x] = run;
            run += c;
        }
    }
    uint32_t tot;
    const uint32_t lex = block_exclusive_scan(run, &tot);
    const uint32_t gex = block_exclusive_scan((int)threadIdx.x < ndig ? hist[(size_t)pass * 256 + threadIdx.x] : 0u, &tot);
    if ((int)threadIdx.x < ndig) {
        lofs[threadIdx.x] = lex;
        uint32_t* look = hist + kRsLookBase + (size_t)pass * ntiles * 256 + threadIdx.x;
        uint32_t excl = 0;
        if (tile == 0) {
            st_relaxed_gpu(look, kRsPrefix | run);
        } else {
            st_relaxed_gpu(look + (size_t)tile * 256, kRsAggregate | run);
            int j = tile - 1, tries = 0;
            while (true) {
                const uint32_t v = ld_relaxed_gpu(look + (size_t)j * 256);
                if ((v & ~kRsCountMask) == 0) {  // tile j has not published yet
                    if (++tries > kRsLookTries) {
                        // report it (the sync calls return VT_ERR_TIMEOUT); positions stay
                        // below the true ones, so every store below stays in bounds
                        if (status) atomicOr(status, VT_STATUS_TIMEOUT);
                        break;
                    }
                    if (tries > 64) __nanosleep(64);
                    continue;
                }
                excl += v & kRsCountMask;
                if ((v & kRsPrefix) || j == 0) break;
                --j;
            }
            st_relaxed_gpu(look + (size_t)tile * 256, kRsPrefix | (excl + run));
        }
        off[threadIdx.x] = gex + excl;
    }
    __syncthreads();
    // the tile's pairs into shared memory in (digit, stable rank) order, then written out
    // by consecutive threads: each digit's run lands in consecutive output positions
#pragma unroll
    for (int j = 0; j < kRsItems; ++j) {
        const int idx = wbase + j * 32 + lane;
        if (idx < n) {
            const uint32_t d = (mk[j] >> shift) & mask;
            const uint32_t lp = lofs[d] + wcnt[warp][d] + mr[j];
            if (!VT_IN_RANGE(lp, 0, kRsTile, status)) continue;
            sk[lp] = mk[j];
            sv[lp] = mv[j];
        }
    }
    __syncthreads();
    const int count = min(kRsTile, n - tile * kRsTile);
    for (int t = threadIdx.x; t < count; t += kBlock) {
        const uint32_t key = sk[t];
        const uint32_t d = (key >> shift) & mask;
        const uint32_t pos = off[d] + ((uint32_t)t - lofs[d]);
        if (!VT_IN_RANGE(pos, 0, n, status)) continue;
        kout[pos] = key;
        vout[pos] = sv[t];
    }
}

// All passes of a sort that fits one tile (n <= 4096) on one block, the pairs in shared
// memory (sk, sv) from before the call to after it: each pass's digit offsets are the
// tile's own prefix sums, so no count kernel, look-back or scratch is needed.  Same
// ranking as k_rs_onesweep, so the same stable order.  Ends with a block barrier.
__device__ __forceinline__ void tile_sort_smem(uint32_t* sk, uint32_t* sv, int32_t n, int passes, int per, int bits,
                                               uint32_t (*wcnt)[256], uint32_t* lofs, int32_t* status)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t lt = (1u << lane) - 1u;
    const int wbase = warp * (32 * kRsItems);
    int shift = 0;
    for (int ps = 0; ps < passes; ++ps) {
        const int nb = min(per, bits - shift);
        const int ndig = 1 << nb;
        const uint32_t mask = (uint32_t)ndig - 1;
        for (int k = threadIdx.x; k < kRsWarps * 256; k += kBlock) (&wcnt[0][0])[k] = 0;
        __syncthreads();  // the pairs are in place and the counters cleared
        uint32_t mk[kRsItems], mv[kRsItems], mr[kRsItems];
#pragma unroll
        for (int j = 0; j < kRsItems; ++j) {
            const int idx = wbase + j * 32 + lane;
            const bool valid = idx < n;
            const uint32_t key = valid ? sk[idx] : 0u;
            const uint32_t val = valid ? sv[idx] : 0u;
            const uint32_t d = valid ? ((key >> shift) & mask) : 0x100u;  // 0x100: not a digit
            const uint32_t peers = __match_any_sync(0xffffffffu, d);
            uint32_t rank = 0;
            if (valid) rank = wcnt[warp][d] + __popc(peers & lt);
            __syncwarp();
            if (valid && lane == __ffs(peers) - 1) wcnt[warp][d] += __popc(peers);
            __syncwarp();
            mk[j] = key;
            mv[j] = val;
            mr[j] = rank;
        }
        __syncthreads();  // every pair is in registers and every warp has counted
        uint32_t run = 0;
        if ((int)threadIdx.x < ndig) {
#pragma unroll
            for (int w = 0; w < kRsWarps; ++w) {
                const uint32_t c = wcnt[w][threadIdx.x];
                wcnt[w][threadIdx.x] = run;
                run += c;
            }
        }
        uint32_t tot;
        const uint32_t lex = block_exclusive_scan(run, &tot);
        if ((int)threadIdx.x < ndig) lofs[threadIdx.x] = lex;
        __syncthreads();
#pragma unroll
        for (int j = 0; j < kRsItems; ++j) {
            const int idx = wbase + j * 32 + lane;
            if (idx < n) {
                const uint32_t d = (mk[j] >> shift) & mask;
                const uint32_t lp = lofs[d] + wcnt[warp][d] + mr[j];
                if (!VT_IN_RANGE(lp, 0, n, status)) continue;
                sk[lp] = mk[j];
                sv[lp] = mv[j];
            }
        }
        shift += nb;
        __syncthreads();  // the pass's pairs are placed and its counters read
    }
    __syncthreads();  // the sorted pairs are in place (also when there is no pass)
}

// The one-tile sort as a kernel (radix_sort_pairs for n <= 4096).
__global__ void __launch_bounds__(kBlock)
k_rs_single_tile(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin, uint32_t* __restrict__ kout,
                 uint32_t* __restrict__ vout, int32_t n, int passes, int per, int bits, int32_t* __restrict__ status)
{
    __shared__ uint32_t lofs[256];
    __shared__ uint32_t wcnt[kRsWarps][256];
    __shared__ uint32_t sk[kRsTile], sv[kRsTile];
    for (int k = threadIdx.x; k < n; k += kBlock) {
        sk[k] = kin[k];
        sv[k] = vin[k];
    }
    tile_sort_smem(sk, sv, n, passes, per, bits, wcnt, lofs, status);
    for (int k = threadIdx.x; k < n; k += kBlock) {
        kout[k] = sk[k];
        vout[k] = sv[k];
    }
}

cudaError_t radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t* keys_tmp, uint32_t* vals_tmp,
                             uint32_t* hist, int32_t n, int32_t bits, cudaStream_t st, int32_t* status)
{
    const int passes = radix_passes(n, bits);
    if (!passes) return cudaSuccess;
    if (passes > kRsMaxPasses || n > (int32_t)kRsCountMask) return cudaErrorInvalidValue;
    const int per = (bits + passes - 1) / passes;
    const int32_t ntiles = (n + kRsTile - 1) / kRsTile;
    // an odd number of passes starts from the temporaries, so the result lands in keys / vals
    uint32_t *ki = keys, *vi = vals, *ko = keys_tmp, *vo = vals_tmp;
    if (passes % 2) {
        ki = keys_tmp; vi = vals_tmp; ko = keys; vo = vals;
    }
    if (ntiles == 1) {
        k_rs_single_tile<<<1, kBlock, 0, st>>>(ki, vi, keys, vals, n, passes, per, bits, status);
        return cudaGetLastError();
    }
    cudaError_t e = cudaMemsetAsync(hist, 0, sizeof(uint32_t) * (kRsLookBase + (size_t)passes * ntiles * 256), st);
    if (e != cudaSuccess) return e;
    k_rs_count<<<ntiles < 1024 ? ntiles : 1024, kBlock, 0, st>>>(ki, n, passes, per, bits, hist);
    int shift = 0;
    for (int ps = 0; ps < passes; ++ps) {
        const int nb = (bits - shift) < per ? (bits - shift) : per;
        k_rs_onesweep<<<ntiles, kBlock, 0, st>>>(ki, vi, ko, vo, n, ps, shift, nb, hist, ntiles, status);
        uint32_t* t;
        t = ki; ki = ko; ko = t;
        t = vi; vi = vo; vo = t;
        shift += nb;
    }
    return cudaGetLastError();
}

// ------------------------------------------------------------------ cell ranges
// FindCellStart_Kernel, SpatialHashGPU.cu:44-77 (cell_start pre-filled with 0xff bytes)
__global__ void __launch_bounds__(kBlock)
k_cell_ranges(const uint32_t* __restrict__ keys, int32_t n, uint32_t* __restrict__ cs,
              uint32_t* __restrict__ ce)
{
    const int t = blockIdx.x * kBlock + (int)threadIdx.x;
    if (t >= n) return;
    const uint32_t h = keys[t];
    if (t == 0 || keys[t - 1] != h) {
        cs[h] = (uint32_t)t;
        if (t > 0) ce[keys[t - 1]] = (uint32_t)t;
    }
    if (t == n - 1) ce[h] = (uint32_t)n;
}

cudaError_t launch_cell_ranges(const uint32_t* keys, int32_t n, uint32_t* cell_start,
                               uint32_t* cell_end, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    k_cell_ranges<<<(n + kBlock - 1) / kBlock, kBlock, 0, st>>>(keys, n, cell_start, cell_end);
    return cudaGetLastError();
}

// Cell ranges, plus the predicted and initial positions copied into sorted-slot order
// (ps[t] = (p[vals[t]].xyz, bits of vals[t]), x0s[t] = x0[vals[t]]), so that the
// neighbour walk reads a bucket's candidates, index included, as contiguous float4 runs
// instead of gathering them through vals.
__global__ void __launch_bounds__(kBlock)
k_cell_ranges_gather(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ vals,
                     const float4* __restrict__ p, const float4* __restrict__ x0, int32_t n,
                     uint2* __restrict__ cells, float4* __restrict__ ps, float4* __restrict__ x0s,
                     int32_t* __restrict__ status)
{
    const int t = blockIdx.x * kBlock + (int)threadIdx.x;
    if (t >= n) return;
    const uint32_t h = keys[t];
    if (t == 0 || keys[t - 1] != h) {
        cells[h].x = (uint32_t)t;
        if (t > 0) cells[keys[t - 1]].y = (uint32_t)t;
    }
    if (t == n - 1) cells[h].y = (uint32_t)n;
    const uint32_t id = vals[t];
    if (!VT_IN_RANGE(id, 0, n, status)) return;
    const float4 q = p[id];
    ps[t] = make_float4(q.x, q.y, q.z, __uint_as_float(id));
    x0s[t] = x0[id];
}

cudaError_t launch_cell_ranges_gather(const DeviceArrays& d, int pin, int32_t n, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    k_cell_ranges_gather<<<(n + kBlock - 1) / kBlock, kBlock, 0, st>>>(d.keys, d.vals, d.p[pin], d.x0, n,
                                                                      d.cells, d.ps, d.x0s, d.status);
    return cudaGetLastError();
}

// The whole hash of a small world (kHashOneTileMaxParticles, within one sort tile), up
// to the neighbour walk, on one block: the cell table cleared, every particle's key, the sort in
// shared memory, the cell ranges and the sorted copies — what the table clear,
// k_hash_keys, the sort and k_cell_ranges_gather do in four launches, with the same
// results.  The sort's pass count is the one radix_sort_pairs takes.
__global__ void __launch_bounds__(kBlock)
k_hash_one_tile(const Tile* __restrict__ tiles, int32_t n_ptiles, const DomainParams* __restrict__ doms,
                const float4* __restrict__ p, const float4* __restrict__ x0, int32_t n, int passes, int per,
                int bits, int32_t total_keys, uint2* __restrict__ cells, uint32_t* __restrict__ keys,
                uint32_t* __restrict__ vals, float4* __restrict__ ps, float4* __restrict__ x0s,
                int32_t* __restrict__ status)
{
    __shared__ uint32_t lofs[256];
    __shared__ uint32_t wcnt[kRsWarps][256];
    __shared__ uint32_t sk[kRsTile], sv[kRsTile];
    const int tid = (int)threadIdx.x;
    for (int k = tid; k < total_keys; k += kBlock) cells[k] = make_uint2(0xffffffffu, 0xffffffffu);
    for (int t = 0; t < n_ptiles; ++t) {
        const Tile tl = tiles[t];
        const int i = tl.begin + tid;
        if (i < tl.end && VT_IN_RANGE(i, 0, n, status)) {
            const DomainParams& D = doms[tl.dom];
            const float4 q = p[i];
            const float sp = D.cell_spacing;
            sk[i] = (uint32_t)D.table_base +
                    hash_coords(int_coord(q.x, sp), int_coord(q.y, sp), int_coord(q.z, sp), D.table_size);
            sv[i] = (uint32_t)i;
        }
    }
    // sorts, and orders the clear above before the range stores below
    tile_sort_smem(sk, sv, n, passes, per, bits, wcnt, lofs, status);
    for (int t = tid; t < n; t += kBlock) {
        const uint32_t h = sk[t];
        if (t == 0 || sk[t - 1] != h) {
            cells[h].x = (uint32_t)t;
            if (t > 0) cells[sk[t - 1]].y = (uint32_t)t;
        }
        if (t == n - 1) cells[h].y = (uint32_t)n;
        const uint32_t id = sv[t];
        keys[t] = h;
        vals[t] = id;
        if (!VT_IN_RANGE(id, 0, n, status)) continue;
        const float4 q = p[id];
        ps[t] = make_float4(q.x, q.y, q.z, __uint_as_float(id));
        x0s[t] = x0[id];
    }
}

static_assert(kHashOneTileMaxParticles <= kRsTile, "the one-block hash sorts one tile");

bool hash_one_tile(int32_t n, int32_t total_keys)
{
    return n >= 1 && n <= kHashOneTileMaxParticles && total_keys <= kHashOneTileMaxKeys;
}

cudaError_t launch_hash_one_tile(const Launch& L, int pin, int32_t bits, int32_t total_keys)
{
    const DeviceArrays& d = *L.d;
    const int passes = radix_passes(L.n_particles, bits);
    const int per = passes ? (bits + passes - 1) / passes : 0;
    k_hash_one_tile<<<1, kBlock, 0, L.st>>>(d.ptiles, L.n_ptiles, d.dom, d.p[pin], d.x0, L.n_particles, passes, per,
                                            bits, total_keys, d.cells, d.keys, d.vals, d.ps, d.x0s, d.status);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ neighbour cache
// CacheNeighbors_Kernel, SpatialHashGPU.cu:79-130, for sorted slot t.
template <typename Pos>
__device__ __forceinline__ void cache_neighbors_one(uint32_t t, const uint32_t* __restrict__ vals,
                                                    const uint32_t* __restrict__ cs,
                                                    const uint32_t* __restrict__ ce, Pos pos, Pos orig,
                                                    uint32_t* __restrict__ out_base, uint32_t id_base,
                                                    int32_t n, int32_t table_base, int32_t table,
                                                    uint64_t M, float sp, float sp2, float diam2,
                                                    int32_t max_nbr)
{
    const uint32_t id = vals[t];
    const vec3 position = pos(id);
    const int32_t ix = int_coord(position.x, sp), iy = int_coord(position.y, sp),
                  iz = int_coord(position.z, sp);
    uint32_t* out = out_base + (id - id_base);
    // the 27 keys are XORs of per-axis products: (x+dx)*A etc. wrap like x*A
    uint32_t hx[3], hy[3], hz[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        hx[k] = (uint32_t)(ix - 1 + k) * 92837111u;
        hy[k] = (uint32_t)(iy - 1 + k) * 689287499u;
        hz[k] = (uint32_t)(iz - 1 + k) * 283923481u;
    }
    bool have_orig = false;
    vec3 originalp = mk3(0, 0, 0);
    int cnt = 0;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
            for (int c = 0; c < 3; ++c) {
                const uint32_t h = (uint32_t)table_base + abs_mod(hx[a] ^ hy[b] ^ hz[c], M, (uint32_t)table);
                const uint32_t start = cs[h];
                if (start == 0xffffffffu) continue;
                uint32_t end = ce[h];
                const uint32_t lim = start + (uint32_t)max_nbr;
                if (lim < end) end = lim;
                for (uint32_t k = start; k < end; ++k) {
                    const uint32_t nb = vals[k];
                    if (nb == id) continue;
                    const vec3 d1 = position - pos(nb);
                    if (!(dot(d1, d1) < sp2)) continue;
                    if (!have_orig) {
                        originalp = orig(id);
                        have_orig = true;
                    }
                    const vec3 d2 = originalp - orig(nb);
                    if (dot(d2, d2) > diam2) {
                        out[(size_t)cnt * n] = nb;
                        ++cnt;
                        if (cnt >= max_nbr) return;
                    }
                }
            }
    out[(size_t)cnt * n] = 0xffffffffu;
}

// The same walk over sorted-slot copies of the positions: candidate k is ps[k] (its
// position, its index in w) and x0s[k], one 16-byte load each, contiguous within a
// bucket; the thread's own object is slot t, so the threads of a warp share buckets.
// Same arithmetic, order and caps.  The list goes to column id - id_base of the domain's
// block (the reference's neighbors[id + k N]), so the collision pass, one thread per
// particle, reads entry k of consecutive particles' lists as consecutive words.  (Lists
// in sorted-slot order, the walk's own thread order, made these stores consecutive but
// cost the collision pass a gather of each particle's own state: 1.36 -> 1.66 ms per
// frame of the mix against no gain in the walk.)  Measured forms of the walk itself:
// threads in object order, a warp per object, a warp per cell group, (start, end) pairs
// loaded three buckets at a time, and the next bucket's range loaded ahead with
// candidates loaded two or four at a time all ran slower — the walk is bound by load
// latency, and this form's 32 registers give the highest occupancy and the most shared
// bucket reads; candidates loaded two at a time at eight blocks per SM (32 registers, a
// few bytes spilled) took the mix's walk from 4.18 to 3.88 ms per frame, the same at 33
// registers and six blocks to 4.58, four at a time spills 112 bytes.  The probes are
// ~4% of the walk (0.15 ms per frame with the candidate loop removed); a flattened loop
// over each thread's candidates of all buckets (the nonempty ranges compacted in shared
// memory first, so a warp's lanes are not held at every bucket by the longest one) ran
// at 4.61 ms.
__device__ __forceinline__ void cache_neighbors_sorted(uint32_t t, const uint2* __restrict__ cells,
                                                       const float4* __restrict__ ps,
                                                       const float4* __restrict__ x0s,
                                                       uint32_t* __restrict__ out_base, uint32_t id_base,
                                                       uint32_t slot_base, int32_t n, int32_t table_base,
                                                       int32_t table, uint64_t M, float sp, float sp2,
                                                       float diam2, int32_t max_nbr, uint32_t slot_end,
                                                       int32_t* status)
{
    const float4 own = ps[t];
    const uint32_t id = __float_as_uint(own.w);
    const vec3 position = xyz(own);
    const int32_t ix = int_coord(position.x, sp), iy = int_coord(position.y, sp),
                  iz = int_coord(position.z, sp);
    if (!VT_IN_RANGE(t, slot_base, (long long)slot_base + n, status)) return;
    uint32_t* out = out_base + (id - id_base);
    // the 27 keys are XORs of per-axis products: (x+dx)*A etc. wrap like x*A
    uint32_t hx[3], hy[3], hz[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        hx[k] = (uint32_t)(ix - 1 + k) * 92837111u;
        hy[k] = (uint32_t)(iy - 1 + k) * 689287499u;
        hz[k] = (uint32_t)(iz - 1 + k) * 283923481u;
    }
    bool have_orig = false;
    vec3 originalp = mk3(0, 0, 0);
    int cnt = 0;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
            for (int c = 0; c < 3; ++c) {
                const uint32_t h = (uint32_t)table_base + abs_mod(hx[a] ^ hy[b] ^ hz[c], M, (uint32_t)table);
                const uint2 range = cells[h];  // start and end in one load
                const uint32_t start = range.x;
                if (start == 0xffffffffu) continue;
                uint32_t end = range.y;
                const uint32_t lim = start + (uint32_t)max_nbr;
                if (lim < end) end = lim;
                if (!VT_IN_RANGE(end, start, (long long)slot_end + 1, status)) continue;
                // two candidates' loads in flight, then taken in order
                for (uint32_t k = start; k < end; k += 2) {
                    const float4 qa = ps[k];
                    const bool two = k + 1 < end;
                    const float4 qb = two ? ps[k + 1] : qa;
#pragma unroll
                    for (int u = 0; u < 2; ++u) {
                        if (u == 1 && !two) break;
                        const float4 qk = u ? qb : qa;
                        const uint32_t kk = k + (uint32_t)u;
                        const uint32_t nb = __float_as_uint(qk.w);
                        if (!VT_IN_RANGE(nb, id_base, id_base + (uint32_t)n, status)) continue;
                        const vec3 d1 = position - xyz(qk);
                        if (nb == id) continue;
                        if (!(dot(d1, d1) < sp2)) continue;
                        if (!have_orig) {
                            originalp = xyz(x0s[t]);
                            have_orig = true;
                        }
                        const vec3 d2 = originalp - xyz(x0s[kk]);
                        if (dot(d2, d2) > diam2) {
                            out[(size_t)cnt * n] = nb;
                            ++cnt;
                            if (cnt >= max_nbr) return;
                        }
                    }
                }
            }
    out[(size_t)cnt * n] = 0xffffffffu;
}

struct PosF4 {
    const float4* __restrict__ a;
    __device__ __forceinline__ vec3 operator()(uint32_t i) const { return xyz(a[i]); }
};
struct PosF3 {
    const float* __restrict__ a;
    __device__ __forceinline__ vec3 operator()(uint32_t i) const
    {
        return mk3(a[3 * (size_t)i], a[3 * (size_t)i + 1], a[3 * (size_t)i + 2]);
    }
};

// One block per particle tile (one domain).  The domain's sorted slots start at its first
// particle's index in the world form and at dslot[domain] in the served form's arena.
__global__ void __launch_bounds__(kBlock, 8)
k_cache_neighbors(const Tile* __restrict__ tiles, const DomainParams* __restrict__ doms,
                  const uint2* __restrict__ cells, const float4* __restrict__ ps, const float4* __restrict__ x0s,
                  uint32_t* __restrict__ nbr, const int32_t* __restrict__ dslot, int32_t* __restrict__ status)
{
    const Tile tl = tiles[blockIdx.x];
    const int t = tl.begin + (int)threadIdx.x;
    if (t >= tl.end) return;
    const DomainParams& D = doms[tl.dom];
    const uint32_t sbase = dslot ? (uint32_t)dslot[tl.dom] : (uint32_t)D.p_begin;
    cache_neighbors_sorted(sbase + (uint32_t)(t - D.p_begin), cells, ps, x0s, nbr + nbr_offset(D),
                           (uint32_t)D.p_begin, sbase, D.p_count, D.table_base, D.table_size,
                           ((uint64_t)D.tmod_hi << 32) | D.tmod_lo, D.cell_spacing, D.cell_spacing2, D.diameter2,
                           D.max_nbr, sbase + (uint32_t)D.p_count, status);
}

// The same lists with a warp per particle, for worlds too small to hide the thread form's
// serial chain of 27 bucket probes: lane q < 27 probes bucket q (q = 9a + 3b + c, the
// walk's order) and tests its candidates, a warp prefix sum of the lanes' counts places
// each bucket's entries after those of the buckets before it, and a second pass over the
// candidates (now in L1) writes the entries that fall within the list's cap.  Same
// tests, order and caps as cache_neighbors_sorted.  Each block serves eight particles of
// one particle tile: block b takes tile b / 32 and its particles 8 (b % 32) .. + 7.
__global__ void __launch_bounds__(kBlock)
k_cache_neighbors_warp(const Tile* __restrict__ tiles, const DomainParams* __restrict__ doms,
                       const uint2* __restrict__ cells, const float4* __restrict__ ps,
                       const float4* __restrict__ x0s, uint32_t* __restrict__ nbr,
                       const int32_t* __restrict__ dslot, int32_t* __restrict__ status)
{
    const Tile tl = tiles[blockIdx.x >> 5];
    const int warp = (int)threadIdx.x >> 5, lane = (int)threadIdx.x & 31;
    const int t = tl.begin + (int)(blockIdx.x & 31) * 8 + warp;
    if (t >= tl.end) return;  // the whole warp
    const DomainParams& D = doms[tl.dom];
    const uint32_t sbase = dslot ? (uint32_t)dslot[tl.dom] : (uint32_t)D.p_begin;
    const uint32_t slot = sbase + (uint32_t)(t - D.p_begin);
    const int32_t n = D.p_count;
    const uint32_t slot_end = sbase + (uint32_t)n, id_base = (uint32_t)D.p_begin;
    const float4 own = ps[slot];
    const uint32_t id = __float_as_uint(own.w);
    const vec3 position = xyz(own);
    const float sp = D.cell_spacing;
    const int32_t ix = int_coord(position.x, sp), iy = int_coord(position.y, sp), iz = int_coord(position.z, sp);
    const int max_nbr = D.max_nbr;
    uint32_t start = 0, end = 0;
    if (lane < 27) {
        const int a = lane / 9, b = (lane / 3) % 3, c = lane % 3;
        const uint32_t key = ((uint32_t)(ix - 1 + a) * 92837111u) ^ ((uint32_t)(iy - 1 + b) * 689287499u) ^
                             ((uint32_t)(iz - 1 + c) * 283923481u);
        const uint32_t h = (uint32_t)D.table_base +
                           abs_mod(key, ((uint64_t)D.tmod_hi << 32) | D.tmod_lo, (uint32_t)D.table_size);
        const uint2 range = cells[h];
        if (range.x != 0xffffffffu) {
            uint32_t e = range.y;
            const uint32_t lim = range.x + (uint32_t)max_nbr;
            if (lim < e) e = lim;
            if (VT_IN_RANGE(e, range.x, (long long)slot_end + 1, status)) {
                start = range.x;
                end = e;
            }
        }
    }
    const vec3 originalp = xyz(x0s[slot]);
    const float sp2 = D.cell_spacing2, diam2 = D.diameter2;
    auto fires = [&](uint32_t k, uint32_t& nb) {
        const float4 qk = ps[k];
        nb = __float_as_uint(qk.w);
        if (!VT_IN_RANGE(nb, id_base, id_base + (uint32_t)n, status)) return false;
        const vec3 d1 = position - xyz(qk);
        if (nb == id) return false;
        if (!(dot(d1, d1) < sp2)) return false;
        const vec3 d2 = originalp - xyz(x0s[k]);
        return dot(d2, d2) > diam2;
    };
    uint32_t cnt = 0;
    for (uint32_t k = start; k < end; ++k) {
        uint32_t nb;
        if (fires(k, nb)) ++cnt;
    }
    uint32_t incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    uint32_t* out = nbr + nbr_offset(D) + (id - id_base);
    uint32_t pos = incl - cnt;
    if (cnt && pos < (uint32_t)max_nbr) {
        for (uint32_t k = start; k < end && pos < (uint32_t)max_nbr; ++k) {
            uint32_t nb;
            if (fires(k, nb)) out[(size_t)(pos++) * n] = nb;
        }
    }
    if (lane == 0 && total < (uint32_t)max_nbr) out[(size_t)total * n] = 0xffffffffu;
}

__global__ void __launch_bounds__(kBlock)
k_cache_neighbors_f3(const uint32_t* __restrict__ vals, const uint32_t* __restrict__ cs,
                     const uint32_t* __restrict__ ce, const float* __restrict__ pos,
                     const float* __restrict__ orig, uint32_t* __restrict__ nbr, int32_t n,
                     int32_t table, uint64_t M, float sp, float sp2, float diam2, int32_t max_nbr)
{
    const int t = blockIdx.x * kBlock + (int)threadIdx.x;
    if (t >= n) return;
    cache_neighbors_one((uint32_t)t, vals, cs, ce, PosF3{pos}, PosF3{orig}, nbr, 0u, n, 0, table, M,
                        sp, sp2, diam2, max_nbr);
}

// ------------------------------------------------------------------ arena form
// The served form keeps each admitted cloth in a range of a sparse particle arena: a
// per-particle domain id (negative for a free slot) replaces the tile -> domain map.
// Free slots get a sentinel key that sorts after every cell, so the first n_active
// sorted entries are the live particles; a domain's particles still sort by (its cell,
// particle index), the order they have when the cloth is simulated alone.
__global__ void __launch_bounds__(kBlock)
k_hash_keys_arena(const int32_t* __restrict__ pdom, const DomainParams* __restrict__ doms,
                  const float4* __restrict__ p, uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                  int32_t hw, uint32_t sentinel)
{
    const int i = blockIdx.x * kBlock + (int)threadIdx.x;
    if (i >= hw) return;
    const int d = pdom[i];
    uint32_t key = sentinel;
    if (d >= 0) {
        const DomainParams& D = doms[d];
        const float4 q = p[i];
        const float sp = D.cell_spacing;
        key = (uint32_t)D.table_base +
              hash_coords(int_coord(q.x, sp), int_coord(q.y, sp), int_coord(q.z, sp), D.table_size);
    }
    keys[i] = key;
    vals[i] = (uint32_t)i;
}

// Cell ranges and sorted copies as k_cell_ranges_gather, plus each domain's first sorted
// slot: a domain's keys form one contiguous run of the sorted order, so the slot where
// the domain of vals[t] differs from that of vals[t - 1] starts it.
__global__ void __launch_bounds__(kBlock)
k_cell_ranges_arena(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ vals,
                    const int32_t* __restrict__ pdom, const float4* __restrict__ p, const float4* __restrict__ x0,
                    int32_t n, uint32_t sentinel, uint2* __restrict__ cells,
                    float4* __restrict__ ps, float4* __restrict__ x0s, int32_t* __restrict__ dslot)
{
    const int t = blockIdx.x * kBlock + (int)threadIdx.x;
    if (t >= n) return;
    const uint32_t h = keys[t];
    if (h == sentinel) return;
    if (t == 0 || keys[t - 1] != h) {
        cells[h].x = (uint32_t)t;
        if (t > 0) cells[keys[t - 1]].y = (uint32_t)t;
    }
    if (t == n - 1 || keys[t + 1] == sentinel) cells[h].y = (uint32_t)(t + 1);
    const uint32_t id = vals[t];
    const int32_t dom = pdom[id];
    if (t == 0 || pdom[vals[t - 1]] != dom) dslot[dom] = t;
    const float4 q = p[id];
    ps[t] = make_float4(q.x, q.y, q.z, __uint_as_float(id));
    x0s[t] = x0[id];
}

cudaError_t launch_hash_arena(const Launch& L, const int32_t* pdom, int pin, int32_t hw,
                              int32_t n_active, uint32_t sentinel, int32_t bits, uint64_t* launches)
{
    const DeviceArrays& d = *L.d;
    const cudaStream_t st = L.st;
    if (hw <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(d.cells, 0xff, sizeof(uint2) * (size_t)sentinel, st);
    if (e != cudaSuccess) return e;
    const int blocks = (hw + kBlock - 1) / kBlock;
    const bool odd = radix_passes(hw, bits) % 2;
    k_hash_keys_arena<<<blocks, kBlock, 0, st>>>(pdom, d.dom, d.p[pin], odd ? d.keys_tmp : d.keys,
                                                 odd ? d.vals_tmp : d.vals, hw, sentinel);
    e = radix_sort_pairs(d.keys, d.vals, d.keys_tmp, d.vals_tmp, d.hist, hw, bits, st, d.status);
    if (e != cudaSuccess) return e;
    k_cell_ranges_arena<<<blocks, kBlock, 0, st>>>(d.keys, d.vals, pdom, d.p[pin], d.x0, hw, sentinel,
                                                   d.cells, d.ps, d.x0s, d.dslot);
    // the walk by particle tiles, each a block of one request's particles
    if (n_active > 0 && L.n_ptiles)
        k_cache_neighbors<<<L.n_ptiles, kBlock, 0, st>>>(d.ptiles, d.dom, d.cells, d.ps, d.x0s, d.nbr, d.dslot,
                                                         d.status);
    if (launches) *launches += 3 + (uint64_t)radix_launches(hw, bits);
    return cudaGetLastError();
}

cudaError_t launch_hash_keys(const Launch& L, int pin, bool to_tmp)
{
    if (!L.n_ptiles) return cudaSuccess;
    const DeviceArrays& d = *L.d;
    k_hash_keys<<<L.n_ptiles, kBlock, 0, L.st>>>(d.ptiles, d.dom, d.p[pin], to_tmp ? d.keys_tmp : d.keys,
                                                 to_tmp ? d.vals_tmp : d.vals);
    return cudaGetLastError();
}

cudaError_t launch_cache_neighbors(const Launch& L, int pin)
{
    if (!L.n_ptiles) return cudaSuccess;
    const DeviceArrays& d = *L.d;
    (void)pin;  // positions come sorted from launch_cell_ranges_gather
    if (L.n_particles <= kWarpWalkMaxParticles)
        k_cache_neighbors_warp<<<L.n_ptiles * 32, kBlock, 0, L.st>>>(d.ptiles, d.dom, d.cells, d.ps, d.x0s, d.nbr,
                                                                     nullptr, d.status);
    else
        k_cache_neighbors<<<L.n_ptiles, kBlock, 0, L.st>>>(d.ptiles, d.dom, d.cells, d.ps, d.x0s, d.nbr, nullptr,
                                                           d.status);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ HashObjects (float3)
// The whole HashObjects pipeline on caller buffers; scratch passed in.
cudaError_t hash_objects_f3(uint32_t* phash, uint32_t* pindex, uint32_t* cell_start,
                            uint32_t* cell_end, uint32_t* neighbors, const float* positions,
                            const float* original, const vt_hash_params& hp,
                            uint32_t* keys_tmp, uint32_t* vals_tmp, uint32_t* hist, cudaStream_t st)
{
    const int32_t n = (int32_t)hp.num_objects;
    cudaError_t e = cudaMemsetAsync(cell_start, 0xff, sizeof(uint32_t) * ((size_t)hp.table_size + 1), st);
    if (e != cudaSuccess || n == 0) return e;
    const int blocks = (n + kBlock - 1) / kBlock;
    int bits = 0;
    while ((1ll << bits) < (long long)hp.table_size) ++bits;  // ceil(log2(tableSize))
    const bool odd = radix_passes(n, bits) % 2;  // the sort reads the temporaries then
    k_hash_keys_f3<<<blocks, kBlock, 0, st>>>(positions, n, hp.cell_spacing, hp.table_size,
                                              odd ? keys_tmp : phash, odd ? vals_tmp : pindex);
    e = radix_sort_pairs(phash, pindex, keys_tmp, vals_tmp, hist, n, bits, st);
    if (e != cudaSuccess) return e;
    k_cell_ranges<<<blocks, kBlock, 0, st>>>(phash, n, cell_start, cell_end);
    const uint64_t magic = ~0ull / (uint64_t)hp.table_size + 1ull;
    k_cache_neighbors_f3<<<blocks, kBlock, 0, st>>>(pindex, cell_start, cell_end, positions, original,
                                                    neighbors, n, hp.table_size, magic, hp.cell_spacing,
                                                    hp.cell_spacing2, hp.particle_diameter2,
                                                    (int32_t)hp.max_num_neighbors);
    return cudaGetLastError();
}

}  // namespace vt
