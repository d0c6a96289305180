// vt_hash_noalloc.cu — HashObjects for callers that cannot allocate device memory.
//
// vt_hash_objects allocates its radix-sort scratch with cudaMalloc on first use (and
// again whenever a larger table arrives), much as the reference's Sort resizes its
// temporary buffer mid-frame (Velvet/SpatialHashGPU.cu:139-152).  Some callers cannot
// allow that: an engine whose frame loop runs under a fixed device-memory budget
// handed out once at start-up, a host that owns every device allocation itself, or a
// real-time loop where cudaMalloc / cudaFree would synchronise the device and stall the
// frame.  vt_hash_objects_noalloc gives them the same computation with the sort scratch
// in a fixed array compiled into this library instead.
//
// The array below is a file-scope __device__ variable of VT_HASH_NOALLOC_MAX_OBJECTS
// objects' worth of scratch (about 2.4 MB).  Every GPU on which the library is loaded
// holds it until the process exits.  In host code its name is only a host-side stand-in
// for the device variable, never a device address: the address is obtained once per
// device with cudaGetSymbolAddress and passed to the kernels.  The address is kept for
// the life of the process, so a cudaDeviceReset after the first call on a device is not
// supported (the module would be reloaded and the kept address would be stale).
#include <mutex>
#include <new>

#include "vt_host.h"

namespace {

constexpr int32_t kMaxObjects = VT_HASH_NOALLOC_MAX_OBJECTS;
// keys_tmp + vals_tmp + the sort's counts and look-back words
constexpr size_t kScratchWords = 2 * (size_t)kMaxObjects + vt::radix_hist_words(kMaxObjects);

static __device__ __align__(256) uint32_t g_noalloc_scratch[kScratchWords];

std::mutex g_mu;
uint32_t* g_scratch_addr[64] = {};  // device address of g_noalloc_scratch, per device ordinal

// Set-up, once per device, with that device current: look the array's device address up.
vt_status scratch_for_current_device(uint32_t** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return vt::cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= 64) {
        vt::set_error("device ordinal beyond 64");
        return VT_ERR_STATE;
    }
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return vt::cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_scratch_addr[dev] = static_cast<uint32_t*>(p);
    }
    *out = g_scratch_addr[dev];
    return VT_OK;
}

}  // namespace

static vt_status hash_objects_noalloc(uint32_t* particle_hash, uint32_t* particle_index, uint32_t* cell_start,
                                      uint32_t* cell_end, uint32_t* neighbors, const float* positions,
                                      const float* original_positions, const vt_hash_params* hp, void* stream)
{
    if (!hp || !cell_start) {
        vt::set_error("params and cell_start must not be NULL");
        return VT_ERR_INVALID_ARGUMENT;
    }
    if (hp->num_objects > (uint32_t)kMaxObjects) {
        vt::set_error("vt_hash_objects_noalloc: num_objects exceeds VT_HASH_NOALLOC_MAX_OBJECTS "
                      "(262144); use vt_hash_objects for larger tables");
        return VT_ERR_CAPACITY;
    }
    if (hp->table_size < 1 || hp->max_num_neighbors < 1 || hp->max_num_neighbors > 64) {
        vt::set_error("table_size must be >= 1 and max_num_neighbors in [1, 64]");
        return VT_ERR_INVALID_ARGUMENT;
    }
    if (hp->num_objects &&
        !(particle_hash && particle_index && cell_end && neighbors && positions && original_positions)) {
        vt::set_error("NULL buffer");
        return VT_ERR_INVALID_ARGUMENT;
    }
    uint32_t* scratch = nullptr;
    vt_status st = scratch_for_current_device(&scratch);
    if (st != VT_OK) return st;
    const int32_t n = (int32_t)hp->num_objects;
    const size_t cap = (size_t)(n > 0 ? n : 1);
    uint32_t* keys_tmp = scratch;
    uint32_t* vals_tmp = keys_tmp + cap;
    uint32_t* hist = vals_tmp + cap;
    // the sort's layout must fit the fixed array
    if (2 * cap + vt::radix_hist_words(n) > kScratchWords) {
        vt::set_error("vt_hash_objects_noalloc: the sort scratch for this table exceeds the fixed array");
        return VT_ERR_CAPACITY;
    }
    // Nothing in the scratch has to start at zero: the sort clears its counts and
    // look-back words on the stream before use and writes every temporary key before
    // reading it, so the previous call's contents are harmless.
    cudaError_t e = vt::hash_objects_f3(particle_hash, particle_index, cell_start, cell_end, neighbors,
                                        positions, original_positions, *hp, keys_tmp, vals_tmp, hist,
                                        (cudaStream_t)stream);
    if (e != cudaSuccess) return vt::cuda_fail(e, "hash_objects (no-alloc)");
    return VT_OK;
}

extern "C" vt_status vt_hash_objects_noalloc(uint32_t* particle_hash, uint32_t* particle_index,
                                             uint32_t* cell_start, uint32_t* cell_end,
                                             uint32_t* neighbors, const float* positions,
                                             const float* original_positions,
                                             const vt_hash_params* hp, void* stream)
{
    try {  // no C++ exception (e.g. from the mutex) crosses the C ABI
        return hash_objects_noalloc(particle_hash, particle_index, cell_start, cell_end, neighbors, positions,
                                    original_positions, hp, stream);
    } catch (const std::bad_alloc&) {
        vt::set_error("host allocation failed");
        return VT_ERR_OUT_OF_MEMORY;
    } catch (...) {
        vt::set_error("unexpected host exception");
        return VT_ERR_STATE;
    }
}
