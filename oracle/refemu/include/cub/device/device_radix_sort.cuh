// cub::DeviceRadixSort::SortPairs for the CPU — TEST INFRASTRUCTURE.  The reference sorts
// its (cell key, particle) pairs with CUB's DeviceRadixSort::SortPairs from the CUDA
// 11.1 toolkit (Velvet/SpatialHashGPU.cu:133-157; README).  CUB is absent here, and its
// published contract is all the reference relies on: pairs ordered by the key bits
// [begin_bit, end_bit) ascending, stable (equal keys keep their input order).  A stable
// sort on those bits has exactly one result, which this restates with a least-
// significant-digit counting sort (8 bits per pass, stable by construction).  Plain loops
// only: the reference's include layout is compiled with -I-, under which libstdc++'s
// <algorithm> does not compile.
#pragma once

#include <cstddef>
#include <vector>

#include <cuda_runtime.h>

namespace cub {

struct DeviceRadixSort {
    template <class K, class V>
    static cudaError_t SortPairs(void* d_temp_storage, size_t& temp_storage_bytes, const K* keys_in, K* keys_out,
                                 const V* values_in, V* values_out, int num_items, int begin_bit = 0,
                                 int end_bit = (int)(sizeof(K) * 8), cudaStream_t = 0, bool = false)
    {
        if (d_temp_storage == nullptr) {  // size query
            temp_storage_bytes = sizeof(K) * (size_t)(num_items > 0 ? num_items : 1);
            return cudaSuccess;
        }
        const size_t n = (size_t)(num_items > 0 ? num_items : 0);
        std::vector<K> k0(keys_in, keys_in + n), k1(n);
        std::vector<V> v0(values_in, values_in + n), v1(n);
        for (int shift = begin_bit; shift < end_bit; shift += 8) {
            const int bits = (end_bit - shift) < 8 ? (end_bit - shift) : 8;
            const K mask = (K)((1u << bits) - 1u);
            size_t count[257] = {0};
            for (size_t t = 0; t < n; ++t) count[((k0[t] >> shift) & mask) + 1]++;
            for (int d = 0; d < 256; ++d) count[d + 1] += count[d];
            for (size_t t = 0; t < n; ++t) {
                const size_t at = count[(k0[t] >> shift) & mask]++;
                k1[at] = k0[t];
                v1[at] = v0[t];
            }
            k0.swap(k1);
            v0.swap(v1);
        }
        for (size_t t = 0; t < n; ++t) {
            keys_out[t] = k0[t];
            values_out[t] = v0[t];
        }
        return cudaSuccess;
    }
};

}  // namespace cub
