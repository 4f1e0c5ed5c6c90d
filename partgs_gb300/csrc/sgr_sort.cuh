// The library's own stable radix sort and prefix sums (sgr_sort.cu), shared
// by the forward's depth order and cell lists and the Chamfer evaluation's
// grids.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace sgr {

// Stable LSD radix sort of (key, id) pairs on key bits [0, end_bit), 8 bits
// a pass; keys_in / vals_in are not modified.  Returns an SGR_* status.
template <class K>
size_t radix_sort_temp_bytes(long long n);
template <class K>
int radix_sort_pairs(const K* keys_in, K* keys_out, const uint32_t* vals_in, uint32_t* vals_out, long long n,
                     int end_bit, void* temp, size_t temp_bytes, cudaStream_t st);

// Inclusive (INCLUSIVE) or exclusive prefix sum; `in` may equal `out`.
template <class T>
size_t scan_temp_bytes(long long n);
template <class T, bool INCLUSIVE>
int prefix_sum(const T* in, T* out, long long n, void* temp, size_t temp_bytes, cudaStream_t st);

}  // namespace sgr
