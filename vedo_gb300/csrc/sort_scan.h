// sort_scan.h - device prefix sums and a stable LSD radix sort, written for the broad
// phase (cell keys -> object ids, object ids -> contact entries).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace vedo {

// Scratch arena used by scans and sorts; grows on demand (owned by the engine).
struct Scratch {
    void* ptr = nullptr;
    size_t bytes = 0;
    cudaError_t reserve(size_t need);
    ~Scratch();
};

// out[i] = sum(in[0..i-1]); *total_dev (device pointer, may be null) receives the sum.
// in and out may alias.
cudaError_t exclusive_scan_u32(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* total_dev,
                               Scratch& scratch, cudaStream_t stream);

// Stable sort of (keys, vals) by keys[begin_bit, end_bit).  Results land in keys/vals;
// keys_alt/vals_alt are caller-provided buffers of the same size.
cudaError_t radix_sort_u64(uint64_t* keys, uint32_t* vals, uint64_t* keys_alt, uint32_t* vals_alt, uint32_t n,
                           int begin_bit, int end_bit, Scratch& scratch, cudaStream_t stream);
cudaError_t radix_sort_u32(uint32_t* keys, uint32_t* vals, uint32_t* keys_alt, uint32_t* vals_alt, uint32_t n,
                           int begin_bit, int end_bit, Scratch& scratch, cudaStream_t stream);

// Number of kernel launches issued by the functions above since the last reset.
extern thread_local uint64_t g_sort_scan_launches;

}  // namespace vedo
