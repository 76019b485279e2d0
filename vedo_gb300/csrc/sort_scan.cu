// sort_scan.cu - exclusive prefix sum and stable LSD radix sort (8-bit digits).
//
// Radix sort pass = histogram kernel (per-tile digit counts, digit-major layout),
// exclusive scan of the counts, and a scatter kernel that ranks each tile's items
// stably (warp match + per-warp digit counts in shared memory, tiles processed in
// rounds of 256 items) before writing them to their global slot.
#include "sort_scan.h"

#include <algorithm>

namespace vedo {

thread_local uint64_t g_sort_scan_launches = 0;

cudaError_t Scratch::reserve(size_t need) {
    if (need <= bytes) return cudaSuccess;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
    size_t n = std::max(need, bytes * 3 / 2);
    cudaError_t e = cudaMalloc(&ptr, n);
    if (e != cudaSuccess) return e;
    bytes = n;
    return cudaSuccess;
}

Scratch::~Scratch() {
    if (ptr) cudaFree(ptr);
}

// ---------------------------------------------------------------------------------------
// scan
constexpr int SCAN_T = 256;
constexpr int SCAN_I = 8;
constexpr uint32_t SCAN_TILE = SCAN_T * SCAN_I;

__global__ void __launch_bounds__(SCAN_T) k_scan_tile(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                                      uint32_t n, uint32_t* __restrict__ block_sums,
                                                      uint32_t* __restrict__ total) {
    __shared__ uint32_t s[SCAN_TILE];
    __shared__ uint32_t warp_sums[SCAN_T / 32];
    const uint32_t base = blockIdx.x * SCAN_TILE;
    const int tid = threadIdx.x;
#pragma unroll
    for (int j = 0; j < SCAN_I; ++j) {
        uint32_t idx = base + j * SCAN_T + tid;
        s[j * SCAN_T + tid] = idx < n ? in[idx] : 0u;
    }
    __syncthreads();
    uint32_t v[SCAN_I];
    uint32_t sum = 0;
#pragma unroll
    for (int j = 0; j < SCAN_I; ++j) {
        v[j] = sum;
        sum += s[tid * SCAN_I + j];
    }
    // block-wide exclusive scan of per-thread sums
    const int lane = tid & 31, warp = tid >> 5;
    uint32_t x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < SCAN_T / 32 ? warp_sums[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < SCAN_T / 32) warp_sums[lane] = w;
    }
    __syncthreads();
    uint32_t excl = x - sum + (warp > 0 ? warp_sums[warp - 1] : 0u);
#pragma unroll
    for (int j = 0; j < SCAN_I; ++j) s[tid * SCAN_I + j] = v[j] + excl;
    if (tid == SCAN_T - 1) {
        uint32_t bsum = excl + sum;
        if (block_sums) block_sums[blockIdx.x] = bsum;
        if (total && gridDim.x == 1) *total = bsum;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < SCAN_I; ++j) {
        uint32_t idx = base + j * SCAN_T + tid;
        if (idx < n) out[idx] = s[j * SCAN_T + tid];
    }
}

__global__ void __launch_bounds__(SCAN_T) k_scan_add(uint32_t* __restrict__ out, uint32_t n,
                                                     const uint32_t* __restrict__ block_off) {
    const uint32_t base = blockIdx.x * SCAN_TILE;
    const uint32_t add = block_off[blockIdx.x];
#pragma unroll
    for (int j = 0; j < SCAN_I; ++j) {
        uint32_t idx = base + j * SCAN_T + threadIdx.x;
        if (idx < n) out[idx] += add;
    }
}

static size_t scan_tmp_words(uint32_t n) {
    size_t w = 0;
    while (n > SCAN_TILE) {
        n = (n + SCAN_TILE - 1) / SCAN_TILE;
        w += n;
    }
    return w + 1;
}

static cudaError_t scan_impl(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* total, uint32_t* tmp,
                             cudaStream_t stream) {
    if (n == 0) {
        if (total) return cudaMemsetAsync(total, 0, sizeof(uint32_t), stream);
        return cudaSuccess;
    }
    uint32_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (nb == 1) {
        k_scan_tile<<<1, SCAN_T, 0, stream>>>(in, out, n, nullptr, total);
        ++g_sort_scan_launches;
        return cudaGetLastError();
    }
    uint32_t* sums = tmp;
    k_scan_tile<<<nb, SCAN_T, 0, stream>>>(in, out, n, sums, nullptr);
    ++g_sort_scan_launches;
    cudaError_t e = scan_impl(sums, sums, nb, total, tmp + nb, stream);
    if (e != cudaSuccess) return e;
    k_scan_add<<<nb, SCAN_T, 0, stream>>>(out, n, sums);
    ++g_sort_scan_launches;
    return cudaGetLastError();
}

cudaError_t exclusive_scan_u32(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* total_dev,
                               Scratch& scratch, cudaStream_t stream) {
    cudaError_t e = scratch.reserve(scan_tmp_words(n) * sizeof(uint32_t));
    if (e != cudaSuccess) return e;
    return scan_impl(in, out, n, total_dev, static_cast<uint32_t*>(scratch.ptr), stream);
}

// ---------------------------------------------------------------------------------------
// radix sort
constexpr int RS_T = 256;
constexpr int RS_ROUNDS = 16;
constexpr uint32_t RS_TILE = RS_T * RS_ROUNDS;
constexpr int RS_WARPS = RS_T / 32;

template <class K>
__global__ void __launch_bounds__(RS_T) k_rs_hist(const K* __restrict__ keys, uint32_t n, int shift,
                                                  uint32_t* __restrict__ counts, uint32_t nb) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * RS_TILE;
#pragma unroll 4
    for (int r = 0; r < RS_ROUNDS; ++r) {
        uint32_t idx = base + r * RS_T + threadIdx.x;
        if (idx < n) atomicAdd(&h[(uint32_t)(keys[idx] >> shift) & 255u], 1u);
    }
    __syncthreads();
    counts[threadIdx.x * nb + blockIdx.x] = h[threadIdx.x];
}

template <class K>
__global__ void __launch_bounds__(RS_T) k_rs_scatter(const K* __restrict__ kin, const uint32_t* __restrict__ vin,
                                                     K* __restrict__ kout, uint32_t* __restrict__ vout, uint32_t n,
                                                     int shift, const uint32_t* __restrict__ offsets, uint32_t nb) {
    __shared__ uint32_t base[256];
    __shared__ uint32_t wcnt[RS_WARPS][256];
    __shared__ uint32_t rtot[256];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    base[tid] = offsets[tid * nb + blockIdx.x];
    const uint32_t tile = blockIdx.x * RS_TILE;
    const uint32_t lt_mask = (1u << lane) - 1u;
    for (int r = 0; r < RS_ROUNDS; ++r) {
        const uint32_t idx = tile + r * RS_T + tid;
        const bool valid = idx < n;
        K key = valid ? kin[idx] : K(0);
        uint32_t val = valid ? vin[idx] : 0u;
        uint32_t d = valid ? ((uint32_t)(key >> shift) & 255u) : 256u;
#pragma unroll
        for (int w = 0; w < RS_WARPS; ++w) wcnt[w][tid] = 0;
        __syncthreads();
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        uint32_t rank = __popc(peers & lt_mask);
        if (valid && rank == 0) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        {
            uint32_t s = 0;
#pragma unroll
            for (int w = 0; w < RS_WARPS; ++w) {
                uint32_t c = wcnt[w][tid];
                wcnt[w][tid] = s;
                s += c;
            }
            rtot[tid] = s;
        }
        __syncthreads();
        if (valid) {
            uint32_t pos = base[d] + wcnt[warp][d] + rank;
            kout[pos] = key;
            vout[pos] = val;
        }
        __syncthreads();
        base[tid] += rtot[tid];
        __syncthreads();
    }
}

template <class K>
static cudaError_t radix_sort_impl(K* keys, uint32_t* vals, K* keys_alt, uint32_t* vals_alt, uint32_t n,
                                   int begin_bit, int end_bit, Scratch& scratch, cudaStream_t stream) {
    if (n <= 1 || end_bit <= begin_bit) return cudaSuccess;
    const uint32_t nb = (n + RS_TILE - 1) / RS_TILE;
    const size_t ncnt = (size_t)256 * nb;
    size_t words = ncnt + scan_tmp_words((uint32_t)ncnt) + 1;
    cudaError_t e = scratch.reserve(words * sizeof(uint32_t));
    if (e != cudaSuccess) return e;
    uint32_t* counts = static_cast<uint32_t*>(scratch.ptr);
    uint32_t* tmp = counts + ncnt;
    K* kin = keys;
    uint32_t* vin = vals;
    K* kout = keys_alt;
    uint32_t* vout = vals_alt;
    int passes = 0;
    for (int shift = begin_bit; shift < end_bit; shift += 8) {
        k_rs_hist<K><<<nb, RS_T, 0, stream>>>(kin, n, shift, counts, nb);
        ++g_sort_scan_launches;
        e = scan_impl(counts, counts, (uint32_t)ncnt, nullptr, tmp, stream);
        if (e != cudaSuccess) return e;
        k_rs_scatter<K><<<nb, RS_T, 0, stream>>>(kin, vin, kout, vout, n, shift, counts, nb);
        ++g_sort_scan_launches;
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        std::swap(kin, kout);
        std::swap(vin, vout);
        ++passes;
    }
    if (passes & 1) {
        e = cudaMemcpyAsync(keys, kin, sizeof(K) * n, cudaMemcpyDeviceToDevice, stream);
        if (e != cudaSuccess) return e;
        e = cudaMemcpyAsync(vals, vin, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, stream);
    }
    return e;
}

cudaError_t radix_sort_u64(uint64_t* keys, uint32_t* vals, uint64_t* keys_alt, uint32_t* vals_alt, uint32_t n,
                           int begin_bit, int end_bit, Scratch& scratch, cudaStream_t stream) {
    return radix_sort_impl<uint64_t>(keys, vals, keys_alt, vals_alt, n, begin_bit, end_bit, scratch, stream);
}

cudaError_t radix_sort_u32(uint32_t* keys, uint32_t* vals, uint32_t* keys_alt, uint32_t* vals_alt, uint32_t n,
                           int begin_bit, int end_bit, Scratch& scratch, cudaStream_t stream) {
    return radix_sort_impl<uint32_t>(keys, vals, keys_alt, vals_alt, n, begin_bit, end_bit, scratch, stream);
}

}  // namespace vedo
