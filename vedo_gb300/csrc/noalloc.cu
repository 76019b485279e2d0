// noalloc.cu - system energy and momentum over caller-owned device arrays, with no device
// allocation at all.
//
// Who needs this: a host program that shares the GPU with the engine and cannot let a library
// call cudaMalloc or cudaFree.  Typical cases are a coupled solver (CFD, FEM) or a framework
// whose caching allocator has already reserved most of HBM for its own pool, so a new
// allocation would fail or fragment that pool; and a monitoring hook on a time-critical loop,
// where cudaFree (and often cudaMalloc) synchronises the whole device and stalls every other
// stream.  Such a caller keeps the object state in its own buffers and asks for the energy
// budget of that state; the reduction's block partial sums live in a fixed array that this
// library declares at file scope, so the call allocates nothing.
//
// The quantities are the ones vedo_gpu_get_observables reports (the engine's own form keeps
// its partial sums in memory the engine allocates): potential, translational and rotational
// energy, speed and angular-speed extremes, the momentum and angular-momentum spread terms
// and the mass-weighted centre, over the objects marked mobile.
#include <cfloat>
#include <cstdint>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "../../include/vedo_gpu.h"
#include "dem_common.cuh"

namespace vedo {
void set_last_error(const std::string& msg);   // capi.cpp: text for vedo_gpu_last_error(NULL)
}

namespace {

using namespace vedo;

constexpr int NA_TPB = 256;
constexpr int NA_PER_THREAD = 8;
constexpr uint32_t NA_OBJ_PER_BLOCK = NA_TPB * NA_PER_THREAD;                  // 2,048
constexpr uint32_t NA_MAX_BLOCKS = VEDO_NOALLOC_MAX_OBJECTS / NA_OBJ_PER_BLOCK; // 8,192
constexpr int NA_W1 = 16;    // first pass: 12 sums, then min |v|, max |v|, min |w|, max |w|
constexpr int NA_W2 = 5;     // second pass: two spread sums, three mass-weighted coordinates
constexpr size_t NA_RES = (size_t)NA_MAX_BLOCKS * NA_W1;                        // results follow the partials
constexpr size_t NA_SCRATCH_DOUBLES = NA_RES + 32;

// The scratch array: block partial sums of both passes, then the reduced values (1 MiB in all).
// Every GPU that loads this library holds it until the process exits.  Every call shares it and
// it keeps the last call's contents; each call writes every slot it later reads, so nothing has
// to be cleared between calls.  In host code `g_na_scratch` is only a stand-in for the symbol:
// the device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) double g_na_scratch[NA_SCRATCH_DOUBLES];

__device__ __forceinline__ d3 ld3(const double* __restrict__ a, uint32_t i) {
    return mk(a[3 * (size_t)i], a[3 * (size_t)i + 1], a[3 * (size_t)i + 2]);
}

template <int W>
__device__ __forceinline__ void block_sum(double (*s)[NA_TPB], int nmin_from) {
    __syncthreads();
    for (int w = NA_TPB / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int q = 0; q < W; ++q) {
                const double a = s[q][threadIdx.x], b = s[q][threadIdx.x + w];
                if (q < nmin_from) s[q][threadIdx.x] = a + b;
                else if (((q - nmin_from) & 1) == 0) s[q][threadIdx.x] = fmin(a, b);
                else s[q][threadIdx.x] = fmax(a, b);
            }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(NA_TPB) k_na_pass1(uint32_t n, const double* __restrict__ pos,
                                                     const double* __restrict__ vel, const double* __restrict__ av,
                                                     const double* __restrict__ mass,
                                                     const double* __restrict__ inertia,
                                                     const uint8_t* __restrict__ mobile, d3 g,
                                                     double* __restrict__ part) {
    __shared__ double s[NA_W1][NA_TPB];
    double v[NA_W1];
    for (int q = 0; q < 12; ++q) v[q] = 0.0;
    v[12] = DBL_MAX; v[13] = -DBL_MAX; v[14] = DBL_MAX; v[15] = -DBL_MAX;
    for (int k = 0; k < NA_PER_THREAD; ++k) {
        const uint32_t i = blockIdx.x * NA_OBJ_PER_BLOCK + k * NA_TPB + threadIdx.x;
        if (i >= n || (mobile && !mobile[i])) continue;
        const d3 V = ld3(vel, i), AV = ld3(av, i), P = ld3(pos, i), I = ld3(inertia, i);
        const double m = mass[i], vl = len(V), al = len(AV);
        v[0] += -m * dot(g, P);
        v[1] += 0.5 * m * vl * vl;
        v[2] += 0.5 * (I.x * AV.x * AV.x + I.y * AV.y * AV.y + I.z * AV.z * AV.z);
        const d3 mo = smul(m, V), am = cross(I, AV);
        v[3] += mo.x; v[4] += mo.y; v[5] += mo.z;
        v[6] += am.x; v[7] += am.y; v[8] += am.z;
        v[9] += 1.0;
        v[10] += m;
        v[12] = fmin(v[12], vl); v[13] = fmax(v[13], vl);
        v[14] = fmin(v[14], al); v[15] = fmax(v[15], al);
    }
    for (int q = 0; q < NA_W1; ++q) s[q][threadIdx.x] = v[q];
    block_sum<NA_W1>(s, 12);
    if (threadIdx.x < NA_W1) part[(size_t)blockIdx.x * NA_W1 + threadIdx.x] = s[threadIdx.x][0];
}

__global__ void __launch_bounds__(NA_TPB) k_na_pass2(uint32_t n, const double* __restrict__ pos,
                                                     const double* __restrict__ vel, const double* __restrict__ av,
                                                     const double* __restrict__ mass,
                                                     const double* __restrict__ inertia,
                                                     const uint8_t* __restrict__ mobile,
                                                     const double* __restrict__ res, double* __restrict__ part) {
    __shared__ double s[NA_W2][NA_TPB];
    double v[NA_W2] = {0.0, 0.0, 0.0, 0.0, 0.0};
    const double cnt = res[9];
    if (cnt > 0.0) {
        const d3 mmean = smul(1.0 / cnt, mk(res[3], res[4], res[5]));
        const d3 amean = smul(1.0 / cnt, mk(res[6], res[7], res[8]));
        for (int k = 0; k < NA_PER_THREAD; ++k) {
            const uint32_t i = blockIdx.x * NA_OBJ_PER_BLOCK + k * NA_TPB + threadIdx.x;
            if (i >= n || (mobile && !mobile[i])) continue;
            const d3 V = ld3(vel, i), AV = ld3(av, i), P = ld3(pos, i), I = ld3(inertia, i);
            const double m = mass[i];
            v[0] += len(sub(smul(m, V), mmean));
            v[1] += len(sub(cross(I, AV), amean));
            v[2] += m * P.x; v[3] += m * P.y; v[4] += m * P.z;
        }
    }
    for (int q = 0; q < NA_W2; ++q) s[q][threadIdx.x] = v[q];
    block_sum<NA_W2>(s, NA_W2);
    if (threadIdx.x < NA_W2) part[(size_t)blockIdx.x * NA_W2 + threadIdx.x] = s[threadIdx.x][0];
}

// One warp per field: lane l folds blocks l, l + 32, ... in order, then a fixed shuffle tree.
__global__ void k_na_reduce(uint32_t nb, int width, int nmin_from, const double* __restrict__ part,
                            double* __restrict__ res) {
    const int q = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (q >= width) return;
    const bool is_sum = q < nmin_from, is_min = !is_sum && ((q - nmin_from) & 1) == 0;
    double acc = is_sum ? 0.0 : (is_min ? DBL_MAX : -DBL_MAX);
    for (uint32_t b = lane; b < nb; b += 32) {
        const double x = part[(size_t)b * width + q];
        acc = is_sum ? acc + x : (is_min ? fmin(acc, x) : fmax(acc, x));
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double x = __shfl_xor_sync(0xffffffffu, acc, o);
        acc = is_sum ? acc + x : (is_min ? fmin(acc, x) : fmax(acc, x));
    }
    if (lane == 0) res[q] = acc;
}

__global__ void k_na_finish(const double* __restrict__ res, double* __restrict__ out) {
    if (threadIdx.x != 0) return;
    const bool any = res[9] > 0.0;
    const double msum = res[10];
    out[0] = res[0]; out[1] = res[1]; out[2] = res[2];
    out[3] = any ? res[12] : 0.0; out[4] = any ? res[13] : 0.0;
    out[5] = any ? res[14] : 0.0; out[6] = any ? res[15] : 0.0;
    out[7] = res[16]; out[8] = res[17];
    out[9] = msum > 0.0 ? res[18] / msum : 0.0;
    out[10] = msum > 0.0 ? res[19] / msum : 0.0;
    out[11] = msum > 0.0 ? res[20] / msum : 0.0;
}

// Device address of the scratch array, looked up once per device with that device current.
constexpr int NA_MAX_DEVICES = 64;
std::mutex g_na_mutex;
double* g_na_addr[NA_MAX_DEVICES] = {};

int scratch_for_current_device(double** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        set_last_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
        return VEDO_ERR_CUDA;
    }
    if (dev < 0 || dev >= NA_MAX_DEVICES) {
        set_last_error("device ordinal beyond the 64 this entry point serves");
        return VEDO_ERR_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_na_scratch);
        if (e != cudaSuccess || !p) {
            set_last_error(std::string("cudaGetSymbolAddress of the scratch array: ") + cudaGetErrorString(e));
            return VEDO_ERR_CUDA;
        }
        g_na_addr[dev] = static_cast<double*>(p);
    }
    *out = g_na_addr[dev];
    return VEDO_OK;
}

}  // namespace

extern "C" int vedo_gpu_system_energy_noalloc(const double* position, const double* velocity,
                                              const double* angular_velocity, const double* mass,
                                              const double* inertia, const uint8_t* mobile, uint32_t num_objects,
                                              const double field_acceleration[3], double* out, void* stream) {
    if (num_objects > VEDO_NOALLOC_MAX_OBJECTS) {
        set_last_error("vedo_gpu_system_energy_noalloc: " + std::to_string(num_objects) +
                       " objects, more than its fixed scratch serves (" +
                       std::to_string(VEDO_NOALLOC_MAX_OBJECTS) + ")");
        return VEDO_ERR_INVALID_ARGUMENT;
    }
    if (!out || !field_acceleration ||
        (num_objects && (!position || !velocity || !angular_velocity || !mass || !inertia))) {
        set_last_error("vedo_gpu_system_energy_noalloc: NULL argument");
        return VEDO_ERR_INVALID_ARGUMENT;
    }
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        set_last_error("vedo_gpu_system_energy_noalloc: no current CUDA device");
        return VEDO_ERR_CUDA;
    }
    // every buffer the kernels touch must be device (or managed) memory of the current device:
    // a host pointer or another GPU's would only fail later, as an asynchronous fault
    const void* bufs[] = {position, velocity, angular_velocity, mass, inertia, mobile, out};
    const char* names[] = {"position", "velocity", "angular_velocity", "mass", "inertia", "mobile", "out"};
    for (int k = 0; k < 7; ++k) {
        if (!bufs[k] || (k < 6 && !num_objects)) continue;
        cudaPointerAttributes at{};
        const cudaError_t pe = cudaPointerGetAttributes(&at, bufs[k]);
        if (pe != cudaSuccess) {
            cudaGetLastError();                       // clear the error the query left
            set_last_error(std::string("vedo_gpu_system_energy_noalloc: ") + names[k] + ": " + cudaGetErrorString(pe));
            return VEDO_ERR_INVALID_ARGUMENT;
        }
        const bool device_mem = at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
        if (!device_mem || (at.type == cudaMemoryTypeDevice && at.device != dev)) {
            set_last_error(std::string("vedo_gpu_system_energy_noalloc: ") + names[k] +
                           " is not device memory of the current device");
            return VEDO_ERR_INVALID_ARGUMENT;
        }
    }
    double* scratch = nullptr;
    const int rc = scratch_for_current_device(&scratch);
    if (rc != VEDO_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const uint32_t nb = num_objects ? (num_objects + NA_OBJ_PER_BLOCK - 1) / NA_OBJ_PER_BLOCK : 1;
    double* part = scratch;
    double* res = scratch + NA_RES;
    const d3 g = mk(field_acceleration[0], field_acceleration[1], field_acceleration[2]);
    k_na_pass1<<<nb, NA_TPB, 0, s>>>(num_objects, position, velocity, angular_velocity, mass, inertia, mobile, g,
                                     part);
    k_na_reduce<<<1, 32 * NA_W1, 0, s>>>(nb, NA_W1, 12, part, res);
    k_na_pass2<<<nb, NA_TPB, 0, s>>>(num_objects, position, velocity, angular_velocity, mass, inertia, mobile, res,
                                     part);
    k_na_reduce<<<1, 32 * NA_W2, 0, s>>>(nb, NA_W2, NA_W2, part, res + NA_W1);
    k_na_finish<<<1, 32, 0, s>>>(res, out);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_last_error(std::string("vedo_gpu_system_energy_noalloc launch: ") + cudaGetErrorString(e));
        return VEDO_ERR_CUDA;
    }
    return VEDO_OK;
}
