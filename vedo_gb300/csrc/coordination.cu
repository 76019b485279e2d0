// coordination.cu - the post-processing tool's coordination number (vedo/knight/CalcCoordinateNum.cpp)
// over the device state.
//
// CalcCoordinateNum compares every sphere with every other one (O(N^2) on the host).  Here the
// spheres go into a uniform cell grid whose edge is a little over the largest radius sum, so
// every pair within reach lies in neighbouring cells; one thread per sphere visits the 27 cells
// around its own and applies the reference's exact FP64 tests (this file is compiled with
// -fmad=false): |p_i - p_j| = sqrt(dx*dx + dy*dy + dz*dz) against r_i + r_j, counting the
// strict test (outputCoordinateNumVTK, :79-126) and the inclusive one (computeAvgCoordinateNum,
// :8-77) in one pass.  The counts are integers, so the result equals the reference's whatever the
// visiting order.
#include "coordination.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "engine_base.h"
#include "sort_scan.h"

namespace vedo {
namespace {

constexpr int TPB = 256;
inline unsigned nblk(uint64_t n) { return (unsigned)((n + TPB - 1) / TPB); }

// order-preserving map of doubles to unsigned 64-bit integers (exact atomic min/max)
__device__ inline unsigned long long ord64(double d) {
    unsigned long long b = (unsigned long long)__double_as_longlong(d);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
inline double dbl_of(unsigned long long o) {
    unsigned long long b = (o >> 63) ? (o & 0x7fffffffffffffffull) : ~o;
    double d;
    std::memcpy(&d, &b, 8);
    return d;
}

__device__ inline bool is_sphere(const ModelDev& m) { return m.shape == SHAPE_SPHERE; }
__device__ inline bool finite3(d3 p) { return isfinite(p.x) && isfinite(p.y) && isfinite(p.z); }

// bounds of the finite sphere centres ([0..2] min, [3..5] max), the largest radius [6] and the
// number of spheres [7]
__global__ void k_cn_bounds(uint32_t n, const uint32_t* __restrict__ model_of, const ModelDev* __restrict__ models,
                            const double4_32a* __restrict__ pos, unsigned long long* __restrict__ red) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const ModelDev& m = models[model_of[i]];
    if (!is_sphere(m)) return;
    atomicAdd(&red[7], 1ull);
    const d3 p = ld(pos, i);
    if (!finite3(p)) return;
    atomicMin(&red[0], ord64(p.x)); atomicMin(&red[1], ord64(p.y)); atomicMin(&red[2], ord64(p.z));
    atomicMax(&red[3], ord64(p.x)); atomicMax(&red[4], ord64(p.y)); atomicMax(&red[5], ord64(p.z));
    atomicMax(&red[6], ord64(m.a0));
}

struct Grid {
    double lo[3], h;
    uint32_t dim[3];
};

__device__ inline uint32_t cell_axis(double x, double lo, double h, uint32_t dim) {
    const double c = floor((x - lo) / h);
    if (!(c >= 0.0)) return 0;                 // below the grid, or not a number
    if (c >= (double)(dim - 1)) return dim - 1;
    return (uint32_t)c;
}

// cell key per sphere (0xffffffff for other shapes: sorted last, never visited)
__global__ void k_cn_keys(uint32_t n, const uint32_t* __restrict__ model_of, const ModelDev* __restrict__ models,
                          const double4_32a* __restrict__ pos, Grid g, uint32_t* __restrict__ key,
                          uint32_t* __restrict__ id) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    id[i] = i;
    if (!is_sphere(models[model_of[i]])) {
        key[i] = 0xffffffffu;
        return;
    }
    const d3 p = ld(pos, i);
    const uint32_t cx = cell_axis(p.x, g.lo[0], g.h, g.dim[0]), cy = cell_axis(p.y, g.lo[1], g.h, g.dim[1]),
                   cz = cell_axis(p.z, g.lo[2], g.h, g.dim[2]);
    key[i] = cx + g.dim[0] * (cy + g.dim[1] * cz);
}

// [start, end) of every occupied cell in the sorted order
__global__ void k_cn_ranges(uint32_t ns, const uint32_t* __restrict__ key, uint32_t* __restrict__ start,
                            uint32_t* __restrict__ end) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ns) return;
    const uint32_t c = key[k];
    if (k == 0 || key[k - 1] != c) start[c] = k;
    if (k + 1 == ns || key[k + 1] != c) end[c] = k + 1;
}

__global__ void k_cn_count(uint32_t ns, const uint32_t* __restrict__ key, const uint32_t* __restrict__ id,
                           const uint32_t* __restrict__ start, const uint32_t* __restrict__ end,
                           const uint32_t* __restrict__ model_of, const ModelDev* __restrict__ models,
                           const double4_32a* __restrict__ pos, Grid g, uint32_t* __restrict__ below,
                           uint32_t* __restrict__ touching) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ns) return;
    const uint32_t i = id[k], c = key[k];
    const uint32_t cx = c % g.dim[0], cy = (c / g.dim[0]) % g.dim[1], cz = c / (g.dim[0] * g.dim[1]);
    const d3 pi = ld(pos, i);
    const double ri = models[model_of[i]].a0;
    uint32_t lt = 0, le = 0;
    for (int dz = -1; dz <= 1; ++dz) {
        const int z = (int)cz + dz;
        if (z < 0 || z >= (int)g.dim[2]) continue;
        for (int dy = -1; dy <= 1; ++dy) {
            const int y = (int)cy + dy;
            if (y < 0 || y >= (int)g.dim[1]) continue;
            for (int dx = -1; dx <= 1; ++dx) {
                const int x = (int)cx + dx;
                if (x < 0 || x >= (int)g.dim[0]) continue;
                const uint32_t cc = (uint32_t)x + g.dim[0] * ((uint32_t)y + g.dim[1] * (uint32_t)z);
                const uint32_t e = end[cc];
                for (uint32_t q = start[cc]; q < e; ++q) {
                    const uint32_t j = id[q];
                    if (j == i) continue;
                    const double d = len(sub(pi, ld(pos, j)));        // (m1 - m2).length()
                    const double rs = ri + models[model_of[j]].a0;    // r1 + r2
                    lt += d < rs ? 1u : 0u;
                    le += d <= rs ? 1u : 0u;
                }
            }
        }
    }
    below[i] = lt;
    touching[i] = le;
}

// computeAvgCoordinateNum's selection: centre strictly inside the box widened by the radius
__global__ void k_cn_average(uint32_t n, const uint32_t* __restrict__ model_of, const ModelDev* __restrict__ models,
                             const double4_32a* __restrict__ pos, const uint32_t* __restrict__ touching, Box6 b,
                             unsigned long long* __restrict__ sums) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const ModelDev& m = models[model_of[i]];
    if (!is_sphere(m)) return;
    const d3 p = ld(pos, i);
    const double r = m.a0;
    if ((p.x < (b.v[1] + r)) && (p.x > (b.v[0] - r)) && (p.y < (b.v[3] + r)) && (p.y > (b.v[2] - r)) &&
        (p.z < (b.v[5] + r)) && (p.z > (b.v[4] - r))) {
        atomicAdd(&sums[0], (unsigned long long)touching[i]);
        atomicAdd(&sums[1], 1ull);
    }
}

}  // namespace

int coordination_device(uint32_t n, const uint32_t* model_of, const ModelDev* models, const double4_32a* pos,
                        uint32_t* below, uint32_t* touching, const double* box, double* average, Scratch& scratch,
                        cudaStream_t s, std::string& err, uint64_t* launches) {
    uint64_t L = 0;
    auto fail = [&](cudaError_t e) {
        err = std::string("coordination: ") + cudaGetErrorString(e);
        return VEDO_ERR_CUDA;
    };
#define CN_CK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) return fail(e_); } while (0)
    CN_CK(cudaMemsetAsync(below, 0, 4 * (size_t)std::max<uint32_t>(n, 1), s));
    CN_CK(cudaMemsetAsync(touching, 0, 4 * (size_t)std::max<uint32_t>(n, 1), s));
    if (n == 0) {
        if (average) *average = NAN;
        return VEDO_OK;
    }
    // bounds of the sphere centres, the largest radius, the sphere count; [8..9]: the average's sums
    unsigned long long* red = nullptr;
    CN_CK(cudaMallocAsync(&red, 10 * sizeof(unsigned long long), s));
    unsigned long long init[10];
    for (int k = 0; k < 3; ++k) init[k] = ~0ull;
    for (int k = 3; k < 10; ++k) init[k] = 0ull;
    CN_CK(cudaMemcpyAsync(red, init, sizeof(init), cudaMemcpyHostToDevice, s));
    k_cn_bounds<<<nblk(n), TPB, 0, s>>>(n, model_of, models, pos, red);
    ++L;
    unsigned long long got[8];
    CN_CK(cudaMemcpyAsync(got, red, sizeof(got), cudaMemcpyDeviceToHost, s));
    CN_CK(cudaStreamSynchronize(s));
    // with no sphere at a finite position no distance test can hold (NaN compares false)
    const bool any = got[6] != 0ull;
    const uint32_t ns = (uint32_t)got[7];
    if (any) {
        Grid g{};
        double hi[3];
        for (int k = 0; k < 3; ++k) {
            g.lo[k] = dbl_of(got[k]);
            hi[k] = dbl_of(got[3 + k]);
        }
        const double rmax = dbl_of(got[6]);
        // a pair within reach is at most 2 r_max apart; the margin keeps the floor() of the cell
        // coordinates of two such centres within one of each other despite rounding
        double h = std::max(2.0 * rmax, 1e-300) * (1.0 + 1e-6);
        for (int k = 0; k < 3; ++k) h = std::max(h, (hi[k] - g.lo[k]) * 1e-9);
        const double cap = std::max(64.0, 4.0 * (double)n);
        for (;;) {
            double cells = 1.0;
            for (int k = 0; k < 3; ++k) cells *= std::floor((hi[k] - g.lo[k]) / h) + 1.0;
            if (cells <= cap) break;
            h *= 2.0;
        }
        g.h = h;
        for (int k = 0; k < 3; ++k) g.dim[k] = (uint32_t)(std::floor((hi[k] - g.lo[k]) / h) + 1.0);
        const uint32_t ncell = g.dim[0] * g.dim[1] * g.dim[2];
        uint32_t *key = nullptr, *id = nullptr, *key2 = nullptr, *id2 = nullptr, *cs = nullptr, *ce = nullptr;
        CN_CK(cudaMallocAsync(&key, 4 * (size_t)n, s));
        CN_CK(cudaMallocAsync(&id, 4 * (size_t)n, s));
        CN_CK(cudaMallocAsync(&key2, 4 * (size_t)n, s));
        CN_CK(cudaMallocAsync(&id2, 4 * (size_t)n, s));
        CN_CK(cudaMallocAsync(&cs, 4 * (size_t)ncell, s));
        CN_CK(cudaMallocAsync(&ce, 4 * (size_t)ncell, s));
        CN_CK(cudaMemsetAsync(cs, 0, 4 * (size_t)ncell, s));
        CN_CK(cudaMemsetAsync(ce, 0, 4 * (size_t)ncell, s));
        k_cn_keys<<<nblk(n), TPB, 0, s>>>(n, model_of, models, pos, g, key, id);
        ++L;
        const uint64_t l0 = g_sort_scan_launches;
        CN_CK(radix_sort_u32(key, id, key2, id2, n, 0, 32, scratch, s));
        L += g_sort_scan_launches - l0;
        // the spheres' keys sort before the other shapes' 0xffffffff: the first ns entries
        if (ns) {
            k_cn_ranges<<<nblk(ns), TPB, 0, s>>>(ns, key, cs, ce);
            k_cn_count<<<nblk(ns), TPB, 0, s>>>(ns, key, id, cs, ce, model_of, models, pos, g, below, touching);
            L += 2;
        }
        CN_CK(cudaFreeAsync(key, s));
        CN_CK(cudaFreeAsync(id, s));
        CN_CK(cudaFreeAsync(key2, s));
        CN_CK(cudaFreeAsync(id2, s));
        CN_CK(cudaFreeAsync(cs, s));
        CN_CK(cudaFreeAsync(ce, s));
    }
    if (average) {
        Box6 b;
        for (int k = 0; k < 6; ++k) b.v[k] = box ? box[k] : 0.0;
        k_cn_average<<<nblk(n), TPB, 0, s>>>(n, model_of, models, pos, touching, b, red + 8);
        ++L;
        unsigned long long sums[2];
        CN_CK(cudaMemcpyAsync(sums, red + 8, sizeof(sums), cudaMemcpyDeviceToHost, s));
        CN_CK(cudaStreamSynchronize(s));
        // the reference sums in an unsigned 32-bit integer and divides by the selected count
        const uint32_t total = (uint32_t)sums[0];
        *average = total / (double)sums[1];
    }
    CN_CK(cudaFreeAsync(red, s));
    CN_CK(cudaStreamSynchronize(s));
    CN_CK(cudaGetLastError());
    if (launches) *launches += L;
#undef CN_CK
    return VEDO_OK;
}

}  // namespace vedo

namespace vedo {

int coordination_host(const DeviceObjects& d, uint32_t* below, uint32_t* touching, const double* box,
                      double* average, std::string& err) {
    if (!d.scene || !d.scratch) {
        err = "coordination needs a single-scene engine";
        return VEDO_ERR_INVALID_ARGUMENT;
    }
    uint32_t* buf = nullptr;
    cudaError_t e = cudaMallocAsync(&buf, 8 * (size_t)std::max<uint32_t>(d.n, 1), d.stream);
    if (e != cudaSuccess) {
        err = std::string("coordination: ") + cudaGetErrorString(e);
        return VEDO_ERR_OUT_OF_MEMORY;
    }
    uint32_t* dlt = buf;
    uint32_t* dle = buf + std::max<uint32_t>(d.n, 1);
    int rc = coordination_device(d.n, d.model_of, d.models, d.pos, dlt, dle, box, average, *d.scratch, d.stream, err,
                                 d.launches);
    if (rc == VEDO_OK && below) e = cudaMemcpyAsync(below, dlt, 4 * (size_t)d.n, cudaMemcpyDeviceToHost, d.stream);
    if (rc == VEDO_OK && e == cudaSuccess && touching)
        e = cudaMemcpyAsync(touching, dle, 4 * (size_t)d.n, cudaMemcpyDeviceToHost, d.stream);
    cudaFreeAsync(buf, d.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(d.stream);
    if (rc == VEDO_OK && e != cudaSuccess) {
        err = std::string("coordination: ") + cudaGetErrorString(e);
        rc = VEDO_ERR_CUDA;
    }
    return rc;
}

int write_vtk_host(EngineBase* eng, const DeviceObjects& d, const char* path, int with_coordination,
                   std::string& err) {
    if (!path) return VEDO_ERR_INVALID_ARGUMENT;
    if (!d.scene) {
        err = "write_vtk needs a single-scene engine";
        return VEDO_ERR_INVALID_ARGUMENT;
    }
    std::vector<double> pos(3 * (size_t)d.n), vel(3 * (size_t)d.n), av(3 * (size_t)d.n);
    vedo_state_view v{};
    v.position = pos.data();
    v.velocity = vel.data();
    v.angular_velocity = av.data();
    int rc = eng->get_state(v);
    if (rc != VEDO_OK) {
        err = eng->error();
        return rc;
    }
    std::vector<uint32_t> cn;
    if (with_coordination) {
        cn.resize(d.n);
        rc = coordination_host(d, cn.data(), nullptr, nullptr, nullptr, err);
        if (rc != VEDO_OK) return rc;
    }
    if (!write_world_vtk(path, *d.scene, pos.data(), vel.data(), av.data(), with_coordination ? cn.data() : nullptr,
                         err))
        return VEDO_ERR_IO;
    return VEDO_OK;
}

}  // namespace vedo
