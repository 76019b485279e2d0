// observables.cuh - DOWorld::CalculateSystemEnergy (DOWorld.cpp:481-660) over the device state,
// mobile objects only, with fixed-shape tree reductions (deterministic run to run).
#pragma once

#include <cfloat>

#include "dem_common.cuh"

namespace vedo {
namespace obs {
namespace {   // internal linkage: the header is compiled into each engine's translation unit

constexpr int TPB = 256;
constexpr int OBS_A = 16;
__global__ void __launch_bounds__(TPB) k_obs_a(uint32_t n, const uint32_t* __restrict__ model_of,
                                               const ModelDev* __restrict__ models, const double4_32a* __restrict__ pos,
                                               const double4_32a* __restrict__ vel, const double4_32a* __restrict__ av,
                                               d3 g, double* __restrict__ part) {
    __shared__ double s[OBS_A][TPB];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[OBS_A];
    for (int q = 0; q < OBS_A; ++q) v[q] = 0.0;
    v[12] = DBL_MAX; v[13] = -DBL_MAX; v[14] = DBL_MAX; v[15] = -DBL_MAX;
    if (i < n) {
        const ModelDev& m = models[model_of[i]];
        if (m.behavior == BEH_MOBILE) {
            const d3 V = ld(vel, i), AV = ld(av, i), P = ld(pos, i);
            const double vl = len(V), al = len(AV);
            const d3 I = mk(m.ix, m.iy, m.iz);
            v[0] = -m.mass * dot(g, P);
            v[1] = 0.5 * m.mass * vl * vl;
            v[2] = 0.5 * (I.x * AV.x * AV.x + I.y * AV.y * AV.y + I.z * AV.z * AV.z);
            const d3 mo = smul(m.mass, V), am = cross(I, AV);
            v[3] = mo.x; v[4] = mo.y; v[5] = mo.z;
            v[6] = am.x; v[7] = am.y; v[8] = am.z;
            v[9] = 1.0;
            v[10] = m.mass;
            v[11] = 0.0;
            v[12] = vl; v[13] = vl; v[14] = al; v[15] = al;
        }
    }
    for (int q = 0; q < OBS_A; ++q) s[q][threadIdx.x] = v[q];
    __syncthreads();
    for (int w = TPB / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            for (int q = 0; q < 12; ++q) s[q][threadIdx.x] += s[q][threadIdx.x + w];
            s[12][threadIdx.x] = fmin(s[12][threadIdx.x], s[12][threadIdx.x + w]);
            s[13][threadIdx.x] = fmax(s[13][threadIdx.x], s[13][threadIdx.x + w]);
            s[14][threadIdx.x] = fmin(s[14][threadIdx.x], s[14][threadIdx.x + w]);
            s[15][threadIdx.x] = fmax(s[15][threadIdx.x], s[15][threadIdx.x + w]);
        }
        __syncthreads();
    }
    if (threadIdx.x < OBS_A) part[(size_t)blockIdx.x * OBS_A + threadIdx.x] = s[threadIdx.x][0];
}

__global__ void k_obs_reduce(uint32_t nb, int width, const double* __restrict__ part, double* __restrict__ res,
                             int nmin_from) {
    // one thread per field, sequential over blocks (deterministic order)
    const int q = threadIdx.x;
    if (q >= width) return;
    double acc = part[q];
    for (uint32_t b = 1; b < nb; ++b) {
        const double x = part[(size_t)b * width + q];
        if (q < nmin_from) acc += x;
        else if (((q - nmin_from) & 1) == 0) acc = fmin(acc, x);
        else acc = fmax(acc, x);
    }
    res[q] = acc;
}

__global__ void __launch_bounds__(TPB) k_obs_b(uint32_t n, const uint32_t* __restrict__ model_of,
                                               const ModelDev* __restrict__ models, const double4_32a* __restrict__ pos,
                                               const double4_32a* __restrict__ vel, const double4_32a* __restrict__ av,
                                               const double* __restrict__ res, uint32_t nact_words,
                                               const uint8_t* __restrict__ flags, uint32_t np,
                                               double* __restrict__ part) {
    __shared__ double s[6][TPB];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[6] = {0, 0, 0, 0, 0, 0};
    const double cnt = res[9];
    const d3 mmean = smul(1.0 / cnt, mk(res[3], res[4], res[5]));
    const d3 amean = smul(1.0 / cnt, mk(res[6], res[7], res[8]));
    if (i < n) {
        const ModelDev& m = models[model_of[i]];
        if (m.behavior == BEH_MOBILE) {
            const d3 V = ld(vel, i), AV = ld(av, i), P = ld(pos, i);
            v[0] = len(sub(smul(m.mass, V), mmean));
            v[1] = len(sub(cross(mk(m.ix, m.iy, m.iz), AV), amean));
            v[2] = m.mass * P.x; v[3] = m.mass * P.y; v[4] = m.mass * P.z;
        }
    }
    for (uint32_t k = i; k < np; k += gridDim.x * blockDim.x) v[5] += (flags[k] & 64u) ? 1.0 : 0.0;
    for (int q = 0; q < 6; ++q) s[q][threadIdx.x] = v[q];
    __syncthreads();
    for (int w = TPB / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int q = 0; q < 6; ++q) s[q][threadIdx.x] += s[q][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < 6) part[(size_t)blockIdx.x * 6 + threadIdx.x] = s[threadIdx.x][0];
}


}  // namespace
}  // namespace obs
}  // namespace vedo
