// prefilter.cuh - conservative FP32 bounds that let the FP64 engine skip exact work.
//
// GB300 executes FP64 at a small fraction of its FP32 rate, so the exact FP64 narrow phase
// and candidate test run only where an FP32 estimate cannot decide.  Positions are kept
// as FP32 offsets from a fixed origin (pos32 = float(p - origin)), plate/cylinder axes as
// unit FP32 vectors (wall32).  Each bound below carries an explicit error term e that
// covers the rounding of those copies (2^-24 relative per coordinate, doubled) and of the
// FP32 arithmetic (a few ulp of the result), so a decision taken from the estimate is the
// one the exact FP64 computation would take: the contact set and the candidate list stay
// identical to the reference's.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace vedo {

// rounding of the FP32 position copies: 2^-23 per unit of |coordinate|
constexpr float PF_POS_EPS = 1.2e-7f;
// relative error allowed for FP32 arithmetic on a length (sqrt, dot, cross: < 8 ulp)
constexpr float PF_ARITH_EPS = 1e-6f;

__device__ __forceinline__ float l1(const float4& a) { return fabsf(a.x) + fabsf(a.y) + fabsf(a.z); }

// Lower/upper-bounded centre distance of two spheres: returns the estimate and its error.
__device__ __forceinline__ float dist32(const float4& a, const float4& b, float& err) {
    const float dx = b.x - a.x, dy = b.y - a.y, dz = b.z - a.z;
    const float l = sqrtf(dx * dx + dy * dy + dz * dz);
    err = PF_POS_EPS * (l1(a) + l1(b)) + PF_ARITH_EPS * l;
    return l;
}

// Lower bound of the distance from a sphere centre a to a plate through b with unit
// normal n (valid when the plate's frame is orthonormal, wall.w != 0): |(a - b) . n|.
__device__ __forceinline__ float plane_dist32(const float4& a, const float4& b, const float4& n, float& err) {
    const float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    const float d = fabsf(dx * n.x + dy * n.y + dz * n.z);
    err = PF_POS_EPS * (l1(a) + l1(b)) + PF_ARITH_EPS * (fabsf(dx) + fabsf(dy) + fabsf(dz));
    return d;
}

// Lower bound of the distance from a sphere centre a to any point of the line through b
// with unit direction u: |(a - b) x u|.
__device__ __forceinline__ float line_dist32(const float4& a, const float4& b, const float4& u, float& err) {
    const float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    const float cx = dy * u.z - dz * u.y, cy = dz * u.x - dx * u.z, cz = dx * u.y - dy * u.x;
    const float d = sqrtf(cx * cx + cy * cy + cz * cz);
    err = PF_POS_EPS * (l1(a) + l1(b)) + PF_ARITH_EPS * (fabsf(dx) + fabsf(dy) + fabsf(dz));
    return d;
}

// Lower-bounded sphere centre distance under a periodic boundary: per axis the least of |d|,
// |d - L|, |d + L| (L = the axis' range, 0 where off), which is at most the minimum-image
// difference the detector takes, whichever image it picks; the shifted differences add the
// rounding of L and of one more subtraction to the error.
__device__ __forceinline__ float dist32_periodic(const float4& a, const float4& b, const float* L, float& err) {
    float d[3] = {b.x - a.x, b.y - a.y, b.z - a.z};
    float ext = 0.0f;
    for (int k = 0; k < 3; ++k) {
        if (L[k] == 0.0f) continue;
        ext += 4.0f * PF_POS_EPS * (fabsf(d[k]) + L[k]);
        d[k] = fminf(fabsf(d[k]), fminf(fabsf(d[k] - L[k]), fabsf(d[k] + L[k])));
    }
    const float l = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    err = PF_POS_EPS * (l1(a) + l1(b)) + ext + PF_ARITH_EPS * l;
    return l;
}

// cd: 1 sphere-sphere, 2 sphere-plate (4, with a hole: tested as the full plate), 3 sphere-cylinder,
// 5 sphere inside a hollow cylinder.  `reach` bounds the distance at which the pair can be in
// contact (radius sum, or radius + plate half-thickness, or sphere + cylinder radius), already
// rounded up; for cd 5 it is stored negated, -(R - r) rounded towards zero: the sphere is clear
// of the shell while its centre is nearer the axis than R - r (so that a pad added to the
// reach narrows that radius).  `periodic`: the FP32 ranges of an active periodic boundary
// (sphere pairs only).  True when the pair is certainly apart.
__device__ __forceinline__ bool certainly_apart(int cd, const float4& s, const float4& m, const float4& wall,
                                                float reach, const float* periodic = nullptr) {
    float e, d;
    if (cd == 1) {
        d = periodic ? dist32_periodic(s, m, periodic, e) : dist32(s, m, e);
    } else if (cd == 2 || cd == 4) {
        if (wall.w == 0.0f) return false;
        d = plane_dist32(s, m, wall, e);
    } else {
        if (wall.w == 0.0f) return false;
        d = line_dist32(s, m, wall, e);
        if (cd == 5) return d + e < -reach * (1.0f - 4.0f * PF_ARITH_EPS);
    }
    return d - e > reach * (1.0f + 4.0f * PF_ARITH_EPS);
}

}  // namespace vedo
