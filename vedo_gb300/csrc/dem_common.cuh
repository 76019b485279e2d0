// dem_common.cuh - device-side data layout and FP64 vector arithmetic of the DEM engine.
//
// The FP64 helpers restate aries::Vector3d (aries/utility/Vector3d.h) operation by
// operation.  Translation units that include them are compiled with -fmad=false, so
// every product and sum is rounded separately, exactly as the reference's host build
// (no -mfma, no -ffast-math, src/Makefile.in:73-77) evaluates them.
#pragma once

#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

namespace vedo {

// ---- enums (DOModel.h:25-27) and engine-internal codes -------------------------------
enum : int { SHAPE_SPHERE = 1, SHAPE_CYL = 6, SHAPE_PLATE = 7, SHAPE_HOLED = 8 };   // 8: QuasiPlateWithCircularHole
// An engine extension with no counterpart in the reference: the inside of a hollow cylinder of
// radius a0 and length a1 about its OrientationZ (a drum shell), global scope, fixed or orbital.
enum : int { SHAPE_INNER_CYL = 32 };
enum : int { BEH_CONSTRAINED = 1, BEH_FIXED = 2, BEH_MOBILE = 3, BEH_ORBITAL = 4 };
enum : int { SCOPE_GLOBAL = 1, SCOPE_LOCAL = 2 };
enum : int { CD_SS = 1, CD_SP = 2, CD_SC = 3, CD_SHP = 4, CD_SIC = 5 };   // CD_SHP: sphere - plate with a circular
                                                                       // hole; CD_SIC: sphere inside a hollow cylinder
// The holed plate is a plate without its hole: distances to it are at least those to the full
// plate, so every conservative plate test (broad phase, prefilter) serves it unchanged.
__host__ __device__ __forceinline__ int cd_plane(int cd) { return cd == CD_SHP ? CD_SP : cd; }
enum : int { IS_BSDBF = 1, IS_BTSDBF = 2, IS_BSDB2F = 3, IS_HERTZ = 4, IS_H = 5 };

// Per-model constants (DOModel::Analysis, DOModel.cpp:17-149, plus the dSudoMass the
// DiscreteObject subclass of each shape/behaviour uses).
struct ModelDev {
    int shape, behavior, scope, group;
    double range;         // DOModel::GetRange
    double mass;          // DOModel::GetMass (energies)
    double sudo;          // DiscreteObject::dSudoMass of this shape/behaviour
    double density;
    double a0, a1, a2;    // shape attributes: sphere r | cylinder r, h | plate w, h, l
    double ix, iy, iz;    // mass moment of inertia
    double ext[3];        // external force
    double inv_sudo;      // 1.0 / sudo, as DOSphere::Response evaluates it (DOSphere.cpp:30)
    double rot_coef;      // 2.5 / sudo / r / r (DOSphere.cpp:39), spheres only
};

// Interaction constants of one (slave model, master model) pair, as the ImpactSolver
// constructors compute them (ISwBSDBF.cpp:7-19 etc.).  cd == 0 means "no interaction".
struct PairParam {
    int cd, is, iact, pad;
    double c[8];
};

// Per-pair status flags (ImpactStatus bContact/bLastContact/bBond/bLastBond).
enum : uint8_t { ST_CONTACT = 1, ST_LAST_CONTACT = 2, ST_BOND = 4, ST_LAST_BOND = 8 };
// Default-constructed ImpactStatus has bLastContact = bLastBond = true (ImpactStatus.cpp:8-9).
constexpr uint8_t ST_DEFAULT = ST_LAST_CONTACT | ST_LAST_BOND;

// Error bits raised by kernels and read by the host after a rebuild.
enum : int { ERR_UNSUPPORTED_PAIR = 1, ERR_CAPACITY = 2, ERR_BAD_SHAPE_PAIR = 4 };

struct d3 { double x, y, z; };

__host__ __device__ __forceinline__ d3 mk(double x, double y, double z) { d3 r; r.x = x; r.y = y; r.z = z; return r; }
__host__ __device__ __forceinline__ d3 add(d3 a, d3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ d3 sub(d3 a, d3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ d3 smul(double s, d3 a) { return mk(s * a.x, s * a.y, s * a.z); }
__host__ __device__ __forceinline__ d3 muls(d3 a, double s) { return mk(a.x * s, a.y * s, a.z * s); }
__host__ __device__ __forceinline__ d3 neg(d3 a) { return mk(-a.x, -a.y, -a.z); }
__host__ __device__ __forceinline__ double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ double len(d3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
// Vector3d::direction (Vector3d.h:117-126).  The reference leaves the result
// uninitialised for a zero vector; every use multiplies it by zero, so (0,0,0) here.
__host__ __device__ __forceinline__ d3 dir(d3 a) {
    double l = len(a);
    if (l != 0) return mk(a.x / l, a.y / l, a.z / l);
    return mk(0.0, 0.0, 0.0);
}
__host__ __device__ __forceinline__ d3 cross(d3 a, d3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__host__ __device__ __forceinline__ d3 project_on(d3 a, d3 v) { return smul(dot(a, v) / len(v), dir(v)); }

// The periodic boundary after Boundary::Correct (Boundary.cpp:79-128): an axis is switched on
// where its bounds differ, `on` is Boundary::Active, range = upper - lower.
struct Periodic {
    int on;
    int sw[3];
    double lo[3], hi[3], range[3];
    float range32[3];    // FP32 copies of the switched ranges for the prefilter, 0 where off
};

// Boundary::DifferenceBoundaryConditions (Boundary.cpp:306-345): the minimum image of a
// difference vector on every switched axis.
__host__ __device__ __forceinline__ double min_image1(double d, double r) {
    if (d >= 0.5 * r) d -= r;
    if (d < -0.5 * r) d += r;
    return d;
}
__host__ __device__ __forceinline__ d3 min_image(const Periodic& b, d3 v) {
    if (b.sw[0]) v.x = min_image1(v.x, b.range[0]);
    if (b.sw[1]) v.y = min_image1(v.y, b.range[1]);
    if (b.sw[2]) v.z = min_image1(v.z, b.range[2]);
    return v;
}

// Boundary::EnforceBoundaryConditions (Boundary.cpp:225-304): a coordinate on a switched axis
// goes back into [lower, upper) by one range, or by fmod (exact in IEEE arithmetic) beyond that.
__host__ __device__ __forceinline__ double wrap1(double p, double lo, double hi, double r) {
    if (p >= hi) {
        p -= r;
        if (p >= hi) p = lo + fmod(p - lo, r);
    }
    if (p < lo) {
        p += r;
        if (p < lo) p = lo + fmod(p - lo, r) + r;
    }
    return p;
}
__host__ __device__ __forceinline__ d3 wrap_position(const Periodic& b, d3 p) {
    if (b.sw[0]) p.x = wrap1(p.x, b.lo[0], b.hi[0], b.range[0]);
    if (b.sw[1]) p.y = wrap1(p.y, b.lo[1], b.hi[1], b.range[1]);
    if (b.sw[2]) p.z = wrap1(p.z, b.lo[2], b.hi[2], b.range[2]);
    return p;
}
#ifdef __CUDACC__
// Vector3d::rotate_around (Vector3d.h:152-178), in two parts: the turn's half-angle terms (its
// axis scaled by sin(a/2), and cos(a/2)), then the rotation of a vector with them, so that an
// object's two orientation vectors share one evaluation of the transcendentals.
struct Turn {
    d3 v;
    double s;
};
__device__ __forceinline__ Turn turn_of(d3 va) {
    d3 u = dir(va);
    double a = len(va);
    // cos(0) = 1 and sin(+0) = +0 exactly: a zero turn (an object not spinning) skips the two FP64
    // transcendental calls, the largest cost of the per-object update on GB300's FP64 pipe
    double s = 1.0, t = 0.0;
    if (a != 0.0) {
        s = cos(0.5 * a);
        t = sin(0.5 * a);
    }
    return Turn{muls(u, t), s};
}
__device__ __forceinline__ d3 rotate_by(d3 p, const Turn& T) {
    const d3 v = T.v;
    const double s = T.s;
    d3 r = add(smul(s * s, p), smul(dot(p, v), v));
    r = add(r, smul(2.0 * s, cross(v, p)));
    return add(r, cross(v, cross(v, p)));
}
__device__ __forceinline__ d3 rotate_around(d3 p, d3 va) { return rotate_by(p, turn_of(va)); }

__device__ __forceinline__ d3 ld(const double4_32a* p, uint32_t i) {
    double4_32a v = p[i];
    return mk(v.x, v.y, v.z);
}
__device__ __forceinline__ void st(double4_32a* p, uint32_t i, d3 a, double w) { p[i] = make_double4_32a(a.x, a.y, a.z, w); }
#endif

}  // namespace vedo
