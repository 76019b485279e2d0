// mixed.cu - mixed-precision DEM engine: one fused tick kernel per time step.
//
// Each sphere thread walks its full neighbour list (both directions) and, for every
// neighbour, evaluates the pair in canonical (slave, master) orientation (the reference's
// Assembler rule, Assembler.cpp:43-67) from inputs both members read identically: the
// previous step's positions (FP64), FP32 velocity copies and the pair's history.  Both
// members therefore obtain bit-identical impulses and Newton's third law holds exactly; the
// history owner (the lower index, or the sphere of a sphere-wall pair) writes the updated
// history into the other buffer.  Impulses are summed per sphere in FP32 with Kahan
// compensation, in the (deterministic) neighbour-list order, and the sphere is integrated
// in FP64 (positions, velocities, angular velocities).
//
// Precision split (per pair): the relative displacement d = x_master - x_slave and the
// overlap numerator R^2 - |d|^2 are double-float (hi/lo FP32 splits of the FP64 positions;
// the overlap of stiff contacts is 1e-9..1e-6 of the radius, beyond FP32's reach); the overlap
// itself, the normal, relative velocities, forces and torques are FP32 in pair-local
// coordinates.  The contact decision (overlap > 0) is the
// FP64 decision: where |R^2 - |d|^2| is within 1e-9 R^2 the reference's own FP64 formula
// (rounded intrinsics, no contraction) decides, so contact sets equal the FP64 engine's.
// Sphere-wall pairs use the reference's FP64 detectors for the geometry.
//
// Broad phase: uniform cell list of edge 2 r_max + skin, stable radix sort on cell key,
// full neighbour lists within r_i + r_j + skin (a conservative FP32 test: a superset), walls
// by a plane/axis lower bound (orbital walls with 8 skins).  The device keeps bounds on the
// spheres' displacement since the rebuild relative to their scene's free-falling frame, on
// their displacement itself and on the orbital walls' approach (list_spent); a step that
// starts with the list possibly incomplete is not taken: the tick and wall kernels copy the
// state unchanged (an identity step) and count it, and the host, which reads the bounds and
// the count every few steps, rebuilds and takes the step again.  Contacts are therefore never
// missed, and the results do not depend on the skin or on when the list is rebuilt.  Spheres
// whose pairs have all been certainly apart since the rebuild skip their walk (quiet spheres).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "dem_common.cuh"
#include "engine_base.h"
#include "observables.cuh"
#include "prefilter.cuh"
#include "scene_host.h"
#include "sort_scan.h"

namespace vedo {
namespace {

constexpr int TPB = 256;
inline unsigned nblk(uint64_t n, int tpb = TPB) { return (unsigned)((n + tpb - 1) / tpb); }

constexpr uint32_t WALL_BIT = 0x80000000u;
// Per-entry facts fixed at rebuild (k_meta), so that the tick reads one word instead of both
// objects' models and the pair's parameters: the pair-parameter index (bits 0-23), the
// contact detector (bits 24-25), "bondable law" (the FP32 prefilter may not skip the pair),
// "history owner" (the entry holds the pair's history) and "this sphere is the slave".
constexpr uint32_t META_PI = 0x00ffffffu;
constexpr int META_CD_SHIFT = 24;            // bits 24-26
constexpr uint32_t META_CD_MASK = 7u;
constexpr uint32_t META_BOND = 1u << 27;
constexpr uint32_t META_OWNER = 1u << 28;
constexpr uint32_t META_SLAVE = 1u << 29;
constexpr uint32_t META_MOVING = 1u << 30;   // the entry's other object is an orbital wall
// A wall entry whose sphere projects inside the plate (or along the rod's or shell's length)
// with a margin that outlasts the list: its distance is the distance to the plane (or axis),
// which only the normal (or transverse) part of the sphere's displacement changes.
constexpr uint32_t META_INTERIOR = 1u << 31;
// Orbital walls move on their own schedule (a drum's end plates turn at a fixed rate), so their
// entries are gathered with a wider skin and carry their own displacement bound; sphere pairs
// and fixed walls keep the sphere bound alone.
constexpr float WALL_SKIN = 8.0f;
constexpr int TICK_GROUP = 4;    // list entries the tick loads and prefilters together
constexpr uint8_t PF_ACTIVE_BIT = 64;
// history flag bit: the status just became clean and the other buffer still holds the old one
constexpr uint8_t HF_PENDING = 16;

// ---- exact FP64 (rounded intrinsics: never contracted into FMA) -----------------------
__device__ __forceinline__ d3 xadd(d3 a, d3 b) { return mk(__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y), __dadd_rn(a.z, b.z)); }
__device__ __forceinline__ d3 xsub(d3 a, d3 b) { return mk(__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y), __dsub_rn(a.z, b.z)); }
__device__ __forceinline__ d3 xsmul(double s, d3 a) { return mk(__dmul_rn(s, a.x), __dmul_rn(s, a.y), __dmul_rn(s, a.z)); }
__device__ __forceinline__ double xdot(d3 a, d3 b) {
    return __dadd_rn(__dadd_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)), __dmul_rn(a.z, b.z));
}
__device__ __forceinline__ double xlen(d3 a) { return __dsqrt_rn(xdot(a, a)); }
__device__ __forceinline__ d3 xdir(d3 a) {
    const double l = xlen(a);
    if (l != 0) return mk(__ddiv_rn(a.x, l), __ddiv_rn(a.y, l), __ddiv_rn(a.z, l));
    return mk(0.0, 0.0, 0.0);
}
__device__ __forceinline__ d3 xcross(d3 a, d3 b) {
    return mk(__dsub_rn(__dmul_rn(a.y, b.z), __dmul_rn(a.z, b.y)), __dsub_rn(__dmul_rn(a.z, b.x), __dmul_rn(a.x, b.z)),
              __dsub_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x)));
}
__device__ __forceinline__ d3 xproject_on(d3 a, d3 v) { return xsmul(__ddiv_rn(xdot(a, v), xlen(v)), xdir(v)); }

// The reference's sphere-plate / sphere-plate-with-hole / sphere-cylinder detectors
// (CDSphere2QuasiPlate.cpp:15-97, CDSphere2QuasiPlateWithCircularHole.cpp:15-133,
// CDSphere2QuasiCylinder.cpp:16-80) in exact FP64: depth, unit normal, impact point.  `hole`:
// hole radius and offsets (the offsets are added to the plate's centre in world coordinates).
__device__ __forceinline__ double wall_detect(int cd, double ra, double b0, double b1, double b2, d3 Ps, d3 Pm, d3 Ox,
                                              d3 Oz, d3& n, d3& point, const double4_32a& hole) {
    double depth;
    if (cd == CD_SHP) {
        const d3 Oy = xcross(Oz, Ox);
        const d3 Cap = xsub(Ps, xproject_on(xsub(Ps, Pm), Oz));
        const double hh = __dmul_rn(0.5, b1), hw = __dmul_rn(0.5, b0), hl = __dmul_rn(0.5, b2);
        const double hr = hole.x, hxo = hole.y, hyo = hole.z;
        const d3 Cha = xsub(Ps, xadd(Pm, mk(hxo, hyo, 0.0)));
        double dx = xdot(xsub(Cap, Pm), Ox);
        if (dx < -hw) dx = -hw; else if (dx > hw) dx = hw;
        double dy = xdot(xsub(Cap, Pm), Oy);
        if (dy < -hl) dy = -hl; else if (dy > hl) dy = hl;
        const double dahx = xdot(Cha, Ox), dahy = xdot(Cha, Oy);
        const double dah = __dsqrt_rn(__dadd_rn(__dmul_rn(dahx, dahx), __dmul_rn(dahy, dahy)));
        if (dah < hr) {
            if (dah == 0.0) {
                dx = hxo;
                dy = hyo;
            } else {
                dx = __dadd_rn(hxo, __dmul_rn(__ddiv_rn(dahx, dah), hr));
                dy = __dadd_rn(hyo, __dmul_rn(__ddiv_rn(dahy, dah), hr));
            }
        }
        const d3 Caps = xadd(xadd(xsmul(dx, Ox), xsmul(dy, Oy)), Pm);
        const d3 vIm = xsub(Caps, Ps);
        const double lv = xlen(vIm);
        depth = dah == 0.0 ? __dsub_rn(__dadd_rn(ra, hh), __dsqrt_rn(__dadd_rn(__dmul_rn(lv, lv), __dmul_rn(hr, hr))))
                           : __dsub_rn(__dadd_rn(ra, hh), lv);
        n = xdir(vIm);
    } else if (cd == CD_SP) {
        const d3 Oy = xcross(Oz, Ox);
        const d3 Cap = xsub(Ps, xproject_on(xsub(Ps, Pm), Oz));
        const double hh = __dmul_rn(0.5, b1), hw = __dmul_rn(0.5, b0), hl = __dmul_rn(0.5, b2);
        double dx = xdot(xsub(Cap, Pm), Ox);
        if (dx < -hw) dx = -hw; else if (dx > hw) dx = hw;
        double dy = xdot(xsub(Cap, Pm), Oy);
        if (dy < -hl) dy = -hl; else if (dy > hl) dy = hl;
        const d3 Caps = xadd(xadd(xsmul(dx, Ox), xsmul(dy, Oy)), Pm);
        const d3 vIm = xsub(Caps, Ps);
        depth = __dsub_rn(__dadd_rn(ra, hh), xlen(vIm));
        n = xdir(vIm);
    } else if (cd == CD_SIC) {
        // engine extension (the reference has no hollow cylinder): the inside of a shell of
        // radius b0 and length b1 about Oz, as the FP64 form's detector computes it
        const double hh = __dmul_rn(0.5, b1);
        const d3 d = xsub(Ps, Pm);
        const double t = xdot(d, Oz);
        const d3 rp = xsub(d, xsmul(t, Oz));
        const d3 u = xdir(rp);
        if (t <= hh && t >= -hh) {
            depth = __dsub_rn(__dadd_rn(ra, xlen(rp)), b0);
            n = u;
        } else {
            const d3 q = xadd(xadd(Pm, xsmul(t > 0.0 ? hh : -hh, Oz)), xsmul(b0, u));
            const d3 vIm = xsub(q, Ps);
            depth = __dsub_rn(ra, xlen(vIm));
            n = xdir(vIm);
        }
    } else {
        const double hh = __dmul_rn(0.5, b1);
        double dap = xdot(xsub(Ps, Pm), Oz);
        if (dap < -hh) dap = -hh; else if (dap > hh) dap = hh;
        const d3 Caps = xadd(Pm, xsmul(dap, Oz));
        const d3 vIm = xsub(Caps, Ps);
        depth = __dsub_rn(__dadd_rn(ra, b0), xlen(vIm));
        n = xdir(vIm);
    }
    point = xadd(Ps, xsmul(__dsub_rn(ra, __dmul_rn(0.5, depth)), n));
    return depth;
}

// ---- FP32 vectors ----------------------------------------------------------------------
struct f3 { float x, y, z; };
__device__ __forceinline__ f3 fm(float x, float y, float z) { f3 r; r.x = x; r.y = y; r.z = z; return r; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return fm(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return fm(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ f3 operator*(float s, f3 a) { return fm(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ f3 operator-(f3 a) { return fm(-a.x, -a.y, -a.z); }
// Every multiply-add below is written out (fmaf) and the file is compiled with -fmad=false, so
// the FP32 sequence is fixed by the source and does not change with the surrounding code (the
// single-law and the multi-law kernels give bit-identical results).
__device__ __forceinline__ float fdot(f3 a, f3 b) { return fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x)); }
__device__ __forceinline__ float flen(f3 a) { return sqrtf(fdot(a, a)); }
__device__ __forceinline__ f3 fdir(f3 a) {
    const float l = flen(a);
    return l != 0.0f ? (1.0f / l) * a : fm(0.0f, 0.0f, 0.0f);
}
__device__ __forceinline__ f3 fcross(f3 a, f3 b) {
    return fm(fmaf(a.y, b.z, -a.z * b.y), fmaf(a.z, b.x, -a.x * b.z), fmaf(a.x, b.y, -a.y * b.x));
}
__device__ __forceinline__ f3 f4to3(float4 v) { return fm(v.x, v.y, v.z); }

// Double-float (hi + lo, ~48 bits) arithmetic from error-free FP32 transforms (Knuth's two-sum,
// the FMA two-product).  Both spheres' positions are split into hi/lo FP32 pairs (split32 below),
// then the relative displacement, |d|^2 and the overlap numerator R^2 - |d|^2 need no FP64 work.
// The splits are either stored once per step (xs arrays) or formed when a pair needs them: the
// same function on the same FP64 positions, so the two ways give identical bits.
struct dfl { float hi, lo; };
__device__ __forceinline__ dfl two_sum(float a, float b) {
    const float s = a + b, bb = s - a;
    return dfl{s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ dfl df_add(dfl a, dfl b) {
    const dfl s = two_sum(a.hi, b.hi);
    return two_sum(s.hi, s.lo + (a.lo + b.lo));
}
// (hm + lm) - (hs + ls)
__device__ __forceinline__ dfl df_diff(float hm, float lm, float hs, float ls) {
    const dfl d = two_sum(hm, -hs);
    return two_sum(d.hi, d.lo + (lm - ls));
}
__device__ __forceinline__ dfl df_sq(dfl a) {
    const float p = a.hi * a.hi;
    return two_sum(p, fmaf(a.hi, a.hi, -p) + 2.0f * a.hi * a.lo);
}
// The nearest periodic image of a double-float difference on an axis of range L (FP32, 0 = off;
// Lhi + Llo = the FP64 range): one range off when the difference reaches half of it, as
// Boundary::DifferenceBoundaryConditions does (pairs that can touch are far from that limit).
__device__ __forceinline__ dfl df_image(dfl d, float L, float Lhi, float Llo) {
    if (L == 0.0f) return d;
    const float v = d.hi + d.lo;
    if (v >= 0.5f * L) return df_add(d, dfl{-Lhi, -Llo});
    if (v < -0.5f * L) return df_add(d, dfl{Lhi, Llo});
    return d;
}

// x = hi + lo with hi = x rounded to FP32 (nearest, ties to even) and lo = (x - hi) rounded to
// FP32, from the bits of x with integer operations (GB300's FP64 pipe is its scarcest): for
// 2^-70 <= |x| < 2^101; zero, tiny and huge values take the FP64 conversions.
// The FP64 conversions of the rare exponents, out of line: GB300 issues FP64 conversions on its
// FP64 pipe (2 lanes per cycle per SM), and a short branch kept inline is predicated rather than
// jumped over, so its FP64 instructions would be issued on every call.
__device__ __noinline__ void split32_wide(double x, float& hi, float& lo) {
    hi = (float)x;
    lo = (float)(x - (double)hi);
}
__device__ __forceinline__ void split32(double x, float& hi, float& lo) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((u >> 52) & 0x7ff) - 1023;           // unbiased exponent
    if (e < -70 || e > 100) {                                  // 2^(e-52) below stays a normal FP32
        split32_wide(x, hi, lo);
        return;
    }
    const unsigned long long mant = u & 0xfffffffffffffull;   // 52 bits
    const unsigned sign = (unsigned)(u >> 63) << 31;
    const unsigned m23 = (unsigned)(mant >> 29);
    const unsigned rem = (unsigned)(mant & 0x1fffffffu);      // 29 bits below FP32's mantissa
    const bool up = rem > 0x10000000u || (rem == 0x10000000u && (m23 & 1u));
    // exponent and mantissa as one integer: a carry out of the mantissa bumps the exponent
    const unsigned body = (((unsigned)(e + 127)) << 23) + m23 + (up ? 1u : 0u);
    hi = __uint_as_float(sign | body);
    // x - hi = (rem or rem - 2^29) units of 2^(e - 52), exactly; its FP32 rounding
    const int r = up ? (int)rem - (int)0x20000000 : (int)rem;
    const float unit = __uint_as_float((unsigned)(e - 52 + 127) << 23);   // 2^(e-52)
    const float lr = __int2float_rn(r) * unit;
    lo = r == 0 ? 0.0f : (sign ? -lr : lr);                     // x - hi = +0 when exact
}

// Exact FP32 <-> FP64 conversions from the bits, with integer operations: the same values as the
// casts (round to nearest, ties to even), without GB300's FP64 pipe, which executes the casts.
// Zero is handled inline; subnormal, huge and non-finite values take the casts out of line.
__device__ __noinline__ double f2d_wide(float f) { return (double)f; }
__device__ __noinline__ float d2f_wide(double x) { return (float)x; }
__device__ __forceinline__ double f2d(float f) {
    const unsigned b = __float_as_uint(f);
    const unsigned ex = (b >> 23) & 0xffu;
    if ((b << 1) == 0u) return __longlong_as_double((long long)((unsigned long long)b << 32));   // +-0
    if (ex == 0u || ex == 0xffu) return f2d_wide(f);
    const unsigned long long u = ((unsigned long long)(b >> 31) << 63) | ((unsigned long long)(ex + 896u) << 52) |
                                 ((unsigned long long)(b & 0x7fffffu) << 29);
    return __longlong_as_double((long long)u);
}
__device__ __forceinline__ float d2f(double x) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    if ((u << 1) == 0ull) return __uint_as_float((unsigned)(u >> 32));                    // +-0
    const int e = (int)((u >> 52) & 0x7ff) - 1023;
    if (e < -126 || e > 126) return d2f_wide(x);
    const unsigned long long mant = u & 0xfffffffffffffull;
    const unsigned m23 = (unsigned)(mant >> 29);
    const unsigned rem = (unsigned)(mant & 0x1fffffffu);
    const bool up = rem > 0x10000000u || (rem == 0x10000000u && (m23 & 1u));
    return __uint_as_float(((unsigned)(u >> 63) << 31) | ((((unsigned)(e + 127)) << 23) + m23 + (up ? 1u : 0u)));
}

// Kahan-compensated FP32 sum of 3-vectors
struct K3 {
    f3 s{0.0f, 0.0f, 0.0f}, c{0.0f, 0.0f, 0.0f};
    __device__ __forceinline__ void add1(float& sum, float& comp, float x) {
        const float y = x - comp;
        const float t = sum + y;
        comp = (t - sum) - y;
        sum = t;
    }
    __device__ __forceinline__ void add(f3 v) {
        add1(s.x, c.x, v.x);
        add1(s.y, c.y, v.y);
        add1(s.z, c.z, v.z);
    }
    __device__ __forceinline__ d3 value() const {
        return mk((double)s.x - (double)c.x, (double)s.y - (double)c.y, (double)s.z - (double)c.z);
    }
};

// The tick's prefilter: certainly_apart (prefilter.cuh) with the positions' rounding bounds
// precomputed in pos32.w and, for spheres and rods, squared distances (no square root): the
// squared test carries the same error allowance as the distance test, so it is as conservative.
// The minimum image of an FP32 difference on an axis of range L (0: no boundary), as a
// magnitude, and the rounding it adds (the range's and one more subtraction's), as
// dist32_periodic (prefilter.cuh) bounds it.
__device__ __forceinline__ float min_image32(float d, float L, float& ext) {
    if (L == 0.0f) return d;
    ext += 4.0f * PF_POS_EPS * (fabsf(d) + L);
    return fminf(fabsf(d), fminf(fabsf(d - L), fabsf(d + L)));
}
__device__ __forceinline__ bool apart32(int cd, const float4& s, const float4& m, const float4& wall, float reach,
                                        const float* L = nullptr) {
    float dx = m.x - s.x, dy = m.y - s.y, dz = m.z - s.z;
    float lim = reach * (1.0f + 4.0f * PF_ARITH_EPS) + s.w + m.w;
    if (cd == CD_SS) {
        if (L) {                                   // a periodic scene: the nearest image
            float ext = 0.0f;
            dx = min_image32(dx, L[0], ext);
            dy = min_image32(dy, L[1], ext);
            dz = min_image32(dz, L[2], ext);
            lim += ext;
        }
        const float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
        return d2 > lim * lim * (1.0f + 4.0f * PF_ARITH_EPS);
    }
    if (wall.w == 0.0f) return false;
    const float lim2 = lim + PF_ARITH_EPS * (fabsf(dx) + fabsf(dy) + fabsf(dz));
    if (cd == CD_SP) return fabsf(fmaf(dz, wall.z, fmaf(dy, wall.y, dx * wall.x))) > lim2;
    const float cx = fmaf(dy, wall.z, -dz * wall.y), cy = fmaf(dz, wall.x, -dx * wall.z),
                cz = fmaf(dx, wall.y, -dy * wall.x);
    const float c2 = fmaf(cz, cz, fmaf(cy, cy, cx * cx));
    if (cd == CD_SIC) {
        // inside a hollow cylinder the reach is -(R - r) (plus the pad): clear while the centre
        // stays nearer the axis than R - r - pad, less every rounding allowance
        const float in = -reach * (1.0f - 4.0f * PF_ARITH_EPS) - s.w - m.w -
                         PF_ARITH_EPS * (fabsf(dx) + fabsf(dy) + fabsf(dz));
        return in > 0.0f && c2 < in * in * (1.0f - 4.0f * PF_ARITH_EPS);
    }
    return c2 > lim2 * lim2 * (1.0f + 4.0f * PF_ARITH_EPS);
}

// ---- the five laws in FP32 (same control flow as the reference's NextStep) -------------
enum : uint8_t { HF_CONTACT = 1, HF_LAST_CONTACT = 2, HF_BOND = 4, HF_LAST_BOND = 8 };

__device__ __forceinline__ f3 shear_rot(f3 F, f3 vs) {                    // ISwModels.cpp:263-273
    return fdot(F, vs) <= 0.0f ? (-flen(F)) * fdir(vs) : flen(F) * fdir(vs);
}

// ISwH's stiffness fixed at first contact from the normal approach speed (ISwH.cpp:79-110):
// coef |vn|^0.4, where coef = (0.957832746294131 / (1 - beta^2), or 479.155951122633 when
// beta >= 0.99) Meff^0.2 knH^0.8 is a constant of the interaction model, computed once in FP64
// on the host (pc32 slot 6).  Out of line: it runs when a contact forms, not on every pass.
__device__ __noinline__ float ish_first_kn(float knH, float coef, float vnl) {
    return vnl == 0.0f ? knH : coef * powf(vnl, 0.4f);
}

// returns 0 (nothing added), 1 (impulse only) or 2 (impulse + torques).  LAW != 0 fixes the
// equation type at compile time (scenes with a single law), LAW == 0 dispatches on `is`.
template <int LAW>
__device__ __forceinline__ int solve32(int is_rt, const float* __restrict__ c, bool active, float depth, f3 n, f3 rA, f3 rB,
                                      f3 va, f3 vb, f3 wa, f3 wb, float dt, uint8_t& f, float4& h, f3& J, f3& tA,
                                      f3& tB) {
    const int is = LAW ? LAW : is_rt;
    const f3 Z = fm(0.0f, 0.0f, 0.0f);
    const bool lsd = is == IS_BSDBF || is == IS_BTSDBF || is == IS_BSDB2F;
    const bool bond = lsd && (depth <= 0.0f) && (c[0] != 0.0f) && (c[4] != 0.0f) && (-depth * c[0] < c[4]);
    if (!active && !bond) {                                                // ImpactStatus::Clean
        f = 0;
        h = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return 0;
    }
    f3 Fn = Z, Fs = Z;
    if (depth > 0.0f) {
        const f3 vRel = (va - vb) + fcross(wa, rA) - fcross(wb, rB);
        const f3 vRn = fdot(vRel, n) * n;
        const f3 vRs = vRel - vRn;
        const f3 sh = fm(h.x, h.y, h.z);
        if (is == IS_BSDBF || is == IS_BSDB2F || is == IS_BTSDBF) {        // ISwBSDBF.cpp:61-112
            const float kn = c[0], ks = c[1], cn = c[2], cs = c[3], bs = c[5], fc = c[6];
            Fn = (-kn * depth) * n - cn * vRn;
            Fs = (is == IS_BTSDBF) ? (-ks * dt) * vRs - cs * vRs : shear_rot(sh, vRs) - (ks * dt) * vRs;
            const float fmax = fc * kn * depth;
            const bool slide = (bs == 0.0f) ? (flen(Fs) > fmax) : (flen(Fs) > bs);
            Fs = slide ? fmax * fdir(Fs) : Fs - cs * vRs;
            if (is != IS_BTSDBF) h = make_float4(Fs.x, Fs.y, Fs.z, h.w);
            f |= HF_CONTACT;
        } else if (is == IS_HERTZ) {                                       // ISwHertz.cpp:53-78
            f |= HF_CONTACT;
            Fn = (-c[0] * depth * sqrtf(depth)) * n - c[1] * vRn;
        } else {                                                           // ISwH.cpp:159-231
            const float knH = c[0], Meff = c[1], ksc1 = c[2], ksc2 = c[3], betan = c[4], fk = c[5];
            float kn;
            if (!(f & HF_CONTACT)) {
                kn = ish_first_kn(knH, c[6], flen(vRn));
                f |= HF_CONTACT;
            } else {
                kn = h.w;
            }
            const float ncd = 2.0f * sqrtf(Meff * kn);
            const float ks = ksc1 * cbrtf(ksc2 * fabsf(kn * depth));
            Fn = (-kn * depth) * n - (ncd * betan) * vRn;
            const float ff = fk * kn * depth;
            Fs = shear_rot(sh, vRs) - (ks * dt) * vRs;
            if (flen(Fs) >= ff) Fs = ff * fdir(Fs);
            h = make_float4(Fs.x, Fs.y, Fs.z, kn);
        }
    } else {                                                               // normal bond at depth <= 0
        const f3 vRel = va - vb;
        const f3 vRn = fdot(vRel, n) * n;
        bool clean = true;
        if (is == IS_BSDB2F && !(f & HF_LAST_BOND)) {
            clean = false;
        } else if (is == IS_BTSDBF) {
            Fn = (-c[0] * depth) * n - c[2] * vRn;
        } else {
            Fn = fdot(vRn, n) < 0.0f ? (-c[0] * depth) * n - c[2] * vRn : (-c[2]) * vRn;
        }
        if (clean) {
            uint8_t nf = 0;
            if (f & HF_CONTACT) nf |= HF_LAST_CONTACT;
            if (f & HF_BOND) nf |= HF_LAST_BOND;
            f = nf;
            h = make_float4(0.0f, 0.0f, 0.0f, h.w);
        }
    }
    if (is == IS_HERTZ) {
        J = dt * Fn;
        return 1;
    }
    const f3 F = Fn + Fs;
    J = dt * F;
    tA = dt * fcross(rA, F);
    tB = (-dt) * fcross(rB, F);
    return 2;
}

// ---- scenes of a batch -----------------------------------------------------------------
// Every scene of a batch keeps its own model/parameter block, cell grid, wall range and time
// step; object indices are the scene's own shifted by its offset, so a scene's results do not
// depend on the other scenes it is batched with.
struct SceneDev {
    uint32_t model_off, nm, pbase, wall_beg, wall_end, obj_off, nobj;
    uint32_t active;               // 0: the scene's job is finished; its objects stay as they are
    uint64_t cell_base;
    uint32_t nc[3];
    float lo[3], inv_h;
    double dt;
    float dtf;                     // dt rounded to FP32 (the pair laws' time step)
    // The scene's drifting frame since the last rebuild: velocity u0 + gdt (k + 1/2) in step k
    // (free fall under the scene's field from the spheres' velocity midrange at the rebuild)
    float u0[3], gdt[3];
    // An active periodic boundary (Boundary.cpp:225-345): the FP64 box for the wrap after each
    // step and the tie band, its ranges in FP32 (0 where an axis is off) for the prefilter and
    // the cell grid, and as double-float pairs for the exact path's minimum image
    Periodic pb;
    float pr_hi[3], pr_lo[3];
};

__device__ __forceinline__ uint32_t pidx(const SceneDev& S, uint32_t mg_slave, uint32_t mg_master) {
    return S.pbase + (mg_slave - S.model_off) * S.nm + (mg_master - S.model_off);
}

// ---- tick ------------------------------------------------------------------------------
struct TickArgs {
    uint32_t n;
    const SceneDev* scenes;
    const uint32_t* scene_of;
    const uint32_t* model_of;
    const ModelDev* models;
    const PairParam* params;
    const float* pc32;             // [nm*nm][8] float constants
    const double4_32a* geom;       // [nm*nm]: ra, b0, b1, b2
    const double4_32a* hole;       // [nm*nm]: hole radius, offsets (sphere - plate with a hole)
    const double4_32a* xA;
    double4_32a* xB;
    double4_32a* v64;
    double4_32a* w64;
    const float4* v32A;
    float4* v32B;
    const float4* w32A;
    float4* w32B;
    const double4_32a* ox;
    const double4_32a* oz;
    const uint32_t* nptr;
    const uint32_t* nent;
    const uint32_t* nslot;
    const uint32_t* nmeta;
    const float4* hA;
    float4* hB;
    const uint8_t* fA;
    uint8_t* fB;
    double4_32a* imp;
    double4_32a* aimp;
    int write_imp;
    int wimp_on;                   // write the wall shares (output steps, and every step of an engine
                                   // with mobile or constrained walls)
    unsigned* vmax_bits;
    const float4* pos32;           // positions at the last rebuild (FP32 offsets)
    // [4]: bounds since the rebuild on any sphere's displacement relative to its scene's frame,
    // on any sphere's displacement, on any orbital wall's displacement; steps since the rebuild
    // (integer bits)
    const float* disp;
    float skin, skin_w;            // list skins: sphere pairs and fixed walls; orbital walls
    const float* reach;
    const float4* wall32;
    float* wimp;                   // [ne][6] impulse and angular impulse on the wall of a wall entry
    const double4_32a* rr;         // [nm*nm] sphere-sphere: R = ra + rb, R^2, tie-band half width 1e-9 R^2
    const float4* rr32;            // [nm*nm] the same for the double-float test: R^2 hi, R^2 lo, band, R
    const float4* xsA;             // [n][2] hi/lo position splits of this step (xs_stored)
    float4* xsB;                   // ... after the step
    int xs_stored;                 // 1: splits stored once per step; 0: formed per pair
    uint32_t* work;                // split tick: spheres deferred to the full tick (else nullptr)
    uint32_t* nwork;               // split tick: spheres in `work`; pair pass: sphere pairs in `pwork`
                                   // (from its start), and nwork[-1] wall pairs (from its end)
    uint4* pwork;                  // pair pass: (owner entry, its sphere, entry word, meta word) of every
                                   // pair on the exact path
    uint8_t* xf;                   // pair pass: [ne] 1 = the entry is on the exact path this step
                                   // (entries after a sphere's first 64)
    unsigned long long* xm;        // pair pass: [n] the same for a sphere's first 64 entries, as a mask
    float4* prec;                  // pair pass: [ne][2] per entry, the pair's share of the entry's
                                   // sphere: (impulse, kind), (torque, 0)
    const uint32_t* pmir;          // pair pass: [ne] at an owner entry of a sphere pair, the
                                   // partner's entry of the same pair
    uint8_t* wk;                   // pair pass: [n] 1 = the sphere is quiet this step
    uint32_t pcap;                 // pair pass: entries `pwork`, `xf` and `prec` hold
    const float4* mf;              // [nm][2]: field + external impulse per step, 1/m~; 2.5/(m~ r^2)
    unsigned* vrel_bits;           // max over spheres of the speed relative to the scene's frame
    const double* ext;             // [2][n][3] external impulse, angular impulse of this step (or nullptr)
    const float2* clear;           // [n] per sphere: every prefilter test of its list says "apart" for
                                   // sphere-pair pads <= x and fixed-wall pads <= y
    uint8_t* qcnt;                 // [n] consecutive clean walks (0..2) since the last rebuild
    const uint32_t* ext_of;        // [n] the caller's index of each object (storage order)
    double4_32a* sox;              // the orientation arrays (ox, oz), turned for spheres by k_turn
    double4_32a* soz;              // when `orient` is set (no kernel of the step reads a sphere's)
    float4* tdav;                  // [n] the step's angular velocity increment, for k_turn
    int orient;
};

// A step whose list may be incomplete is an identity step.  A sphere pair may have closed by
// both spheres' displacements relative to their scene's frame (the frame's own motion moves
// both alike), a sphere and a fixed wall by the sphere's displacement, a sphere and an orbital
// wall by that and the wall's.
__host__ __device__ __forceinline__ bool list_spent(float drel, float dabs, float dw, float skin, float skin_w) {
    return 2.0f * drel > skin || dabs > skin || dabs + dw > skin_w;
}
__device__ __forceinline__ bool held_step(const TickArgs& a) {
    return list_spent(a.disp[0], a.disp[1], a.disp[2], a.skin, a.skin_w);
}

// identity step: the next buffers receive the current state and history unchanged
__device__ __forceinline__ void hold_state(const TickArgs& a, uint32_t i) {
    if (i >= a.n || a.models[a.model_of[i]].scope != SCOPE_LOCAL) return;
    if (a.qcnt[i]) a.qcnt[i] = 0;          // the copy below makes both history buffers alike
    a.xB[i] = a.xA[i];
    if (a.xs_stored) {
        a.xsB[2 * i] = a.xsA[2 * i];
        a.xsB[2 * i + 1] = a.xsA[2 * i + 1];
    }
    a.v32B[i] = a.v32A[i];
    a.w32B[i] = a.w32A[i];
    const uint32_t e1 = a.nptr[i + 1];
    for (uint32_t e = a.nptr[i]; e < e1; ++e)
        if (a.nslot[e] == e) {
            a.hB[e] = a.hA[e];
            a.fB[e] = a.fA[e];
        }
}

// The rare FP64 parts of the exact path, out of line: GB300 issues FP64 arithmetic, compares
// and conversions on its FP64 pipe (2 lanes per cycle per SM), and a short branch kept inline is
// predicated rather than jumped over, so its FP64 instructions would be issued for every pair.
// Sphere pair in the tie band: the reference's formula, (ra + rb) - |x_m - x_s| in FP64.
__device__ __noinline__ double tie_depth(const TickArgs& a, uint32_t pi, uint32_t s, uint32_t m, const Periodic& pb) {
    const double4_32a gg = a.geom[pi];
    d3 d = sub(ld(a.xA, m), ld(a.xA, s));
    if (pb.on) d = min_image(pb, d);              // CDSphere2Sphere.cpp:19-22
    return __dsub_rn(__dadd_rn(gg.x, gg.y), xlen(d));
}
// Sphere-wall pair: the reference's detector in FP64 (wall_detect), the contact normal and
// lever arms rounded to FP32.
__device__ __noinline__ void wall_pair(const TickArgs& a, int cd, uint32_t pi, uint32_t s, uint32_t m, bool& active,
                                       float& depth, f3& n, f3& rA, f3& rB, const Periodic& pb) {
    const double4_32a gg = a.geom[pi];
    const d3 Ps = ld(a.xA, s), Pm = ld(a.xA, m);
    d3 nd, pt;
    const double dex = wall_detect(cd, gg.x, gg.y, gg.z, gg.w, Ps, Pm, ld(a.ox, m), ld(a.oz, m), nd, pt,
                                   cd == CD_SHP ? a.hole[pi] : make_double4_32a(0, 0, 0, 0));
    active = dex > 0.0;
    depth = (float)dex;
    n = fm((float)nd.x, (float)nd.y, (float)nd.z);
    d3 ra = sub(pt, Ps), rb = sub(pt, Pm);
    if (pb.on) {                               // both lever arms take the nearest image (ISwBSDBF.cpp:69-73)
        ra = min_image(pb, ra);
        rb = min_image(pb, rb);
    }
    rA = fm((float)ra.x, (float)ra.y, (float)ra.z);
    rB = fm((float)rb.x, (float)rb.y, (float)rb.z);
}

// The rare writes of an entry that is certainly apart, out of line: the wall's zero share on an
// output step, and the cleaning of an owned history that is set or pending.
__device__ __noinline__ void apart_wall_share(const TickArgs& a, uint32_t e) {
    float* o = a.wimp + 6 * (size_t)e;
    o[0] = o[1] = o[2] = o[3] = o[4] = o[5] = 0.0f;
}
__device__ __noinline__ bool clean_history(const TickArgs& a, uint32_t e, uint8_t f0) {
    a.hB[e] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (f0 & 15) {                             // ImpactStatus::Clean
        a.fB[e] = HF_PENDING;
        return true;
    }
    a.fB[e] = 0;                               // HF_PENDING: both buffers clean again
    return false;
}

// Phase 1 of a sphere's neighbour walk, for the group of entries at `base`: the entries and
// neighbour positions are loaded together (the loads overlap) and the FP32 prefilter settles
// the pairs that are certainly apart (rebuild-time distance minus both spheres' travel since
// then): their history is cleaned and their wall-impulse share zeroed.  Returns the mask of
// entries that need the exact path.  The side effects are idempotent, so a walk that is
// abandoned and redone (the split tick) leaves the same state.
template <bool PBC>
__device__ __forceinline__ uint32_t prefilter_group(const TickArgs& a, uint32_t base, uint32_t e1, const float4& p32i,
                                                    float pad, bool& dirty, uint32_t& owned, uint32_t& walls,
                                                    const float* L) {
    uint32_t ge[TICK_GROUP], gm[TICK_GROUP];
    uint8_t gf[TICK_GROUP];
    float4 gp[TICK_GROUP];
#pragma unroll
    for (int k = 0; k < TICK_GROUP; ++k) {
        const bool ok = base + k < e1;
        ge[k] = ok ? a.nent[base + k] : 0u;
        gm[k] = ok ? a.nmeta[base + k] : 0u;     // cd 0: nothing to do
        gf[k] = ok ? a.fA[base + k] : (uint8_t)0;
    }
#pragma unroll
    for (int k = 0; k < TICK_GROUP; ++k)
        gp[k] = (gm[k] >> META_CD_SHIFT) & META_CD_MASK ? a.pos32[ge[k] & ~WALL_BIT] : p32i;
    uint32_t exact = 0;
#pragma unroll
    for (int k = 0; k < TICK_GROUP; ++k) {
        const uint32_t meta = gm[k];
        const int cd = (int)((meta >> META_CD_SHIFT) & META_CD_MASK);
        if (cd == 0) continue;
        const uint32_t e = base + k;
        const uint32_t j = ge[k] & ~WALL_BIT;
        const bool wall = ge[k] & WALL_BIT;
        const bool i_slave = meta & META_SLAVE;
        if (meta & META_BOND) {
            exact |= 1u << k;
            if (meta & META_OWNER) owned |= 1u << k;
            if (wall) walls |= 1u << k;
            continue;
        }
        const float4 ws = wall ? a.wall32[j] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        // a wall entry: the sphere's whole displacement, or for an interior one (the smaller of the
        // two bounds) the part across the wall: the frame's drift across it (the wall's w,
        // k_walls) plus the deviation from the frame; an orbital wall's approach adds
        float pk = pad;
        if (wall) {
            pk = (meta & META_INTERIOR) ? fminf(a.disp[1], a.disp[0] + ws.w) : a.disp[1];
            if (meta & META_MOVING) pk += a.disp[2];
        }
        if (!apart32(cd, i_slave ? p32i : gp[k], i_slave ? gp[k] : p32i, ws, a.reach[meta & META_PI] + pk,
                     PBC && !wall ? L : nullptr)) {
            exact |= 1u << k;
            if (meta & META_OWNER) owned |= 1u << k;
            if (wall) walls |= 1u << k;
            continue;
        }
        if (wall && a.wimp_on) apart_wall_share(a, e);
        if ((meta & META_OWNER) && (gf[k] & (15 | HF_PENDING))) dirty |= clean_history(a, e, gf[k]);
    }
    return exact;
}

// The group's prefilter with the periodic image only where the scene has a periodic boundary
// (a separate instance: the common path carries none of it).
__device__ __forceinline__ uint32_t prefilter_any(const TickArgs& a, uint32_t base, uint32_t e1, const float4& p32i,
                                                  float pad, bool& dirty, uint32_t& owned, uint32_t& walls,
                                                  const float* L) {
    return L ? prefilter_group<true>(a, base, e1, p32i, pad, dirty, owned, walls, L)
             : prefilter_group<false>(a, base, e1, p32i, pad, dirty, owned, walls, nullptr);
}

// Quiet spheres.  Between rebuilds a sphere's list, the rebuild-time positions and the fixed
// walls' normals do not change, and the prefilter's "apart" is monotone in the pad, so two
// numbers per sphere (`clear`, k_clear: sphere pairs, fixed walls) settle the whole walk: with
// the pads at or below them every entry is apart.  Such a walk writes history only to clean it: an owned entry whose status is set is
// cleaned to HF_PENDING, and a HF_PENDING one clears the other buffer.  After two consecutive
// walks that cleaned nothing (`qcnt` = 2) both buffers of every owned entry hold a clean status
// that a further walk rewrites with the same values, so the walk is skipped and the sphere is
// finished with its field impulse alone: the state is the walk's, bit for bit.  A walk that
// cleans a status or needs the exact path resets the count; so do rebuilds and identity steps.
__device__ __forceinline__ void note_walk(const TickArgs& a, uint32_t i, uint32_t qc, bool reset) {
    const uint32_t q2 = reset ? 0u : (qc < 2u ? qc + 1u : 2u);
    if (q2 != qc) a.qcnt[i] = (uint8_t)q2;
}

// The end of a sphere's step: field and external impulse join the compensated sum (the
// increments dv, dw are FP32, the state update FP64), the impulses are recorded on the last
// step of a call, and the sphere is integrated.  Returns the squared speed bounds of the step
// (the square roots are taken once per warp):
//  x: the step moves the sphere by dt (V + dv/2), at most max(|V|, |V + dv|), formed in FP32
//     from the new velocity and the increment, |V| as |vn - dv| (the margin covers roundings);
//  y: the frame's velocity in this step is u = u0 + gdt (k + 1/2), and the sphere's step
//     velocity vmid = vn - dv/2 is compared with it in FP32 with an allowance s for the
//     roundings: 2 |vmid - u|^2 + 2 s^2 >= (|vmid - u| + s)^2.
// A quiet sphere had no torque in its last two steps, so both buffers of its FP32 angular
// velocity already hold the value the copy would write.
template <bool XS>
__device__ __forceinline__ float2 finish_sphere(const TickArgs& a, uint32_t i, bool mobile, bool quiet,
                                                const SceneDev& S, const d3& Pi, const d3& V, const float4& mf0,
                                                const float4& mf1, K3& J, K3& JA) {
    const double dt = S.dt;
    // DOContainer.cpp:20-27, DiscreteObject.cpp:160-163
    J.add(fm(mf0.x, mf0.y, mf0.z));
    if (a.ext) {                   // SimMediator::Run(external impacts): DOContainer::AddImpact (SimMediator.cpp:1015-1018)
        const double* e = a.ext + 3 * (size_t)i;
        const double* ea = a.ext + 3 * ((size_t)a.n + i);
        J.add(fm((float)e[0], (float)e[1], (float)e[2]));
        JA.add(fm((float)ea[0], (float)ea[1], (float)ea[2]));
    }
    if (a.write_imp) {
        st(a.imp, i, J.value(), 0.0);
        st(a.aimp, i, JA.value(), 0.0);
    }
    if (mobile) {
        const f3 Jf = fm(J.s.x - J.c.x, J.s.y - J.c.y, J.s.z - J.c.z);
        const f3 JAf = fm(JA.s.x - JA.c.x, JA.s.y - JA.c.y, JA.s.z - JA.c.z);
        const f3 dv = mf0.w * Jf, dw = mf1.x * JAf;
        const d3 dvd = mk(f2d(dv.x), f2d(dv.y), f2d(dv.z));
        const d3 P2 = mk(fma(dt, fma(0.5, dvd.x, V.x), Pi.x), fma(dt, fma(0.5, dvd.y, V.y), Pi.y),
                         fma(dt, fma(0.5, dvd.z, V.z), Pi.z));
        const d3 V2 = add(V, dvd);
        st(a.xB, i, P2, 0.0);
        st(a.v64, i, V2, 0.0);
        if (XS) {
            float4 h2, l2;
            split32(P2.x, h2.x, l2.x);
            split32(P2.y, h2.y, l2.y);
            split32(P2.z, h2.z, l2.z);
            h2.w = l2.w = 0.0f;
            a.xsB[2 * i] = h2;
            a.xsB[2 * i + 1] = l2;
        }
        if (a.orient) a.tdav[i] = make_float4(dw.x, dw.y, dw.z, 0.0f);   // for k_turn
        if (dw.x != 0.0f || dw.y != 0.0f || dw.z != 0.0f) {
            const d3 W2 = add(ld(a.w64, i), mk(f2d(dw.x), f2d(dw.y), f2d(dw.z)));
            st(a.w64, i, W2, 0.0);
            a.w32B[i] = make_float4(d2f(W2.x), d2f(W2.y), d2f(W2.z), 0.0f);
        } else if (!quiet) {                       // no torque: omega + 0 is omega
            a.w32B[i] = a.w32A[i];
        }
        const float4 vn = make_float4(d2f(V2.x), d2f(V2.y), d2f(V2.z), 0.0f);
        a.v32B[i] = vn;
        const float ox = vn.x - dv.x, oy = vn.y - dv.y, oz = vn.z - dv.z;
        const float vabs2 = fmaxf(fmaf(oz, oz, fmaf(oy, oy, ox * ox)), fmaf(vn.z, vn.z, fmaf(vn.y, vn.y, vn.x * vn.x)));
        const float kh = (float)__float_as_uint(a.disp[3]) + 0.5f;
        const float ux = fmaf(S.gdt[0], kh, S.u0[0]), uy = fmaf(S.gdt[1], kh, S.u0[1]), uz = fmaf(S.gdt[2], kh, S.u0[2]);
        const float rx = fmaf(-0.5f, dv.x, vn.x) - ux, ry = fmaf(-0.5f, dv.y, vn.y) - uy,
                    rz = fmaf(-0.5f, dv.z, vn.z) - uz;
        const float sl = 1e-6f * (fabsf(vn.x) + fabsf(vn.y) + fabsf(vn.z) + fabsf(dv.x) + fabsf(dv.y) + fabsf(dv.z) +
                                  fabsf(ux) + fabsf(uy) + fabsf(uz));
        return make_float2(vabs2, 2.0f * fmaf(rz, rz, fmaf(ry, ry, fmaf(rx, rx, sl * sl))));
    }
    st(a.xB, i, Pi, 0.0);
    if (XS) {
        a.xsB[2 * i] = a.xsA[2 * i];
        a.xsB[2 * i + 1] = a.xsA[2 * i + 1];
    }
    a.v32B[i] = a.v32A[i];
    a.w32B[i] = a.w32A[i];
    return make_float2(0.0f, 0.0f);
}

// The exact path of one list entry e of sphere i (entry `meta`): the pair in canonical (slave,
// master) orientation from the previous positions, FP32 velocity copies and the pair's history,
// so both members of a sphere pair obtain the same bits; the history owner writes the new status
// into the other buffer, a wall entry writes the wall's share of the impulse.  Returns 0 (nothing
// added), 1 (impulse J only) or 2 (J and the torques tA on the slave, tB on the master).
// KIND: 0 any entry; 1 a sphere pair, 2 a wall pair (the other branch is not compiled: a kernel
// without the out-of-line wall detector's call keeps its locals in registers).
template <int LAW, bool XS, int KIND = 0>
__device__ __forceinline__ int exact_pair(const TickArgs& a, const SceneDev& S, uint32_t i, const d3& Pi, uint32_t e,
                                          uint32_t ent, uint32_t meta, f3& Jp, f3& tA, f3& tB) {
    const float dtf = S.dtf;
    const uint32_t j = ent & ~WALL_BIT;
    const bool wall = ent & WALL_BIT;
    // canonical orientation (Assembler.cpp:43-67), fixed at rebuild; sphere-wall: the sphere is the slave
    const bool i_slave = meta & META_SLAVE;
    const bool owner = meta & META_OWNER;
    const uint32_t s = i_slave ? i : j, m = i_slave ? j : i;
    const uint32_t pi = meta & META_PI;
    const uint32_t slot = owner ? e : a.nslot[e];
    const PairParam& P = a.params[pi];
    bool active;
    float depth;
    f3 n, rA, rB;
    if (KIND == 1 || (KIND == 0 && P.cd == CD_SS)) {
        // d = x_master - x_slave, |d|^2 and R^2 - |d|^2 in double-float from the two
        // positions' hi/lo splits; where the numerator is within 1e-9 R^2 of zero the
        // reference's FP64 formula decides
        float4 hi_i, lo_i, hj, lj;
        if (XS) {
            hj = a.xsA[2 * j];
            lj = a.xsA[2 * j + 1];
            hi_i = a.xsA[2 * i];
            lo_i = a.xsA[2 * i + 1];
        } else {
            const d3 Pj = ld(a.xA, j);
            split32(Pj.x, hj.x, lj.x);
            split32(Pj.y, hj.y, lj.y);
            split32(Pj.z, hj.z, lj.z);
            split32(Pi.x, hi_i.x, lo_i.x);
            split32(Pi.y, hi_i.y, lo_i.y);
            split32(Pi.z, hi_i.z, lo_i.z);
        }
        const float4 hs = i_slave ? hi_i : hj, ls = i_slave ? lo_i : lj;
        const float4 hm = i_slave ? hj : hi_i, lm = i_slave ? lj : lo_i;
        dfl dx = df_diff(hm.x, lm.x, hs.x, ls.x), dy = df_diff(hm.y, lm.y, hs.y, ls.y),
            dz = df_diff(hm.z, lm.z, hs.z, ls.z);
        if (S.pb.on) {                             // a periodic scene: the nearest image
            dx = df_image(dx, S.pb.range32[0], S.pr_hi[0], S.pr_lo[0]);
            dy = df_image(dy, S.pb.range32[1], S.pr_hi[1], S.pr_lo[1]);
            dz = df_image(dz, S.pb.range32[2], S.pr_hi[2], S.pr_lo[2]);
        }
        const dfl s2 = df_add(df_add(df_sq(dx), df_sq(dy)), df_sq(dz));
        const float4 rq = a.rr32[pi];                // R^2 hi, R^2 lo, band, R
        const dfl num = df_add(dfl{rq.x, rq.y}, dfl{-s2.hi, -s2.lo});
        if (num.hi < -rq.z || num.hi > rq.z) {
            active = num.hi > 0.0f;
            depth = (num.hi + num.lo) / (rq.w + sqrtf(s2.hi));
        } else {                               // tie band: the reference's formula decides
            const double dex = tie_depth(a, pi, s, m, S.pb);
            active = dex > 0.0;
            depth = (float)dex;
        }
        const f3 df = fm(dx.hi + dx.lo, dy.hi + dy.lo, dz.hi + dz.lo);
        n = fdir(df);
        rA = (a.pc32[8 * (size_t)pi + 7] - 0.5f * depth) * n;   // slot 7: the slave's radius
        rB = rA - df;
    } else if (KIND != 1) {
        wall_pair(a, P.cd, pi, s, m, active, depth, n, rA, rB, S.pb);
    }
    const uint8_t f0 = a.fA[slot];
    uint8_t f = f0 & 15;
    float4 h = (f != 0 || active) ? a.hA[slot] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    Jp = fm(0.0f, 0.0f, 0.0f);
    tA = Jp;
    tB = Jp;
    const int app = solve32<LAW>(P.is, a.pc32 + 8 * (size_t)pi, active, depth, n, rA, rB, f4to3(a.v32A[s]),
                                 f4to3(a.v32A[m]), f4to3(a.w32A[s]), f4to3(a.w32A[m]), dtf, f, h, Jp, tA, tB);
    if (e == slot) {                           // history owner writes the new status
        if (f != 0 || (f0 & 15) != 0) {
            a.hB[slot] = h;
            a.fB[slot] = (uint8_t)(f | ((f == 0) ? HF_PENDING : 0));
        } else if (f0 & HF_PENDING) {
            a.hB[slot] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            a.fB[slot] = 0;
        }
    }
    if (wall && a.wimp_on) {                   // the wall's share, summed per wall later
        float* o = a.wimp + 6 * (size_t)e;
        o[0] = app ? -Jp.x : 0.0f; o[1] = app ? -Jp.y : 0.0f; o[2] = app ? -Jp.z : 0.0f;
        o[3] = app == 2 ? tB.x : 0.0f; o[4] = app == 2 ? tB.y : 0.0f; o[5] = app == 2 ? tB.z : 0.0f;
    }
    return app;
}

// One sphere's step: neighbour walk (prefilter, then the exact path in entry order), sums,
// integration.  Returns its squared speed bounds of the step.
template <int LAW, bool XS>
__device__ __forceinline__ float2 tick_sphere(const TickArgs& a, uint32_t i) {
    float2 vmax_local = make_float2(0.0f, 0.0f);
    {
        // every load that depends on the index alone is issued here, together, so that their
        // latencies overlap; the model- and list-dependent ones follow
        const uint32_t mi = a.model_of[i];
        const uint32_t si = a.scene_of[i];
        const uint32_t e0 = a.nptr[i], e1 = a.nptr[i + 1];
        const d3 Pi = ld(a.xA, i);
        const d3 V = ld(a.v64, i);
        const float4 p32i = a.pos32[i];
        const float disp = a.disp[0];
        const ModelDev& M = a.models[mi];
        const SceneDev& S = a.scenes[si];
        if (M.scope == SCOPE_LOCAL && S.active) {
            const float pad = 2.0f * disp;
            const float4 mf0 = a.mf[2 * mi], mf1 = a.mf[2 * mi + 1];
            const bool mobile = M.behavior == BEH_MOBILE;
            // the clean-walk count is kept by the light tick when there is one
            const uint32_t qc = a.work ? 0u : a.qcnt[i];
            const float2 cl = a.clear[i];
            const bool quiet = qc >= 2u && !a.write_imp && pad <= cl.x && a.disp[1] <= cl.y;
            bool dirty = false, any_exact = false;
            K3 J, JA;
            // The list is walked in chunks of 64 entries (one chunk for nearly every sphere):
            // phase 1 prefilters the whole chunk into a mask, phase 2 runs the exact path over
            // it.  A warp then iterates phase 2 as often as its busiest sphere has exact entries
            // in the chunk, not as often as the busiest sphere of each group of entries has.
            for (uint32_t c0 = e0; c0 < e1 && !quiet; c0 += 64) {
                const uint32_t c1 = min(e1, c0 + 64);
                unsigned long long exact = 0ull;
                uint32_t owned = 0u, walls = 0u;       // (unused here)
                for (uint32_t base = c0; base < c1; base += TICK_GROUP)
                    exact |= (unsigned long long)prefilter_any(a, base, c1, p32i, pad, dirty, owned, walls,
                                                               S.pb.on ? S.pb.range32 : nullptr)
                             << (base - c0);
                any_exact |= exact != 0ull;
                // Phase 2: the exact path for the flagged entries, in entry order
                while (exact) {
                    const int k = __ffsll(exact) - 1;
                    exact &= exact - 1;
                    const uint32_t e = c0 + k;
                    const uint32_t meta = a.nmeta[e];
                    f3 Jp, tA, tB;
                    const int app = exact_pair<LAW, XS>(a, S, i, Pi, e, a.nent[e], meta, Jp, tA, tB);
                    if (app) {
                        if (meta & META_SLAVE) {
                            J.add(Jp);
                            if (app == 2) JA.add(tA);
                        } else {
                            J.add(-Jp);
                            if (app == 2) JA.add(tB);
                        }
                    }
                }
            }
            if (!a.work && !quiet) note_walk(a, i, qc, dirty || any_exact);
            vmax_local = finish_sphere<XS>(a, i, mobile, quiet, S, Pi, V, mf0, mf1, J, JA);
        } else if (M.scope == SCOPE_LOCAL) {
            hold_state(a, i);                      // a finished scene waits, unchanged
        }
    }
    return vmax_local;
}

// the warp's squared speed bounds (absolute, relative to the frame): their square roots, with
// a margin for the roundings, join the step's maxima
__device__ __forceinline__ void reduce_vmax(const TickArgs& a, float2 v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v.x = fmaxf(v.x, __shfl_xor_sync(0xffffffffu, v.x, o));
        v.y = fmaxf(v.y, __shfl_xor_sync(0xffffffffu, v.y, o));
    }
    if ((threadIdx.x & 31) == 0) {
        // the maxima only grow within a step, so a value at or below one already read (from L2)
        // needs no atomic: most warps skip it
        const unsigned bx = __float_as_uint(sqrtf(v.x) * 1.0001f), by = __float_as_uint(sqrtf(v.y) * 1.0001f);
        if (v.x > 0.0f && bx > __ldcg(a.vmax_bits)) atomicMax(a.vmax_bits, bx);
        if (v.y > 0.0f && by > __ldcg(a.vrel_bits)) atomicMax(a.vrel_bits, by);
    }
}
__device__ __forceinline__ float2 fmax2(float2 a, float2 b) { return make_float2(fmaxf(a.x, b.x), fmaxf(a.y, b.y)); }

// Programmatic dependent launch (sm_90 and later): the per-step kernels are launched so that the
// next one may be scheduled while this one drains.  Each first waits until the grid before it
// has finished and its writes are visible (a no-op for a plain launch), then lets the next grid
// launch; that one is released only once every block of this grid has started, so its waiting
// blocks never hold resources this grid still needs.
__device__ __forceinline__ void step_order() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// The full tick, one thread per sphere.
template <int LAW, bool XS>
__global__ void __launch_bounds__(TPB) k_tick(TickArgs a) {
    step_order();
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    float2 vmax_local = make_float2(0.0f, 0.0f);
    if (held_step(a)) {                          // the same value for every thread of the launch
        hold_state(a, t);
    } else if (t < a.n) {
        vmax_local = tick_sphere<LAW, XS>(a, t);
    }
    reduce_vmax(a, vmax_local);
}

// The full tick of the split tick: a grid sized to the resident threads strides over the
// spheres the light kernel deferred (none in a held step).
template <int LAW, bool XS>
__global__ void __launch_bounds__(TPB) k_tick_work(TickArgs a) {
    step_order();
    float2 vmax_local = make_float2(0.0f, 0.0f);
    if (!held_step(a)) {
        const uint32_t nw = *a.nwork;
        for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nw; q += gridDim.x * blockDim.x)
            vmax_local = fmax2(vmax_local, tick_sphere<LAW, XS>(a, a.work[q]));
    }
    reduce_vmax(a, vmax_local);
}

// The light half of the split tick: every sphere's neighbour walk in FP32 prefilter form only,
// at a register count that keeps the SM full.  A sphere whose pairs are all certainly apart is
// finished here (its sums hold the field impulse alone); a sphere with any pair that needs the
// exact path is deferred, whole, to k_tick over the worklist.  Either way one thread computes
// the sphere with the same operations, so results are those of the single tick.
template <bool XS>
__global__ void __launch_bounds__(TPB, 6) k_tick_light(TickArgs a) {   // 6 blocks of 256 per SM (40 registers; the rare walk spills a little)
    step_order();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool hold = held_step(a);
    float2 vmax_local = make_float2(0.0f, 0.0f);
    bool defer = false;
    if (hold) {
        hold_state(a, i);
    } else if (i < a.n) {
        // the state is read after the quiet test (or the walk): start bringing it to L2 now
        asm volatile("prefetch.global.L2 [%0];" ::"l"(a.xA + i));
        asm volatile("prefetch.global.L2 [%0];" ::"l"(a.v64 + i));
        const uint32_t mi = a.model_of[i];
        const uint32_t si = a.scene_of[i];
        const uint32_t qc = a.qcnt[i];
        const float2 clear = a.clear[i];
        const float disp = a.disp[0];
        const ModelDev& M = a.models[mi];
        const SceneDev& S = a.scenes[si];
        if (M.scope == SCOPE_LOCAL && S.active) {
            const float pad = 2.0f * disp;
            const bool quiet = qc >= 2u && !a.write_imp && pad <= clear.x && a.disp[1] <= clear.y;
            if (!quiet) {                          // walk the list
                const uint32_t e0 = a.nptr[i], e1 = a.nptr[i + 1];
                const float4 p32i = a.pos32[i];
                bool dirty = false;
                uint32_t owned = 0u, walls = 0u;       // (unused here)
                // a periodic scene's spheres go to the full tick, whose prefilter takes the images
                defer = S.pb.on != 0;
                for (uint32_t base = e0; base < e1 && !defer; base += TICK_GROUP)
                    defer = prefilter_group<false>(a, base, e1, p32i, pad, dirty, owned, walls, nullptr) != 0u;
                note_walk(a, i, a.qcnt[i], dirty || defer);    // (reread: fewer live registers in the walk)
            }
            if (!defer) {                          // state loaded after the walk: fewer live registers
                const d3 Pi = ld(a.xA, i);
                const d3 V = ld(a.v64, i);
                const uint32_t mj = a.model_of[i];     // (reread: fewer live registers in the walk)
                const float4 mf0 = a.mf[2 * mj], mf1 = a.mf[2 * mj + 1];
                K3 J, JA;
                vmax_local = finish_sphere<XS>(a, i, a.models[mj].behavior == BEH_MOBILE, quiet,
                                               a.scenes[a.scene_of[i]], Pi, V, mf0, mf1, J, JA);
            }
        } else if (M.scope == SCOPE_LOCAL) {
            hold_state(a, i);
        }
    }
    const unsigned dm = __ballot_sync(0xffffffffu, defer);
    if (dm) {                                      // warp-aggregated append to the worklist
        const int lane = threadIdx.x & 31, lead = __ffs(dm) - 1;
        uint32_t at = 0;
        if (lane == lead) at = atomicAdd(a.nwork, (uint32_t)__popc(dm));
        at = __shfl_sync(0xffffffffu, at, lead);
        if (defer) a.work[at + __popc(dm & ((1u << lane) - 1u))] = i;
    }
    reduce_vmax(a, vmax_local);
}

// DOSphere::Response (DOSphere.cpp:40-44): the orientation turns by dw = dt (w + dav/2) with the
// angular velocity w before the step and its increment dav, by Vector3d::rotate_around in FP64 for
// both axes; a zero turn leaves them.  Run after the tick when the caller asks for orientations,
// from the new angular velocity w + dav and the increment: dt (w + dav - dav/2).
__device__ __forceinline__ void turn_sphere(const TickArgs& a, uint32_t i) {
    if (i >= a.n) return;
    const ModelDev& M = a.models[a.model_of[i]];
    const SceneDev& S = a.scenes[a.scene_of[i]];
    if (M.scope != SCOPE_LOCAL || !S.active || M.behavior != BEH_MOBILE) return;
    const float4 dav = a.tdav[i];
    const d3 W2 = ld(a.w64, i);
    const d3 dwv = smul(S.dt, sub(W2, smul(0.5, mk(f2d(dav.x), f2d(dav.y), f2d(dav.z)))));
    if (dwv.x == 0.0 && dwv.y == 0.0 && dwv.z == 0.0) return;
    const Turn T = turn_of(dwv);
    st(a.sox, i, rotate_by(ld(a.sox, i), T), 0.0);
    st(a.soz, i, rotate_by(ld(a.soz, i), T), 0.0);
}
__global__ void __launch_bounds__(TPB) k_turn(TickArgs a) {
    step_order();
    if (!held_step(a)) turn_sphere(a, blockIdx.x * blockDim.x + threadIdx.x);
}

// SimMediator.cpp:746: after the response every object of a periodic scene goes back into the
// periodic box (Boundary::EnforceBoundaryConditions, wrap_position); run after the tick, only
// when a scene is periodic, so that the tick itself carries no FP64 wrap.  A wrapped sphere's
// position splits are formed anew.
__device__ __forceinline__ void wrap_sphere(const TickArgs& a, uint32_t i) {
    if (i >= a.n) return;
    const SceneDev& S = a.scenes[a.scene_of[i]];
    if (!S.pb.on || !S.active || a.models[a.model_of[i]].scope != SCOPE_LOCAL) return;
    const d3 P = ld(a.xB, i);
    const d3 W = wrap_position(S.pb, P);
    if (W.x == P.x && W.y == P.y && W.z == P.z) return;
    st(a.xB, i, W, 0.0);
    if (a.xs_stored) {
        float4 h2, l2;
        split32(W.x, h2.x, l2.x);
        split32(W.y, h2.y, l2.y);
        split32(W.z, h2.z, l2.z);
        h2.w = l2.w = 0.0f;
        a.xsB[2 * i] = h2;
        a.xsB[2 * i + 1] = l2;
    }
}
__global__ void __launch_bounds__(TPB) k_wrap(TickArgs a) {
    step_order();
    if (!held_step(a)) wrap_sphere(a, blockIdx.x * blockDim.x + threadIdx.x);
}

// ---- pair pass ------------------------------------------------------------------------------
// The tick in three stages, each pair on the exact path evaluated once:
//  k_tick_pf     every sphere's list walk in prefilter form (with the single tick's history
//                cleaning and clean-walk count), marking the entries on the exact path and
//                appending each such pair once, at its history owner, to a worklist;
//  k_tick_pairs  one thread per pair of the worklist, the wall pairs and the sphere pairs in two
//                kernels that run side by side: the exact path (exact_pair, the single tick's
//                arithmetic) writes each member's share of the impulse and torque at that
//                member's own entry of the pair;
//  k_tick_sum    one thread per sphere: the shares at its marked entries, in entry order, join
//                the compensated sums, then the sphere is integrated (finish_sphere).
// Both members of a pair add the one evaluation that the single tick computes twice with
// identical bits, in the same order, so results are the single tick's.  The pair kernel runs
// with every lane on a pair, where the single tick's lanes wait for the sphere of their warp with
// the most pairs.
// One sphere's prefilter walk (i >= n: a lane without a sphere); every lane of the warp calls it.
__device__ __forceinline__ void pf_sphere(const TickArgs& a, uint32_t i) {
    const int lane = threadIdx.x & 31;
    uint32_t c0 = 0u, e0 = 0u, e1 = 0u, qc = 0u;
    float4 p32i = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float pad = 0.0f;
    const float* L = nullptr;
    bool walk = false, dirty = false, any_exact = false;
    if (i < a.n) {
        const ModelDev& M = a.models[a.model_of[i]];
        const SceneDev& S = a.scenes[a.scene_of[i]];
        if (S.pb.on) L = S.pb.range32;
        if (M.scope == SCOPE_LOCAL && S.active) {
            qc = a.qcnt[i];
            const float2 cl = a.clear[i];
            pad = 2.0f * a.disp[0];
            const bool quiet = qc >= 2u && !a.write_imp && pad <= cl.x && a.disp[1] <= cl.y;
            a.wk[i] = quiet ? 1u : 0u;
            if (!quiet) {
                e0 = a.nptr[i];
                e1 = a.nptr[i + 1];
                c0 = e0;
                p32i = a.pos32[i];
                walk = true;
                if (e0 == e1) a.xm[i] = 0ull;      // an empty list: no chunk writes the mask
            }
        }
    }
    // the warp walks its spheres' lists 64 entries at a time, in step, so that every chunk's
    // pairs are appended with one atomic per warp
    bool more = walk && c0 < e1;
    while (__any_sync(0xffffffffu, more)) {
        unsigned long long own = 0ull, wown = 0ull;
        if (more) {
            const uint32_t c1 = min(e1, c0 + 64);
            unsigned long long exact = 0ull;
            for (uint32_t base = c0; base < c1; base += TICK_GROUP) {
                uint32_t owned = 0u, walls = 0u;
                exact |= (unsigned long long)prefilter_any(a, base, c1, p32i, pad, dirty, owned, walls, L)
                         << (base - c0);
                own |= (unsigned long long)(owned & ~walls) << (base - c0);
                wown |= (unsigned long long)(owned & walls) << (base - c0);
            }
            any_exact |= exact != 0ull;
            if (c0 == e0) {
                a.xm[i] = exact;
            } else {
                for (uint32_t e = c0; e < c1; ++e) a.xf[e] = (uint8_t)((exact >> (e - c0)) & 1ull);
            }
        }
        // sphere pairs fill the worklist from its start, wall pairs from its end, so that each
        // kind has a pair kernel of its own, in full warps (a wall pair's detector is FP64 work,
        // and a warp issues it once for every lane that needs it)
        const uint32_t cnt = (uint32_t)__popcll(own), wcnt = (uint32_t)__popcll(wown);
        uint32_t incl = cnt, wincl = wcnt;         // inclusive prefixes over the warp
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
            const uint32_t w = __shfl_up_sync(0xffffffffu, wincl, o);
            if (lane >= o) {
                incl += v;
                wincl += w;
            }
        }
        uint32_t at = 0u, wat = 0u;
        if (lane == 31 && incl) at = atomicAdd(a.nwork, incl);
        if (lane == 31 && wincl) wat = atomicAdd(a.nwork - 1, wincl);
        at = __shfl_sync(0xffffffffu, at, 31) + incl - cnt;
        wat = __shfl_sync(0xffffffffu, wat, 31) + wincl - wcnt;
        while (own) {
            const int k = __ffsll(own) - 1;
            own &= own - 1;
            const uint32_t e = c0 + (uint32_t)k;   // (its words are in L1 from the prefilter)
            if (at < a.pcap) a.pwork[at] = make_uint4(e, i, a.nent[e], a.nmeta[e]);   // (at most one per entry)
            ++at;
        }
        while (wown) {
            const int k = __ffsll(wown) - 1;
            wown &= wown - 1;
            const uint32_t e = c0 + (uint32_t)k;
            if (wat < a.pcap) a.pwork[a.pcap - 1u - wat] = make_uint4(e, i, a.nent[e], a.nmeta[e]);
            ++wat;
        }
        if (more) {
            c0 += 64;
            more = c0 < e1;
        }
    }
    if (walk) note_walk(a, i, qc, dirty || any_exact);
}
__global__ void __launch_bounds__(TPB, 4) k_tick_pf(TickArgs a) {
    step_order();
    if (held_step(a)) return;                      // k_tick_sum holds the state (uniform branch)
    pf_sphere(a, blockIdx.x * blockDim.x + threadIdx.x);
}

// One pair of the worklist: the exact path and both members' shares.
template <int LAW, bool XS, int KIND>
__device__ __forceinline__ void pair_item(const TickArgs& a, const uint4& it) {
    const uint32_t e = it.x, i = it.y, ent = it.z, meta = it.w;
    const d3 Pi = XS ? mk(0.0, 0.0, 0.0) : ld(a.xA, i);
    f3 Jp, tA, tB;
    const int app = exact_pair<LAW, XS, KIND>(a, a.scenes[a.scene_of[i]], i, Pi, e, ent, meta, Jp, tA, tB);
    // each member's share at its own entry: the slave adds J and tA, the master -J and tB
    // (the negation is exact, so the sums see the single tick's values)
    const bool i_slave = meta & META_SLAVE;
    const float kind = __int_as_float(app);
    const f3 Ji = i_slave ? Jp : -Jp, ti = i_slave ? tA : tB;
    a.prec[2 * (size_t)e] = make_float4(Ji.x, Ji.y, Ji.z, kind);
    if (app == 2) a.prec[2 * (size_t)e + 1] = make_float4(ti.x, ti.y, ti.z, 0.0f);
    if (!(ent & WALL_BIT)) {                   // a sphere pair: the partner's share at its entry
        const uint32_t q2 = a.pmir[e];
        const f3 Jj = i_slave ? -Jp : Jp, tj = i_slave ? tB : tA;
        a.prec[2 * (size_t)q2] = make_float4(Jj.x, Jj.y, Jj.z, kind);
        if (app == 2) a.prec[2 * (size_t)q2 + 1] = make_float4(tj.x, tj.y, tj.z, 0.0f);
    }
}

// The worklist's pairs from `first` in strides of `stride`: KIND 1 the sphere pairs (from the
// worklist's start), KIND 2 the wall pairs (from its end).  Two kernels: the sphere-pair one
// carries no call of the wall detector, and so no spills.
template <int LAW, bool XS, int KIND>
__device__ __forceinline__ void pairs_from(const TickArgs& a, uint32_t first, uint32_t stride) {
    const uint32_t nw = min(a.nwork[0], a.pcap), nww = min(a.nwork[-1], a.pcap - nw);
    if (KIND == 1) {
        for (uint32_t q = first; q < nw; q += stride) pair_item<LAW, XS, 1>(a, a.pwork[q]);
    } else {
        for (uint32_t q = first; q < nww; q += stride) pair_item<LAW, XS, 2>(a, a.pwork[a.pcap - 1u - q]);
    }
}
// AFTER_WALLS: launched after the wall-pair kernel, whose blocks all waited for the prefilter pass
// before releasing this one, so the worklist is complete when it starts; it waits for the
// wall-pair kernel only at its end, so that the two run side by side (the wall pairs' FP64 work
// and the sphere pairs' gathers use different units), and the sum kernel after it, waiting for
// it, then waits for both.
template <int LAW, bool XS, int KIND, bool AFTER_WALLS>
__global__ void __launch_bounds__(TPB, 4) k_tick_pairs(TickArgs a) {     // sphere pairs: 56 registers, no spills
    if (AFTER_WALLS) {
        asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
        if (!held_step(a)) pairs_from<LAW, XS, KIND>(a, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
        asm volatile("griddepcontrol.wait;" ::: "memory");
        return;
    }
    step_order();
    if (held_step(a)) return;
    pairs_from<LAW, XS, KIND>(a, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// One sphere's sums and integration (or, in an identity step, its state carried over); returns its
// squared speed bounds.
template <bool XS>
__device__ __forceinline__ float2 sum_sphere(const TickArgs& a, uint32_t i, bool hold) {
    float2 vmax_local = make_float2(0.0f, 0.0f);
    if (hold) {
        hold_state(a, i);
    } else if (i < a.n) {
        const uint32_t mi = a.model_of[i];
        const uint32_t si = a.scene_of[i];
        const uint32_t e0 = a.nptr[i], e1 = a.nptr[i + 1];
        const d3 Pi = ld(a.xA, i);
        const d3 V = ld(a.v64, i);
        const ModelDev& M = a.models[mi];
        const SceneDev& S = a.scenes[si];
        if (M.scope == SCOPE_LOCAL && S.active) {
            const bool quiet = a.wk[i] != 0u;
            const float4 mf0 = a.mf[2 * mi], mf1 = a.mf[2 * mi + 1];
            K3 J, JA;
            auto add_pair = [&](const float4& r0, const float4& t0) {
                const int app = __float_as_int(r0.w);
                if (app) {
                    J.add(f4to3(r0));
                    if (app == 2) JA.add(f4to3(t0));
                }
            };
            if (!quiet) {
                // the records of two marked entries at a time are loaded together (both halves of an
                // entry's record share one 32-byte sector), then summed in entry order
                unsigned long long m = a.xm[i];
                while (m) {
                    float4 r[2], t[2];
                    uint32_t cnt = 0;
#pragma unroll
                    for (int k = 0; k < 2; ++k) {
                        if (m) {
                            const size_t e = e0 + (uint32_t)(__ffsll(m) - 1);
                            m &= m - 1;
                            r[k] = a.prec[2 * e];
                            t[k] = a.prec[2 * e + 1];
                            cnt = (uint32_t)k + 1u;
                        }
                    }
#pragma unroll
                    for (int k = 0; k < 2; ++k)
                        if ((uint32_t)k < cnt) add_pair(r[k], t[k]);
                }
                for (uint32_t e = e0 + 64; e < e1; ++e)         // long lists: entries after the first 64
                    if (a.xf[e]) add_pair(a.prec[2 * (size_t)e], a.prec[2 * (size_t)e + 1]);
            }
            vmax_local = finish_sphere<XS>(a, i, M.behavior == BEH_MOBILE, quiet, S, Pi, V, mf0, mf1, J, JA);
        } else if (M.scope == SCOPE_LOCAL) {
            hold_state(a, i);
        }
    }
    return vmax_local;
}
template <bool XS>
__global__ void __launch_bounds__(TPB, 5) k_tick_sum(TickArgs a) {      // 48 registers: 5 blocks of 256 per SM
    step_order();
    reduce_vmax(a, sum_sphere<XS>(a, blockIdx.x * blockDim.x + threadIdx.x, held_step(a)));
}

// A wall's FP32 record carries in w the drift of its scene's frame across it after k steps
// since the rebuild: |D . n| for a plate, |D x a| for a rod, D = dt k (u0 + gdt k / 2), with an
// allowance for the roundings of the frame's per-step velocities, of this closed form and of
// the FP32 normal; w = 0 marks a wall without a usable normal, so a valid one keeps w > 0.
__device__ __forceinline__ float frame_drift_across(const SceneDev& S, uint32_t k, int shape, float nx, float ny,
                                                    float nz) {
    const float kf = (float)k, dtk = (float)S.dt * kf, hk = 0.5f * kf;
    const float Dx = dtk * fmaf(S.gdt[0], hk, S.u0[0]), Dy = dtk * fmaf(S.gdt[1], hk, S.u0[1]),
                Dz = dtk * fmaf(S.gdt[2], hk, S.u0[2]);
    float across;
    if (shape == SHAPE_PLATE || shape == SHAPE_HOLED) {
        across = fabsf(fmaf(Dz, nz, fmaf(Dy, ny, Dx * nx)));
    } else {
        const float cx = fmaf(Dy, nz, -Dz * ny), cy = fmaf(Dz, nx, -Dx * nz), cz = fmaf(Dx, ny, -Dy * nx);
        across = sqrtf(fmaf(cz, cz, fmaf(cy, cy, cx * cx)));
    }
    const float slack = 1e-6f * (fabsf(Dx) + fabsf(Dy) + fabsf(Dz) +
                                 dtk * (fabsf(S.u0[0]) + fabsf(S.u0[1]) + fabsf(S.u0[2]) +
                                        kf * (fabsf(S.gdt[0]) + fabsf(S.gdt[1]) + fabsf(S.gdt[2]))));
    return fmaxf(across + slack, 1e-30f);
}

// Vector3d::rotate_around (Vector3d.h:152-178) split in two: the half-angle terms of the turn
// omega dt (v = axis sin(a/2), s = cos(a/2)), fixed for an orbital wall (prescribed omega, fixed
// dt), and the rotation of a vector with them, in rotate_around's operation order.
__device__ __forceinline__ double4_32a turn_terms(d3 va) {
    const d3 u = dir(va);
    const double ang = len(va);
    const double c = cos(0.5 * ang), sn = sin(0.5 * ang);
    const d3 v = muls(u, sn);
    return make_double4_32a(v.x, v.y, v.z, c);
}
__device__ __forceinline__ d3 rotate_quat(d3 p, const double4_32a& R) {
    const d3 v = mk(R.x, R.y, R.z);
    const double s = R.w;
    d3 r = add(smul(s * s, p), smul(dot(p, v), v));
    r = add(r, smul(2.0 * s, cross(v, p)));
    return add(r, cross(v, cross(v, p)));
}
__global__ void k_wall_rot(uint32_t nglob, const uint32_t* __restrict__ glob, const uint32_t* __restrict__ model_of,
                           const ModelDev* __restrict__ models, const SceneDev* __restrict__ scenes,
                           const uint32_t* __restrict__ scene_of, const double4_32a* __restrict__ w64,
                           double4_32a* __restrict__ wrot) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nglob) return;
    const uint32_t w = glob[q];
    wrot[q] = models[model_of[w]].behavior == BEH_ORBITAL ? turn_terms(muls(ld(w64, w), scenes[scene_of[w]].dt))
                                                           : make_double4_32a(0.0, 0.0, 0.0, 1.0);
}

// Scope-global objects (walls): fixed ones keep their state, orbital ones move with their
// prescribed V and omega (DOOrbitalQuasiPlate.cpp:18-34).  Thread 0 also writes the
// displacement bounds and the step count after the step into the other parity slot
// (disp_out), or, when the step is an identity step, carries them over and counts the step in
// *held; every wall's FP32 record gets the frame's drift across it for the next step.
struct WallArgs {
    uint32_t nglob;
    const uint32_t* glob;
    const uint32_t* model_of;
    const ModelDev* models;
    const SceneDev* scenes;
    const uint32_t* scene_of;
    const double4_32a* xA;
    double4_32a* xB;
    double4_32a* v64;
    double4_32a* w64;
    const float4* v32A;
    float4* v32B;
    const float4* w32A;
    float4* w32B;
    double4_32a* ox;
    double4_32a* oz;
    float dt_max;
    unsigned* vmax_bits;
    unsigned* vrel_bits;
    const float* disp_in;
    float* disp_out;
    float skin, skin_w, pos_eps;
    const unsigned* wall_speed_bits;
    const double4_32a* wrot;
    unsigned* held;
    float4* wall32;
    unsigned* nwork;
    const double4_32a* imp;
    const double4_32a* aimp;
    unsigned* dyn_bits;
};
__device__ __forceinline__ void walls_item(const WallArgs& W, uint32_t q) {
    const uint32_t nglob = W.nglob;
    const uint32_t* __restrict__ glob = W.glob;
    const uint32_t* __restrict__ model_of = W.model_of;
    const ModelDev* __restrict__ models = W.models;
    const SceneDev* __restrict__ scenes = W.scenes;
    const uint32_t* __restrict__ scene_of = W.scene_of;
    const double4_32a* xA = W.xA;
    double4_32a* xB = W.xB;
    double4_32a* v64 = W.v64;
    double4_32a* w64 = W.w64;
    const float4* v32A = W.v32A;
    float4* v32B = W.v32B;
    const float4* w32A = W.w32A;
    float4* w32B = W.w32B;
    double4_32a* ox = W.ox;
    double4_32a* oz = W.oz;
    const float dt_max = W.dt_max;
    unsigned* vmax_bits = W.vmax_bits;
    unsigned* vrel_bits = W.vrel_bits;
    const float* disp_in = W.disp_in;
    float* disp_out = W.disp_out;
    const float skin = W.skin, skin_w = W.skin_w, pos_eps = W.pos_eps;
    const unsigned* wall_speed_bits = W.wall_speed_bits;
    const double4_32a* __restrict__ wrot = W.wrot;
    unsigned* held = W.held;
    float4* wall32 = W.wall32;
    unsigned* nwork = W.nwork;
    const double4_32a* imp = W.imp;
    const double4_32a* aimp = W.aimp;
    unsigned* dyn_bits = W.dyn_bits;
    const float drel = disp_in[0], dabs = disp_in[1], dw = disp_in[2];
    const bool hold = list_spent(drel, dabs, dw, skin, skin_w);
    if (q == 0) {
        nwork[0] = nwork[1] = 0u;                  // the worklists' counts (pair pass: wall pairs, then
                                                   // sphere pairs and the split tick's spheres), empty
                                                   // for the next step
        if (hold) {
            for (int k = 0; k < 4; ++k) disp_out[k] = disp_in[k];
            *held += 1u;
        } else {
            // pos_eps: the FP64 rounding of a position update, which the speeds do not see
            disp_out[0] = drel + dt_max * __uint_as_float(*vrel_bits) + pos_eps;
            disp_out[1] = dabs + dt_max * __uint_as_float(*vmax_bits) + pos_eps;
            disp_out[2] = dw + dt_max * __uint_as_float(*wall_speed_bits) + pos_eps;
            disp_out[3] = __uint_as_float(__float_as_uint(disp_in[3]) + 1u);
        }
        *vmax_bits = 0u;
        *vrel_bits = 0u;
    }
    if (q >= nglob) return;
    const uint32_t w = glob[q];
    if (hold || !scenes[scene_of[w]].active) {
        xB[w] = xA[w];
        v32B[w] = v32A[w];
        w32B[w] = w32A[w];
        return;
    }
    const ModelDev& M = models[model_of[w]];
    const SceneDev& S = scenes[scene_of[w]];
    const double dt = S.dt;
    const uint32_t k1 = __float_as_uint(disp_in[3]) + 1u;     // steps since the rebuild, after this one
    d3 P = ld(xA, w);
    if (M.behavior == BEH_FIXED) {
        float4 ws = wall32[w];
        if (ws.w != 0.0f) {
            ws.w = frame_drift_across(S, k1, M.shape, ws.x, ws.y, ws.z);
            wall32[w] = ws;
        }
    } else if (M.behavior != BEH_ORBITAL) {
        // a mobile or constrained wall moved by its impulses this step (summed exactly by
        // k_wall_max/acc/fin, field and external force included), as the FP64 form's
        // respond_object: DOQuasiPlate.cpp:20-41 / DOConstrainedQuasiPlate.cpp:18-35
        const d3 J = ld(imp, w), JA = ld(aimp, w);
        d3 V = ld(v64, w), AV = ld(w64, w), Ox = ld(ox, w), Oz = ld(oz, w);
        const d3 P0 = P;
        d3 dw;
        if (M.behavior == BEH_CONSTRAINED) {
            const d3 dv = smul(M.inv_sudo, smul(dot(J, Oz), dir(Oz)));
            P = add(P, smul(dt, add(V, smul(0.5, dv))));
            dw = muls(AV, dt);
            V = add(V, dv);
        } else {
            const d3 dv = smul(M.inv_sudo, J);
            const d3 dav = mk(dot(JA, Ox) / M.ix, dot(JA, cross(Oz, Ox)) / M.iy, dot(JA, Oz) / M.iz);
            P = add(P, smul(dt, add(V, smul(0.5, dv))));
            dw = smul(dt, add(AV, smul(0.5, dav)));
            V = add(V, dv);
            AV = add(AV, dav);
        }
        const Turn T = turn_of(dw);
        Ox = rotate_by(Ox, T);
        Oz = rotate_by(Oz, T);
        st(ox, w, Ox, 0.0);
        st(oz, w, Oz, 0.0);
        st(v64, w, V, 0.0);
        st(w64, w, AV, 0.0);
        st(xB, w, P, 0.0);
        v32B[w] = make_float4((float)V.x, (float)V.y, (float)V.z, 0.0f);
        w32B[w] = make_float4((float)AV.x, (float)AV.y, (float)AV.z, 0.0f);
        const double lz = len(Oz), lx = len(Ox);
        bool ok = lz > 0.0;
        if (M.shape == SHAPE_PLATE || M.shape == SHAPE_HOLED) ok = ok && lx > 0.0 && fabs(dot(Ox, Oz)) <= 1e-9 * lx * lz;
        const float nx = (float)(Oz.x / lz), ny = (float)(Oz.y / lz), nz = (float)(Oz.z / lz);
        wall32[w] = ok ? make_float4(nx, ny, nz, frame_drift_across(S, k1, M.shape, nx, ny, nz))
                       : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        // how far any point of the wall went this step: its centre's travel and the turn of its
        // farthest point (k_wall_bound adds the largest to the walls' displacement bound)
        const double R = M.shape == SHAPE_INNER_CYL ? sqrt(M.a0 * M.a0 + 0.25 * M.a1 * M.a1)
                                                    : 0.5 * sqrt(M.a0 * M.a0 + M.a1 * M.a1 + M.a2 * M.a2);
        const double d = len(sub(P, P0)) + len(dw) * R;
        atomicMax(dyn_bits, __float_as_uint((float)(d * 1.0001) + 1e-30f));
        return;
    } else {
        const d3 V = ld(v64, w);
        P = add(P, muls(V, dt));
        // rotate_around(O, omega dt) with its cos/sin terms computed once per list (k_wall_rot)
        const double4_32a R = wrot[q];
        const d3 Ox = rotate_quat(ld(ox, w), R), Oz = rotate_quat(ld(oz, w), R);
        st(ox, w, Ox, 0.0);
        st(oz, w, Oz, 0.0);
        const double lz = len(Oz), lx = len(Ox);
        bool ok = lz > 0.0;
        if (M.shape == SHAPE_PLATE || M.shape == SHAPE_HOLED) ok = ok && lx > 0.0 && fabs(dot(Ox, Oz)) <= 1e-9 * lx * lz;
        const float nx = (float)(Oz.x / lz), ny = (float)(Oz.y / lz), nz = (float)(Oz.z / lz);
        wall32[w] = ok ? make_float4(nx, ny, nz, frame_drift_across(S, k1, M.shape, nx, ny, nz))
                       : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    st(xB, w, P, 0.0);
    v32B[w] = v32A[w];
    w32B[w] = w32A[w];
}
__global__ void k_walls(WallArgs W) {
    step_order();
    walls_item(W, blockIdx.x * blockDim.x + threadIdx.x);
}

// After k_walls, when mobile or constrained walls move: the largest distance any point of such a
// wall went this step joins the walls' displacement bound (not in a step that was held).
__global__ void k_wall_bound(const float* __restrict__ disp_in, float* __restrict__ disp_out, float skin,
                             float skin_w, unsigned* __restrict__ dyn_bits) {
    step_order();
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    if (!list_spent(disp_in[0], disp_in[1], disp_in[2], skin, skin_w)) disp_out[2] += __uint_as_float(*dyn_bits);
    *dyn_bits = 0u;
}

// ---- persistent tick ------------------------------------------------------------------------
// One cooperative launch runs a whole check interval: the steps' stages (the kernels above, as
// device functions, with the same operations in the same order per sphere, pair and wall) are
// separated by grid barriers instead of kernel boundaries.  A cooperative launch has every block
// resident at once (the launch fails rather than start otherwise), so the barrier's wait always
// ends; it is still bounded: a block that has waited `limit_ns` on the global timer, or polled
// a bounded number of times, records the barrier's site and sets the expiry flag, and every block
// that sees the flag leaves at its next barrier, so the kernel ends and the host reports the
// error.  Words: [0] arrivals, [1] generation, [2] expired, [3] the site of the first expiry.
struct GridBar {
    unsigned* w;
    uint32_t nblocks;
    unsigned long long limit_ns;
};
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ bool grid_sync(const GridBar& g, unsigned site) {
    __shared__ int ok_s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 0;
        unsigned* w = g.w;
        if (ld_acquire(w + 2) == 0u) {
            const unsigned gen = ld_acquire(w + 1);
            __threadfence();                       // this block's writes, before its arrival
            if (atomicAdd(w, 1u) == g.nblocks - 1u) {
                atomicExch(w, 0u);                 // the count is reset before the generation moves
                __threadfence();
                atomicAdd(w + 1, 1u);
                ok = 1;
            } else {
                const unsigned long long t0 = global_ns();
                const unsigned long long polls = g.limit_ns / 16u + 4096u;
                for (unsigned long long k = 0;; ++k) {
                    if (ld_acquire(w + 1) != gen) {
                        ok = 1;
                        break;
                    }
                    if (ld_acquire(w + 2) != 0u) break;
                    if (k > polls || global_ns() - t0 > g.limit_ns) {
                        atomicCAS(w + 3, 0u, site);
                        atomicExch(w + 2, 1u);
                        break;
                    }
                    __nanosleep(32);
                }
            }
            __threadfence();                       // the other blocks' writes, after the barrier
        }
        ok_s = ok;
    }
    __syncthreads();
    return ok_s != 0;
}

struct PersistArgs {
    TickArgs t[2];                 // the steps that start from the first step's buffers, and the others
    WallArgs w[2];
    uint32_t steps;
    int pbc;                       // a scene is periodic: spheres back into the box after each step
    GridBar bar;
};
static_assert(sizeof(PersistArgs) <= 4096, "the persistent tick's arguments must fit the classic parameter space");

// FORM 0: the full tick (one thread per sphere), then the walls; FORM 2: the pair pass's prefilter
// pass, pair pass and sums, then the walls.  Spheres go to the warps of the whole grid in turn
// (consecutive warps of a block on different SMs), so a small scene spreads over every SM.
template <int FORM, int LAW, bool XS>
__global__ void __launch_bounds__(FORM == 2 ? 1024 : 512, 1) k_persist(PersistArgs p) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t W = gridDim.x * (blockDim.x >> 5);
    const uint32_t gw = (threadIdx.x >> 5) * gridDim.x + blockIdx.x;
    uint32_t site = 1;
    for (uint32_t k = 0; k < p.steps; ++k) {
        const TickArgs& a = p.t[k & 1u];
        const uint32_t n = a.n;
        const bool hold = list_spent(__ldcg(a.disp), __ldcg(a.disp + 1), __ldcg(a.disp + 2), a.skin, a.skin_w);
        float2 vm = make_float2(0.0f, 0.0f);
        if (FORM == 2) {
            if (!hold)
                for (uint32_t s = gw; s * 32u < n; s += W) pf_sphere(a, s * 32u + lane);
            if (!grid_sync(p.bar, site++)) return;
            if (!hold) {
                pairs_from<LAW, XS, 1>(a, gw * 32u + lane, W * 32u);
                pairs_from<LAW, XS, 2>(a, gw * 32u + lane, W * 32u);
            }
            if (!grid_sync(p.bar, site++)) return;
            for (uint32_t s = gw; s * 32u < n; s += W) {
                const uint32_t i = s * 32u + lane;
                vm = fmax2(vm, sum_sphere<XS>(a, i, hold));
                if (!hold && p.pbc) wrap_sphere(a, i);
                if (!hold && a.orient) turn_sphere(a, i);
            }
        } else {
            for (uint32_t s = gw; s * 32u < n; s += W) {
                const uint32_t i = s * 32u + lane;
                if (hold) {
                    hold_state(a, i);
                } else if (i < n) {
                    vm = fmax2(vm, tick_sphere<LAW, XS>(a, i));
                    if (p.pbc) wrap_sphere(a, i);
                    if (a.orient) turn_sphere(a, i);
                }
            }
        }
        reduce_vmax(a, vm);
        if (!grid_sync(p.bar, site++)) return;
        const WallArgs& wa = p.w[k & 1u];
        for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < max(wa.nglob, 1u); q += gridDim.x * blockDim.x)
            walls_item(wa, q);
        if (k + 1u < p.steps && !grid_sync(p.bar, site++)) return;
    }
}

// The barrier alone, for its check: `rounds` barriers over a cooperative grid that expects
// `nblocks` arrivals (more than the grid has: a barrier that nothing completes, which must expire
// and end the kernel).  Each block adds its round count; out[0] gets the rounds every block saw
// complete, out[1] the blocks that saw a round's counts wrong.
__global__ void k_bar_check(GridBar g, uint32_t rounds, unsigned* cnt, unsigned* out) {
    for (uint32_t r = 0; r < rounds; ++r) {
        if (threadIdx.x == 0) atomicAdd(cnt + (r & 1u), 1u);
        if (!grid_sync(g, r + 1u)) return;
        if (threadIdx.x == 0) {
            if (__ldcg(cnt + (r & 1u)) != gridDim.x * (r / 2u + 1u)) atomicAdd(out + 1, 1u);
            if (blockIdx.x == 0) atomicExch(out, r + 1u);
        }
    }
}

// ---- broad phase -------------------------------------------------------------------------
// Per scene, the componentwise range of its mobile spheres' velocities (ordered float bits in
// vred[6 * scene + k]: [0..2] min, [3..5] max): its midrange is the frame velocity of the list.
__global__ void __launch_bounds__(TPB) k_vrange(uint32_t n, const uint32_t* __restrict__ model_of,
                                                const ModelDev* __restrict__ models,
                                                const uint32_t* __restrict__ scene_of,
                                                const double4_32a* __restrict__ v, unsigned* __restrict__ vred) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned mn[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, mx[3] = {0, 0, 0};
    uint32_t sc = 0xffffffffu;
    if (i < n && models[model_of[i]].scope == SCOPE_LOCAL && models[model_of[i]].behavior == BEH_MOBILE) {
        sc = scene_of[i];
        const d3 q = ld(v, i);
        const float f[3] = {(float)q.x, (float)q.y, (float)q.z};
        for (int k = 0; k < 3; ++k) {
            const unsigned b = __float_as_uint(f[k]);
            mn[k] = mx[k] = (b >> 31) ? ~b : (b | 0x80000000u);
        }
    }
    const uint32_t sc0 = __shfl_sync(0xffffffffu, sc, 0);
    const bool one = __all_sync(0xffffffffu, sc == sc0 || sc == 0xffffffffu) && sc0 != 0xffffffffu;
    if (one) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                mn[k] = min(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], o));
                mx[k] = max(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], o));
            }
    }
    if ((one && (threadIdx.x & 31) == 0) || (!one && sc != 0xffffffffu)) {
        unsigned* r = vred + 6 * (size_t)(one ? sc0 : sc);
        for (int k = 0; k < 3; ++k) {
            atomicMin(&r[k], mn[k]);
            atomicMax(&r[3 + k], mx[k]);
        }
    }
}

__global__ void __launch_bounds__(TPB) k_bounds(uint32_t n, const uint32_t* __restrict__ model_of,
                                                const ModelDev* __restrict__ models,
                                                const uint32_t* __restrict__ scene_of, const double4_32a* __restrict__ x,
                                                d3 origin, float4* __restrict__ pos32, unsigned* __restrict__ red) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    // red[8 * scene + k]: [0..2] min (ordered float bits), [3..5] max, [6] max radius
    unsigned mn[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, mx[3] = {0, 0, 0}, rm = 0;
    const uint32_t sc = i < n ? scene_of[i] : 0xffffffffu;
    if (i < n) {
        const ModelDev& M = models[model_of[i]];
        const d3 p = ld(x, i);
        float4 q = make_float4((float)(p.x - origin.x), (float)(p.y - origin.y), (float)(p.z - origin.z), 0.0f);
        q.w = PF_POS_EPS * (fabsf(q.x) + fabsf(q.y) + fabsf(q.z));   // bound on this copy's rounding
        pos32[i] = q;
        if (M.scope == SCOPE_LOCAL) {
            auto ordf = [](float f) {
                unsigned b = __float_as_uint(f);
                return (b >> 31) ? ~b : (b | 0x80000000u);
            };
            mn[0] = mx[0] = ordf(q.x);
            mn[1] = mx[1] = ordf(q.y);
            mn[2] = mx[2] = ordf(q.z);
            rm = __float_as_uint((float)M.range);
        }
    }
    const uint32_t sc0 = __shfl_sync(0xffffffffu, sc, 0);
    if (__all_sync(0xffffffffu, sc == sc0 || sc == 0xffffffffu)) {   // one scene in this warp
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                mn[k] = min(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], o));
                mx[k] = max(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], o));
            }
            rm = max(rm, __shfl_xor_sync(0xffffffffu, rm, o));
        }
        if ((threadIdx.x & 31) == 0 && sc0 != 0xffffffffu) {
            unsigned* r = red + 8 * (size_t)sc0;
            for (int k = 0; k < 3; ++k) {
                atomicMin(&r[k], mn[k]);
                atomicMax(&r[3 + k], mx[k]);
            }
            atomicMax(&r[6], rm);
        }
    } else if (sc != 0xffffffffu) {                                  // scene boundary inside the warp
        unsigned* r = red + 8 * (size_t)sc;
        for (int k = 0; k < 3; ++k) {
            atomicMin(&r[k], mn[k]);
            atomicMax(&r[3 + k], mx[k]);
        }
        atomicMax(&r[6], rm);
    }
}

__global__ void __launch_bounds__(TPB) k_keys(uint32_t n, const uint32_t* __restrict__ model_of,
                                              const ModelDev* __restrict__ models,
                                              const uint32_t* __restrict__ scene_of, const SceneDev* __restrict__ scenes,
                                              const float4* __restrict__ pos32, uint64_t sentinel,
                                              uint64_t* __restrict__ key, uint32_t* __restrict__ sid) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint64_t k = sentinel;
    if (models[model_of[i]].scope == SCOPE_LOCAL) {
        const SceneDev& S = scenes[scene_of[i]];
        const float4 p = pos32[i];
        const float pc[3] = {p.x, p.y, p.z};
        uint32_t c[3];
        for (int a = 0; a < 3; ++a) {
            float u = pc[a] - S.lo[a];
            if (S.pb.sw[a]) {                      // periodic axis: the image inside the box
                const float L = S.pb.range32[a];
                u -= L * floorf(u / L);
            }
            c[a] = min((uint32_t)fmaxf(u * S.inv_h, 0.0f), S.nc[a] - 1);
        }
        k = S.cell_base + ((uint64_t)c[0] * S.nc[1] + c[1]) * S.nc[2] + c[2];
    }
    key[i] = k;
    sid[i] = i;
}

__global__ void __launch_bounds__(TPB) k_cells(uint32_t nloc, const uint64_t* __restrict__ key,
                                               uint32_t* __restrict__ grid_start, uint32_t* __restrict__ grid_end) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nloc) return;
    const uint64_t k = key[p];
    if (p == 0 || key[p - 1] != k) grid_start[k] = p;
    if (p == nloc - 1 || key[p + 1] != k) grid_end[k] = p + 1;
}

// Full neighbour list of every local sphere: 27 cells in a fixed order, j ascending within a
// cell, then the walls; candidate when the pair may come within reach + skin (conservative).
template <bool FILL>
__global__ void __launch_bounds__(TPB) k_nbr(uint32_t nloc, const uint32_t* __restrict__ sid,
                                             const uint64_t* __restrict__ key, const uint32_t* __restrict__ grid_start,
                                             const uint32_t* __restrict__ grid_end,
                                             const uint32_t* __restrict__ scene_of, const SceneDev* __restrict__ scenes,
                                             const uint32_t* __restrict__ glob,
                                             const uint32_t* __restrict__ model_of, const ModelDev* __restrict__ models,
                                             const PairParam* __restrict__ params, const float* __restrict__ reach,
                                             const float4* __restrict__ pos32,
                                             const float4* __restrict__ wall32, float skin,
                                             const uint32_t* __restrict__ ext_of, const uint32_t* __restrict__ int_of,
                                             uint32_t* __restrict__ cnt_or_ptr, uint32_t* __restrict__ ent) {
    const uint32_t P = blockIdx.x * blockDim.x + threadIdx.x;
    if (P >= nloc) return;
    const uint32_t i = sid[P];
    const SceneDev& S = scenes[scene_of[i]];
    const uint32_t nx = S.nc[0], ny = S.nc[1], nz = S.nc[2];
    const uint64_t k = key[P] - S.cell_base;
    const uint32_t cz = (uint32_t)(k % nz), cy = (uint32_t)((k / nz) % ny), cx = (uint32_t)(k / ((uint64_t)nz * ny));
    const uint32_t mi = model_of[i];
    const float4 pi = pos32[i];
    uint32_t c = 0;
    uint32_t off = FILL ? cnt_or_ptr[i] : 0u;
    // the fill pass knows the sphere's count from the scanned pointers: it stops once every entry
    // is found (the entries are put in canonical order below, whatever order they were found in)
    const uint32_t want = FILL ? cnt_or_ptr[i + 1] - off : 0xffffffffu;
    // a neighbour cell index on an axis, wrapping on a periodic one (at least three cells: the
    // three are distinct); 0xffffffff outside a bounded grid
    auto ncell = [&](int a, uint32_t cc, uint32_t nn, int d) -> uint32_t {
        if (S.pb.sw[a]) return (cc + nn + (uint32_t)(d + 1) - 1u) % nn;
        if ((d < 0 && cc == 0) || (d > 0 && cc + 1 >= nn)) return 0xffffffffu;
        return cc + (uint32_t)d;
    };
    const float* L = S.pb.on ? S.pb.range32 : nullptr;
    for (int dx = -1; dx <= 1 && c < want; ++dx) {
        const uint32_t xx = ncell(0, cx, nx, dx);
        if (xx == 0xffffffffu) continue;
        for (int dy = -1; dy <= 1 && c < want; ++dy) {
            const uint32_t yy = ncell(1, cy, ny, dy);
            if (yy == 0xffffffffu) continue;
            for (int dz = -1; dz <= 1 && c < want; ++dz) {
                const uint32_t zz = ncell(2, cz, nz, dz);
                if (zz == 0xffffffffu) continue;
                const uint64_t nk = S.cell_base + ((uint64_t)xx * ny + yy) * nz + zz;
                const uint32_t b = grid_start[nk], e = grid_end[nk];
                for (uint32_t q = b; q < e && c < want; ++q) {
                    const uint32_t j = sid[q];
                    if (j == i) continue;
                    const uint32_t mj = model_of[j];
                    const uint32_t pa = pidx(S, mi, mj), pb = pidx(S, mj, mi);
                    if (params[pa].cd == 0 && params[pb].cd == 0) continue;
                    const float r = fmaxf(reach[pa], reach[pb]);
                    float err;
                    const float d = L ? dist32_periodic(pi, pos32[j], L, err) : dist32(pi, pos32[j], err);
                    if (d - err > (r + skin) * (1.0f + 4.0f * PF_ARITH_EPS)) continue;
                    if (FILL) ent[off + c] = ext_of[j];          // sorted below by the caller's index
                    ++c;
                }
            }
        }
    }
    for (uint32_t q = S.wall_beg; q < S.wall_end && c < want; ++q) {
        const uint32_t w = glob[q];
        const uint32_t pw = pidx(S, mi, model_of[w]);
        const int cd = cd_plane(params[pw].cd);
        if (cd == 0) continue;
        const float4 wl = wall32[w];
        if (wl.w != 0.0f) {
            float err;
            const float d = cd == CD_SP ? plane_dist32(pi, pos32[w], wl, err) : line_dist32(pi, pos32[w], wl, err);
            const float sk = models[model_of[w]].behavior != BEH_FIXED ? WALL_SKIN * skin : skin;
            if (cd == CD_SIC) {                        // clear of the shell by more than the skin
                if (d + err < -(reach[pw] + sk) * (1.0f - 4.0f * PF_ARITH_EPS)) continue;
            } else if (d - err > (reach[pw] + sk) * (1.0f + 4.0f * PF_ARITH_EPS)) {
                continue;
            }
        }
        if (FILL) ent[off + c] = ext_of[w] | WALL_BIT;
        ++c;
    }
    if (!FILL) {
        cnt_or_ptr[i] = c;
        return;
    }
    // Canonical order: spheres by the caller's index, then walls by the caller's index.  Every
    // per-sphere sum then runs in an order that depends neither on the cell grid nor on when
    // the list was rebuilt, nor on where the scene sits in a batch (indices only shift by the
    // scene's offset), nor on the engine's storage order.
    for (uint32_t q = 1; q < c; ++q) {
        const uint32_t v = ent[off + q];
        uint32_t r = q;
        while (r > 0 && ent[off + r - 1] > v) {
            ent[off + r] = ent[off + r - 1];
            --r;
        }
        ent[off + r] = v;
    }
    for (uint32_t q = 0; q < c; ++q) {                  // back to storage indices
        const uint32_t v = ent[off + q];
        ent[off + q] = (v & WALL_BIT) | int_of[v & ~WALL_BIT];
    }
}

// History slot of every entry: the entry itself for the owner (lower index, or a wall
// entry), else the owner's entry for the same pair in the neighbour's list.
__global__ void __launch_bounds__(TPB) k_slots(uint32_t n, const uint32_t* __restrict__ ptr,
                                               const uint32_t* __restrict__ ent, uint32_t* __restrict__ slot,
                                               int* __restrict__ err) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (uint32_t e = ptr[i]; e < ptr[i + 1]; ++e) {
        const uint32_t v = ent[e];
        if ((v & WALL_BIT) || i < v) {
            slot[e] = e;
            continue;
        }
        const uint32_t j = v;
        uint32_t found = 0xffffffffu;
        for (uint32_t q = ptr[j]; q < ptr[j + 1]; ++q)
            if (ent[q] == i) { found = q; break; }
        if (found == 0xffffffffu) atomicOr(err, 1);
        slot[e] = found == 0xffffffffu ? e : found;
    }
}

// Pair pass: at each owner entry of a sphere pair, the partner's entry of the same pair (every
// entry first names itself, then, in a second launch, each non-owner entry names itself at its
// owner entry; an entry without partner keeps its own index).
template <bool PARTNER>
__global__ void __launch_bounds__(TPB) k_mirror(uint32_t n, const uint32_t* __restrict__ ptr,
                                                const uint32_t* __restrict__ slot, uint32_t* __restrict__ mir) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (uint32_t e = ptr[i]; e < ptr[i + 1]; ++e) {
        if (!PARTNER) {
            mir[e] = e;
        } else {
            const uint32_t o = slot[e];
            if (o != e) mir[o] = e;
        }
    }
}

// Per-entry facts for the tick (META_*): orientation by the Assembler's rule
// (Assembler.cpp:43-67: the density-0 object is the master, else the lower index is the
// slave; a wall is always the master), the oriented pair's parameter index, its contact
// detector, whether its law may bond (then the FP32 prefilter may not skip it), and
// whether the entry holds the pair's history.
__global__ void __launch_bounds__(TPB) k_meta(uint32_t n, const uint32_t* __restrict__ ptr,
                                              const uint32_t* __restrict__ ent, const uint32_t* __restrict__ slot,
                                              const uint32_t* __restrict__ model_of,
                                              const ModelDev* __restrict__ models,
                                              const uint32_t* __restrict__ scene_of,
                                              const SceneDev* __restrict__ scenes,
                                              const PairParam* __restrict__ params, const uint32_t* __restrict__ ext_of,
                                              uint32_t* __restrict__ meta) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t mi = model_of[i];
    const ModelDev& M = models[mi];
    const SceneDev& S = scenes[scene_of[i]];
    for (uint32_t e = ptr[i]; e < ptr[i + 1]; ++e) {
        const uint32_t v = ent[e];
        const uint32_t j = v & ~WALL_BIT;
        const uint32_t mj = model_of[j];
        bool i_slave;
        if (v & WALL_BIT) {
            i_slave = true;
        } else {
            const ModelDev& N = models[mj];
            if (M.density == 0.0 && N.density != 0.0) i_slave = false;
            else if (N.density == 0.0 && M.density != 0.0) i_slave = true;
            else i_slave = ext_of[i] < ext_of[j];
        }
        const uint32_t pi = pidx(S, i_slave ? mi : mj, i_slave ? mj : mi);
        const PairParam& P = params[pi];
        const bool bond = (P.is == IS_BSDBF || P.is == IS_BTSDBF || P.is == IS_BSDB2F) && P.c[4] != 0.0;
        const bool moving = (v & WALL_BIT) && models[mj].behavior != BEH_FIXED;
        meta[e] = (pi & META_PI) | ((uint32_t)(cd_plane(P.cd) & META_CD_MASK) << META_CD_SHIFT) | (bond ? META_BOND : 0u) |
                  (slot[e] == e ? META_OWNER : 0u) | (i_slave ? META_SLAVE : 0u) | (moving ? META_MOVING : 0u);
    }
}

// New owner entries take the status of the same pair in the old list (if it was listed).
__global__ void __launch_bounds__(TPB) k_carry(uint32_t n, const uint32_t* __restrict__ ptr,
                                               const uint32_t* __restrict__ ent, const uint32_t* __restrict__ slot,
                                               const uint32_t* __restrict__ optr, const uint32_t* __restrict__ oent,
                                               const uint32_t* __restrict__ oslot, const float4* __restrict__ oh,
                                               const uint8_t* __restrict__ of, float4* __restrict__ h,
                                               uint8_t* __restrict__ f, float4* __restrict__ h2,
                                               uint8_t* __restrict__ f2, int have_old) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (uint32_t e = ptr[i]; e < ptr[i + 1]; ++e) {
        if (slot[e] != e) continue;
        const uint32_t v = ent[e];
        float4 hv = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        uint8_t fv = HF_LAST_CONTACT | HF_LAST_BOND;       // default-constructed ImpactStatus
        if (have_old) {
            for (uint32_t q = optr[i]; q < optr[i + 1]; ++q)
                if (oent[q] == v) {
                    const uint32_t os = oslot[q];
                    hv = oh[os];
                    fv = of[os] & (uint8_t)15;
                    break;
                }
        }
        h[e] = hv;
        f[e] = fv;
        h2[e] = hv;
        f2[e] = fv;
    }
}



// Per sphere, the largest pads (the prefilter's allowance for the travel since the rebuild:
// sphere pairs in x, fixed walls in y) at which every entry of its new list is still certainly
// apart, checked with the prefilter itself: an estimate from the rebuild-time gap, backed off
// until apart32 confirms it.  -1 (never quiet) for a sphere with a bondable entry, an entry that
// failed the check, or an entry with an orbital wall (its normal is recomputed every step).
// Resets the clean-walk count.
__global__ void __launch_bounds__(TPB) k_clear(uint32_t n, const uint32_t* __restrict__ ptr,
                                               const uint32_t* __restrict__ ent, const uint32_t* __restrict__ meta,
                                               const uint32_t* __restrict__ model_of,
                                               const ModelDev* __restrict__ models, const float4* __restrict__ pos32,
                                               const float4* __restrict__ wall32, const float* __restrict__ reach,
                                               float2* __restrict__ clear, uint8_t* __restrict__ qcnt, int enable,
                                               const uint32_t* __restrict__ scene_of, const SceneDev* __restrict__ scenes) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    qcnt[i] = 0;
    float c = -1.0f, cw = -1.0f;                   // sphere pairs, fixed walls
    // (the spheres of a periodic scene always walk their lists: these limits use plain differences)
    if (enable && models[model_of[i]].scope == SCOPE_LOCAL && !scenes[scene_of[i]].pb.on) {
        c = cw = 3.0e38f;
        const float4 pi = pos32[i];
        for (uint32_t e = ptr[i]; e < ptr[i + 1]; ++e) {
            const uint32_t m = meta[e];
            const int cd = (int)((m >> META_CD_SHIFT) & META_CD_MASK);
            if (cd == 0) continue;
            const uint32_t j = ent[e] & ~WALL_BIT;
            const bool wall = ent[e] & WALL_BIT;
            if ((m & META_BOND) || (wall && models[model_of[j]].behavior != BEH_FIXED)) {
                c = cw = -1.0f;
                break;
            }
            const float4 pj = pos32[j];
            const float4 ws = wall ? wall32[j] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            const float4 ps = (m & META_SLAVE) ? pi : pj, pm = (m & META_SLAVE) ? pj : pi;
            const float dx = pm.x - ps.x, dy = pm.y - ps.y, dz = pm.z - ps.z;
            float gap;
            if (cd == CD_SS) {
                gap = sqrtf(dx * dx + dy * dy + dz * dz);
            } else if (cd == CD_SP) {
                gap = fabsf(dx * ws.x + dy * ws.y + dz * ws.z);
            } else {
                const float cx = dy * ws.z - dz * ws.y, cy = dz * ws.x - dx * ws.z, cz = dx * ws.y - dy * ws.x;
                gap = sqrtf(cx * cx + cy * cy + cz * cz);
            }
            const float r = reach[m & META_PI];
            const float slack = ps.w + pm.w + PF_ARITH_EPS * (fabsf(dx) + fabsf(dy) + fabsf(dz));
            // inside a hollow cylinder (r = -(R - r_s)): the room left between the centre's axis
            // distance and R - r_s
            float t = cd == CD_SIC ? (-r - gap - slack) * (1.0f - 1e-4f) : (gap - slack) * (1.0f - 1e-4f) - r;
            bool ok = false;
            for (int k = 0; k < 4 && t >= 0.0f && !ok; ++k) {
                ok = apart32(cd, ps, pm, ws, r + t);
                if (!ok) t = k < 2 ? 0.5f * t : 0.0f;
            }
            if (!ok) {
                c = cw = -1.0f;
                break;
            }
            if (wall) cw = fminf(cw, t);
            else c = fminf(c, t);
        }
    }
    clear[i] = make_float2(c, cw);
}

// Interior wall entries of the new list (META_INTERIOR): the sphere's projection lies inside
// the plate's rectangle (or within the rod's length) by more than any in-plane travel before
// the list is spent: the sphere's (at most the skin) and, for an orbital wall, the wall's own
// (together at most the wall skin).
__global__ void __launch_bounds__(TPB) k_interior(uint32_t n, const uint32_t* __restrict__ ptr,
                                                  const uint32_t* __restrict__ ent, uint32_t* __restrict__ meta,
                                                  const uint32_t* __restrict__ model_of,
                                                  const ModelDev* __restrict__ models,
                                                  const double4_32a* __restrict__ x, const double4_32a* __restrict__ ox,
                                                  const double4_32a* __restrict__ oz, float skin, float skin_w) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || models[model_of[i]].scope != SCOPE_LOCAL) return;
    const d3 P = ld(x, i);
    for (uint32_t e = ptr[i]; e < ptr[i + 1]; ++e) {
        const uint32_t v = ent[e];
        if (!(v & WALL_BIT)) continue;
        const uint32_t w = v & ~WALL_BIT;
        const ModelDev& W = models[model_of[w]];
        const d3 Oz = ld(oz, w);
        const double lz = len(Oz);
        if (!(lz > 0.0)) continue;
        const d3 d = sub(P, ld(x, w));
        const double m = (W.behavior != BEH_FIXED ? skin_w : skin) + 1e-9 * (len(d) + 1.0);
        const d3 uz = muls(Oz, 1.0 / lz);
        bool in = false;                           // a holed plate's hole edge is not modelled here
        if (W.shape == SHAPE_PLATE) {
            const d3 Ox = ld(ox, w);
            const double lx = len(Ox);
            if (!(lx > 0.0)) continue;
            const d3 ux = muls(Ox, 1.0 / lx), uy = cross(uz, ux);
            in = fabs(dot(d, ux)) <= 0.5 * W.a0 - m && fabs(dot(d, uy)) <= 0.5 * W.a2 - m;
        } else if (W.shape == SHAPE_CYL || W.shape == SHAPE_INNER_CYL) {
            in = fabs(dot(d, uz)) <= 0.5 * W.a1 - m;
        }
        if (in) meta[e] |= META_INTERIOR;
    }
}

// Spheres whose next step skips the walk: the tick's own test, with the current bound.
__global__ void __launch_bounds__(TPB) k_quiet_count(uint32_t n, const float2* __restrict__ clear,
                                                     const uint8_t* __restrict__ qcnt, const float* __restrict__ disp,
                                                     unsigned* __restrict__ count) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool q = i < n && qcnt[i] >= 2u && 2.0f * disp[0] <= clear[i].x && disp[1] <= clear[i].y;
    const unsigned m = __ballot_sync(0xffffffffu, q);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(count, (unsigned)__popc(m));
}

// Wall entries of every sphere, in ascending entry order, keyed by the wall's global index.
__global__ void __launch_bounds__(TPB) k_wall_count(uint32_t n, const uint32_t* __restrict__ ptr,
                                                    const uint32_t* __restrict__ ent, uint32_t* __restrict__ cnt) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t c = 0;
    for (uint32_t e = ptr[i]; e < ptr[i + 1]; ++e) c += (ent[e] & WALL_BIT) ? 1u : 0u;
    cnt[i] = c;
}
__global__ void __launch_bounds__(TPB) k_wall_fill(uint32_t n, const uint32_t* __restrict__ ptr,
                                                   const uint32_t* __restrict__ ent, const uint32_t* __restrict__ off,
                                                   const uint32_t* __restrict__ gidx, uint32_t* __restrict__ key,
                                                   uint32_t* __restrict__ val) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t o = off[i];
    for (uint32_t e = ptr[i]; e < ptr[i + 1]; ++e)
        if (ent[e] & WALL_BIT) {
            key[o] = gidx[ent[e] & ~WALL_BIT];
            val[o] = e;
            ++o;
        }
}
__global__ void __launch_bounds__(TPB) k_wall_ptr(uint32_t nglob, const uint32_t* __restrict__ key, uint32_t m,
                                                  uint32_t* __restrict__ wptr) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q > nglob) return;
    uint32_t lo = 0, hi = m;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (key[mid] < q) lo = mid + 1; else hi = mid;
    }
    wptr[q] = lo;
}

// Impulse on each wall, summed exactly: the six components of every wall entry are scaled by a
// power of two fixed by the wall's largest entry (|x| 2^s <= 2^42) and added as 64-bit integers.
// Integer addition is associative, so the sum is the same in any order and in parallel, and
// entries that carry zero (spheres near the wall but not touching it) change nothing: the
// result does not depend on the skin, on the list's rebuilds or on the scene's place in a
// batch.  Relative resolution 2^-42 of the largest term, far below the FP32 inputs' rounding.
__device__ __forceinline__ int wall_scale(unsigned maxbits) {
    const float m = __uint_as_float(maxbits);
    return m > 0.0f ? 42 - ilogbf(m) : 0;
}

__global__ void __launch_bounds__(TPB) k_wall_max(uint32_t nw, const uint32_t* __restrict__ wkey,
                                                  const uint32_t* __restrict__ wval, const float* __restrict__ wimp,
                                                  unsigned* __restrict__ wmax) {
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nw) return;
    const float* o = wimp + 6 * (size_t)wval[e];
    const float a = fmaxf(fmaxf(fabsf(o[0]), fabsf(o[1])), fabsf(o[2]));
    const float b = fmaxf(fmaxf(fabsf(o[3]), fabsf(o[4])), fabsf(o[5]));
    if (a > 0.0f) atomicMax(wmax + 2 * wkey[e], __float_as_uint(a));
    if (b > 0.0f) atomicMax(wmax + 2 * wkey[e] + 1, __float_as_uint(b));
}

__global__ void __launch_bounds__(TPB) k_wall_acc(uint32_t nw, const uint32_t* __restrict__ wkey,
                                                  const uint32_t* __restrict__ wval, const float* __restrict__ wimp,
                                                  const unsigned* __restrict__ wmax,
                                                  unsigned long long* __restrict__ wacc) {
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nw) return;
    const uint32_t q = wkey[e];
    const float* o = wimp + 6 * (size_t)wval[e];
    const int s0 = wall_scale(wmax[2 * q]), s1 = wall_scale(wmax[2 * q + 1]);
    for (int k = 0; k < 6; ++k) {
        const float x = o[k];
        if (x == 0.0f) continue;
        const long long v = __double2ll_rn(ldexp((double)x, k < 3 ? s0 : s1));
        atomicAdd(wacc + 6 * (size_t)q + k, (unsigned long long)v);
    }
}

__global__ void k_wall_fin(uint32_t nglob, const uint32_t* __restrict__ glob, const unsigned* __restrict__ wmax,
                           const unsigned long long* __restrict__ wacc, const uint32_t* __restrict__ model_of,
                           const ModelDev* __restrict__ models, const SceneDev* __restrict__ scenes,
                           const uint32_t* __restrict__ scene_of, const double* __restrict__ gfield,
                           double4_32a* __restrict__ imp, double4_32a* __restrict__ aimp) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nglob) return;
    const int s0 = wall_scale(wmax[2 * q]), s1 = wall_scale(wmax[2 * q + 1]);
    const unsigned long long* a = wacc + 6 * (size_t)q;
    d3 J = mk(ldexp((double)(long long)a[0], -s0), ldexp((double)(long long)a[1], -s0),
              ldexp((double)(long long)a[2], -s0));
    const d3 JA = mk(ldexp((double)(long long)a[3], -s1), ldexp((double)(long long)a[4], -s1),
                     ldexp((double)(long long)a[5], -s1));
    const uint32_t w = glob[q];
    const ModelDev& M = models[model_of[w]];
    const uint32_t sc = scene_of[w];
    const double dt = scenes[sc].dt;
    const d3 fimp = muls(mk(gfield[3 * sc], gfield[3 * sc + 1], gfield[3 * sc + 2]), dt);
    J = add(J, muls(fimp, M.sudo));
    J = add(J, smul(dt, mk(M.ext[0], M.ext[1], M.ext[2])));
    st(imp, w, J, 0.0);
    st(aimp, w, JA, 0.0);
}

// Contact activity of every owner entry at the current positions (for queries).
__global__ void __launch_bounds__(TPB) k_active(uint32_t n, TickArgs a, uint8_t* __restrict__ act) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t mi = a.model_of[i];
    for (uint32_t e = a.nptr[i]; e < a.nptr[i + 1]; ++e) {
        act[e] = 0;
        if (a.nslot[e] != e) continue;
        const uint32_t ent = a.nent[e];
        const uint32_t j = ent & ~WALL_BIT;
        const bool wall = ent & WALL_BIT;
        const uint32_t mj = a.model_of[j];
        bool i_slave = true;
        if (!wall) {
            const ModelDev& M = a.models[mi];
            const ModelDev& N = a.models[mj];
            if (M.density == 0.0 && N.density != 0.0) i_slave = false;
            else if (N.density == 0.0 && M.density != 0.0) i_slave = true;
            else i_slave = a.ext_of[i] < a.ext_of[j];
        }
        const uint32_t s = i_slave ? i : j, m = i_slave ? j : i;
        const uint32_t pi = pidx(a.scenes[a.scene_of[i]], i_slave ? mi : mj, i_slave ? mj : mi);
        const PairParam& P = a.params[pi];
        if (P.cd == 0) continue;
        const double4_32a gg = a.geom[pi];
        const d3 Ps = ld(a.xA, s), Pm = ld(a.xA, m);
        double depth;
        if (P.cd == CD_SS) {
            d3 d = xsub(Pm, Ps);
            const Periodic& pb = a.scenes[a.scene_of[i]].pb;
            if (pb.on) d = min_image(pb, d);      // CDSphere2Sphere.cpp:19-22
            depth = __dsub_rn(__dadd_rn(gg.x, gg.y), xlen(d));
        } else {
            d3 nd, pt;
            depth = wall_detect(P.cd, gg.x, gg.y, gg.z, gg.w, Ps, Pm, ld(a.ox, m), ld(a.oz, m), nd, pt,
                                P.cd == CD_SHP ? a.hole[pi] : make_double4_32a(0, 0, 0, 0));
        }
        act[e] = depth > 0.0 ? PF_ACTIVE_BIT : 0;
    }
}

__global__ void __launch_bounds__(TPB) k_pack3m(uint32_t n, const double* __restrict__ src, double4_32a* __restrict__ dst) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = make_double4_32a(src[3 * (size_t)i], src[3 * (size_t)i + 1], src[3 * (size_t)i + 2], 0.0);
}
// vedo_gpu_set_state: one field of every object from the staged host copy.  With `jump`, the
// field is the position and each sphere's jump (rounded up) joins a maximum, so that the list
// can stay when the displacement bound absorbs it; any change to a wall's position, velocity,
// angular velocity or orientation is flagged (its cached motion terms need a rebuild).
__global__ void __launch_bounds__(TPB) k_place(uint32_t n, const double* __restrict__ src, double4_32a* __restrict__ dst,
                                               const uint32_t* __restrict__ ext_of,
                                               const uint32_t* __restrict__ model_of,
                                               const ModelDev* __restrict__ models, int wall_field,
                                               unsigned* __restrict__ jump, unsigned* __restrict__ wall_moved) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float d = 0.0f;
    if (i < n) {
        const size_t e = ext_of[i];                   // the caller's index of stored object i
        const double nx = src[3 * e], ny = src[3 * e + 1], nz = src[3 * e + 2];
        const double4_32a o = dst[i];
        if (models[model_of[i]].scope == SCOPE_LOCAL) {
            if (jump) {
                const double dx = __dsub_rn(nx, o.x), dy = __dsub_rn(ny, o.y), dz = __dsub_rn(nz, o.z);
                const double l = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
                d = __fmul_ru(__double2float_ru(l), 1.000001f);
                if (!(d == d)) d = 3.0e38f;            // a NaN jump spends the list
            }
        } else if (wall_field && (nx != o.x || ny != o.y || nz != o.z)) {
            atomicOr(wall_moved, 1u);
        }
        dst[i] = make_double4_32a(nx, ny, nz, 0.0);
    }
    if (jump) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) d = fmaxf(d, __shfl_xor_sync(0xffffffffu, d, o));
        if ((threadIdx.x & 31) == 0 && d > 0.0f) atomicMax(jump, __float_as_uint(d));
    }
}
// n objects of the caller's order starting at `off` into [n][3] doubles: object off + i is
// stored at int_of[off + i]
__global__ void __launch_bounds__(TPB) k_unpack3m(uint32_t n, uint32_t off, const uint32_t* __restrict__ int_of,
                                                  const double4_32a* __restrict__ src, double* __restrict__ dst) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const double4_32a v = src[int_of[off + i]];
        dst[3 * (size_t)i] = v.x;
        dst[3 * (size_t)i + 1] = v.y;
        dst[3 * (size_t)i + 2] = v.z;
    }
}
// [n][3] doubles of the caller's order into storage order
__global__ void __launch_bounds__(TPB) k_gather3(uint32_t n, const uint32_t* __restrict__ ext_of,
                                                 const double* __restrict__ src, double* __restrict__ dst) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t e = ext_of[i];
    dst[3 * (size_t)i] = src[3 * e];
    dst[3 * (size_t)i + 1] = src[3 * e + 1];
    dst[3 * (size_t)i + 2] = src[3 * e + 2];
}
// positions and models in the caller's order, for the observables that list every object
__global__ void __launch_bounds__(TPB) k_to_caller(uint32_t n, const uint32_t* __restrict__ int_of,
                                                   const double4_32a* __restrict__ x, const uint32_t* __restrict__ model_of,
                                                   double4_32a* __restrict__ xe, uint32_t* __restrict__ me) {
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const uint32_t i = int_of[e];
    xe[e] = x[i];
    me[e] = model_of[i];
}
// positions as hi/lo FP32 splits, for the stored way of the double-float pair test
__global__ void __launch_bounds__(TPB) k_split(uint32_t n, const double4_32a* __restrict__ x, float4* __restrict__ xs) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double4_32a p = x[i];
    float4 h, l;
    split32(p.x, h.x, l.x);
    split32(p.y, h.y, l.y);
    split32(p.z, h.z, l.z);
    h.w = l.w = 0.0f;
    xs[2 * (size_t)i] = h;
    xs[2 * (size_t)i + 1] = l;
}
__global__ void __launch_bounds__(TPB) k_copy32(uint32_t n, const double4_32a* __restrict__ v, float4* __restrict__ o) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const double4_32a q = v[i];
        o[i] = make_float4((float)q.x, (float)q.y, (float)q.z, 0.0f);
    }
}
// Spinning orbital plates whose sweeping edges may meet a sphere: edge[q] is set when a sphere
// lies within reach + skin_w of the plate's plane (the band it can reach before the list is
// spent) but outside the plate's inscribed circle shrunk by skin_w.  Inside that circle the
// plate covers the sphere's projection whatever its turn, so a plate turning about its own
// normal changes no distance there.
__global__ void __launch_bounds__(TPB) k_wall_edge(uint32_t n, const uint32_t* __restrict__ model_of,
                                                   const ModelDev* __restrict__ models,
                                                   const uint32_t* __restrict__ scene_of,
                                                   const SceneDev* __restrict__ scenes,
                                                   const uint32_t* __restrict__ glob,
                                                   const double4_32a* __restrict__ x,
                                                   const double4_32a* __restrict__ oz, float skin_w,
                                                   unsigned* __restrict__ edge) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const ModelDev& M = models[model_of[i]];
    if (M.scope != SCOPE_LOCAL) return;
    const SceneDev& S = scenes[scene_of[i]];
    const d3 P = ld(x, i);
    for (uint32_t q = S.wall_beg; q < S.wall_end; ++q) {
        const uint32_t w = glob[q];
        const ModelDev& W = models[model_of[w]];
        if (W.behavior != BEH_ORBITAL || W.shape != SHAPE_PLATE) continue;
        const d3 Oz = ld(oz, w);
        const double lz = len(Oz);
        if (!(lz > 0.0)) continue;
        const d3 d = sub(P, ld(x, w));
        const double sd = dot(d, Oz) / lz;
        const double tol = 1e-9 * (len(d) + 1.0);
        if (fabs(sd) > M.range + 0.5 * W.a1 + skin_w + tol) continue;
        const double rho = sqrt(fmax(dot(d, d) - sd * sd, 0.0));
        if (rho > 0.5 * fmin(W.a0, W.a2) - skin_w - tol) atomicOr(&edge[q], 1u);
    }
}

// Bound on how fast an orbital wall's plane (plate) or axis line (cylinder) can move towards
// a sphere that may touch it: |V| + |omega| R, R = half the wall's diagonal + 2 r_max.  A rod
// spinning about its own axis keeps its surface, and a plate spinning about its own normal
// keeps its plane and, where no sphere is near its sweeping edges (k_wall_edge), every
// distance: then only the normal (plate) or transverse (rod) part of V counts.  V and omega of
// an orbital wall are prescribed, so the bound holds until the state is set again.
__global__ void k_wall_speed(uint32_t nglob, const uint32_t* __restrict__ glob, const uint32_t* __restrict__ model_of,
                             const ModelDev* __restrict__ models, const double4_32a* __restrict__ v64,
                             const double4_32a* __restrict__ w64, const double4_32a* __restrict__ oz, float reach,
                             const unsigned* __restrict__ edge, unsigned* __restrict__ out_bits) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nglob) return;
    const uint32_t w = glob[q];
    const ModelDev& M = models[model_of[w]];
    if (M.behavior != BEH_ORBITAL) return;
    const d3 V = ld(v64, w), W = ld(w64, w), Oz = ld(oz, w);
    const double lz = len(Oz);
    // the wall's farthest point from its centre (a hollow cylinder: its rim), plus the reach
    const double R = (M.shape == SHAPE_INNER_CYL ? sqrt(M.a0 * M.a0 + 0.25 * M.a1 * M.a1)
                                                 : 0.5 * sqrt(M.a0 * M.a0 + M.a1 * M.a1 + M.a2 * M.a2)) + (double)reach;
    double sp = len(V) + len(W) * R;
    if (lz > 0.0) {
        const d3 u = muls(Oz, 1.0 / lz);
        const d3 c = cross(W, u);
        if (len(c) <= 1e-12 * len(W) && !(M.shape == SHAPE_PLATE && edge[q])) {   // spins about its normal / axis
            const double vn = dot(V, u);
            sp = (M.shape == SHAPE_PLATE) ? fabs(vn) : len(sub(V, muls(u, vn)));
        }
    }
    atomicMax(out_bits, __float_as_uint((float)(sp * 1.0001) + 1e-30f));
}

__global__ void __launch_bounds__(TPB) k_wall32(uint32_t n, const uint32_t* __restrict__ model_of,
                                                const ModelDev* __restrict__ models, const double4_32a* __restrict__ ox,
                                                const double4_32a* __restrict__ oz, float4* __restrict__ wall32) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const ModelDev& M = models[model_of[i]];
    if (M.shape == SHAPE_SPHERE) {
        wall32[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return;
    }
    const d3 Ox = ld(ox, i), Oz = ld(oz, i);
    const double lz = len(Oz), lx = len(Ox);
    bool ok = lz > 0.0;
    if (M.shape == SHAPE_PLATE || M.shape == SHAPE_HOLED) ok = ok && lx > 0.0 && fabs(dot(Ox, Oz)) <= 1e-9 * lx * lz;
    wall32[i] = ok ? make_float4((float)(Oz.x / lz), (float)(Oz.y / lz), (float)(Oz.z / lz), 1e-30f)   // no drift yet
                   : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

// ---- moving scenes into a new engine (continuous batching) --------------------------------
// One entry per scene of the new engine, in object order: its objects come from the previous
// engine's device arrays (kind 0) or from host data staged on the device (kind 1).
struct MoveScene {
    uint32_t new_off, nobj, src_off, kind;
};

__device__ __forceinline__ const MoveScene& find_move(const MoveScene* __restrict__ mv, uint32_t nmv, uint32_t i) {
    uint32_t lo = 0, hi = nmv;                      // last entry with new_off <= i
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (mv[mid].new_off <= i) lo = mid; else hi = mid;
    }
    return mv[lo];
}

struct StateArrays {
    const double4_32a *x, *v, *w, *ox, *oz, *imp, *aimp;
};

__global__ void __launch_bounds__(TPB) k_move_state(uint32_t n, const MoveScene* __restrict__ mv, uint32_t nmv,
                                                    StateArrays prev, const double* __restrict__ stage,
                                                    size_t stage_stride, double4_32a* __restrict__ x,
                                                    double4_32a* __restrict__ v, double4_32a* __restrict__ w,
                                                    double4_32a* __restrict__ ox, double4_32a* __restrict__ oz,
                                                    double4_32a* __restrict__ imp, double4_32a* __restrict__ aimp,
                                                    float4* __restrict__ v32, float4* __restrict__ w32) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const MoveScene& m = find_move(mv, nmv, i);
    const uint32_t j = m.src_off + (i - m.new_off);
    double4_32a* dst[7] = {x, v, w, ox, oz, imp, aimp};
    if (m.kind == 0) {
        const double4_32a* src[7] = {prev.x, prev.v, prev.w, prev.ox, prev.oz, prev.imp, prev.aimp};
        for (int k = 0; k < 7; ++k) dst[k][i] = src[k][j];
    } else {
        for (int k = 0; k < 7; ++k) {
            const double* q = stage + (size_t)k * stage_stride + 3 * (size_t)j;
            dst[k][i] = make_double4_32a(q[0], q[1], q[2], 0.0);
        }
    }
    const double4_32a vv = v[i], ww = w[i];
    v32[i] = make_float4((float)vv.x, (float)vv.y, (float)vv.z, 0.0f);
    w32[i] = make_float4((float)ww.x, (float)ww.y, (float)ww.z, 0.0f);
}

// A neighbour list (CSR rows, history at the same entry positions) that the first rebuild
// of the new engine carries histories from: rows of kept scenes are copied from the previous
// engine's current list with object and entry indices shifted; rows of new scenes come from
// their IactRecordTab records, staged on the device.
struct ListArrays {
    const uint32_t *ptr, *ent, *slot;
    const float4* h;
    const uint8_t* f;
};

__global__ void __launch_bounds__(TPB) k_row_count(uint32_t n, const MoveScene* __restrict__ mv, uint32_t nmv,
                                                   ListArrays prev, ListArrays stage, uint32_t* __restrict__ cnt) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n) return;
    if (i == n) { cnt[n] = 0u; return; }
    const MoveScene& m = find_move(mv, nmv, i);
    const uint32_t j = m.src_off + (i - m.new_off);
    const ListArrays& L = m.kind == 0 ? prev : stage;
    cnt[i] = L.ptr ? L.ptr[j + 1] - L.ptr[j] : 0u;
}

__global__ void __launch_bounds__(TPB) k_row_fill(uint32_t n, const MoveScene* __restrict__ mv, uint32_t nmv,
                                                  ListArrays prev, ListArrays stage, const uint32_t* __restrict__ ptr,
                                                  uint32_t* __restrict__ ent, uint32_t* __restrict__ slot,
                                                  float4* __restrict__ h, uint8_t* __restrict__ f) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const MoveScene& m = find_move(mv, nmv, i);
    const uint32_t j = m.src_off + (i - m.new_off);
    const ListArrays& L = m.kind == 0 ? prev : stage;
    if (!L.ptr) return;
    // object indices of a kept scene move by the scene's shift; staged rows already use the
    // new indices.  Entry indices (slots) move by the shift of the scene's first row.
    const uint32_t dobj = m.kind == 0 ? m.new_off - m.src_off : 0u;
    const uint32_t dent = ptr[m.new_off] - L.ptr[m.src_off];
    const uint32_t b = L.ptr[j], e1 = L.ptr[j + 1], o = ptr[i];
    for (uint32_t q = b; q < e1; ++q) {
        const uint32_t v = L.ent[q];
        ent[o + (q - b)] = (v & WALL_BIT) | ((v & ~WALL_BIT) + dobj);
        slot[o + (q - b)] = L.slot[q] + dent;
        h[o + (q - b)] = L.h[q];
        f[o + (q - b)] = L.f[q];
    }
}

// Morton (Z-order) code of a cell triple, 21 bits per axis.
inline uint64_t morton3(uint64_t x, uint64_t y, uint64_t z) {
    auto spread = [](uint64_t v) {
        v &= 0x1fffffull;
        v = (v | v << 32) & 0x1f00000000ffffull;
        v = (v | v << 16) & 0x1f0000ff0000ffull;
        v = (v | v << 8) & 0x100f00f00f00f00full;
        v = (v | v << 4) & 0x10c30c30c30c30c3ull;
        v = (v | v << 2) & 0x1249249249249249ull;
        return v;
    };
    return spread(x) | spread(y) << 1 | spread(z) << 2;
}

// The order in which the engine stores a scene's objects: its spheres by the Z-order code of
// the cell of edge 2 r_max that holds their centre (ties by index), then its walls in their
// own order.  Spheres near one another in space sit near one another in memory, so the
// neighbours a warp gathers share cache lines whatever order the caller numbered them in.
// Returns perm with perm[internal] = the caller's (scene-local) index.
std::vector<uint32_t> spatial_order(const HScene& h, const Tables& t) {
    std::vector<uint32_t> sph, wal;
    double lo[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, rmax = 0.0;
    for (uint32_t i = 0; i < h.n; ++i) {
        const ModelDev& M = t.models[h.model_of[i]];
        if (M.scope == SCOPE_LOCAL) {
            sph.push_back(i);
            rmax = std::max(rmax, M.a0);
            for (int k = 0; k < 3; ++k) lo[k] = std::min(lo[k], h.pos[3 * (size_t)i + k]);
        } else {
            wal.push_back(i);
        }
    }
    const double cell = rmax > 0.0 ? 2.0 * rmax : 1.0;
    std::vector<std::pair<uint64_t, uint32_t>> key(sph.size());
    for (size_t q = 0; q < sph.size(); ++q) {
        uint64_t c[3];
        for (int k = 0; k < 3; ++k) {
            const double f = std::floor((h.pos[3 * (size_t)sph[q] + k] - lo[k]) / cell);
            c[k] = f > 0.0 ? (uint64_t)std::min(f, 2097151.0) : 0u;   // NaN and negative: cell 0
        }
        key[q] = {morton3(c[0], c[1], c[2]), sph[q]};
    }
    std::sort(key.begin(), key.end());
    std::vector<uint32_t> perm;
    perm.reserve(h.n);
    for (const auto& kv : key) perm.push_back(kv.second);
    perm.insert(perm.end(), wal.begin(), wal.end());
    return perm;
}

}  // namespace

// ==========================================================================================
class MixedEngine : public EngineBase {
public:
    ~MixedEngine() override;
    int init(const HScene& scene, const vedo_engine_opts& opts) override {
        return init_batch(std::vector<const HScene*>{&scene}, opts);
    }
    int init_batch(const std::vector<const HScene*>& scenes, const vedo_engine_opts& opts) {
        std::vector<SceneSource> src;
        for (const HScene* h : scenes) src.push_back(SceneSource{h, -1});
        return init_from(src, nullptr, opts);
    }
    // A scene of a new engine: a host scene (prev_scene < 0) or scene prev_scene of `prev`,
    // whose state and contact history move over on the device.
    struct SceneSource {
        const HScene* host;
        int prev_scene;
    };
    int init_from(const std::vector<SceneSource>& src, const MixedEngine* prev, const vedo_engine_opts& opts);
    // Freeze (or resume) one scene: a frozen scene's objects keep their state and its time stops.
    int set_scene_active(uint32_t s, bool on);
    bool scene_active(uint32_t s) const { return s < sc_.size() && sc_[s].active; }
    // State of objects [off, off + cnt) into [cnt][3] host arrays.
    int get_state_slice(uint32_t off, uint32_t cnt, const vedo_state_view& v);
    uint64_t steps_of_scene(uint32_t s) const { return s < sc_.size() ? sc_[s].steps : 0; }
    int run(uint32_t nsteps, int* keep_running) override;
    int get_state(const vedo_state_view& v) override;
    int set_state(const vedo_state_view& v) override;
    int num_interactions(uint32_t* n) override;
    int get_interactions(const vedo_contact_view& v) override;
    int get_observables(double out[13]) override;
    int write_ido(const char* path) override;
    int coordination(uint32_t* below, uint32_t* touching, const double* box, double* average) override;
    int write_vtk(const char* path, int with_coordination) override;
    DeviceObjects objects();
    int caller_view();
    double time() const override { return sc_.empty() ? 0.0 : sc_[0].t; }
    uint64_t steps() const override { return round_; }
    uint64_t steps_remaining() const override {
        return sc_.empty() ? 0 : count_steps(sc_[0].t, sc_[0].dt, sc_[0].t_stop);
    }
    uint32_t num_objects() const override { return n_; }
    uint64_t last_profile(double out[4]) const override {
        for (int k = 0; k < 4; ++k) out[k] = prof_[k];
        return launches_;
    }
    void set_profiling(bool on) override { profiling_ = on; }
    const std::string& error() const override { return err_; }
    // batch accessors
    uint32_t num_scenes() const { return (uint32_t)sc_.size(); }
    int scene_range(uint32_t s, uint32_t* off, uint32_t* n) const {
        if (s >= sc_.size()) return VEDO_ERR_INVALID_ARGUMENT;
        *off = sc_[s].obj_off;
        *n = sc_[s].nobj;
        return VEDO_OK;
    }
    double scene_time(uint32_t s) const { return s < sc_.size() ? sc_[s].t : 0.0; }
    int quiet_spheres(uint64_t* count) override;
    int run_with_impulses(const double* impulse, const double* angular_impulse, int* keep_running) override;
    int list_status(double out[6]) override;
    int tuning(float out[6]) const override {
        out[0] = skin_frac_;
        out[1] = cell_scale_;
        out[2] = (float)tpb_;
        out[3] = xs_stored_ ? 1.0f : 0.0f;
        out[4] = pair_pass_ ? 2.0f : (split_tick_ ? 1.0f : 0.0f);
        out[5] = persistent_ ? 1.0f : 0.0f;
        return VEDO_OK;
    }

private:
    struct NList {
        uint32_t cap = 0, ne = 0;
        uint32_t* ptr = nullptr;   // [n+1]
        uint32_t* ent = nullptr;
        uint32_t* slot = nullptr;
        uint32_t* meta = nullptr;
        float4* h[2] = {nullptr, nullptr};
        uint8_t* f[2] = {nullptr, nullptr};
    };
    struct SceneHost {
        uint32_t obj_off = 0, nobj = 0, model_off = 0, nm = 0, pbase = 0, wall_beg = 0, wall_end = 0, nloc = 0;
        double dt = 0, t = 0, t_stop = 0, g[3] = {0, 0, 0};
        float skin = 0, rmax = 0;
        bool active = true;
        uint64_t steps = 0;         // steps this scene has taken (in this engine and before)
        // the scene's objects in the engine's storage order: perm[internal] = the caller's
        // scene-local index (spatial_order)
        std::shared_ptr<const std::vector<uint32_t>> perm;
        Periodic pb{};              // the scene's periodic boundary (on = 0: none)
    };
    int fail(int c, const std::string& m) { err_ = m; return c; }
    int cuda_fail(cudaError_t e, const char* where) {
        err_ = std::string("CUDA error ") + cudaGetErrorString(e) + " at " + where;
        return e == cudaErrorMemoryAllocation ? VEDO_ERR_OUT_OF_MEMORY : VEDO_ERR_CUDA;
    }
    int rebuild();
    void launch_step(bool write_imp);
    cudaError_t launch_err_ = cudaSuccess;   // the first failed launch of the step kernels
    int step_chunk(uint32_t chunk, bool imp_last, float* use_after);
    int autotune(uint32_t max_steps, uint32_t* taken);
    void set_skin(float frac);
    void drop_graphs();
    int ensure_nlist(NList& L, uint32_t cap);
    void free_nlist(NList& L);
    TickArgs args(bool write_imp);
    WallArgs wargs(int c);

    std::vector<std::shared_ptr<const HScene>> host_;   // per scene: models, interactions, initial state
    std::vector<SceneHost> sc_;
    std::vector<SceneDev> sdev_;
    std::vector<ModelDev> models_;
    std::vector<PairParam> params_;
    vedo_engine_opts opts_{};
    std::string err_;
    uint32_t n_ = 0, nm_ = 0, nloc_ = 0, np_ = 0;
    double origin_[3] = {0, 0, 0};
    float dt_max_ = 0.0f, skin_min_ = 0.0f;
    float skin_frac_ = 0.15f;       // skin as a fraction of each scene's largest radius
    float cell_scale_ = 1.0f;       // cell edge = cell_scale * (2 r_max + skin)
    int tpb_ = TPB;                 // threads per block of the tick kernel
    bool tune_pending_ = false;
    // one check interval of steps, by start parity (+1), with the per-kernel timing events of
    // profiling (+2), with the impulse output of a call's last step (+4)
    cudaGraphExec_t graph_[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    uint64_t graph_launches_[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    unsigned ev_flags_ = cudaEventRecordDefault;      // cudaEventRecordExternal while capturing
    std::vector<cudaEvent_t> pev_;  // profiling: per step, events before the tick, after it, after the walls
    uint32_t pev_used_ = 0;
    uint64_t round_ = 0;
    int cur_ = 0;                   // which of the A/B buffers is "A" (current)
    bool need_rebuild_ = true;
    bool profiling_ = false;
    double prof_[4] = {0, 0, 0, 0};
    uint64_t prof_ticks_ = 0;       // tick launches timed in the last run (profiling on)
    uint64_t launches_ = 0;
    uint64_t rebuilds_ = 0;
    uint64_t since_rebuild_ = 0;
    int law_ = 0;                   // the single equation type of the batch, or 0 (several laws)
    cudaStream_t stream_ = nullptr;
    cudaEvent_t ev_[4] = {};

    ModelDev* d_models_ = nullptr;
    PairParam* d_params_ = nullptr;
    float* d_pc32_ = nullptr;
    double4_32a* d_geom_ = nullptr;
    double4_32a* d_hole_ = nullptr;                // [nm*nm] hole radius and offsets (CD_SHP pairs)
    double4_32a* d_rr_ = nullptr;
    float4* d_mf_ = nullptr;
    float* d_reach_ = nullptr;
    uint32_t* d_model_of_ = nullptr;
    uint32_t* d_scene_of_ = nullptr;
    SceneDev* d_scenes_ = nullptr;
    double* d_gfield_ = nullptr;
    uint32_t* d_glob_ = nullptr;
    std::vector<uint32_t> glob_;
    double4_32a* d_x_[2] = {nullptr, nullptr};
    double4_32a *d_v64_ = nullptr, *d_w64_ = nullptr, *d_ox_ = nullptr, *d_oz_ = nullptr;
    double4_32a *d_imp_ = nullptr, *d_aimp_ = nullptr;
    float4* d_v32_[2] = {nullptr, nullptr};
    float4* d_w32_[2] = {nullptr, nullptr};
    float4 *d_pos32_ = nullptr, *d_wall32_ = nullptr;
    float4* d_rr32_ = nullptr;
    float4* d_xs_[2] = {nullptr, nullptr};        // hi/lo position splits by step parity (stored way)
    bool xs_stored_ = false;
    bool split_tick_ = false;                     // light + deferred full tick (identical results)
    uint32_t* d_work_ = nullptr;                  // [n] spheres deferred by the light tick
    bool pair_pass_ = false;                      // prefilter pass, pair pass, per-sphere sums (identical results)
    uint32_t pcap_ = 0;                           // entries the pair pass's buffers hold
    uint4* d_pwork_ = nullptr;                    // [pcap] pairs on the exact path (owner entry, sphere)
    uint8_t* d_xf_ = nullptr;                     // [pcap] entry on the exact path this step
    float4* d_prec_ = nullptr;                    // [pcap][2] each entry's share of its pair
    uint32_t* d_pmir_ = nullptr;                  // [pcap] partner entry of an owner entry
    uint8_t* d_wk_ = nullptr;                     // [n] quiet this step (pair pass)
    unsigned long long* d_xm_ = nullptr;          // [n] exact-path mask of the first 64 entries (pair pass)
    int ensure_pair_bufs(uint32_t ne);
    void free_pair_bufs();
    void fill_mirror(const NList& L) {
        k_mirror<false><<<nblk(n_), TPB, 0, stream_>>>(n_, L.ptr, L.slot, d_pmir_);
        k_mirror<true><<<nblk(n_), TPB, 0, stream_>>>(n_, L.ptr, L.slot, d_pmir_);
    }
    // blocks of tpb_ threads of kernel k resident on the whole GPU at once (cached per kernel
    // and block size)
    const void* grid_k_ = nullptr;
    int grid_tpb_ = 0;
    unsigned grid_blocks_ = 0;
    unsigned resident_grid(const void* k) {
        if (k != grid_k_ || tpb_ != grid_tpb_) {
            int b = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k, tpb_, 0) != cudaSuccess || b < 1) b = 1;
            grid_k_ = k;
            grid_tpb_ = tpb_;
            grid_blocks_ = (unsigned)b * (unsigned)sms_;
        }
        return grid_blocks_;
    }
    bool quiet_ok_ = true;                        // quiet spheres skip their walk (identical results)
    // one cooperative launch per check interval (the full tick or the pair pass; identical results)
    bool persistent_ = false;
    const void* pk_ = nullptr;                    // the persistent kernel of the grid below
    unsigned pk_grid_ = 0;
    bool persist_usable() const {
        return persistent_ && !split_tick_ && !dyn_walls_ && !profiling_;
    }
    int launch_persistent(uint32_t chunk);
    bool orient_ = false;                         // integrate the spheres' orientations
    bool any_pbc_ = false;                        // a scene has a periodic boundary
    bool dyn_walls_ = false;                      // a wall is mobile or constrained (moved by its impulses)
    float4* d_tdav_ = nullptr;                    // [n] angular velocity increments (orientations)
    int sms_ = 1;                                 // streaming multiprocessors of the device
    float2* d_clear_ = nullptr;                   // [n] quiet-sphere pad limits of the current list
    double* d_ext_ = nullptr;                     // [2][n][3] external impulses of run_with_impulses
    bool ext_on_ = false;
    unsigned* d_vred_ = nullptr;                  // [scenes][6] velocity ranges at the rebuild
    float pos_eps_ = 0.0f;                        // FP64 rounding of a position update (bound)
    uint8_t* d_qcnt_ = nullptr;                   // [n] clean walks since the rebuild (0..2)
    unsigned* d_red_ = nullptr;     // [8] vmax bits, [9], [10] scan totals, [11] identity steps, [12] wall speed
    unsigned* d_sred_ = nullptr;    // [scenes][8] per-scene bounds
    float* d_disp_ = nullptr;       // [2][4] displacement bounds and steps since the rebuild, by step parity (cur_)
    int* d_err_ = nullptr;
    NList nl_[2];
    int nlc_ = 0;                   // current neighbour list
    Scratch scratch_;
    uint64_t *d_key_ = nullptr, *d_key_alt_ = nullptr;
    uint32_t *d_sid_ = nullptr, *d_sid_alt_ = nullptr, *d_cnt_ = nullptr;
    uint32_t *d_gs_ = nullptr, *d_ge_ = nullptr;
    uint64_t grid_cap_ = 0;
    uint8_t* d_act_ = nullptr;
    uint32_t act_cap_ = 0;
    uint32_t* d_gidx_ = nullptr;
    uint32_t *d_wkey_ = nullptr, *d_wval_ = nullptr, *d_wkey_alt_ = nullptr, *d_wval_alt_ = nullptr, *d_wptr_ = nullptr;
    uint32_t wcap_ = 0, nwall_ent_ = 0;
    float* d_wimp_ = nullptr;
    unsigned long long* d_wred_ = nullptr;
    double4_32a* d_wrot_ = nullptr;          // per wall: half-angle terms of its turn per step
    unsigned* d_wedge_ = nullptr;            // per wall: a sphere is near a spinning plate's sweeping edges
    uint32_t wimp_cap_ = 0;
    double* d_stage_ = nullptr;
    double* d_obs_ = nullptr;
    // storage order: internal index -> the caller's (global) index, and back
    uint32_t* d_ext_of_ = nullptr;
    uint32_t* d_int_of_ = nullptr;
    double4_32a* d_xe_ = nullptr;                 // positions in the caller's order (observables)
    uint32_t* d_model_e_ = nullptr;               // models in the caller's order (observables)
};

#define MCK(call)                                                 \
    do {                                                          \
        cudaError_t _e = (call);                                  \
        if (_e != cudaSuccess) return cuda_fail(_e, #call);       \
    } while (0)

template <class T>
static cudaError_t mal(T** p, size_t count) {
    *p = nullptr;
    return cudaMalloc((void**)p, sizeof(T) * (count ? count : 1));
}

void MixedEngine::free_nlist(NList& L) {
    cudaFree(L.ptr); cudaFree(L.ent); cudaFree(L.slot); cudaFree(L.meta);
    for (int b = 0; b < 2; ++b) { cudaFree(L.h[b]); cudaFree(L.f[b]); }
    L = NList{};
}

// The pair pass's per-entry buffers, sized to the list (allocated only while the pair pass is
// used or tried).
int MixedEngine::ensure_pair_bufs(uint32_t ne) {
    if (!d_wk_) MCK(mal(&d_wk_, n_));
    if (!d_xm_) MCK(mal(&d_xm_, n_));
    if (ne <= pcap_ && d_prec_) return VEDO_OK;
    for (void* p : {(void*)d_pwork_, (void*)d_xf_, (void*)d_prec_, (void*)d_pmir_})
        if (p) cudaFree(p);
    const uint64_t c = std::max<uint64_t>(1024, (uint64_t)ne + ne / 4);
    pcap_ = (uint32_t)std::min<uint64_t>(c, 0x7fffffffull);
    MCK(mal(&d_pwork_, pcap_));
    MCK(mal(&d_xf_, pcap_));
    MCK(mal(&d_prec_, 2 * (size_t)pcap_));
    MCK(mal(&d_pmir_, pcap_));
    return VEDO_OK;
}
void MixedEngine::free_pair_bufs() {
    for (void* p : {(void*)d_pwork_, (void*)d_xf_, (void*)d_prec_, (void*)d_pmir_, (void*)d_wk_, (void*)d_xm_})
        if (p) cudaFree(p);
    d_pwork_ = nullptr;
    d_xf_ = nullptr;
    d_prec_ = nullptr;
    d_pmir_ = nullptr;
    d_wk_ = nullptr;
    d_xm_ = nullptr;
    pcap_ = 0;
}

int MixedEngine::ensure_nlist(NList& L, uint32_t cap) {
    if (!L.ptr) MCK(mal(&L.ptr, (size_t)n_ + 1));
    if (cap <= L.cap && L.ent) return VEDO_OK;
    uint32_t* ptr = L.ptr;
    L.ptr = nullptr;
    free_nlist(L);
    L.ptr = ptr;
    uint64_t c = std::max<uint64_t>(1024, (uint64_t)cap + cap / 4);
    L.cap = (uint32_t)std::min<uint64_t>(c, 0x7fffffffull);
    MCK(mal(&L.ent, L.cap));
    MCK(mal(&L.slot, L.cap));
    MCK(mal(&L.meta, L.cap));
    for (int b = 0; b < 2; ++b) {
        MCK(mal(&L.h[b], L.cap));
        MCK(mal(&L.f[b], L.cap));
    }
    return VEDO_OK;
}

MixedEngine::~MixedEngine() {
    if (stream_) cudaStreamSynchronize(stream_);
    free_nlist(nl_[0]);
    free_nlist(nl_[1]);
    void* ptrs[] = {d_models_, d_params_, d_pc32_, d_geom_, d_hole_, d_rr_, d_mf_, d_reach_, d_model_of_, d_scene_of_,
                    d_scenes_, d_gfield_, d_glob_, d_x_[0], d_x_[1], d_v64_, d_w64_, d_ox_, d_oz_, d_imp_, d_aimp_,
                    d_v32_[0], d_v32_[1], d_w32_[0], d_w32_[1], d_rr32_, d_xs_[0], d_xs_[1], d_work_, d_tdav_, d_clear_, d_vred_, d_ext_, d_qcnt_, d_pos32_, d_wall32_, d_red_, d_sred_, d_disp_, d_err_,
                    d_key_, d_key_alt_, d_sid_, d_sid_alt_, d_cnt_, d_gs_, d_ge_, d_act_, d_stage_, d_obs_, d_gidx_,
                    d_wkey_, d_wval_, d_wkey_alt_, d_wval_alt_, d_wptr_, d_wimp_, d_wred_, d_wrot_, d_wedge_, d_ext_of_, d_int_of_, d_xe_, d_model_e_};
    for (void* p : ptrs) if (p) cudaFree(p);
    free_pair_bufs();
    drop_graphs();
    for (auto& e : pev_) cudaEventDestroy(e);
    for (auto& e : ev_) if (e) cudaEventDestroy(e);
    if (stream_) cudaStreamDestroy(stream_);
}

void MixedEngine::drop_graphs() {
    for (auto& g : graph_) {
        if (g) cudaGraphExecDestroy(g);
        g = nullptr;
    }
}

void MixedEngine::set_skin(float frac) {
    skin_frac_ = frac;
    for (size_t k = 0; k < sc_.size(); ++k) {
        sc_[k].skin = frac * sc_[k].rmax;
        skin_min_ = k == 0 ? sc_[k].skin : std::min(skin_min_, sc_[k].skin);
    }
    need_rebuild_ = true;
}

int MixedEngine::init_from(const std::vector<SceneSource>& src, const MixedEngine* prev,
                           const vedo_engine_opts& opts) {
    opts_ = opts;
    if (opts_.check_interval == 0) opts_.check_interval = 10;
    skin_frac_ = opts.skin > 0 ? opts.skin : 0.15f;
    cell_scale_ = opts.cell_scale >= 1.0f ? opts.cell_scale : 1.0f;
    tpb_ = opts.tick_block ? (int)opts.tick_block : TPB;
    if (tpb_ < 32 || tpb_ > TPB || tpb_ % 32) return fail(VEDO_ERR_INVALID_ARGUMENT, "tick_block must be 32..256, a multiple of 32");
    tune_pending_ = opts.autotune != 0;
    xs_stored_ = opts.stored_splits != 0;
    split_tick_ = opts.split_tick == 1;
    pair_pass_ = opts.split_tick == 2;
    if (opts.split_tick > 2) return fail(VEDO_ERR_INVALID_ARGUMENT, "split_tick must be 0, 1 or 2");
    quiet_ok_ = opts.full_walks == 0;
    orient_ = opts.orientations != 0;
    persistent_ = opts.persistent != 0;
    if (opts.persistent > 1) return fail(VEDO_ERR_INVALID_ARGUMENT, "persistent must be 0 or 1");
    if (prev) {                    // a repacked engine keeps the tuning of the one it replaces
        skin_frac_ = prev->skin_frac_;
        cell_scale_ = prev->cell_scale_;
        tpb_ = prev->tpb_;
        xs_stored_ = prev->xs_stored_;
        split_tick_ = prev->split_tick_;
        pair_pass_ = prev->pair_pass_;
        quiet_ok_ = prev->quiet_ok_;
        persistent_ = prev->persistent_;
        tune_pending_ = prev->tune_pending_;
    }
    if (src.empty()) return fail(VEDO_ERR_INVALID_SCENE, "empty batch");
    // ---- per-scene tables, concatenated
    std::vector<uint32_t> model_of, scene_of, ext_of;
    std::vector<double> st[7];                 // staged host state of the new scenes
    std::vector<double4_32a> geo, rr, hole;
    std::vector<float4> rr32;
    std::vector<float> pc, reach;
    std::vector<float4> mf;
    std::vector<double> gfield;
    std::vector<MoveScene> moves;
    struct Rec { uint32_t a, b; float4 h; uint8_t f; };
    std::vector<std::vector<Rec>> recs;        // per new-scene object offset in staging order
    uint32_t n_stage = 0;
    int law = -1;
    for (const SceneSource& so : src) {
        const bool kept = so.prev_scene >= 0;
        if (kept && (!prev || (size_t)so.prev_scene >= prev->sc_.size()))
            return fail(VEDO_ERR_INVALID_ARGUMENT, "scene source out of range");
        std::shared_ptr<const HScene> hp = kept ? prev->host_[so.prev_scene] : std::make_shared<HScene>(*so.host);
        const HScene& h = *hp;
        host_.push_back(hp);
        Tables t;
        std::string msg;
        int rc = build_tables(h, t, msg);
        if (rc != VEDO_OK) return fail(rc, msg);
        SceneHost S;
        S.pb = t.pbc;
        if (t.pbc.on) {
            // Periodic scenes: sphere pairs take the nearest image and mobile spheres go back into
            // the box after every step.  Walls and spheres that do not move stay where they are,
            // which the reference's wrap agrees with only inside the box: other layouts are refused.
            for (uint32_t i = 0; i < h.n; ++i) {
                const ModelDev& M = t.models[h.model_of[i]];
                const bool moves = M.scope == SCOPE_LOCAL && M.behavior == BEH_MOBILE;
                bool inside = true;
                for (int k = 0; k < 3; ++k) {
                    const double p = h.pos[3 * (size_t)i + k];
                    if (t.pbc.sw[k] && (p < t.pbc.lo[k] || p >= t.pbc.hi[k])) inside = false;
                }
                if (!moves && !inside)
                    return fail(VEDO_ERR_UNSUPPORTED_MODEL, "mixed form, periodic boundary: a wall or a sphere that does "
                                                            "not move lies outside the periodic box");
                if (M.scope != SCOPE_LOCAL && M.behavior == BEH_ORBITAL)
                    for (int k = 0; k < 3; ++k)
                        if (t.pbc.sw[k] && h.vel[3 * (size_t)i + k] != 0.0)
                            return fail(VEDO_ERR_UNSUPPORTED_MODEL, "mixed form, periodic boundary: an orbital wall "
                                                                    "moves along a periodic axis");
            }
            any_pbc_ = true;
        }
        S.obj_off = n_;
        S.nobj = h.n;
        S.model_off = nm_;
        S.nm = (uint32_t)t.models.size();
        S.pbase = np_;
        S.dt = h.time_interval;
        S.t = kept ? prev->sc_[so.prev_scene].t : h.time_current;
        S.steps = kept ? prev->sc_[so.prev_scene].steps : 0;
        S.t_stop = h.time_stop;
        for (int k = 0; k < 3; ++k) S.g[k] = h.g[k];
        double rmax = 0.0;
        S.perm = kept ? prev->sc_[so.prev_scene].perm
                      : std::make_shared<const std::vector<uint32_t>>(spatial_order(h, t));
        const std::vector<uint32_t>& perm = *S.perm;
        std::vector<uint32_t> inv(h.n);
        for (uint32_t q = 0; q < h.n; ++q) inv[perm[q]] = q;
        for (uint32_t q = 0; q < h.n; ++q) ext_of.push_back(n_ + perm[q]);
        S.wall_beg = (uint32_t)glob_.size();
        for (uint32_t i = 0; i < h.n; ++i) {
            const ModelDev& M = t.models[h.model_of[perm[i]]];
            if (M.scope == SCOPE_LOCAL) {
                if (M.shape != SHAPE_SPHERE)
                    return fail(VEDO_ERR_UNSUPPORTED_MODEL, "mixed form: local (scope) objects must be spheres");
                rmax = std::max(rmax, M.a0);
                ++S.nloc;
            } else {
                if (M.behavior == BEH_MOBILE || M.behavior == BEH_CONSTRAINED) dyn_walls_ = true;
                glob_.push_back(n_ + i);
            }
            model_of.push_back(S.model_off + h.model_of[perm[i]]);
            scene_of.push_back((uint32_t)sc_.size());
        }
        S.wall_end = (uint32_t)glob_.size();
        S.rmax = (float)rmax;
        S.skin = skin_frac_ * S.rmax;
        if (kept) {
            moves.push_back(MoveScene{n_, h.n, prev->sc_[so.prev_scene].obj_off, 0u});
        } else {
            moves.push_back(MoveScene{n_, h.n, n_stage, 1u});
            const std::vector<double>* a[7] = {&h.pos, &h.vel, &h.av, &h.ox, &h.oz, &h.imp, &h.aimp};
            for (int k = 0; k < 7; ++k)              // staged in storage order
                for (uint32_t i = 0; i < h.n; ++i)
                    st[k].insert(st[k].end(), a[k]->begin() + 3 * (size_t)perm[i], a[k]->begin() + 3 * (size_t)perm[i] + 3);
            // IactRecordTab records, owned by the lower sphere (or the sphere of a wall pair),
            // with their objects in storage order
            recs.resize((size_t)n_stage + h.n);
            for (uint32_t q = 0; q < h.rec.size(); ++q) {
                uint32_t ra = h.rec.first[q], rb = h.rec.second[q];
                if (ra >= h.n || rb >= h.n) continue;
                ra = inv[ra];
                rb = inv[rb];
                const bool aw = t.models[h.model_of[perm[ra]]].scope != SCOPE_LOCAL;
                const bool bw = t.models[h.model_of[perm[rb]]].scope != SCOPE_LOCAL;
                if (aw && !bw) std::swap(ra, rb);
                else if (!aw && !bw && rb < ra) std::swap(ra, rb);   // the row of the history owner
                Rec r;
                r.a = n_stage + ra;
                r.b = (n_ + rb) | ((aw || bw) ? WALL_BIT : 0u);
                r.h = make_float4((float)h.rec.shear[3 * q], (float)h.rec.shear[3 * q + 1],
                                  (float)h.rec.shear[3 * q + 2], (float)h.rec.kn[q]);
                r.f = (uint8_t)(HF_LAST_CONTACT | HF_LAST_BOND | (h.rec.contact[q] ? HF_CONTACT : 0) |
                                (h.rec.bond[q] ? HF_BOND : 0));
                recs[r.a].push_back(r);
            }
            n_stage += h.n;
        }
        for (const ModelDev& M : t.models) models_.push_back(M);
        const size_t nq = (size_t)S.nm * S.nm;
        for (size_t q = 0; q < nq; ++q) {
            const PairParam& P = t.params[q];
            params_.push_back(P);
            if (P.cd) law = (law == -1 || law == P.is) ? P.is : 0;
            for (int k = 0; k < 8; ++k) pc.push_back((float)P.c[k]);
            pc[pc.size() - 1] = (float)t.geom[4 * q];   // slot 7: the slave sphere's radius (no law reads c[7])
            if (P.is == IS_H) {        // ISwH first-contact stiffness coefficient (see ish_first_kn)
                const double knH = P.c[0], Meff = P.c[1], betan = P.c[4];
                const double k0 = betan < 0.99 ? 0.957832746294131 / (1.0 - betan * betan) : 479.155951122633;
                pc[pc.size() - 2] = (float)(k0 * std::pow(Meff, 0.2) * std::pow(knH, 0.8));
            }
            const double* g = &t.geom[4 * q];
            geo.push_back(make_double4_32a(g[0], g[1], g[2], g[3]));
            hole.push_back(make_double4_32a(t.hole[4 * q], t.hole[4 * q + 1], t.hole[4 * q + 2], 0.0));
            const double R = g[0] + g[1];
            rr.push_back(make_double4_32a(R, R * R, 1e-9 * R * R, 0.0));
            const double R2 = R * R;
            const float R2h = (float)R2;
            rr32.push_back(make_float4(R2h, (float)(R2 - (double)R2h), (float)(1e-9 * R2), (float)R));
            double r = 0.0;
            if (P.cd == CD_SS) r = g[0] + g[1];
            else if (cd_plane(P.cd) == CD_SP) r = g[0] + 0.5 * g[2];
            else if (P.cd == CD_SC) r = g[0] + g[1];
            // inside a hollow cylinder: -(R - r), its magnitude rounded down (apart32)
            reach.push_back(P.cd == CD_SIC ? (float)(g[0] - g[1]) * (1.0f - 1e-6f) : (float)r * (1.0f + 1e-6f));
        }
        for (const ModelDev& M : t.models) {
            double gi[3];
            for (int q = 0; q < 3; ++q) gi[q] = h.g[q] * S.dt * M.sudo + S.dt * M.ext[q];
            mf.push_back(make_float4((float)gi[0], (float)gi[1], (float)gi[2], (float)M.inv_sudo));
            mf.push_back(make_float4((float)M.rot_coef, 0.0f, 0.0f, 0.0f));
        }
        for (int k = 0; k < 3; ++k) gfield.push_back(h.g[k]);
        n_ += h.n;
        nm_ += S.nm;
        np_ += (uint32_t)nq;
        nloc_ += S.nloc;
        dt_max_ = std::max(dt_max_, (float)S.dt);
        skin_min_ = sc_.empty() ? S.skin : std::min(skin_min_, S.skin);
        sc_.push_back(S);
    }
    law_ = law < 0 ? 0 : law;
    if (np_ > META_PI) return fail(VEDO_ERR_INVALID_SCENE, "too many interaction-model pairs in one batch (2^24)");
    // ---- device
    MCK(cudaSetDevice(opts.device));
    MCK(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, opts.device));
    MCK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    for (auto& e : ev_) MCK(cudaEventCreate(&e));
    auto up = [&](auto** d, const auto& v) -> int {
        MCK(mal(d, v.size()));
        if (!v.empty()) MCK(cudaMemcpy(*d, v.data(), sizeof(v[0]) * v.size(), cudaMemcpyHostToDevice));
        return VEDO_OK;
    };
    int rc;
    if ((rc = up(&d_models_, models_)) || (rc = up(&d_params_, params_)) || (rc = up(&d_pc32_, pc)) ||
        (rc = up(&d_geom_, geo)) || (rc = up(&d_hole_, hole)) || (rc = up(&d_rr_, rr)) || (rc = up(&d_rr32_, rr32)) || (rc = up(&d_mf_, mf)) || (rc = up(&d_reach_, reach)) ||
        (rc = up(&d_model_of_, model_of)) || (rc = up(&d_scene_of_, scene_of)) || (rc = up(&d_gfield_, gfield)) ||
        (rc = up(&d_glob_, glob_)) || (rc = up(&d_ext_of_, ext_of)))
        return rc;
    {
        std::vector<uint32_t> int_of(n_);
        for (uint32_t i = 0; i < n_; ++i) int_of[ext_of[i]] = i;
        if ((rc = up(&d_int_of_, int_of))) return rc;
    }
    {
        std::vector<uint32_t> gidx(n_, 0xffffffffu);
        for (uint32_t q = 0; q < glob_.size(); ++q) gidx[glob_[q]] = q;
        if ((rc = up(&d_gidx_, gidx))) return rc;
        MCK(mal(&d_wptr_, glob_.size() + 1));
        MCK(mal(&d_wred_, 7 * glob_.size()));
        MCK(mal(&d_wrot_, glob_.size()));
        MCK(mal(&d_wedge_, glob_.size()));
    }
    sdev_.resize(sc_.size());
    MCK(mal(&d_scenes_, sc_.size()));
    MCK(mal(&d_sred_, 8 * sc_.size()));
    MCK(mal(&d_vred_, 6 * sc_.size()));
    MCK(mal(&d_work_, n_));
    if (orient_) MCK(mal(&d_tdav_, n_));

    MCK(mal(&d_clear_, n_));
    MCK(mal(&d_qcnt_, n_));
    MCK(cudaMemset(d_qcnt_, 0, n_));
    for (int b = 0; b < 2; ++b) {
        MCK(mal(&d_xs_[b], 2 * (size_t)n_));
        MCK(mal(&d_x_[b], n_));
        MCK(mal(&d_v32_[b], n_));
        MCK(mal(&d_w32_[b], n_));
    }
    MCK(mal(&d_v64_, n_)); MCK(mal(&d_w64_, n_)); MCK(mal(&d_ox_, n_)); MCK(mal(&d_oz_, n_));
    MCK(mal(&d_imp_, n_)); MCK(mal(&d_aimp_, n_)); MCK(mal(&d_pos32_, n_)); MCK(mal(&d_wall32_, n_));
    MCK(mal(&d_red_, 16)); MCK(mal(&d_disp_, 8)); MCK(mal(&d_err_, 1));
    MCK(mal(&d_key_, n_)); MCK(mal(&d_key_alt_, n_)); MCK(mal(&d_sid_, n_)); MCK(mal(&d_sid_alt_, n_));
    MCK(mal(&d_cnt_, (size_t)n_ + 1));
    MCK(mal(&d_stage_, 7 * 3 * (size_t)n_));
    MCK(mal(&d_obs_, (size_t)(nblk(n_) + 2) * 16 + 64));
    MCK(cudaMemset(d_red_, 0, 64));
    MCK(cudaMemset(d_disp_, 0, 32));
    if (prev) {
        for (int k = 0; k < 3; ++k) origin_[k] = prev->origin_[k];
    } else {
        double lo[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, hi[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
        for (uint32_t i = 0; i < n_stage; ++i)
            for (int k = 0; k < 3; ++k) {
                lo[k] = std::min(lo[k], st[0][3 * (size_t)i + k]);
                hi[k] = std::max(hi[k], st[0][3 * (size_t)i + k]);
            }
        for (int k = 0; k < 3; ++k) origin_[k] = n_stage ? 0.5 * (lo[k] + hi[k]) : 0.0;
    }
    // state: staged host scenes and scenes moved from the previous engine, one kernel
    const size_t stride = 3 * (size_t)n_;
    for (int k = 0; k < 7; ++k)
        if (n_stage) MCK(cudaMemcpy(d_stage_ + k * stride, st[k].data(), 8 * st[k].size(), cudaMemcpyHostToDevice));
    MoveScene* d_moves = nullptr;
    MCK(mal(&d_moves, moves.size()));
    MCK(cudaMemcpy(d_moves, moves.data(), sizeof(MoveScene) * moves.size(), cudaMemcpyHostToDevice));
    StateArrays ps{};
    ListArrays pl{}, sl{};
    if (prev) {
        const int pc_ = prev->cur_;
        ps = StateArrays{prev->d_x_[pc_], prev->d_v64_, prev->d_w64_, prev->d_ox_, prev->d_oz_, prev->d_imp_,
                         prev->d_aimp_};
        const NList& PL = prev->nl_[prev->nlc_];
        if (PL.ent) pl = ListArrays{PL.ptr, PL.ent, PL.slot, PL.h[pc_], PL.f[pc_]};
    }
    k_move_state<<<nblk(n_), TPB, 0, stream_>>>(n_, d_moves, (uint32_t)moves.size(), ps, d_stage_, stride,
                                                d_x_[cur_], d_v64_, d_w64_, d_ox_, d_oz_, d_imp_, d_aimp_,
                                                d_v32_[cur_], d_w32_[cur_]);
    // histories to carry: the previous engine's list rows and the new scenes' records
    uint32_t* s_buf = nullptr;
    float4* s_h = nullptr;
    uint8_t* s_f = nullptr;
    size_t nrec = 0;
    for (auto& r : recs) nrec += r.size();
    if (nrec) {
        std::vector<uint32_t> sptr(n_stage + 1, 0), sent, sslot;
        std::vector<float4> shv;
        std::vector<uint8_t> sfv;
        for (uint32_t i = 0; i < n_stage; ++i) {
            sptr[i] = (uint32_t)sent.size();
            for (const Rec& r : recs[i]) {
                sslot.push_back((uint32_t)sent.size());
                sent.push_back(r.b);
                shv.push_back(r.h);
                sfv.push_back(r.f);
            }
        }
        sptr[n_stage] = (uint32_t)sent.size();
        MCK(mal(&s_buf, sptr.size() + 2 * sent.size()));
        MCK(mal(&s_h, sent.size()));
        MCK(mal(&s_f, sent.size()));
        MCK(cudaMemcpy(s_buf, sptr.data(), 4 * sptr.size(), cudaMemcpyHostToDevice));
        MCK(cudaMemcpy(s_buf + sptr.size(), sent.data(), 4 * sent.size(), cudaMemcpyHostToDevice));
        MCK(cudaMemcpy(s_buf + sptr.size() + sent.size(), sslot.data(), 4 * sslot.size(), cudaMemcpyHostToDevice));
        MCK(cudaMemcpy(s_h, shv.data(), sizeof(float4) * shv.size(), cudaMemcpyHostToDevice));
        MCK(cudaMemcpy(s_f, sfv.data(), sfv.size(), cudaMemcpyHostToDevice));
        sl = ListArrays{s_buf, s_buf + sptr.size(), s_buf + sptr.size() + sent.size(), s_h, s_f};
    }
    if (pl.ent || sl.ent) {
        NList& O = nl_[1];
        if (!O.ptr) MCK(mal(&O.ptr, (size_t)n_ + 1));
        k_row_count<<<nblk((size_t)n_ + 1), TPB, 0, stream_>>>(n_, d_moves, (uint32_t)moves.size(), pl, sl, d_cnt_);
        MCK(exclusive_scan_u32(d_cnt_, O.ptr, n_ + 1, d_red_ + 9, scratch_, stream_));
        uint32_t ne = 0;
        MCK(cudaMemcpyAsync(&ne, d_red_ + 9, 4, cudaMemcpyDeviceToHost, stream_));
        MCK(cudaStreamSynchronize(stream_));
        if ((rc = ensure_nlist(O, ne)) != VEDO_OK) return rc;
        O.ne = ne;
        k_row_fill<<<nblk(n_), TPB, 0, stream_>>>(n_, d_moves, (uint32_t)moves.size(), pl, sl, O.ptr, O.ent, O.slot,
                                                  O.h[cur_], O.f[cur_]);
        nlc_ = 1;
    }
    MCK(cudaStreamSynchronize(stream_));
    MCK(cudaGetLastError());
    cudaFree(d_moves);
    if (s_buf) cudaFree(s_buf);
    if (s_h) cudaFree(s_h);
    if (s_f) cudaFree(s_f);
    need_rebuild_ = true;
    rc = rebuild();
    if (rc != VEDO_OK) return rc;
    MCK(cudaStreamSynchronize(stream_));
    return VEDO_OK;
}

int MixedEngine::set_scene_active(uint32_t s, bool on) {
    if (s >= sc_.size()) return fail(VEDO_ERR_INVALID_ARGUMENT, "scene index out of range");
    // a resumed scene rebuilds: its spheres stood still while its frame moved on
    if (on && !sc_[s].active) need_rebuild_ = true;
    sc_[s].active = on;
    sdev_[s].active = on ? 1u : 0u;
    MCK(cudaMemcpyAsync(d_scenes_ + s, &sdev_[s], sizeof(SceneDev), cudaMemcpyHostToDevice, stream_));
    MCK(cudaStreamSynchronize(stream_));
    drop_graphs();
    return VEDO_OK;
}

int MixedEngine::get_state_slice(uint32_t off, uint32_t cnt, const vedo_state_view& v) {
    if ((uint64_t)off + cnt > n_) return fail(VEDO_ERR_INVALID_ARGUMENT, "object range out of bounds");
    double* dst[] = {v.position, v.velocity, v.angular_velocity, v.orientation_x, v.orientation_z, v.impact,
                     v.angular_impact};
    const double4_32a* src[] = {d_x_[cur_], d_v64_, d_w64_, d_ox_, d_oz_, d_imp_, d_aimp_};
    for (int k = 0; k < 7; ++k) {
        if (!dst[k] || !cnt) continue;
        double* stg = d_stage_ + (size_t)k * 3 * n_;
        k_unpack3m<<<nblk(cnt), TPB, 0, stream_>>>(cnt, off, d_int_of_, src[k], stg);
        MCK(cudaMemcpyAsync(dst[k], stg, 24 * (size_t)cnt, cudaMemcpyDeviceToHost, stream_));
    }
    MCK(cudaStreamSynchronize(stream_));
    MCK(cudaGetLastError());
    return VEDO_OK;
}

// The wall kernel's arguments for a step that starts from buffer parity c.
WallArgs MixedEngine::wargs(int c) {
    WallArgs w;
    w.nglob = (uint32_t)glob_.size();
    w.glob = d_glob_;
    w.model_of = d_model_of_;
    w.models = d_models_;
    w.scenes = d_scenes_;
    w.scene_of = d_scene_of_;
    w.xA = d_x_[c];
    w.xB = d_x_[c ^ 1];
    w.v64 = d_v64_;
    w.w64 = d_w64_;
    w.v32A = d_v32_[c];
    w.v32B = d_v32_[c ^ 1];
    w.w32A = d_w32_[c];
    w.w32B = d_w32_[c ^ 1];
    w.ox = d_ox_;
    w.oz = d_oz_;
    w.dt_max = dt_max_;
    w.vmax_bits = d_red_ + 8;
    w.vrel_bits = d_red_ + 2;
    w.disp_in = d_disp_ + 4 * c;
    w.disp_out = d_disp_ + 4 * (c ^ 1);
    w.skin = skin_min_;
    w.skin_w = WALL_SKIN * skin_min_;
    w.pos_eps = pos_eps_;
    w.wall_speed_bits = d_red_ + 12;
    w.wrot = d_wrot_;
    w.held = d_red_ + 11;
    w.wall32 = d_wall32_;
    w.nwork = d_red_ + 13;
    w.imp = d_imp_;
    w.aimp = d_aimp_;
    w.dyn_bits = d_red_ + 3;
    return w;
}

TickArgs MixedEngine::args(bool write_imp) {
    NList& L = nl_[nlc_];
    TickArgs a;
    a.n = n_;
    a.scenes = d_scenes_;
    a.scene_of = d_scene_of_;
    a.model_of = d_model_of_;
    a.models = d_models_;
    a.params = d_params_;
    a.pc32 = d_pc32_;
    a.geom = d_geom_;
    a.hole = d_hole_;
    a.xA = d_x_[cur_];
    a.xB = d_x_[cur_ ^ 1];
    a.v64 = d_v64_;
    a.w64 = d_w64_;
    a.v32A = d_v32_[cur_];
    a.v32B = d_v32_[cur_ ^ 1];
    a.w32A = d_w32_[cur_];
    a.w32B = d_w32_[cur_ ^ 1];
    a.ox = d_ox_;
    a.oz = d_oz_;
    a.nptr = L.ptr;
    a.nent = L.ent;
    a.nslot = L.slot;
    a.nmeta = L.meta;
    a.hA = L.h[cur_];
    a.hB = L.h[cur_ ^ 1];
    a.fA = L.f[cur_];
    a.fB = L.f[cur_ ^ 1];
    a.imp = d_imp_;
    a.aimp = d_aimp_;
    a.write_imp = write_imp ? 1 : 0;
    a.wimp_on = (write_imp || dyn_walls_) ? 1 : 0;
    a.vmax_bits = d_red_ + 8;
    a.pos32 = d_pos32_;
    a.disp = d_disp_ + 4 * cur_;
    a.vrel_bits = d_red_ + 2;
    a.skin = skin_min_;
    a.skin_w = WALL_SKIN * skin_min_;
    a.reach = d_reach_;
    a.wall32 = d_wall32_;
    a.wimp = d_wimp_;
    a.rr = d_rr_;
    a.rr32 = d_rr32_;
    a.xsA = d_xs_[cur_];
    a.xsB = d_xs_[cur_ ^ 1];
    a.xs_stored = xs_stored_ ? 1 : 0;
    a.work = split_tick_ ? d_work_ : nullptr;
    a.nwork = d_red_ + 14;
    a.pwork = d_pwork_;
    a.xf = d_xf_;
    a.prec = d_prec_;
    a.pmir = d_pmir_;
    a.wk = d_wk_;
    a.xm = d_xm_;
    a.pcap = pcap_;
    a.mf = d_mf_;
    a.clear = d_clear_;
    a.qcnt = d_qcnt_;
    a.ext = ext_on_ ? d_ext_ : nullptr;
    a.ext_of = d_ext_of_;
    a.sox = d_ox_;
    a.soz = d_oz_;
    a.tdav = d_tdav_;
    a.orient = orient_ ? 1 : 0;
    return a;
}

int MixedEngine::rebuild() {
    drop_graphs();   // the captured launches name this list's buffers
    const uint64_t l0 = g_sort_scan_launches;
    uint64_t own = 0;
    const uint32_t S = (uint32_t)sc_.size();
    const d3 org = mk(origin_[0], origin_[1], origin_[2]);
    std::vector<unsigned> red0(8 * (size_t)S, 0u);
    for (uint32_t s = 0; s < S; ++s) red0[8 * s] = red0[8 * s + 1] = red0[8 * s + 2] = 0xffffffffu;
    MCK(cudaMemcpyAsync(d_sred_, red0.data(), 4 * red0.size(), cudaMemcpyHostToDevice, stream_));
    k_bounds<<<nblk(n_), TPB, 0, stream_>>>(n_, d_model_of_, d_models_, d_scene_of_, d_x_[cur_], org, d_pos32_,
                                            d_sred_);
    k_wall32<<<nblk(n_), TPB, 0, stream_>>>(n_, d_model_of_, d_models_, d_ox_, d_oz_, d_wall32_);
    std::vector<unsigned> vred0(6 * (size_t)S, 0u);
    for (uint32_t s = 0; s < S; ++s) vred0[6 * s] = vred0[6 * s + 1] = vred0[6 * s + 2] = 0xffffffffu;
    MCK(cudaMemcpyAsync(d_vred_, vred0.data(), 4 * vred0.size(), cudaMemcpyHostToDevice, stream_));
    k_vrange<<<nblk(n_), TPB, 0, stream_>>>(n_, d_model_of_, d_models_, d_scene_of_, d_v64_, d_vred_);
    own += 3;
    std::vector<unsigned> red(8 * (size_t)S), vred(6 * (size_t)S);
    MCK(cudaMemcpyAsync(red.data(), d_sred_, 4 * red.size(), cudaMemcpyDeviceToHost, stream_));
    MCK(cudaMemcpyAsync(vred.data(), d_vred_, 4 * vred.size(), cudaMemcpyDeviceToHost, stream_));
    MCK(cudaStreamSynchronize(stream_));
    auto unord = [](unsigned o) {
        unsigned b = (o >> 31) ? (o & 0x7fffffffu) : ~o;
        float f;
        memcpy(&f, &b, 4);
        return f;
    };
    // per-scene cell grids (edge 2 r_max + skin), packed one after the other
    uint64_t cells = 0;
    float pos_eps = 0.0f;
    for (uint32_t s = 0; s < S; ++s) {
        SceneDev& D = sdev_[s];
        const SceneHost& H = sc_[s];
        D.model_off = H.model_off;
        D.nm = H.nm;
        D.pbase = H.pbase;
        D.wall_beg = H.wall_beg;
        D.wall_end = H.wall_end;
        D.obj_off = H.obj_off;
        D.nobj = H.nobj;
        D.active = H.active ? 1u : 0u;
        D.dt = H.dt;
        D.dtf = (float)H.dt;
        D.pb = H.pb;
        for (int k = 0; k < 3; ++k) {
            const float hi = (float)H.pb.range[k];
            D.pr_hi[k] = H.pb.sw[k] ? hi : 0.0f;
            D.pr_lo[k] = H.pb.sw[k] ? (float)(H.pb.range[k] - (double)hi) : 0.0f;
        }
        // the frame: free fall under the scene's field from its spheres' velocity midrange
        const bool moving = vred[6 * s] != 0xffffffffu;
        for (int k = 0; k < 3; ++k) {
            D.u0[k] = moving ? 0.5f * (unord(vred[6 * s + k]) + unord(vred[6 * s + 3 + k])) : 0.0f;
            D.gdt[k] = (float)(H.g[k] * H.dt);
        }
        float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
        if (H.nloc)
            for (int k = 0; k < 3; ++k) {
                lo[k] = unord(red[8 * s + k]);
                hi[k] = unord(red[8 * s + 3 + k]);
                // a position update's FP64 rounding is at most half an ulp of the coordinate
                const double m = std::max(std::fabs(origin_[k] + lo[k]), std::fabs(origin_[k] + hi[k])) + 1.0;
                pos_eps = std::max(pos_eps, (float)std::ldexp(m, -50));
            }
        float rmax;
        memcpy(&rmax, &red[8 * s + 6], 4);
        float h = (2.0f * rmax + H.skin) * (1.0f + 1e-5f) * cell_scale_;
        if (!(h > 0.0f)) h = 1.0f;
        const uint64_t budget = std::max<uint64_t>(8ull * std::max<uint32_t>(H.nobj, 1), 1ull << 12);
        uint32_t nc[3] = {1, 1, 1};
        // a periodic axis: the grid spans the box, ranges of at least one cell edge each, and the
        // cells wrap around (k_keys, k_nbr)
        for (int k = 0; k < 3; ++k)
            if (H.pb.sw[k]) lo[k] = (float)(H.pb.lo[k] - origin_[k]);
        // a periodic axis holds at least three cells (the three neighbour cells are then distinct):
        // the cells may be made no wider than a third of the shortest periodic range
        const float hmin = (2.0f * rmax + H.skin) * (1.0f + 1e-5f);
        float hcap = 3.0e38f;
        for (int k = 0; k < 3; ++k)
            if (H.pb.sw[k]) hcap = std::min(hcap, H.pb.range32[k] / 3.0f);
        if (hmin > hcap)
            return fail(VEDO_ERR_UNSUPPORTED_MODEL, "mixed form, periodic boundary: a periodic range shorter than "
                                                    "three times 2 r_max + skin");
        h = std::min(h, hcap);
        for (int pass = 0; pass < 8; ++pass) {
            for (int k = 0; k < 3; ++k)
                nc[k] = H.pb.sw[k] ? std::max<uint32_t>(3, (uint32_t)std::floor(H.pb.range32[k] / h))
                                   : std::max<uint32_t>(1, (uint32_t)std::floor((hi[k] - lo[k]) / h) + 1);
            const uint64_t c = (uint64_t)nc[0] * nc[1] * nc[2];
            if (c <= budget || h >= hcap) break;
            h = std::min(hcap, h * (float)std::cbrt((double)c / budget) * 1.01f);   // sparse scene: coarser cells
        }
        for (int k = 0; k < 3; ++k) {
            D.nc[k] = nc[k];
            D.lo[k] = lo[k];
        }
        D.inv_h = 1.0f / h;
        D.cell_base = cells;
        cells += (uint64_t)nc[0] * nc[1] * nc[2];
    }
    pos_eps_ = pos_eps;
    MCK(cudaMemcpyAsync(d_scenes_, sdev_.data(), sizeof(SceneDev) * S, cudaMemcpyHostToDevice, stream_));
    if (cells > grid_cap_) {
        if (d_gs_) cudaFree(d_gs_);
        if (d_ge_) cudaFree(d_ge_);
        grid_cap_ = cells + cells / 4;
        MCK(mal(&d_gs_, grid_cap_));
        MCK(mal(&d_ge_, grid_cap_));
    }
    MCK(cudaMemsetAsync(d_gs_, 0, 4 * cells, stream_));
    MCK(cudaMemsetAsync(d_ge_, 0, 4 * cells, stream_));
    k_keys<<<nblk(n_), TPB, 0, stream_>>>(n_, d_model_of_, d_models_, d_scene_of_, d_scenes_, d_pos32_, cells,
                                          d_key_, d_sid_);
    ++own;
    int bits = 1;
    while (bits < 64 && (cells >> bits)) ++bits;
    MCK(radix_sort_u64(d_key_, d_sid_, d_key_alt_, d_sid_alt_, n_, 0, bits, scratch_, stream_));
    if (nloc_) {
        k_cells<<<nblk(nloc_), TPB, 0, stream_>>>(nloc_, d_key_, d_gs_, d_ge_);
        ++own;
    }
    // count, scan, fill
    const int newl = nlc_ ^ 1;
    NList& L = nl_[newl];
    NList& O = nl_[nlc_];
    if (!L.ptr) MCK(mal(&L.ptr, (size_t)n_ + 1));
    MCK(cudaMemsetAsync(d_cnt_, 0, 4 * ((size_t)n_ + 1), stream_));
    if (nloc_) {
        k_nbr<false><<<nblk(nloc_), TPB, 0, stream_>>>(nloc_, d_sid_, d_key_, d_gs_, d_ge_, d_scene_of_, d_scenes_,
                                                       d_glob_, d_model_of_, d_models_, d_params_, d_reach_,
                                                       d_pos32_, d_wall32_, skin_min_, d_ext_of_, d_int_of_, d_cnt_,
                                                       nullptr);
        ++own;
    }
    MCK(exclusive_scan_u32(d_cnt_, L.ptr, n_ + 1, d_red_ + 9, scratch_, stream_));
    uint32_t ne = 0;
    MCK(cudaMemcpyAsync(&ne, d_red_ + 9, 4, cudaMemcpyDeviceToHost, stream_));
    MCK(cudaStreamSynchronize(stream_));
    int rc = ensure_nlist(L, ne);
    if (rc != VEDO_OK) return rc;
    L.ne = ne;
    if (pair_pass_ && (rc = ensure_pair_bufs(ne)) != VEDO_OK) return rc;
    if (nloc_) {
        k_nbr<true><<<nblk(nloc_), TPB, 0, stream_>>>(nloc_, d_sid_, d_key_, d_gs_, d_ge_, d_scene_of_, d_scenes_,
                                                      d_glob_, d_model_of_, d_models_, d_params_, d_reach_, d_pos32_,
                                                      d_wall32_, skin_min_, d_ext_of_, d_int_of_, L.ptr, L.ent);
        ++own;
    }
    MCK(cudaMemsetAsync(d_err_, 0, 4, stream_));
    k_slots<<<nblk(n_), TPB, 0, stream_>>>(n_, L.ptr, L.ent, L.slot, d_err_);
    if (pair_pass_) {
        fill_mirror(L);
        own += 2;
    }
    k_meta<<<nblk(n_), TPB, 0, stream_>>>(n_, L.ptr, L.ent, L.slot, d_model_of_, d_models_, d_scene_of_, d_scenes_,
                                          d_params_, d_ext_of_, L.meta);
    ++own;
    k_carry<<<nblk(n_), TPB, 0, stream_>>>(n_, L.ptr, L.ent, L.slot, O.ptr, O.ent, O.slot, O.h[cur_], O.f[cur_],
                                           L.h[cur_], L.f[cur_], L.h[cur_ ^ 1], L.f[cur_ ^ 1],
                                           O.ent != nullptr ? 1 : 0);
    k_interior<<<nblk(n_), TPB, 0, stream_>>>(n_, L.ptr, L.ent, L.meta, d_model_of_, d_models_, d_x_[cur_], d_ox_,
                                              d_oz_, skin_min_, WALL_SKIN * skin_min_);
    k_clear<<<nblk(n_), TPB, 0, stream_>>>(n_, L.ptr, L.ent, L.meta, d_model_of_, d_models_, d_pos32_, d_wall32_,
                                           d_reach_, d_clear_, d_qcnt_, quiet_ok_ ? 1 : 0, d_scene_of_, d_scenes_);
    own += 3;
    // per-wall entry lists for the wall impulse output
    if (!glob_.empty()) {
        k_wall_count<<<nblk(n_), TPB, 0, stream_>>>(n_, L.ptr, L.ent, d_cnt_);
        MCK(exclusive_scan_u32(d_cnt_, d_cnt_, n_ + 1, d_red_ + 10, scratch_, stream_));
        uint32_t nw = 0;
        MCK(cudaMemcpyAsync(&nw, d_red_ + 10, 4, cudaMemcpyDeviceToHost, stream_));
        MCK(cudaStreamSynchronize(stream_));
        if (nw > wcap_) {
            for (uint32_t** p : {&d_wkey_, &d_wval_, &d_wkey_alt_, &d_wval_alt_}) {
                if (*p) cudaFree(*p);
                *p = nullptr;
            }
            wcap_ = nw + nw / 4 + 64;
            MCK(mal(&d_wkey_, wcap_)); MCK(mal(&d_wval_, wcap_)); MCK(mal(&d_wkey_alt_, wcap_));
            MCK(mal(&d_wval_alt_, wcap_));
        }
        nwall_ent_ = nw;
        k_wall_fill<<<nblk(n_), TPB, 0, stream_>>>(n_, L.ptr, L.ent, d_cnt_, d_gidx_, d_wkey_, d_wval_);
        int wb = 1;
        while (wb < 32 && (((uint32_t)glob_.size() - 1) >> wb)) ++wb;
        MCK(radix_sort_u32(d_wkey_, d_wval_, d_wkey_alt_, d_wval_alt_, nw, 0, wb, scratch_, stream_));
        k_wall_ptr<<<nblk(glob_.size() + 1), TPB, 0, stream_>>>((uint32_t)glob_.size(), d_wkey_, nw, d_wptr_);
        own += 3;
        if (6ull * ne > wimp_cap_) {
            if (d_wimp_) cudaFree(d_wimp_);
            wimp_cap_ = (uint32_t)std::min<uint64_t>(6ull * (ne + ne / 4 + 64), 0xffffffffull);
            MCK(mal(&d_wimp_, wimp_cap_));
        }
    }
    // orbital walls' plane speed (the spheres' speed is measured every step)
    float rmax_all = 0.0f;
    for (uint32_t s = 0; s < S; ++s) {
        float r;
        memcpy(&r, &red[8 * s + 6], 4);
        rmax_all = std::max(rmax_all, r);
    }
    MCK(cudaMemsetAsync(d_red_ + 11, 0, 8, stream_));
    if (!glob_.empty()) {
        k_wall_rot<<<nblk(glob_.size()), TPB, 0, stream_>>>((uint32_t)glob_.size(), d_glob_, d_model_of_, d_models_,
                                                           d_scenes_, d_scene_of_, d_w64_, d_wrot_);
        ++own;
        MCK(cudaMemsetAsync(d_wedge_, 0, 4 * glob_.size(), stream_));
        k_wall_edge<<<nblk(n_), TPB, 0, stream_>>>(n_, d_model_of_, d_models_, d_scene_of_, d_scenes_, d_glob_,
                                                   d_x_[cur_], d_oz_, WALL_SKIN * skin_min_, d_wedge_);
        k_wall_speed<<<nblk(glob_.size()), TPB, 0, stream_>>>((uint32_t)glob_.size(), d_glob_, d_model_of_, d_models_,
                                                             d_v64_, d_w64_, d_oz_, 2.0f * rmax_all, d_wedge_,
                                                             d_red_ + 12);
        own += 2;
    }
    int herr = 0;
    MCK(cudaMemcpyAsync(&herr, d_err_, 4, cudaMemcpyDeviceToHost, stream_));
    MCK(cudaMemsetAsync(d_disp_, 0, 32, stream_));
    MCK(cudaStreamSynchronize(stream_));
    MCK(cudaGetLastError());
    if (herr) return fail(VEDO_ERR_CUDA, "mixed form: asymmetric neighbour lists");
    if (xs_stored_) {              // the stored splits follow the positions from here on
        k_split<<<nblk(n_), TPB, 0, stream_>>>(n_, d_x_[cur_], d_xs_[cur_]);
        ++own;
    }
    nlc_ = newl;
    need_rebuild_ = false;
    since_rebuild_ = 0;
    ++rebuilds_;
    launches_ += own + (g_sort_scan_launches - l0);
    return VEDO_OK;
}

// One time step's launches: the fused tick, the wall impulse sums on the last step of a call,
// and the wall kernel (wall motion and the displacement bound after the step).
// A per-step kernel launch; `dep`: with programmatic dependent launch (the kernel orders itself
// after the previous one with step_order()).
template <typename... P, typename... A>
static cudaError_t step_launch(bool dep, void (*k)(P...), unsigned grid, unsigned block, cudaStream_t s, A... args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = dep ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k, args...);
}

void MixedEngine::launch_step(bool write_imp) {
    TickArgs a = args(write_imp);
    const unsigned nb = (unsigned)((n_ + tpb_ - 1) / tpb_);
    cudaEvent_t* pe = nullptr;
    if (profiling_ && pev_used_ + 3 <= pev_.size()) {
        pe = &pev_[pev_used_];
        pev_used_ += 3;
        // external records while capturing (the flag is valid only then): a captured step keeps
        // them as event nodes
        cudaEventRecordWithFlags(pe[0], stream_, ev_flags_);
    }
    // dependent launches between the step's kernels, except where event records sit between them
    const bool dep = pe == nullptr;
    auto note = [&](cudaError_t e) {
        if (e != cudaSuccess && launch_err_ == cudaSuccess) launch_err_ = e;
    };
    unsigned nb_full = nb;
    if (pair_pass_) {               // prefilter pass, pair pass over its worklist, per-sphere sums
        // (the worklist count is zeroed by k_walls at the end of every step)
        note(step_launch(dep, k_tick_pf, nblk(n_), TPB, stream_, a));
        // the pair kernel strides over the worklist with the grid that is resident at once
#define VEDO_PAIRS(L)                                                                                       \
    {                                                                                                       \
        auto kw = xs_stored_ ? k_tick_pairs<L, true, 2, false> : k_tick_pairs<L, false, 2, false>;          \
        if (!glob_.empty() && dep) {   /* the wall pairs, then the sphere pairs beside them */             \
            auto kp = xs_stored_ ? k_tick_pairs<L, true, 1, true> : k_tick_pairs<L, false, 1, true>;        \
            note(step_launch(dep, kw, (unsigned)sms_ * 4u, (unsigned)tpb_, stream_, a));                     \
            note(step_launch(dep, kp, resident_grid((const void*)kp), (unsigned)tpb_, stream_, a));         \
            ++launches_;                                                                                    \
        } else {                                                                                            \
            auto kp = xs_stored_ ? k_tick_pairs<L, true, 1, false> : k_tick_pairs<L, false, 1, false>;      \
            note(step_launch(dep, kp, resident_grid((const void*)kp), (unsigned)tpb_, stream_, a));         \
            if (!glob_.empty()) {                                                                           \
                note(step_launch(dep, kw, (unsigned)sms_ * 4u, (unsigned)tpb_, stream_, a));                 \
                ++launches_;                                                                                \
            }                                                                                               \
        }                                                                                                   \
    }
        switch (law_) {
        case IS_BSDBF: VEDO_PAIRS(IS_BSDBF); break;
        case IS_BTSDBF: VEDO_PAIRS(IS_BTSDBF); break;
        case IS_BSDB2F: VEDO_PAIRS(IS_BSDB2F); break;
        case IS_HERTZ: VEDO_PAIRS(IS_HERTZ); break;
        case IS_H: VEDO_PAIRS(IS_H); break;
        default: VEDO_PAIRS(0); break;
        }
#undef VEDO_PAIRS
        note(step_launch(dep, xs_stored_ ? k_tick_sum<true> : k_tick_sum<false>, nblk(n_), TPB, stream_, a));
        launches_ += 3;
    } else {
    if (split_tick_) {              // light tick over all spheres, then the full tick over the deferred
        // (the worklist count is zeroed by k_walls at the end of every step)
        note(step_launch(dep, xs_stored_ ? k_tick_light<true> : k_tick_light<false>, nblk(n_), TPB, stream_, a));
        ++launches_;
        // the full tick at its residency (128 registers: 16 warps per SM) strides over the worklist
        nb_full = std::min<unsigned>(nb, (unsigned)sms_ * 512u / (unsigned)tpb_);
    }
#define VEDO_TICK(L)                                                                                        \
    note(step_launch(dep, split_tick_ ? (xs_stored_ ? k_tick_work<L, true> : k_tick_work<L, false>)          \
                                      : (xs_stored_ ? k_tick<L, true> : k_tick<L, false>),                   \
                     split_tick_ ? nb_full : nb, (unsigned)tpb_, stream_, a))
    switch (law_) {
    case IS_BSDBF: VEDO_TICK(IS_BSDBF); break;
    case IS_BTSDBF: VEDO_TICK(IS_BTSDBF); break;
    case IS_BSDB2F: VEDO_TICK(IS_BSDB2F); break;
    case IS_HERTZ: VEDO_TICK(IS_HERTZ); break;
    case IS_H: VEDO_TICK(IS_H); break;
    default: VEDO_TICK(0); break;
    }
#undef VEDO_TICK
    ++launches_;
    }
    if (any_pbc_) {                 // periodic scenes: spheres back into the box
        note(step_launch(dep, k_wrap, nblk(n_), TPB, stream_, a));
        ++launches_;
    }
    if (orient_) {                  // sphere orientations, from the tick's angular velocity increments
        note(step_launch(dep, k_turn, nblk(n_), TPB, stream_, a));
        ++launches_;
    }
    if (pe) cudaEventRecordWithFlags(pe[1], stream_, ev_flags_);
    if ((write_imp || dyn_walls_) && !glob_.empty()) {      // the walls' impulses (every step when walls respond)
        const uint32_t ng = (uint32_t)glob_.size();
        cudaMemsetAsync(d_wred_, 0, (size_t)ng * (8 + 48), stream_);
        unsigned* wmax = reinterpret_cast<unsigned*>(d_wred_ + 6 * (size_t)ng);
        if (nwall_ent_) {
            k_wall_max<<<nblk(nwall_ent_), TPB, 0, stream_>>>(nwall_ent_, d_wkey_, d_wval_, d_wimp_, wmax);
            k_wall_acc<<<nblk(nwall_ent_), TPB, 0, stream_>>>(nwall_ent_, d_wkey_, d_wval_, d_wimp_, wmax, d_wred_);
            launches_ += 2;
        }
        k_wall_fin<<<nblk(ng), TPB, 0, stream_>>>(ng, d_glob_, wmax, d_wred_, d_model_of_, d_models_, d_scenes_,
                                                  d_scene_of_, d_gfield_, d_imp_, d_aimp_);
        ++launches_;
    }
    note(step_launch(dep, k_walls, nblk(std::max<size_t>(glob_.size(), 1)), TPB, stream_, wargs(cur_)));
    ++launches_;
    if (dyn_walls_) {
        note(step_launch(dep, k_wall_bound, 1u, 32u, stream_, (const float*)(d_disp_ + 4 * cur_),
                         d_disp_ + 4 * (cur_ ^ 1), skin_min_, WALL_SKIN * skin_min_, d_red_ + 3));
        ++launches_;
    }
    if (pe) cudaEventRecordWithFlags(pe[2], stream_, ev_flags_);
    cur_ ^= 1;
}

// `chunk` steps as one cooperative launch of the persistent tick; 0 = launched, -1 = the kernel
// cannot have a block resident on every SM (the caller launches the steps one by one), > 0 an
// error code.
int MixedEngine::launch_persistent(uint32_t chunk) {
    const unsigned block = pair_pass_ ? 1024u : 512u;
    const void* k = nullptr;
#define VEDO_PK(L)                                                                                     \
    k = pair_pass_ ? (xs_stored_ ? (const void*)k_persist<2, L, true> : (const void*)k_persist<2, L, false>) \
                   : (xs_stored_ ? (const void*)k_persist<0, L, true> : (const void*)k_persist<0, L, false>)
    switch (law_) {
    case IS_BSDBF: VEDO_PK(IS_BSDBF); break;
    case IS_BTSDBF: VEDO_PK(IS_BTSDBF); break;
    case IS_BSDB2F: VEDO_PK(IS_BSDB2F); break;
    case IS_HERTZ: VEDO_PK(IS_HERTZ); break;
    case IS_H: VEDO_PK(IS_H); break;
    default: VEDO_PK(0); break;
    }
#undef VEDO_PK
    if (k != pk_) {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k, (int)block, 0) != cudaSuccess) b = 0;
        (void)cudaGetLastError();
        pk_ = k;
        pk_grid_ = (unsigned)std::max(b, 0) * (unsigned)sms_;
    }
    if (pk_grid_ == 0) return -1;
    PersistArgs p;
    const int c0 = cur_;
    p.t[0] = args(false);
    p.w[0] = wargs(c0);
    cur_ = c0 ^ 1;
    p.t[1] = args(false);
    p.w[1] = wargs(c0 ^ 1);
    cur_ = c0;
    p.steps = chunk;
    p.pbc = any_pbc_ ? 1 : 0;
    p.bar.w = d_red_ + 4;
    p.bar.nblocks = pk_grid_;
    p.bar.limit_ns = 2000000000ull;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(pk_grid_);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream_;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    void* kargs[] = {&p};
    MCK(cudaLaunchKernelExC(&cfg, k, kargs));
    ++launches_;
    if (chunk & 1) cur_ ^= 1;
    return 0;
}

// `chunk` steps, then one read of the displacement bound and of the held-step count.  A full
// check interval without impulse output replays a CUDA graph captured once per list, or runs as
// one persistent launch.
int MixedEngine::step_chunk(uint32_t chunk, bool imp_last, float* use_after) {
    const uint32_t ci = opts_.check_interval;
    if (profiling_ && pev_.size() < 3 * (size_t)ci) {
        while (pev_.size() < 3 * (size_t)ci) {
            cudaEvent_t e = nullptr;
            MCK(cudaEventCreate(&e));
            pev_.push_back(e);
        }
    }
    pev_used_ = 0;
    int persisted = -1;
    if (!imp_last && persist_usable()) {
        persisted = launch_persistent(chunk);
        if (persisted > 0) return persisted;
    }
    if (persisted == 0) {
        // (launched)
    } else if (opts_.graphs && chunk == ci) {
        const int c0 = cur_;
        const int gi = c0 + (profiling_ ? 2 : 0) + (imp_last ? 4 : 0);
        if (!graph_[gi]) {
            cudaGraph_t g = nullptr;
            const uint64_t l0 = launches_;
            MCK(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
            ev_flags_ = cudaEventRecordExternal;
            for (uint32_t k = 0; k < chunk; ++k) launch_step(imp_last && k + 1 == chunk);
            ev_flags_ = cudaEventRecordDefault;
            const cudaError_t ce = cudaStreamEndCapture(stream_, &g);
            graph_launches_[gi] = launches_ - l0;
            launches_ = l0;
            cur_ = c0;
            if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
            pev_used_ = 0;
            const cudaError_t ie = cudaGraphInstantiate(&graph_[gi], g, 0);
            cudaGraphDestroy(g);
            if (ie != cudaSuccess) return cuda_fail(ie, "cudaGraphInstantiate");
        }
        MCK(cudaGraphLaunch(graph_[gi], stream_));
        if (profiling_) pev_used_ = 3 * chunk;           // the graph records every step's events
        launches_ += graph_launches_[gi];
        if (chunk & 1) cur_ ^= 1;
    } else {
        for (uint32_t k = 0; k < chunk; ++k) launch_step(imp_last && k + 1 == chunk);
    }
    if (launch_err_ != cudaSuccess) {
        const cudaError_t le = launch_err_;
        launch_err_ = cudaSuccess;
        return cuda_fail(le, "kernel launch");
    }
    float dd[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    unsigned red[8] = {0, 0, 0, 0, 0, 0, 0, 0};    // [2], [3]: barrier expiry and its site; [7]: held steps
    MCK(cudaMemcpyAsync(dd, d_disp_ + 4 * cur_, 16, cudaMemcpyDeviceToHost, stream_));
    MCK(cudaMemcpyAsync(red, d_red_ + 4, 32, cudaMemcpyDeviceToHost, stream_));
    MCK(cudaStreamSynchronize(stream_));
    const unsigned held = red[7];
    if (red[2]) {
        MCK(cudaMemsetAsync(d_red_ + 4, 0, 16, stream_));
        MCK(cudaStreamSynchronize(stream_));
        return fail(VEDO_ERR_CUDA, "persistent tick: a grid barrier waited past its limit (barrier " +
                                       std::to_string(red[3]) + " of the interval); the state is undefined");
    }
    for (uint32_t q = 0; q + 3 <= pev_used_; q += 3) {   // profiling: tick and wall kernel times
        float a = 0.0f, b = 0.0f;
        cudaEventElapsedTime(&a, pev_[q], pev_[q + 1]);
        cudaEventElapsedTime(&b, pev_[q + 1], pev_[q + 2]);
        prof_[0] += a;
        prof_[1] += b;
        prof_ticks_ += 1;
    }
    pev_used_ = 0;
    const uint32_t taken = chunk - std::min(held, chunk);
    round_ += taken;
    since_rebuild_ += taken;
    for (auto& S : sc_) {
        if (!S.active) continue;
        for (uint32_t k = 0; k < taken; ++k) S.t += S.dt;     // SystemParameter::NextStep (SystemParameter.h:113-116), once per step
        S.steps += taken;
    }
    // the share of the list's life used so far: 1 = the next step would be an identity step
    const float use = std::max(std::max(2.0f * dd[0], dd[1]) / skin_min_, (dd[1] + dd[2]) / (WALL_SKIN * skin_min_));
    if (held || list_spent(dd[0], dd[1], dd[2], skin_min_, WALL_SKIN * skin_min_) || use > 1.0f) {
        // held steps are taken again after the rebuild; a bound already past half the skin
        // would hold the next step, and contact queries need a complete list too
        need_rebuild_ = true;
    } else if (since_rebuild_ % ci == 0) {
        // Rebuild before the bound can reach half the skin: the bound so far plus twice its
        // mean growth per step over the next check interval.
        const float growth = use / (float)since_rebuild_;
        if (use + 2.0f * growth * (float)ci > 1.0f) need_rebuild_ = true;
    }
    if (use_after) *use_after = use;
    return (int)taken == (int)chunk ? VEDO_OK : -(int)(chunk - taken);
}

// Online tuning of the tick block size, the skin and the cell scale.  The trials are ordinary
// steps of the run: results do not depend on any of the three (the list is complete for any
// skin and rebuild schedule, and the per-sphere sums follow the canonical list order), so the
// run's results are those of an untuned run.  Costs are CUDA-event device times: the tick
// per step, and for the skin the rebuild time spread over the steps a list of that skin is
// expected to last at the displacement growth just measured.
int MixedEngine::autotune(uint32_t max_steps, uint32_t* taken) {
    *taken = 0;
    const uint32_t ci = opts_.check_interval;
    const int blocks[] = {64, 128, 256};
    const float skins[] = {0.05f, 0.1f, 0.15f, 0.25f, 0.4f};
    const float cells[] = {1.0f, 1.25f, 1.5f};
    // at most four chunks per timed trial (a rebuild between may add two), two per skin trial
    const uint32_t need = ci * (uint32_t)(4 * (3 + 2 + 3 + 1) + 2 * 5);
    if (max_steps < need) return VEDO_OK;            // too short a call: tune in a later one
    cudaEvent_t e0 = ev_[2], e1 = ev_[3];
    auto timed_rebuild = [&](float* ms) -> int {
        MCK(cudaEventRecord(e0, stream_));
        int rc = rebuild();
        if (rc != VEDO_OK) return rc;
        MCK(cudaEventRecord(e1, stream_));
        MCK(cudaEventSynchronize(e1));
        MCK(cudaEventElapsedTime(ms, e0, e1));
        return VEDO_OK;
    };
    auto timed_chunk = [&](float* ms_per_step, float* growth) -> int {
        const uint64_t r0 = round_;
        float use = 0.0f, use0 = 0.0f;
        // an untimed chunk first: it captures the graph of this configuration (after a rebuild,
        // another, so that the clean-walk counts have settled when the timing starts).  A list
        // past half its life is rebuilt first: a list that runs out inside the timed chunk makes
        // its remaining steps identity steps, which would time the configuration far too fast.
        int wrc = step_chunk(ci, false, &use0);
        if (wrc > 0) return wrc;
        if (need_rebuild_ || use0 > 0.5f) {
            if ((wrc = rebuild()) != VEDO_OK) return wrc;
            wrc = step_chunk(ci, false, nullptr);
            if (wrc > 0) return wrc;
            if (need_rebuild_ && (wrc = rebuild()) != VEDO_OK) return wrc;
        }
        const uint64_t rt = round_;
        MCK(cudaEventRecord(e0, stream_));
        int rc = step_chunk(ci, false, &use);
        if (rc > 0) return rc;
        MCK(cudaEventRecord(e1, stream_));
        MCK(cudaEventSynchronize(e1));
        float ms = 0.0f;
        MCK(cudaEventElapsedTime(&ms, e0, e1));
        // per step taken (should the list still have run out, its identity steps do not count
        // as steps: an overestimate, never an underestimate)
        *ms_per_step = ms / (float)std::max<uint64_t>(1, round_ - rt);
        if (growth) *growth = since_rebuild_ ? use / (float)since_rebuild_ : 0.0f;
        *taken += (uint32_t)(round_ - r0);
        return VEDO_OK;
    };
    int rc;
    if (need_rebuild_ && (rc = rebuild()) != VEDO_OK) return rc;
    // 1. tick block size (the list is unchanged, the tick time alone decides)
    float best = FLT_MAX;
    int best_tpb = tpb_;
    for (int b : blocks) {
        tpb_ = b;
        drop_graphs();
        float t = 0.0f;
        if ((rc = timed_chunk(&t, nullptr)) != VEDO_OK) return rc;
        if (need_rebuild_ && (rc = rebuild()) != VEDO_OK) return rc;
        if (t < best) { best = t; best_tpb = b; }
    }
    tpb_ = best_tpb;
    // 2. the pair test's hi/lo position splits: formed per pair, or stored once per step (the
    //    two ways give identical bits)
    {
        float t_form = 0.0f, t_store = 0.0f;
        xs_stored_ = false;
        drop_graphs();
        if ((rc = timed_chunk(&t_form, nullptr)) != VEDO_OK) return rc;
        xs_stored_ = true;
        drop_graphs();
        k_split<<<nblk(n_), TPB, 0, stream_>>>(n_, d_x_[cur_], d_xs_[cur_]);
        if ((rc = timed_chunk(&t_store, nullptr)) != VEDO_OK) return rc;
        if (need_rebuild_ && (rc = rebuild()) != VEDO_OK) return rc;
        xs_stored_ = t_store < t_form;
        drop_graphs();
    }
    // 2b. one full tick, the split tick (a light tick at full occupancy, the full tick over the
    //     spheres with a pair on the exact path) or the pair pass (each pair on the exact path
    //     evaluated once); identical results
    {
        float t_one = 0.0f, t_split = 0.0f, t_pair = 0.0f;
        split_tick_ = false;
        pair_pass_ = false;
        drop_graphs();
        if ((rc = timed_chunk(&t_one, nullptr)) != VEDO_OK) return rc;
        split_tick_ = true;
        drop_graphs();
        if ((rc = timed_chunk(&t_split, nullptr)) != VEDO_OK) return rc;
        if (need_rebuild_ && (rc = rebuild()) != VEDO_OK) return rc;
        split_tick_ = false;
        pair_pass_ = true;
        drop_graphs();
        if ((rc = ensure_pair_bufs(nl_[nlc_].ne)) != VEDO_OK) return rc;
        fill_mirror(nl_[nlc_]);
        if ((rc = timed_chunk(&t_pair, nullptr)) != VEDO_OK) return rc;
        if (need_rebuild_ && (rc = rebuild()) != VEDO_OK) return rc;
        pair_pass_ = t_pair < t_one && t_pair < t_split;
        split_tick_ = !pair_pass_ && t_split < t_one;
        if (!pair_pass_) free_pair_bufs();
        drop_graphs();
        // 2c. the chosen tick's check interval as one persistent launch, against the replayed
        //     graph of per-step kernels just timed (the full tick and the pair pass)
        persistent_ = false;
        if (!split_tick_ && !dyn_walls_) {
            const float t_graph = pair_pass_ ? t_pair : t_one;
            float t_pers = 0.0f;
            persistent_ = true;
            if ((rc = timed_chunk(&t_pers, nullptr)) != VEDO_OK) return rc;
            if (need_rebuild_ && (rc = rebuild()) != VEDO_OK) return rc;
            persistent_ = pk_grid_ > 0 && t_pers < t_graph;
        }
    }
    // 3. skin: tick time per step plus the amortised rebuild
    best = FLT_MAX;
    float best_skin = skin_frac_;
    for (float f : skins) {
        bool fits = true;                   // a periodic range must hold three cells of 2 r_max + skin
        for (const SceneHost& H : sc_)
            for (int k = 0; k < 3; ++k)
                if (H.pb.sw[k] && (2.0f + f) * H.rmax * (1.0f + 1e-5f) > H.pb.range32[k] / 3.0f) fits = false;
        if (!fits) continue;
        set_skin(f);
        // what a rebuild costs: the rebuild, then the first chunk of the new list (its steps walk
        // every list while the clean-walk counts settle, and its graph is captured)
        float trb = 0.0f, t = 0.0f, growth = 0.0f;
        {
            const uint64_t r0 = round_;
            MCK(cudaEventRecord(e0, stream_));
            if ((rc = rebuild()) != VEDO_OK) return rc;
            int wrc = step_chunk(ci, false, nullptr);
            if (wrc > 0) return wrc;
            MCK(cudaEventRecord(e1, stream_));
            MCK(cudaEventSynchronize(e1));
            MCK(cudaEventElapsedTime(&trb, e0, e1));
            *taken += (uint32_t)(round_ - r0);
        }
        if (need_rebuild_) {                           // the list did not last one chunk
            if ((rc = rebuild()) != VEDO_OK) return rc;
            continue;
        }
        {                                              // a settled chunk of the same list
            const uint64_t r0 = round_;
            float use = 0.0f, ms = 0.0f;
            MCK(cudaEventRecord(e0, stream_));
            int wrc = step_chunk(ci, false, &use);
            if (wrc > 0) return wrc;
            MCK(cudaEventRecord(e1, stream_));
            MCK(cudaEventSynchronize(e1));
            MCK(cudaEventElapsedTime(&ms, e0, e1));
            t = ms / (float)ci;
            growth = since_rebuild_ ? use / (float)since_rebuild_ : 0.0f;
            const bool short_list = round_ - r0 < ci;   // identity steps: the list did not last
            *taken += (uint32_t)(round_ - r0);
            if (short_list) {
                if ((rc = rebuild()) != VEDO_OK) return rc;
                continue;
            }
        }
        trb = std::max(0.0f, trb - t * (float)ci);
        // steps until the list's life is used up at this growth (the rebuild rule's margin)
        const float life = growth > 0.0f ? std::max((float)ci, 1.0f / growth - 2.0f * (float)ci) : 1e6f;
        const float cost = t + trb / life;
        if (cost < best) { best = cost; best_skin = f; }
    }
    set_skin(best_skin);
    // 4. cell scale: the rebuild time alone (the list does not depend on it)
    best = FLT_MAX;
    float best_cell = cell_scale_;
    for (float c : cells) {
        cell_scale_ = c;
        float trb = 0.0f;
        if ((rc = timed_rebuild(&trb)) != VEDO_OK) return rc;
        if (trb < best) { best = trb; best_cell = c; }
    }
    cell_scale_ = best_cell;
    need_rebuild_ = true;
    tune_pending_ = false;
    return VEDO_OK;
}

int MixedEngine::run(uint32_t nsteps, int* keep_running) {
    prof_[0] = prof_[1] = prof_[2] = prof_[3] = 0;
    prof_ticks_ = 0;
    launches_ = 0;
    MCK(cudaSetDevice(opts_.device));
    MCK(cudaEventRecord(ev_[0], stream_));
    const uint32_t ci = opts_.check_interval;
    uint32_t done = 0;
    if (tune_pending_ && nsteps > 1) {
        // the tuner's steps are steps of this call; the last one stays for the impulse output
        uint32_t t = 0;
        int rc = autotune(nsteps - 1, &t);
        if (rc != VEDO_OK) return rc;
        done += t;
    }
    while (done < nsteps) {
        if (need_rebuild_) {
            if (profiling_) MCK(cudaEventRecord(ev_[2], stream_));
            int rc = rebuild();
            if (rc != VEDO_OK) return rc;
            if (profiling_) {
                MCK(cudaEventRecord(ev_[3], stream_));
                MCK(cudaEventSynchronize(ev_[3]));
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, ev_[2], ev_[3]);
                prof_[2] += ms;
            }
        }
        const uint32_t chunk = std::min<uint32_t>(nsteps - done, ci - (uint32_t)(since_rebuild_ % ci));
        const uint64_t r0 = round_;
        int rc = step_chunk(chunk, done + chunk == nsteps, nullptr);
        if (rc > 0) return rc;
        done += (uint32_t)(round_ - r0);
    }
    MCK(cudaEventRecord(ev_[1], stream_));
    MCK(cudaStreamSynchronize(stream_));
    MCK(cudaGetLastError());
    float ms = 0;
    cudaEventElapsedTime(&ms, ev_[0], ev_[1]);
    prof_[3] = ms;
    if (keep_running) *keep_running = sc_[0].t < sc_[0].t_stop ? 1 : 0;
    return VEDO_OK;
}

int MixedEngine::get_state(const vedo_state_view& v) {
    double* dst[] = {v.position, v.velocity, v.angular_velocity, v.orientation_x, v.orientation_z, v.impact,
                     v.angular_impact};
    const double4_32a* src[] = {d_x_[cur_], d_v64_, d_w64_, d_ox_, d_oz_, d_imp_, d_aimp_};
    for (int k = 0; k < 7; ++k) {
        if (!dst[k]) continue;
        double* st = d_stage_ + (size_t)k * 3 * n_;
        k_unpack3m<<<nblk(n_), TPB, 0, stream_>>>(n_, 0u, d_int_of_, src[k], st);
        MCK(cudaMemcpyAsync(dst[k], st, 24 * (size_t)n_, cudaMemcpyDeviceToHost, stream_));
    }
    MCK(cudaStreamSynchronize(stream_));
    MCK(cudaGetLastError());
    return VEDO_OK;
}

// One step with per-object external impulses (SimMediator::Run(external impacts),
// SimMediator.cpp:987-1119): added to each sphere's compensated sums after the field and
// constrained impulses (walls, fixed or orbital, do not respond to impulses).
int MixedEngine::run_with_impulses(const double* impulse, const double* angular_impulse, int* keep_running) {
    MCK(cudaSetDevice(opts_.device));
    if (!d_ext_) MCK(cudaMalloc(&d_ext_, 2 * 24 * (size_t)n_));
    const double* src[2] = {impulse, angular_impulse};
    for (int k = 0; k < 2; ++k) {
        double* dst = d_ext_ + (size_t)k * 3 * n_;
        if (src[k]) {                              // the caller's order, gathered into storage order
            double* stg = d_stage_ + (size_t)k * 3 * n_;
            MCK(cudaMemcpyAsync(stg, src[k], 24 * (size_t)n_, cudaMemcpyHostToDevice, stream_));
            k_gather3<<<nblk(n_), TPB, 0, stream_>>>(n_, d_ext_of_, stg, dst);
        } else {
            MCK(cudaMemsetAsync(dst, 0, 24 * (size_t)n_, stream_));
        }
    }
    ext_on_ = true;
    const int rc = run(1, keep_running);
    ext_on_ = false;
    return rc;
}

int MixedEngine::list_status(double out[6]) {
    float dd[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    MCK(cudaMemcpyAsync(dd, d_disp_ + 4 * cur_, 16, cudaMemcpyDeviceToHost, stream_));
    MCK(cudaStreamSynchronize(stream_));
    uint32_t k;
    memcpy(&k, &dd[3], 4);
    out[0] = (double)k;
    out[1] = (double)rebuilds_;
    out[2] = dd[0];
    out[3] = dd[1];
    out[4] = dd[2];
    out[5] = skin_min_ > 0.0f ? std::max(std::max(2.0 * dd[0], (double)dd[1]) / skin_min_,
                                          ((double)dd[1] + dd[2]) / (WALL_SKIN * skin_min_))
                              : 0.0;
    return VEDO_OK;
}

int MixedEngine::quiet_spheres(uint64_t* count) {
    *count = 0;
    if (need_rebuild_ || !n_) return VEDO_OK;         // the next step starts with a new list
    unsigned c = 0;
    MCK(cudaMemsetAsync(d_red_ + 15, 0, 4, stream_));
    k_quiet_count<<<nblk(n_), TPB, 0, stream_>>>(n_, d_clear_, d_qcnt_, d_disp_ + 4 * cur_, d_red_ + 15);
    MCK(cudaMemcpyAsync(&c, d_red_ + 15, 4, cudaMemcpyDeviceToHost, stream_));
    MCK(cudaStreamSynchronize(stream_));
    *count = c;
    return VEDO_OK;
}

int MixedEngine::set_state(const vedo_state_view& v) {
    const double* srcs[] = {v.position, v.velocity, v.angular_velocity, v.orientation_x, v.orientation_z, v.impact,
                            v.angular_impact};
    double4_32a* dst[] = {d_x_[cur_], d_v64_, d_w64_, d_ox_, d_oz_, d_imp_, d_aimp_};
    // The list survives new state when no wall changed and the spheres' largest jump fits the
    // displacement bound: the jump is added to the bound (every pair may have closed by it).
    MCK(cudaMemsetAsync(d_red_, 0, 8, stream_));      // [0] largest sphere jump, [1] a wall changed
    for (int k = 0; k < 7; ++k) {
        if (!srcs[k]) continue;
        double* st = d_stage_ + (size_t)k * 3 * n_;
        MCK(cudaMemcpyAsync(st, srcs[k], 24 * (size_t)n_, cudaMemcpyHostToDevice, stream_));
        k_place<<<nblk(n_), TPB, 0, stream_>>>(n_, st, dst[k], d_ext_of_, d_model_of_, d_models_, k < 5 ? 1 : 0,
                                               k == 0 ? d_red_ : nullptr, d_red_ + 1);
    }
    k_copy32<<<nblk(n_), TPB, 0, stream_>>>(n_, d_v64_, d_v32_[cur_]);
    k_copy32<<<nblk(n_), TPB, 0, stream_>>>(n_, d_w64_, d_w32_[cur_]);
    unsigned jw[2] = {0u, 0u};
    float dd[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    MCK(cudaMemcpyAsync(jw, d_red_, 8, cudaMemcpyDeviceToHost, stream_));
    MCK(cudaMemcpyAsync(dd, d_disp_ + 4 * cur_, 16, cudaMemcpyDeviceToHost, stream_));
    MCK(cudaStreamSynchronize(stream_));
    MCK(cudaGetLastError());
    if (need_rebuild_ || jw[1]) {
        need_rebuild_ = true;
        return VEDO_OK;
    }
    if (jw[0]) {
        float j;
        memcpy(&j, &jw[0], 4);
        // the jump moves a sphere against its frame and absolutely (roundings of the sums: up)
        dd[0] = std::nextafter(dd[0] + j, FLT_MAX);
        dd[1] = std::nextafter(dd[1] + j, FLT_MAX);
        if (list_spent(dd[0], dd[1], dd[2], skin_min_, WALL_SKIN * skin_min_)) {
            need_rebuild_ = true;
            return VEDO_OK;
        }
        MCK(cudaMemcpyAsync(d_disp_ + 4 * cur_, dd, 8, cudaMemcpyHostToDevice, stream_));
        if (xs_stored_) k_split<<<nblk(n_), TPB, 0, stream_>>>(n_, d_x_[cur_], d_xs_[cur_]);
        MCK(cudaStreamSynchronize(stream_));
        MCK(cudaGetLastError());
    }
    return VEDO_OK;
}

int MixedEngine::num_interactions(uint32_t* n) {
    if (need_rebuild_) {
        int rc = rebuild();
        if (rc != VEDO_OK) return rc;
    }
    NList& L = nl_[nlc_];
    std::vector<uint32_t> slot(L.ne);
    if (L.ne) MCK(cudaMemcpy(slot.data(), L.slot, 4 * L.ne, cudaMemcpyDeviceToHost));
    uint32_t c = 0;
    for (uint32_t e = 0; e < L.ne; ++e) c += slot[e] == e;
    *n = c;
    return VEDO_OK;
}

int MixedEngine::get_interactions(const vedo_contact_view& v) {
    if (need_rebuild_) {
        int rc = rebuild();
        if (rc != VEDO_OK) return rc;
    }
    NList& L = nl_[nlc_];
    const uint32_t ne = L.ne;
    if (ne > act_cap_) {
        if (d_act_) cudaFree(d_act_);
        act_cap_ = ne + ne / 4 + 16;
        MCK(mal(&d_act_, act_cap_));
    }
    if (ne) k_active<<<nblk(n_), TPB, 0, stream_>>>(n_, args(false), d_act_);
    std::vector<uint32_t> ptr(n_ + 1), ent(ne), slot(ne);
    std::vector<uint8_t> act(ne), fl(ne);
    std::vector<float4> h(ne);
    MCK(cudaMemcpyAsync(ptr.data(), L.ptr, 4 * (n_ + 1), cudaMemcpyDeviceToHost, stream_));
    if (ne) {
        MCK(cudaMemcpyAsync(ent.data(), L.ent, 4 * ne, cudaMemcpyDeviceToHost, stream_));
        MCK(cudaMemcpyAsync(slot.data(), L.slot, 4 * ne, cudaMemcpyDeviceToHost, stream_));
        MCK(cudaMemcpyAsync(act.data(), d_act_, ne, cudaMemcpyDeviceToHost, stream_));
        MCK(cudaMemcpyAsync(fl.data(), L.f[cur_], ne, cudaMemcpyDeviceToHost, stream_));
        MCK(cudaMemcpyAsync(h.data(), L.h[cur_], sizeof(float4) * ne, cudaMemcpyDeviceToHost, stream_));
    }
    MCK(cudaStreamSynchronize(stream_));
    struct Row { uint32_t a, b, sl, ms; uint32_t e; };
    std::vector<uint32_t> ext(n_);
    MCK(cudaMemcpy(ext.data(), d_ext_of_, 4 * (size_t)n_, cudaMemcpyDeviceToHost));
    std::vector<Row> rows;
    for (uint32_t i = 0; i < n_; ++i)
        for (uint32_t e = ptr[i]; e < ptr[i + 1]; ++e) {
            if (slot[e] != e) continue;
            const uint32_t ei = ext[i], ej = ext[ent[e] & ~WALL_BIT];   // the caller's indices
            const bool wall = ent[e] & WALL_BIT;
            Row r;
            r.a = std::min(ei, ej);
            r.b = std::max(ei, ej);
            r.sl = wall ? ei : std::min(ei, ej);
            r.ms = wall ? ej : std::max(ei, ej);
            r.e = e;
            rows.push_back(r);
        }
    std::sort(rows.begin(), rows.end(), [](const Row& x, const Row& y) { return x.a != y.a ? x.a < y.a : x.b < y.b; });
    for (size_t k = 0; k < rows.size(); ++k) {
        const Row& r = rows[k];
        if (v.first) v.first[k] = r.a;
        if (v.second) v.second[k] = r.b;
        if (v.slave) v.slave[k] = r.sl;
        if (v.master) v.master[k] = r.ms;
        if (v.active) v.active[k] = act[r.e] ? 1 : 0;
        if (v.contact) v.contact[k] = (fl[r.e] & HF_CONTACT) ? 1 : 0;
        if (v.kn) v.kn[k] = h[r.e].w;
        if (v.shear) {
            v.shear[3 * k] = h[r.e].x;
            v.shear[3 * k + 1] = h[r.e].y;
            v.shear[3 * k + 2] = h[r.e].z;
        }
    }
    return VEDO_OK;
}

int MixedEngine::get_observables(double out[13]) {
    if (need_rebuild_) {
        int rc = rebuild();
        if (rc != VEDO_OK) return rc;
    }
    NList& L = nl_[nlc_];
    if (L.ne > act_cap_) {
        if (d_act_) cudaFree(d_act_);
        act_cap_ = L.ne + L.ne / 4 + 16;
        MCK(mal(&d_act_, act_cap_));
    }
    if (L.ne) k_active<<<nblk(n_), TPB, 0, stream_>>>(n_, args(false), d_act_);
    const unsigned nb = std::max(1u, nblk(n_));
    double* part = d_obs_;
    double* res = d_obs_ + (size_t)nb * 16 + 16;
    const d3 g = mk(sc_[0].g[0], sc_[0].g[1], sc_[0].g[2]);
    obs::k_obs_a<<<nb, TPB, 0, stream_>>>(n_, d_model_of_, d_models_, d_x_[cur_], d_v64_, d_w64_, g, part);
    obs::k_obs_reduce<<<1, 32, 0, stream_>>>(nb, 16, part, res, 12);
    obs::k_obs_b<<<nb, TPB, 0, stream_>>>(n_, d_model_of_, d_models_, d_x_[cur_], d_v64_, d_w64_, res, 0, d_act_,
                                          L.ne, part);
    obs::k_obs_reduce<<<1, 32, 0, stream_>>>(nb, 6, part, res + 16, 6);
    double r[22];
    MCK(cudaMemcpyAsync(r, res, sizeof(r), cudaMemcpyDeviceToHost, stream_));
    MCK(cudaStreamSynchronize(stream_));
    const bool any = r[9] > 0;
    out[0] = r[0]; out[1] = r[1]; out[2] = r[2];
    out[3] = any ? r[12] : 0.0; out[4] = any ? r[13] : 0.0; out[5] = any ? r[14] : 0.0; out[6] = any ? r[15] : 0.0;
    out[7] = r[16]; out[8] = r[17]; out[9] = r[21];
    const double msum = r[10];
    out[10] = msum > 0 ? r[18] / msum : 0.0;
    out[11] = msum > 0 ? r[19] / msum : 0.0;
    out[12] = msum > 0 ? r[20] / msum : 0.0;
    return VEDO_OK;
}

// the observables' view of the state: positions of the current parity, single-scene engines only
// Positions and models in the caller's object order (the coordination numbers and the VTK file
// list objects in that order).
int MixedEngine::caller_view() {
    if (!d_xe_) {
        MCK(mal(&d_xe_, n_));
        MCK(mal(&d_model_e_, n_));
    }
    k_to_caller<<<nblk(n_), TPB, 0, stream_>>>(n_, d_int_of_, d_x_[cur_], d_model_of_, d_xe_, d_model_e_);
    MCK(cudaGetLastError());
    return VEDO_OK;
}

DeviceObjects MixedEngine::objects() {
    DeviceObjects d;
    d.n = n_; d.model_of = d_model_e_; d.models = d_models_; d.pos = d_xe_;
    d.stream = stream_; d.scratch = &scratch_; d.launches = &launches_;
    d.scene = sc_.size() == 1 ? host_[0].get() : nullptr;
    return d;
}

int MixedEngine::coordination(uint32_t* below, uint32_t* touching, const double* box, double* average) {
    const int vr = caller_view();
    if (vr != VEDO_OK) return vr;
    std::string m;
    const int rc = coordination_host(objects(), below, touching, box, average, m);
    return rc == VEDO_OK ? rc : fail(rc, m);
}

int MixedEngine::write_vtk(const char* path, int with_coordination) {
    const int vr = caller_view();
    if (vr != VEDO_OK) return vr;
    std::string m;
    const int rc = write_vtk_host(this, objects(), path, with_coordination, m);
    return rc == VEDO_OK ? rc : fail(rc, m);
}

int MixedEngine::write_ido(const char* path) {
    if (sc_.size() != 1) return fail(VEDO_ERR_INVALID_ARGUMENT, "write_ido needs a single-scene engine");
    HScene hs = *host_[0];
    vedo_state_view v{hs.pos.data(), hs.vel.data(), hs.av.data(), hs.ox.data(), hs.oz.data(), hs.imp.data(),
                      hs.aimp.data()};
    int rc = get_state(v);
    if (rc != VEDO_OK) return rc;
    hs.time_current = sc_[0].t;
    uint32_t np = 0;
    rc = num_interactions(&np);
    if (rc != VEDO_OK) return rc;
    std::vector<uint32_t> a(np), b(np);
    std::vector<uint8_t> act(np), con(np);
    std::vector<double> sh(3 * (size_t)np), kn(np);
    vedo_contact_view cv{a.data(), b.data(), nullptr, nullptr, act.data(), sh.data(), kn.data(), con.data()};
    rc = get_interactions(cv);
    if (rc != VEDO_OK) return rc;
    HRecords R;
    for (uint32_t k = 0; k < np; ++k) {
        if (!act[k]) continue;
        R.first.push_back(a[k]); R.second.push_back(b[k]);
        R.contact.push_back(con[k]); R.bond.push_back(0);
        R.kn.push_back(kn[k]); R.v0.push_back(0.0);
        for (int q = 0; q < 3; ++q) {
            R.shear.push_back(sh[3 * k + q]);
            R.point.push_back(0.0); R.dirn.push_back(0.0); R.imp.push_back(0.0); R.aimp.push_back(0.0);
        }
        R.overlap.push_back(0.0);
    }
    HScene s = hs;
    s.rec = R;
    std::string msg;
    if (!vedo::write_ido(path, s, msg)) return fail(VEDO_ERR_IO, msg);
    return VEDO_OK;
}

EngineBase* make_mixed_engine() { return new (std::nothrow) MixedEngine(); }

// batch construction for the C ABI (capi.cpp)
EngineBase* make_mixed_batch(const std::vector<const HScene*>& scenes, const vedo_engine_opts& opts, int* rc,
                             std::string* err) {
    MixedEngine* e = new (std::nothrow) MixedEngine();
    if (!e) {
        *rc = VEDO_ERR_OUT_OF_MEMORY;
        return nullptr;
    }
    *rc = e->init_batch(scenes, opts);
    if (*rc != VEDO_OK) {
        *err = e->error();
        delete e;
        return nullptr;
    }
    return e;
}

int mixed_scene_range(EngineBase* e, uint32_t s, uint32_t* off, uint32_t* n, double* t) {
    MixedEngine* m = dynamic_cast<MixedEngine*>(e);
    if (!m) return VEDO_ERR_INVALID_ARGUMENT;
    int rc = m->scene_range(s, off, n);
    if (rc == VEDO_OK && t) *t = m->scene_time(s);
    return rc;
}

// Continuous batching (serve.cpp): a new engine from scenes `keep` of `prev` (their device
// state and histories move over) followed by the host scenes `add`.
EngineBase* mixed_repack(EngineBase* prev, const std::vector<uint32_t>& keep, const std::vector<const HScene*>& add,
                         const vedo_engine_opts& opts, int* rc, std::string* err) {
    MixedEngine* p = prev ? dynamic_cast<MixedEngine*>(prev) : nullptr;
    if (prev && !p) {
        *rc = VEDO_ERR_INVALID_ARGUMENT;
        *err = "repack needs a MIXED-form engine";
        return nullptr;
    }
    std::vector<MixedEngine::SceneSource> src;
    for (uint32_t k : keep) src.push_back(MixedEngine::SceneSource{nullptr, (int)k});
    for (const HScene* h : add) src.push_back(MixedEngine::SceneSource{h, -1});
    MixedEngine* e = new (std::nothrow) MixedEngine();
    if (!e) {
        *rc = VEDO_ERR_OUT_OF_MEMORY;
        return nullptr;
    }
    *rc = e->init_from(src, p, opts);
    if (*rc != VEDO_OK) {
        *err = e->error();
        delete e;
        return nullptr;
    }
    return e;
}

int mixed_set_scene_active(EngineBase* e, uint32_t s, bool on) {
    MixedEngine* m = dynamic_cast<MixedEngine*>(e);
    return m ? m->set_scene_active(s, on) : VEDO_ERR_INVALID_ARGUMENT;
}

int mixed_get_state_slice(EngineBase* e, uint32_t off, uint32_t cnt, const vedo_state_view& v) {
    MixedEngine* m = dynamic_cast<MixedEngine*>(e);
    return m ? m->get_state_slice(off, cnt, v) : VEDO_ERR_INVALID_ARGUMENT;
}

uint64_t mixed_scene_steps(EngineBase* e, uint32_t s) {
    MixedEngine* m = dynamic_cast<MixedEngine*>(e);
    return m ? m->steps_of_scene(s) : 0;
}

uint32_t mixed_num_scenes(EngineBase* e) {
    MixedEngine* m = dynamic_cast<MixedEngine*>(e);
    return m ? m->num_scenes() : 1u;
}

// The persistent tick's grid barrier on its own (vedo_gpu_barrier_check).
static int barrier_check_on(int device, uint32_t rounds, uint32_t extra, uint64_t limit_ns, uint32_t out[4]) {
    if (cudaSetDevice(device) != cudaSuccess) return VEDO_ERR_CUDA;
    int sms = 0, b = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return VEDO_ERR_CUDA;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_bar_check, 256, 0) != cudaSuccess || b < 1)
        return VEDO_ERR_CUDA;
    unsigned* d = nullptr;
    if (cudaMalloc(&d, 8 * sizeof(unsigned)) != cudaSuccess) return VEDO_ERR_OUT_OF_MEMORY;
    int rc = VEDO_OK;
    unsigned h[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    GridBar g;
    g.w = d;
    g.nblocks = (uint32_t)(sms * b) + extra;
    g.limit_ns = limit_ns;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)(sms * b));
    cfg.blockDim = dim3(256);
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    if (cudaMemset(d, 0, 8 * sizeof(unsigned)) != cudaSuccess ||
        cudaLaunchKernelEx(&cfg, k_bar_check, g, rounds, d + 4, d + 6) != cudaSuccess ||
        cudaDeviceSynchronize() != cudaSuccess || cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess)
        rc = VEDO_ERR_CUDA;
    cudaFree(d);
    out[0] = h[6];
    out[1] = h[7];
    out[2] = h[2];
    out[3] = h[3];
    return rc;
}
// (the caller's current device is left as it was)
static int barrier_check(int device, uint32_t rounds, uint32_t extra, uint64_t limit_ns, uint32_t out[4]) {
    int prev = 0;
    if (cudaGetDevice(&prev) != cudaSuccess) return VEDO_ERR_CUDA;
    const int rc = barrier_check_on(device, rounds, extra, limit_ns, out);
    cudaSetDevice(prev);
    return rc;
}

}  // namespace vedo

extern "C" int vedo_gpu_barrier_check(int32_t device, uint32_t rounds, uint32_t extra, uint64_t limit_ns,
                                      uint32_t out[4]) {
    if (!out || rounds == 0 || limit_ns == 0) return VEDO_ERR_INVALID_ARGUMENT;
    return vedo::barrier_check(device, rounds, extra, limit_ns, out);
}
