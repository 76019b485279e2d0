// engine.cu - FP64 DEM time step and NBS broad phase on the GPU.
//
// Built with -fmad=false: the FP64 arithmetic below reproduces the reference's IEEE
// operation sequence (see dem_physics.cuh).  Per time step (SimMediator::Run,
// SimMediator.cpp:714-842) two kernels run:
//   k_pair_pf, k_pair_exact - the FP32 prefilter over every candidate pair, then for the
//             pairs it leaves (in full warps): narrow phase at the current positions (the
//             ContactInfo the reference computed at the end of the previous step) + impact
//             solver + status update; the impulses go to a per-pair output record.
//   k_obj   - one thread per local object: the pair impulses in candidate-list order
//             (the reference's IactContainer order), the field impulse, the external
//             force and DiscreteObject::Response.  Scope-global objects (walls) are
//             summed by one warp each in k_obj_global (ordered, warp-cooperative loads).
// Every UpIact steps the candidate list is rebuilt with NBSConsultant's rule
// (NBSConsultant.cpp:85-374): cell keys, a stable radix sort, cell ranges, then a count
// and a fill pass over (object, neighbour slot) tasks laid out in the reference's
// traversal order, so the new list equals the reference's list element for element.
#include "engine.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>

#include "dem_physics.cuh"
#include "prefilter.cuh"
#include "observables.cuh"

namespace vedo {

namespace {

constexpr int TPB = 256;
inline unsigned blocks_for(uint64_t n, int tpb = TPB) { return (unsigned)((n + tpb - 1) / tpb); }
// Candidate lists up to this length take the one-pass pair kernel (the step is launch-bound there)
constexpr uint32_t FUSED_PAIRS = 1u << 17;

// Neighbour visiting order of NBSConsultant::Reset (NBSConsultant.cpp:202-270):
// 12 = the cell itself (i < j), 13 = all scope-global objects.
__constant__ int c_slot[15][3] = {{-1, -1, -1}, {-1, -1, 0}, {-1, -1, 1}, {0, -1, -1}, {0, -1, 0},
                                  {0, -1, 1},   {1, -1, -1}, {1, -1, 0},  {1, -1, 1},  {-1, 0, -1},
                                  {-1, 0, 0},   {0, 0, -1},  {0, 0, 0},   {0, 0, 0},   {1, 0, -1}};
constexpr int SLOT_SELF = 12;
constexpr int SLOT_GLOBAL = 13;
constexpr int NSLOT = 15;
// LeapConsultant::subReset (LeapConsultant.h:195-446): the 13 half-shell neighbours, then the
// cell itself (13), then the scope-global objects (14).
__constant__ int c_slot_leap[13][3] = {{-1, -1, -1}, {-1, -1, 0}, {-1, -1, 1}, {0, -1, -1}, {0, -1, 0},
                                       {0, -1, 1},   {1, -1, -1}, {1, -1, 0},  {1, -1, 1},  {-1, 0, -1},
                                       {-1, 0, 0},   {0, 0, -1},  {1, 0, -1}};

// The broad phase's cell-key layout: the axis order of the key (the consultant's comparator:
// NBS and TrirLeX x, y, z; TrirLeY y, x, z; TrirLeZ z, x, y, NBSConsultant.h:62-128), the key's
// extent per axis, the number of zones per axis and, for the Leap consultant, its periodic axes.
struct CellGrid {
    int mode;                  // key order: 0 x, y, z (NBS, TrirLeX); 1 y, x, z (TrirLeY); 2 z, x, y (TrirLeZ)
    uint64_t dim[3];           // key extent per axis (x, y, z)
    uint32_t ncel[3];          // zones per axis (x, y, z): the last zone is ncel - 1
    int leap;                  // 1: LeapConsultant's traversal
    int pbc[3], has_pbc;       // Leap: axes whose neighbours wrap (LeapConsultant.h:146-150)
};
// (fixed indices per mode: the zone coordinates stay in registers)
__host__ __device__ inline uint64_t grid_key(const CellGrid& g, const uint64_t c[3]) {
    if (g.mode == 1) return (c[1] * g.dim[0] + c[0]) * g.dim[2] + c[2];
    if (g.mode == 2) return (c[2] * g.dim[0] + c[0]) * g.dim[1] + c[1];
    return (c[0] * g.dim[1] + c[1]) * g.dim[2] + c[2];
}
__device__ inline void grid_cell(const CellGrid& g, uint64_t key, uint64_t c[3]) {
    if (g.mode == 1) {
        c[2] = key % g.dim[2]; key /= g.dim[2]; c[0] = key % g.dim[0]; c[1] = key / g.dim[0];
    } else if (g.mode == 2) {
        c[1] = key % g.dim[1]; key /= g.dim[1]; c[0] = key % g.dim[0]; c[2] = key / g.dim[0];
    } else {
        c[2] = key % g.dim[2]; key /= g.dim[2]; c[1] = key % g.dim[1]; c[0] = key / g.dim[1];
    }
}

// order-preserving map of doubles to unsigned 64-bit integers (for exact atomic min/max)
__host__ __device__ inline unsigned long long ord_of(double d) {
    unsigned long long b;
    memcpy(&b, &d, 8);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__host__ __device__ inline double dbl_of(unsigned long long o) {
    unsigned long long b = (o >> 63) ? (o & 0x7fffffffffffffffull) : ~o;
    double d;
    memcpy(&d, &b, 8);
    return d;
}

// ------------------------------------------------------------------------------------
// time step
// CalculateImpact in two passes, so that the FP64 work runs in full warps (the FP64 pipe issues a
// warp instruction at the same cost however few of its lanes are active, and most candidate pairs
// are apart):
//  k_pair_pf     one thread per candidate pair: the FP32 prefilter; a pair that is certainly apart
//                and carries no normal bond gets ImpactStatus::Clean and no impulse, the others are
//                appended to the worklist (warp-aggregated);
//  k_pair_exact  the worklist's pairs: narrow phase at the current positions + impact solver +
//                status update, each pair's operations exactly those of a single pass, written to
//                the pair's own records (the order of the worklist does not matter).
__global__ void __launch_bounds__(TPB) k_pair_pf(uint32_t np, const uint2* __restrict__ sm,
                                                 const uint32_t* __restrict__ param,
                                                 const PairParam* __restrict__ params, const float* __restrict__ reach,
                                                 const float4* __restrict__ pos32, const float4* __restrict__ wall32,
                                                 double4_32a* __restrict__ hist, double* __restrict__ v0,
                                                 uint8_t* __restrict__ flags, Periodic pb, uint32_t* __restrict__ work,
                                                 uint32_t* __restrict__ nwork) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    bool near = false;
    if (k < np) {
        const uint2 p = sm[k];
        const uint32_t pi = param[k];
        const int cd = params[pi].cd, is = params[pi].is;
        // Pairs that are certainly apart and carry no normal bond: ImpactStatus::Clean, no impulse.
        const bool bondable = (is == IS_BSDBF || is == IS_BTSDBF || is == IS_BSDB2F) && params[pi].c[4] != 0.0;
        if (!bondable &&
            certainly_apart(cd, pos32[p.x], pos32[p.y], wall32[p.y], reach[pi], pb.on ? pb.range32 : nullptr)) {
            const uint8_t f0 = flags[k];
            if (f0 & PF_NONZERO) {
                hist[k] = make_double4_32a(0.0, 0.0, 0.0, 0.0);
                v0[k] = 0.0;
            }
            if (f0 != 0) flags[k] = 0;
        } else {
            near = true;
        }
    }
    const unsigned m = __ballot_sync(0xffffffffu, near);
    if (m) {
        const int lane = threadIdx.x & 31, lead = __ffs(m) - 1;
        uint32_t at = 0;
        if (lane == lead) at = atomicAdd(nwork, (uint32_t)__popc(m));
        at = __shfl_sync(0xffffffffu, at, lead);
        if (near) work[at + __popc(m & ((1u << lane) - 1u))] = k;
    }
}

__device__ __forceinline__ void pair_exact(uint32_t k, const uint2* __restrict__ sm,
                                           const uint32_t* __restrict__ param, const PairParam* __restrict__ params,
                                           const double4_32a* __restrict__ geom, const double4_32a* __restrict__ hole,
                                           const double4_32a* __restrict__ pos,
                                           const double4_32a* __restrict__ vel, const double4_32a* __restrict__ av,
                                           const double4_32a* __restrict__ ox, const double4_32a* __restrict__ oz,
                                           double4_32a* __restrict__ hist, double* __restrict__ v0,
                                           uint8_t* __restrict__ flags, double* __restrict__ out, double dt,
                                           int backup, const Periodic& pb, uint8_t* __restrict__ touched) {
    const uint2 p = sm[k];
    const uint32_t pi = param[k];
    const int cd = params[pi].cd, is = params[pi].is;
    const double4_32a gg = geom[pi];
    PairGeom g{gg.x, gg.y, gg.z, gg.w, 0.0, 0.0, 0.0};
    if (cd == CD_SHP) {
        const double4_32a hh = hole[pi];
        g.hr = hh.x; g.hxo = hh.y; g.hyo = hh.z;
    }
    const d3 Ps = ld(pos, p.x), Pm = ld(pos, p.y);
    double depth;
    d3 n, point;
    detect_pair(cd, g, Ps, Pm, ox, oz, p.y, pb, depth, n, point);
    const bool active = depth > 0.0;
    const uint8_t f0 = flags[k];
    PairStatus st;
    st.f = f0 & (PF_STATUS | PF_NONZERO);
    if (backup) {                                             // ImpactStatus::Backup (ImpactStatus.h:174-178)
        uint8_t s2 = st.f & (uint8_t)~(ST_LAST_CONTACT | ST_LAST_BOND);
        if (st.f & ST_CONTACT) s2 |= ST_LAST_CONTACT;
        if (st.f & ST_BOND) s2 |= ST_LAST_BOND;
        st.f = s2;
    }
    const double* c = params[pi].c;
    const bool bonded = (is == IS_BSDBF || is == IS_BTSDBF || is == IS_BSDB2F) && normal_bond(c[0], c[4], depth);
    if (!active && !bonded) {                                 // ImpactStatus::Clean, nothing added
        if (st.f & PF_NONZERO) {
            hist[k] = make_double4_32a(0.0, 0.0, 0.0, 0.0);
            v0[k] = 0.0;
        }
        if (f0 != 0) flags[k] = 0;
        return;
    }
    if (st.f & PF_NONZERO) {
        double4_32a h = hist[k];
        st.shear = mk(h.x, h.y, h.z);
        st.kn = h.w;
        st.v0 = v0[k];
    } else {
        st.shear = mk(0.0, 0.0, 0.0);
        st.kn = 0.0;
        st.v0 = 0.0;
    }
    const d3 Va = ld(vel, p.x), Vb = ld(vel, p.y), AVa = ld(av, p.x), AVb = ld(av, p.y);
    d3 J, tA, tB;
    const uint8_t app = solve_pair(is, c, active, depth, n, point, Ps, Pm, Va, Vb, AVa, AVb, dt, pb, st, J, tA, tB);
    if (st.f & PF_NONZERO) {
        hist[k] = make_double4_32a(st.shear.x, st.shear.y, st.shear.z, st.kn);
        v0[k] = st.v0;
    }
    flags[k] = st.f | app | (active ? PF_ACTIVE : 0);
    if (app) {
        double* o = out + 9 * (size_t)k;
        o[0] = J.x; o[1] = J.y; o[2] = J.z;
        o[3] = tA.x; o[4] = tA.y; o[5] = tA.z;
        o[6] = tB.x; o[7] = tB.y; o[8] = tB.z;
        touched[p.x] = 1;              // both objects have an impulse to gather this step
        touched[p.y] = 1;
    }
}

// Both passes in one thread per candidate pair, for short lists (one launch less per step where
// the step is launch-bound; the same operations per pair).
__global__ void __launch_bounds__(TPB) k_pair_fused(uint32_t np, const uint2* __restrict__ sm,
                                                    const uint32_t* __restrict__ param,
                                                    const PairParam* __restrict__ params,
                                                    const double4_32a* __restrict__ geom,
                                                    const double4_32a* __restrict__ hole,
                                                    const float* __restrict__ reach,
                                                    const double4_32a* __restrict__ pos,
                                                    const double4_32a* __restrict__ vel,
                                                    const double4_32a* __restrict__ av,
                                                    const double4_32a* __restrict__ ox,
                                                    const double4_32a* __restrict__ oz,
                                                    const float4* __restrict__ pos32,
                                                    const float4* __restrict__ wall32, double4_32a* __restrict__ hist,
                                                    double* __restrict__ v0, uint8_t* __restrict__ flags,
                                                    double* __restrict__ out, double dt, int backup, Periodic pb,
                                                    uint8_t* __restrict__ touched) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= np) return;
    const uint2 p = sm[k];
    const uint32_t pi = param[k];
    const int cd = params[pi].cd, is = params[pi].is;
    const bool bondable = (is == IS_BSDBF || is == IS_BTSDBF || is == IS_BSDB2F) && params[pi].c[4] != 0.0;
    if (!bondable && certainly_apart(cd, pos32[p.x], pos32[p.y], wall32[p.y], reach[pi], pb.on ? pb.range32 : nullptr)) {
        const uint8_t f0 = flags[k];
        if (f0 & PF_NONZERO) {
            hist[k] = make_double4_32a(0.0, 0.0, 0.0, 0.0);
            v0[k] = 0.0;
        }
        if (f0 != 0) flags[k] = 0;
        return;
    }
    pair_exact(k, sm, param, params, geom, hole, pos, vel, av, ox, oz, hist, v0, flags, out, dt, backup, pb, touched);
}

__global__ void __launch_bounds__(TPB) k_pair_exact(const uint32_t* __restrict__ work,
                                                    const uint32_t* __restrict__ nwork, const uint2* __restrict__ sm,
                                                    const uint32_t* __restrict__ param,
                                                    const PairParam* __restrict__ params,
                                                    const double4_32a* __restrict__ geom,
                                                    const double4_32a* __restrict__ hole,
                                                    const double4_32a* __restrict__ pos,
                                                    const double4_32a* __restrict__ vel,
                                                    const double4_32a* __restrict__ av,
                                                    const double4_32a* __restrict__ ox,
                                                    const double4_32a* __restrict__ oz, double4_32a* __restrict__ hist,
                                                    double* __restrict__ v0, uint8_t* __restrict__ flags,
                                                    double* __restrict__ out, double dt, int backup, Periodic pb,
                                                    uint8_t* __restrict__ touched) {
    const uint32_t nw = *nwork;
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nw; q += gridDim.x * blockDim.x)
        pair_exact(work[q], sm, param, params, geom, hole, pos, vel, av, ox, oz, hist, v0, flags, out, dt, backup, pb,
                   touched);
}

__device__ __forceinline__ void add_entry(uint32_t ent, uint8_t f, const double* __restrict__ out, d3& J, d3& JA) {
    if (!(f & PF_APPLIED)) return;
    const double* o = out + 9 * (size_t)(ent >> 1);
    const d3 Jk = mk(o[0], o[1], o[2]);
    if (ent & 1) {                                            // master: B->AddImpact(-1.0 * ImpactA, tB)
        J = add(J, neg(Jk));
        if (f & PF_ANGULAR) JA = add(JA, mk(o[6], o[7], o[8]));
    } else {                                                  // slave: A->AddImpact(ImpactA, tA)
        J = add(J, Jk);
        if (f & PF_ANGULAR) JA = add(JA, mk(o[3], o[4], o[5]));
    }
}

// FP32 copies used by the prefilters: position relative to `origin`, and for plates and
// cylinders the unit axis with a validity flag (plates need an orthogonal Ox/Oz frame for
// the plane bound).
__device__ __forceinline__ void write32(uint32_t i, int shape, d3 P, d3 Ox, d3 Oz, d3 origin,
                                        float4* __restrict__ pos32, float4* __restrict__ wall32) {
    pos32[i] = make_float4((float)(P.x - origin.x), (float)(P.y - origin.y), (float)(P.z - origin.z), 0.0f);
    if (shape != SHAPE_SPHERE) {
        const double lz = len(Oz), lx = len(Ox);
        bool ok = lz > 0.0;
        if (shape == SHAPE_PLATE || shape == SHAPE_HOLED) ok = ok && lx > 0.0 && fabs(dot(Ox, Oz)) <= 1e-9 * lx * lz;
        wall32[i] = ok ? make_float4((float)(Oz.x / lz), (float)(Oz.y / lz), (float)(Oz.z / lz), 1.0f)
                       : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
}

__device__ __forceinline__ void finish_object(uint32_t i, const ModelDev& m, d3 J, d3 JA, double dt, d3 fimp,
                                              double4_32a* __restrict__ pos, double4_32a* __restrict__ vel,
                                              double4_32a* __restrict__ av, double4_32a* __restrict__ ox,
                                              double4_32a* __restrict__ oz, double4_32a* __restrict__ imp,
                                              double4_32a* __restrict__ aimp, int write_imp, d3 origin,
                                              float4* __restrict__ pos32, float4* __restrict__ wall32,
                                              const double* __restrict__ ext_imp, const double* __restrict__ ext_aimp,
                                              const Periodic& pb) {
    J = add(J, muls(fimp, m.sudo));                           // DOContainer::AddFieldImpact (DOContainer.cpp:25)
    J = add(J, smul(dt, mk(m.ext[0], m.ext[1], m.ext[2])));   // DiscreteObject::AddConstrainedImpact (:160-163)
    if (ext_imp) {                 // SimMediator::Run(external impacts): DOContainer::AddImpact (SimMediator.cpp:1015-1018)
        J = add(J, mk(ext_imp[3 * (size_t)i], ext_imp[3 * (size_t)i + 1], ext_imp[3 * (size_t)i + 2]));
        JA = add(JA, mk(ext_aimp[3 * (size_t)i], ext_aimp[3 * (size_t)i + 1], ext_aimp[3 * (size_t)i + 2]));
    }
    if (m.behavior != BEH_FIXED) {
        d3 P = ld(pos, i), V = ld(vel, i), AV = ld(av, i), Ox = ld(ox, i), Oz = ld(oz, i);
        respond_object(m, dt, J, JA, P, V, AV, Ox, Oz);
        if (pb.on) P = wrap_position(pb, P);                 // DOContainer::EnforcePeriodicBoundaryConditions
        st(pos, i, P, 0.0);
        st(ox, i, Ox, 0.0);
        st(oz, i, Oz, 0.0);
        if (m.behavior != BEH_ORBITAL) {
            st(vel, i, V, 0.0);
            st(av, i, AV, 0.0);
        }
        write32(i, m.shape, P, Ox, Oz, origin, pos32, wall32);
    } else if (pb.on) {            // the wrap moves every object, fixed ones included (SimMediator.cpp:746)
        const d3 P = ld(pos, i), W = wrap_position(pb, P);
        if (W.x != P.x || W.y != P.y || W.z != P.z) {
            st(pos, i, W, 0.0);
            write32(i, m.shape, W, ld(ox, i), ld(oz, i), origin, pos32, wall32);
        }
    }
    if (write_imp) {                                          // DiscreteObject::ClearImpact (:141-147)
        st(imp, i, J, 0.0);
        st(aimp, i, JA, 0.0);
    }
}

__global__ void __launch_bounds__(TPB) k_obj(uint32_t n, const uint32_t* __restrict__ model_of,
                                             const ModelDev* __restrict__ models, double4_32a* __restrict__ pos,
                                             double4_32a* __restrict__ vel, double4_32a* __restrict__ av,
                                             double4_32a* __restrict__ ox, double4_32a* __restrict__ oz,
                                             double4_32a* __restrict__ imp, double4_32a* __restrict__ aimp,
                                             const uint32_t* __restrict__ csr_ptr, const uint32_t* __restrict__ csr_ent,
                                             const uint8_t* __restrict__ flags, const double* __restrict__ out,
                                             double dt, d3 fimp, int write_imp, d3 origin, float4* __restrict__ pos32,
                                             float4* __restrict__ wall32, const double* __restrict__ ext_imp,
                                             const double* __restrict__ ext_aimp, Periodic pb,
                                             uint8_t* __restrict__ touched, uint32_t* __restrict__ nwork) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) *nwork = 0u;                                   // the pair worklist, empty for the next step
    if (i >= n) return;
    const ModelDev& m = models[model_of[i]];
    if (m.scope == SCOPE_GLOBAL) return;
    d3 J = mk(0.0, 0.0, 0.0), JA = mk(0.0, 0.0, 0.0);
    // an object no pair applied an impulse to keeps zero sums: its ordered walk adds nothing
    if (touched[i]) {
        touched[i] = 0;
        const uint32_t e0 = csr_ptr[i], e1 = csr_ptr[i + 1];
        // the entries that applied an impulse are marked first (integer work), then summed in entry
        // order: a warp issues each FP64 add once per marked entry of its busiest object, not once
        // per candidate entry (most candidates of an object apply nothing)
        const uint32_t c1 = min(e1, e0 + 64u);
        unsigned long long mark = 0ull;
        for (uint32_t e = e0; e < c1; ++e)
            if (flags[csr_ent[e] >> 1] & PF_APPLIED) mark |= 1ull << (e - e0);
        for (; mark; mark &= mark - 1) {
            const uint32_t ent = csr_ent[e0 + (uint32_t)(__ffsll(mark) - 1)];
            add_entry(ent, flags[ent >> 1], out, J, JA);
        }
        for (uint32_t e = c1; e < e1; ++e) {                   // long lists: the entries after 64
            const uint32_t ent = csr_ent[e];
            add_entry(ent, flags[ent >> 1], out, J, JA);
        }
    }
    finish_object(i, m, J, JA, dt, fimp, pos, vel, av, ox, oz, imp, aimp, write_imp, origin, pos32, wall32, ext_imp,
                  ext_aimp, pb);
}

// One warp per scope-global object: lanes load 32 entries at a time, then every lane adds
// them in order (shuffle broadcast), which keeps the reference's summation order.
__global__ void k_obj_global(uint32_t nglob, const uint32_t* __restrict__ glob, const uint32_t* __restrict__ model_of,
                             const ModelDev* __restrict__ models, double4_32a* __restrict__ pos,
                             double4_32a* __restrict__ vel, double4_32a* __restrict__ av, double4_32a* __restrict__ ox,
                             double4_32a* __restrict__ oz, double4_32a* __restrict__ imp, double4_32a* __restrict__ aimp,
                             const uint32_t* __restrict__ csr_ptr, const uint32_t* __restrict__ csr_ent,
                             const uint8_t* __restrict__ flags, const double* __restrict__ out, double dt, d3 fimp,
                             int write_imp, d3 origin, float4* __restrict__ pos32, float4* __restrict__ wall32,
                             const double* __restrict__ ext_imp, const double* __restrict__ ext_aimp, Periodic pb,
                             uint8_t* __restrict__ touched) {
    const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= nglob) return;
    const uint32_t i = glob[w];
    if (lane == 0 && touched[i]) touched[i] = 0;
    const ModelDev& m = models[model_of[i]];
    d3 J = mk(0.0, 0.0, 0.0), JA = mk(0.0, 0.0, 0.0);
    const bool need_sum = write_imp || m.behavior == BEH_MOBILE || m.behavior == BEH_CONSTRAINED || ext_imp;
    if (need_sum) {
        const uint32_t e0 = csr_ptr[i], e1 = csr_ptr[i + 1];
        for (uint32_t base = e0; base < e1; base += 32) {
            const uint32_t e = base + lane;
            double jx = 0, jy = 0, jz = 0, ax = 0, ay = 0, az = 0;
            int app = 0;
            if (e < e1) {
                const uint32_t ent = csr_ent[e];
                const uint8_t f = flags[ent >> 1];
                if (f & PF_APPLIED) {
                    const double* o = out + 9 * (size_t)(ent >> 1);
                    app = 1;
                    if (ent & 1) {
                        jx = -o[0]; jy = -o[1]; jz = -o[2];
                        if (f & PF_ANGULAR) { ax = o[6]; ay = o[7]; az = o[8]; app = 2; }
                    } else {
                        jx = o[0]; jy = o[1]; jz = o[2];
                        if (f & PF_ANGULAR) { ax = o[3]; ay = o[4]; az = o[5]; app = 2; }
                    }
                }
            }
            // only the entries that applied an impulse, in entry order (a wall's candidate list is
            // long and few of its spheres touch it)
            for (unsigned am = __ballot_sync(0xffffffffu, app != 0); am; am &= am - 1) {
                const int q = __ffs(am) - 1;
                const int a = __shfl_sync(0xffffffffu, app, q);
                const double bx = __shfl_sync(0xffffffffu, jx, q), by = __shfl_sync(0xffffffffu, jy, q),
                             bz = __shfl_sync(0xffffffffu, jz, q);
                const double cx = __shfl_sync(0xffffffffu, ax, q), cy = __shfl_sync(0xffffffffu, ay, q),
                             cz = __shfl_sync(0xffffffffu, az, q);
                if (a) J = add(J, mk(bx, by, bz));
                if (a == 2) JA = add(JA, mk(cx, cy, cz));
            }
        }
    }
    if (lane == 0)
        finish_object(i, m, J, JA, dt, fimp, pos, vel, av, ox, oz, imp, aimp, write_imp, origin, pos32, wall32,
                      ext_imp, ext_aimp, pb);
}

// Narrow phase only: PF_ACTIVE of every pair at the current positions (the IsActive()
// that NBSConsultant::RebuildIactRecordTab reads, NBSConsultant.cpp:384).
__global__ void __launch_bounds__(TPB) k_detect_active(uint32_t np, const uint2* __restrict__ sm,
                                                       const uint32_t* __restrict__ param,
                                                       const PairParam* __restrict__ params,
                                                       const double4_32a* __restrict__ geom,
                                                       const double4_32a* __restrict__ hole,
                                                       const float* __restrict__ reach,
                                                       const double4_32a* __restrict__ pos, const double4_32a* __restrict__ ox,
                                                       const double4_32a* __restrict__ oz,
                                                       const float4* __restrict__ pos32,
                                                       const float4* __restrict__ wall32, uint8_t* __restrict__ flags,
                                                       Periodic pb) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= np) return;
    const uint2 p = sm[k];
    const uint32_t pi = param[k];
    const uint8_t f = flags[k];
    double depth = -1.0;
    if (!certainly_apart(params[pi].cd, pos32[p.x], pos32[p.y], wall32[p.y], reach[pi], pb.on ? pb.range32 : nullptr)) {
        const double4_32a gg = geom[pi];
        PairGeom g{gg.x, gg.y, gg.z, gg.w, 0.0, 0.0, 0.0};
        if (params[pi].cd == CD_SHP) {
            const double4_32a hh = hole[pi];
            g.hr = hh.x; g.hxo = hh.y; g.hyo = hh.z;
        }
        d3 n, point;
        detect_pair(params[pi].cd, g, ld(pos, p.x), ld(pos, p.y), ox, oz, p.y, pb, depth, n, point);
    }
    const uint8_t nf = depth > 0.0 ? (uint8_t)(f | PF_ACTIVE) : (uint8_t)(f & ~PF_ACTIVE);
    if (nf != f) flags[k] = nf;
}

// ------------------------------------------------------------------------------------
// broad phase (NBSConsultant::Reset, NBSConsultant.cpp:85-316)
__global__ void __launch_bounds__(TPB) k_safe(uint32_t n, const uint32_t* __restrict__ model_of,
                                              const ModelDev* __restrict__ models, const double4_32a* __restrict__ pos,
                                              const double4_32a* __restrict__ vel, double sf, double dtu, double glen,
                                              double* __restrict__ safe, unsigned long long* __restrict__ red) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long mn[3] = {~0ull, ~0ull, ~0ull}, mx[3] = {0, 0, 0}, vm = 0, last = 0;
    if (i < n) {
        const ModelDev& m = models[model_of[i]];
        const double vl = len(ld(vel, i));
        safe[i] = sf * (2.0 * m.range + dtu * vl + 0.5 * dtu * dtu * glen);   // :127-129
        if (m.scope == SCOPE_LOCAL) {                                          // :131-141
            const double4_32a p = pos[i];
            mn[0] = mx[0] = ord_of(p.x);
            mn[1] = mx[1] = ord_of(p.y);
            mn[2] = mx[2] = ord_of(p.z);
            vm = ord_of(vl);
            last = (unsigned long long)i + 1;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            mn[q] = min(mn[q], __shfl_xor_sync(0xffffffffu, mn[q], o));
            mx[q] = max(mx[q], __shfl_xor_sync(0xffffffffu, mx[q], o));
        }
        vm = max(vm, __shfl_xor_sync(0xffffffffu, vm, o));
        last = max(last, __shfl_xor_sync(0xffffffffu, last, o));
    }
    if ((threadIdx.x & 31) == 0) {
        for (int q = 0; q < 3; ++q) {
            atomicMin(&red[2 * q], mn[q]);
            atomicMax(&red[2 * q + 1], mx[q]);
        }
        atomicMax(&red[6], vm);
        atomicMax(&red[7], last);
    }
}

__global__ void __launch_bounds__(TPB) k_cellkey(uint32_t n, const uint32_t* __restrict__ model_of,
                                                 const ModelDev* __restrict__ models, const double4_32a* __restrict__ pos,
                                                 double xmin, double ymin, double zmin, double zone, CellGrid g,
                                                 uint64_t sentinel, uint64_t* __restrict__ key,
                                                 uint32_t* __restrict__ sid) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint64_t k = sentinel;
    if (models[model_of[i]].scope == SCOPE_LOCAL) {          // NBS :163-178, Leap LeapConsultant.h:160-170
        const double4_32a p = pos[i];
        const uint64_t c[3] = {(uint32_t)((p.x - xmin) / zone), (uint32_t)((p.y - ymin) / zone),
                               (uint32_t)((p.z - zmin) / zone)};
        k = grid_key(g, c);
    }
    key[i] = k;
    sid[i] = i;
}

// One axis of the local objects' positions as sortable keys (others sort last): the Leap
// consultant's spans come from the sorted positions (LeapConsultant.cpp:143-168).
__global__ void __launch_bounds__(TPB) k_axis_key(uint32_t n, const uint32_t* __restrict__ model_of,
                                                  const ModelDev* __restrict__ models,
                                                  const double4_32a* __restrict__ pos, int axis,
                                                  uint64_t* __restrict__ key, uint32_t* __restrict__ sid) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint64_t k = ~0ull;
    if (models[model_of[i]].scope == SCOPE_LOCAL) {
        const double4_32a p = pos[i];
        k = ord_of(axis == 0 ? p.x : axis == 1 ? p.y : p.z);
    }
    key[i] = k;
    sid[i] = i;
}

__global__ void __launch_bounds__(TPB) k_cell_flags(uint32_t nloc, const uint64_t* __restrict__ key,
                                                    uint32_t* __restrict__ flag) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nloc) return;
    flag[p] = (p == 0 || key[p] != key[p - 1]) ? 1u : 0u;
}

__global__ void __launch_bounds__(TPB) k_cell_fill(uint32_t nloc, const uint64_t* __restrict__ key,
                                                   const uint32_t* __restrict__ flag_excl,
                                                   uint64_t* __restrict__ cell_key, uint32_t* __restrict__ cell_start,
                                                   uint32_t* __restrict__ cellof, const uint32_t* __restrict__ ncells) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nloc) return;
    const bool head = (p == 0 || key[p] != key[p - 1]);
    const uint32_t c = head ? flag_excl[p] : flag_excl[p] - 1u;   // index of p's cell
    cellof[p] = c;
    if (head) {
        cell_key[c] = key[p];
        cell_start[c] = p;
    }
    if (p == nloc - 1) cell_start[*ncells] = nloc;
}

// Candidate test of BuildIactTab (NBSConsultant.cpp:318-345): DOMap::CalDistance <= safe_i +
// safe_j, decided from FP32 bounds where they are conclusive and in exact FP64 otherwise.
// pb: the Leap consultant's distance takes the boundary's minimum image (nullptr: NBS's does not)
__device__ __forceinline__ bool candidate(const ModelDev& mi, const ModelDev& mj, uint32_t i, uint32_t j, double si,
                                          double sj, float si32, float sj32, const double4_32a* __restrict__ pos,
                                          const double4_32a* __restrict__ ox, const double4_32a* __restrict__ oz,
                                          const float4* __restrict__ pos32, const float4* __restrict__ wall32,
                                          int* __restrict__ err, const Periodic* pb) {
    const float thr = si32 + sj32;                     // float sums of the rounded-to-float safe lengths
    const float tlo = thr * (1.0f - 4.0f * PF_ARITH_EPS), thi = thr * (1.0f + 4.0f * PF_ARITH_EPS);
    if (pb) {
        // periodic: the least distance over the images bounds the detector's from below (the
        // certain-candidate shortcut is not taken: the image the reference picks may be another)
        if (mi.shape == SHAPE_SPHERE && mj.shape == SHAPE_SPHERE) {
            float e;
            const float d = dist32_periodic(pos32[i], pos32[j], pb->range32, e);
            if (d - e > thi) return false;
        }
    } else if (mi.shape == SHAPE_SPHERE && mj.shape == SHAPE_SPHERE) {
        float e;
        const float d = dist32(pos32[i], pos32[j], e);
        if (d - e > thi) return false;
        if (d + e < tlo) return true;
    } else {
        const bool ip = mi.shape != SHAPE_SPHERE;      // the non-sphere member
        const uint32_t w = ip ? i : j, sp = ip ? j : i;
        const int wshape = ip ? mi.shape : mj.shape;
        const float4 wl = wall32[w];
        if (wl.w != 0.0f && (wshape == SHAPE_PLATE || wshape == SHAPE_HOLED || wshape == SHAPE_CYL) &&
            (ip ? mj.shape : mi.shape) == SHAPE_SPHERE) {
            float e;
            const float d = wshape != SHAPE_CYL ? plane_dist32(pos32[sp], pos32[w], wl, e)
                                                  : line_dist32(pos32[sp], pos32[w], wl, e);
            if (d - e > thi) return false;
        } else if (wl.w != 0.0f && wshape == SHAPE_INNER_CYL && (ip ? mj.shape : mi.shape) == SHAPE_SPHERE) {
            // the distance to the shell is at least R minus the axis distance (rim included)
            float e;
            const float d = line_dist32(pos32[sp], pos32[w], wl, e);
            const float R = (float)(ip ? mi.a0 : mj.a0) * (1.0f - 4.0f * PF_ARITH_EPS);
            if (R - (d + e) > thi) return false;
        }
    }
    bool ok;
    const double d = cal_distance(mi, mj, i, j, pos, ox, oz, pb, ok);
    if (!ok) {
        atomicOr(err, ERR_BAD_SHAPE_PAIR);
        return false;
    }
    return !(d > (si + sj));
}

// One thread per (slot, object) task, slot-major so that a warp works on one slot.  Tasks
// are numbered in the reference's traversal order: cell by cell (ix, iy, iz lexicographic),
// within a cell by slot, within a slot by the object's position in the cell (ascending id).
template <bool FILL>
__global__ void __launch_bounds__(TPB) k_pairs(uint32_t nloc, const uint32_t* __restrict__ sid,
                                               const uint64_t* __restrict__ cell_key,
                                               const uint32_t* __restrict__ cell_start,
                                               const uint32_t* __restrict__ ncells_p, const uint32_t* __restrict__ cellof,
                                               const uint32_t* __restrict__ grid, uint64_t grid_cells,
                                               const uint32_t* __restrict__ glob, uint32_t nglob,
                                               const uint32_t* __restrict__ model_of, const ModelDev* __restrict__ models,
                                               const int* __restrict__ group_iact, int G,
                                               const double4_32a* __restrict__ pos, const double4_32a* __restrict__ ox,
                                               const double4_32a* __restrict__ oz, const float4* __restrict__ pos32,
                                               const float4* __restrict__ wall32, const double* __restrict__ safe,
                                               CellGrid g, Periodic pbv,
                                               uint32_t* __restrict__ task, uint32_t* __restrict__ first,
                                               uint32_t* __restrict__ second, int* __restrict__ err) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (uint64_t)nloc * NSLOT) return;
    const int s = (int)(t / nloc);
    const uint32_t P = (uint32_t)(t % nloc);
    const uint32_t c = cellof[P];
    uint64_t cc[3];
    grid_cell(g, cell_key[c], cc);
    const uint32_t cs = cell_start[c], csize = cell_start[c + 1] - cs;
    const uint64_t tid = (uint64_t)cs * NSLOT + (uint64_t)s * csize + (P - cs);
    // NBS: only cells inside the loops are primary (:186-190); Leap visits every zone of its map
    if (!g.leap && (cc[0] >= g.ncel[0] || cc[1] >= g.ncel[1] || cc[2] >= g.ncel[2])) {
        if (!FILL) task[tid] = 0;
        return;
    }
    const int slot_self = g.leap ? 13 : SLOT_SELF, slot_global = g.leap ? 14 : SLOT_GLOBAL;
    const uint32_t* js = nullptr;
    uint32_t jn = 0;
    // the cell whose zone coordinates are w (its index, or none)
    auto find_cell = [&](const uint64_t w[3]) -> uint32_t {
#pragma unroll
        for (int a = 0; a < 3; ++a)
            if (w[a] >= g.dim[a]) return 0xffffffffu;
        const uint64_t nk = grid_key(g, w);
        if (grid) return nk < grid_cells ? grid[nk] : 0xffffffffu;
        const uint32_t nc = *ncells_p;
        uint32_t lo = 0, hi = nc;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (cell_key[mid] < nk) lo = mid + 1; else hi = mid;
        }
        return (lo < nc && cell_key[lo] == nk) ? lo : 0xffffffffu;
    };
    if (s == slot_self) {                                     // BuildIactTab(v), :347-374
        js = sid + P + 1;
        jn = cs + csize - (P + 1);
    } else if (s == slot_global) {                            // BuildIactTab(v, GlobalElement), :266
        js = glob;
        jn = nglob;
    } else if (g.leap || s < NSLOT) {
        int d[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) d[a] = g.leap ? c_slot_leap[s][a] : c_slot[s][a];
        uint32_t c2 = 0xffffffffu;
        if (!((cc[0] == 0 && d[0] < 0) || (cc[1] == 0 && d[1] < 0) || (cc[2] == 0 && d[2] < 0))) {
            const uint64_t w[3] = {cc[0] + d[0], cc[1] + d[1], cc[2] + d[2]};
            c2 = find_cell(w);
        }
        if (c2 == 0xffffffffu && g.leap && g.has_pbc) {
            // the neighbour's periodic image (LeapConsultant.h:199-440): on an axis stepping down
            // from zone 0 (up from the last zone) it wraps when that axis is periodic; ids are
            // _uint_t, and an image that names the opposite neighbour is skipped
            bool at_edge = false, dup = false, valid = true;
            uint64_t w[3];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const uint32_t ia = (uint32_t)cc[a], mx = g.ncel[a] - 1u;
                uint32_t wa = ia;
                if (d[a] < 0) {
                    at_edge |= ia == 0u;
                    wa = g.pbc[a] ? mx : ia - 1u;
                    dup |= wa == ia + 1u;
                } else if (d[a] > 0) {
                    at_edge |= ia == mx;
                    wa = g.pbc[a] ? 0u : ia + 1u;
                    dup |= wa == ia - 1u;
                }
                valid &= wa != 0xffffffffu;
                w[a] = wa;
            }
            if (at_edge && !dup && valid) c2 = find_cell(w);
        }
        if (c2 != 0xffffffffu) {
            js = sid + cell_start[c2];
            jn = cell_start[c2 + 1] - cell_start[c2];
        }
    }
    const uint32_t i = sid[P];
    const ModelDev& mi = models[model_of[i]];
    const double si = safe[i];
    const float si32 = (float)si;
    const int gi = mi.group;
    uint32_t cnt = 0;
    const uint32_t off = FILL ? task[tid] : 0u;
    // the fill pass knows each task's count from the scanned offsets (the next task's offset, or
    // the total after the last one): it stops at its last candidate and skips empty tasks
    uint32_t want = 0xffffffffu;
    if (FILL) want = ((uint64_t)tid + 1 < (uint64_t)nloc * NSLOT ? task[tid + 1] : ncells_p[1]) - off;
    for (uint32_t q = 0; q < jn && cnt < want; ++q) {
        const uint32_t j = js[q];
        const ModelDev& mj = models[model_of[j]];
        if (group_iact[gi * G + mj.group] < 0) continue;
        const double sj = safe[j];
        if (!candidate(mi, mj, i, j, si, sj, si32, (float)sj, pos, ox, oz, pos32, wall32, err,
                       g.leap && pbv.on ? &pbv : nullptr)) continue;
        if (FILL) {
            first[off + cnt] = i < j ? i : j;
            second[off + cnt] = i < j ? j : i;
        }
        ++cnt;
    }
    if (!FILL) task[tid] = cnt;
}

__global__ void __launch_bounds__(TPB) k_grid_fill(const uint32_t* __restrict__ ncells_p,
                                                   const uint64_t* __restrict__ cell_key, uint32_t* __restrict__ grid) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < *ncells_p) grid[cell_key[c]] = c;
}

__global__ void __launch_bounds__(TPB) k_refresh32(uint32_t n, const uint32_t* __restrict__ model_of,
                                                   const ModelDev* __restrict__ models,
                                                   const double4_32a* __restrict__ pos,
                                                   const double4_32a* __restrict__ ox,
                                                   const double4_32a* __restrict__ oz, d3 origin,
                                                   float4* __restrict__ pos32, float4* __restrict__ wall32) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    write32(i, models[model_of[i]].shape, ld(pos, i), ld(ox, i), ld(oz, i), origin, pos32, wall32);
}

// Assembler::CreateInteraction orientation and model selection (Assembler.cpp:15-87)
__global__ void __launch_bounds__(TPB) k_setup(uint32_t np, const uint32_t* __restrict__ first,
                                               const uint32_t* __restrict__ second,
                                               const uint32_t* __restrict__ model_of,
                                               const ModelDev* __restrict__ models,
                                               const PairParam* __restrict__ params, uint32_t nm,
                                               uint2* __restrict__ sm, uint32_t* __restrict__ param,
                                               int* __restrict__ err) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= np) return;
    const uint32_t a = first[k], b = second[k];
    const uint32_t ma = model_of[a], mb = model_of[b];
    const ModelDev& A = models[ma];
    const ModelDev& B = models[mb];
    uint32_t sl = a, ms = b;
    // no interaction of an object with itself (Assembler.cpp:27-30): the Leap consultant lists such
    // pairs when a periodic axis is one zone wide, and the reference then drops them, leaving its
    // pair table and interactions misaligned; here the list is refused
    bool bad = a == b || (B.density < 0.0 || A.density < 0.0) || (B.density == 0.0 && A.density == 0.0);
    if (A.shape > B.shape) { sl = b; ms = a; }
    else if (A.shape < B.shape) { sl = a; ms = b; }
    else if (A.density == 0.0) { sl = b; ms = a; }
    else if (B.density == 0.0) { sl = a; ms = b; }
    const uint32_t pi = model_of[sl] * nm + model_of[ms];
    if (bad || params[pi].cd == 0) {
        atomicOr(err, ERR_UNSUPPORTED_PAIR);
        sm[k] = make_uint2(a, b);
        param[k] = 0;
        return;
    }
    sm[k] = make_uint2(sl, ms);
    param[k] = pi;
}

// History carry: a new pair takes the status of the same (first, second) pair of the old
// list when that pair was active (RebuildIactRecordTab + Initiate, NBSConsultant.cpp:376-395,
// SimMediator.cpp:690-707); otherwise a default-constructed ImpactStatus.
__global__ void __launch_bounds__(TPB) k_history_old(uint32_t np, const uint32_t* __restrict__ first,
                                                     const uint32_t* __restrict__ second,
                                                     const uint2* __restrict__ sm, const uint32_t* __restrict__ param,
                                                     const PairParam* __restrict__ params,
                                                     const float* __restrict__ reach,
                                                     const float4* __restrict__ pos32,
                                                     const float4* __restrict__ wall32,
                                                     const uint32_t* __restrict__ o_ptr,
                                                     const uint32_t* __restrict__ o_ent,
                                                     const uint32_t* __restrict__ o_first,
                                                     const uint32_t* __restrict__ o_second,
                                                     const uint8_t* __restrict__ o_flags,
                                                     const double4_32a* __restrict__ o_hist,
                                                     const double* __restrict__ o_v0, double4_32a* __restrict__ hist,
                                                     double* __restrict__ v0, uint8_t* __restrict__ flags,
                                                     Periodic pb) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= np) return;
    const uint32_t a = first[k], b = second[k];
    uint8_t f = ST_DEFAULT;
    double4_32a h = make_double4_32a(0.0, 0.0, 0.0, 0.0);
    double vv = 0.0;
    const uint2 p = sm[k];
    const uint32_t pi = param[k];
    // a pair certainly apart now was not active at this position in the old list either
    const bool maybe = !certainly_apart(params[pi].cd, pos32[p.x], pos32[p.y], wall32[p.y], reach[pi],
                                        pb.on ? pb.range32 : nullptr);
    const uint32_t e1 = maybe ? o_ptr[a + 1] : 0u;
    for (uint32_t e = maybe ? o_ptr[a] : 0u; e < e1; ++e) {
        const uint32_t ko = o_ent[e] >> 1;
        if (o_first[ko] == a && o_second[ko] == b) {
            const uint8_t of = o_flags[ko];
            if (of & PF_ACTIVE) {
                f = of & (PF_STATUS | PF_NONZERO);
                if (of & PF_NONZERO) {
                    h = o_hist[ko];
                    vv = o_v0[ko];
                }
            }
            break;
        }
    }
    hist[k] = h;
    v0[k] = vv;
    flags[k] = f;
}

// History from the IactRecordTab read with the scene (IactRecordTab::GetImpactStatus,
// IactRecordTab.cpp:20-25); records are sorted by (first << 32 | second).
__global__ void __launch_bounds__(TPB) k_history_rec(uint32_t np, const uint32_t* __restrict__ first,
                                                     const uint32_t* __restrict__ second,
                                                     const uint64_t* __restrict__ rkey, uint32_t nrec,
                                                     const double4_32a* __restrict__ rhist, const double* __restrict__ rv0,
                                                     const uint8_t* __restrict__ rflags, double4_32a* __restrict__ hist,
                                                     double* __restrict__ v0, uint8_t* __restrict__ flags) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= np) return;
    const uint64_t key = ((uint64_t)first[k] << 32) | second[k];
    uint32_t lo = 0, hi = nrec;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (rkey[mid] < key) lo = mid + 1; else hi = mid;
    }
    if (lo < nrec && rkey[lo] == key) {
        hist[k] = rhist[lo];
        v0[k] = rv0[lo];
        flags[k] = rflags[lo];
    } else {
        hist[k] = make_double4_32a(0.0, 0.0, 0.0, 0.0);
        v0[k] = 0.0;
        flags[k] = ST_DEFAULT;
    }
}

__global__ void __launch_bounds__(TPB) k_csr_keys(uint32_t np, const uint2* __restrict__ sm, uint32_t* __restrict__ key,
                                                  uint32_t* __restrict__ val) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= np) return;
    const uint2 p = sm[k];
    key[2 * k] = p.x;
    val[2 * k] = 2 * k;
    key[2 * k + 1] = p.y;
    val[2 * k + 1] = 2 * k + 1;
}

__global__ void __launch_bounds__(TPB) k_csr_ptr(uint32_t n, const uint32_t* __restrict__ key, uint32_t m,
                                                 uint32_t* __restrict__ ptr) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n) return;
    uint32_t lo = 0, hi = m;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (key[mid] < i) lo = mid + 1; else hi = mid;
    }
    ptr[i] = lo;
}

}  // namespace

// ====================================================================================
#define CK(call)                                                  \
    do {                                                          \
        cudaError_t _e = (call);                                  \
        if (_e != cudaSuccess) return cuda_fail(_e, #call);       \
    } while (0)

int Engine::cuda_fail(cudaError_t e, const char* where) {
    err_ = std::string("CUDA error ") + cudaGetErrorString(e) + " at " + where;
    return e == cudaErrorMemoryAllocation ? VEDO_ERR_OUT_OF_MEMORY : VEDO_ERR_CUDA;
}

template <class T>
static cudaError_t dalloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    return cudaMalloc((void**)p, sizeof(T) * count);
}

void Engine::free_list(PairList& L) {
    cudaFree(L.first); cudaFree(L.second); cudaFree(L.sm); cudaFree(L.param); cudaFree(L.hist); cudaFree(L.v0);
    cudaFree(L.flags); cudaFree(L.out); cudaFree(L.csr_ent); cudaFree(L.csr_ptr); cudaFree(L.work);
    L = PairList{};
}

int Engine::ensure_list(PairList& L, uint32_t cap) {
    if (L.csr_ptr == nullptr) CK(dalloc(&L.csr_ptr, (size_t)n_ + 1));
    if (cap <= L.cap && L.first) return VEDO_OK;
    uint32_t* ptr = L.csr_ptr;
    L.csr_ptr = nullptr;
    free_list(L);
    L.csr_ptr = ptr;
    uint64_t c = std::max<uint64_t>(1024, (uint64_t)cap + cap / 4);
    if (c > 0x7fffffffull) c = 0x7fffffffull;
    L.cap = (uint32_t)c;
    CK(dalloc(&L.first, c)); CK(dalloc(&L.second, c)); CK(dalloc(&L.sm, c)); CK(dalloc(&L.param, c));
    CK(dalloc(&L.hist, c)); CK(dalloc(&L.v0, c)); CK(dalloc(&L.flags, c)); CK(dalloc(&L.out, 9 * c));
    CK(dalloc(&L.csr_ent, 2 * c));
    CK(dalloc(&L.work, c));
    return VEDO_OK;
}

Engine::~Engine() {
    if (status_) std::fclose(status_);
    if (stream_) cudaStreamSynchronize(stream_);
    free_list(cur_);
    free_list(old_);
    void* ptrs[] = {d_models_, d_params_, d_geom_, d_group_iact_, d_model_of_, d_err_, d_pos_, d_vel_, d_av_, d_ox_,
                    d_oz_, d_imp_, d_aimp_, d_global_, d_safe_, d_red_, d_key_, d_key_alt_, d_cell_key_, d_sid_,
                    d_sid_alt_, d_cell_start_, d_cellof_, d_flag_, d_task_, d_total_, d_ck_, d_cv_, d_ck_alt_,
                    d_cv_alt_, d_cnt_, d_rec_key_, d_rec_hist_, d_rec_v0_, d_rec_flags_, d_obs_, d_stage_,
                    d_pos32_, d_wall32_, d_reach_, d_grid_, d_ext_, d_hole_, d_touched_, d_nwork_};
    for (void* p : ptrs) if (p) cudaFree(p);
    for (auto& e : ev_) if (e) cudaEventDestroy(e);
    if (stream_) cudaStreamDestroy(stream_);
}

static void upload3(std::vector<double4_32a>& tmp, const std::vector<double>& v, uint32_t n) {
    tmp.resize(n);
    for (uint32_t i = 0; i < n; ++i) tmp[i] = make_double4_32a(v[3 * i], v[3 * i + 1], v[3 * i + 2], 0.0);
}

int Engine::init(const HScene& scene, const vedo_engine_opts& opts) {
    host_ = scene;
    opts_ = opts;
    if (opts_.up_iact == 0) opts_.up_iact = 1;
    if (opts_.consultant > 1) return fail(VEDO_ERR_INVALID_ARGUMENT, "unknown consultant");
    leap_ = opts_.consultant == 1;
    out_prefix_ = opts.output_prefix ? opts.output_prefix : "";
    std::string msg;
    int rc = build_tables(host_, tab_, msg);
    if (rc != VEDO_OK) return fail(rc, msg);
    zoi_on_ = host_.zoi_switch[0] || host_.zoi_switch[1] || host_.zoi_switch[2];
    n_ = host_.n;
    nm_ = (uint32_t)tab_.models.size();
    dt_ = host_.time_interval;
    t_ = host_.time_current;
    t_stop_ = host_.time_stop;
    sf_ = host_.safety_factor;
    for (int k = 0; k < 3; ++k) g_[k] = host_.g[k];
    device_ = opts.device;
    CK(cudaSetDevice(device_));
    CK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    for (auto& e : ev_) CK(cudaEventCreate(&e));
    // constant tables
    CK(dalloc(&d_models_, nm_));
    CK(cudaMemcpy(d_models_, tab_.models.data(), sizeof(ModelDev) * nm_, cudaMemcpyHostToDevice));
    CK(dalloc(&d_params_, (size_t)nm_ * nm_));
    CK(cudaMemcpy(d_params_, tab_.params.data(), sizeof(PairParam) * nm_ * nm_, cudaMemcpyHostToDevice));
    std::vector<double4_32a> geo((size_t)nm_ * nm_);
    for (size_t q = 0; q < geo.size(); ++q)
        geo[q] = make_double4_32a(tab_.geom[4 * q], tab_.geom[4 * q + 1], tab_.geom[4 * q + 2], tab_.geom[4 * q + 3]);
    CK(dalloc(&d_geom_, geo.size()));
    CK(cudaMemcpy(d_geom_, geo.data(), sizeof(double4_32a) * geo.size(), cudaMemcpyHostToDevice));
    for (size_t q = 0; q < geo.size(); ++q)
        geo[q] = make_double4_32a(tab_.hole[4 * q], tab_.hole[4 * q + 1], tab_.hole[4 * q + 2], 0.0);
    CK(dalloc(&d_hole_, geo.size()));
    CK(cudaMemcpy(d_hole_, geo.data(), sizeof(double4_32a) * geo.size(), cudaMemcpyHostToDevice));
    const int G = tab_.ngroups;
    CK(dalloc(&d_group_iact_, (size_t)G * G));
    CK(cudaMemcpy(d_group_iact_, tab_.group_iact.data(), sizeof(int) * G * G, cudaMemcpyHostToDevice));
    CK(dalloc(&d_model_of_, n_));
    CK(cudaMemcpy(d_model_of_, host_.model_of.data(), sizeof(uint32_t) * n_, cudaMemcpyHostToDevice));
    CK(dalloc(&d_err_, 1));
    CK(cudaMemset(d_err_, 0, sizeof(int)));
    // objects
    std::vector<double4_32a> tmp;
    double4_32a** dst[] = {&d_pos_, &d_vel_, &d_av_, &d_ox_, &d_oz_, &d_imp_, &d_aimp_};
    const std::vector<double>* src[] = {&host_.pos, &host_.vel, &host_.av, &host_.ox, &host_.oz, &host_.imp, &host_.aimp};
    for (int k = 0; k < 7; ++k) {
        CK(dalloc(dst[k], n_));
        upload3(tmp, *src[k], n_);
        CK(cudaMemcpy(*dst[k], tmp.data(), sizeof(double4_32a) * n_, cudaMemcpyHostToDevice));
    }
    for (uint32_t i = 0; i < n_; ++i)
        if (tab_.models[host_.model_of[i]].scope != SCOPE_LOCAL) global_ids_.push_back(i);
        else leap_rmax_ = std::max(leap_rmax_, tab_.models[host_.model_of[i]].range);
    if (leap_ && global_ids_.size() == n_)           // the reference indexes an empty vector
        return fail(VEDO_ERR_INVALID_SCENE, "the Leap consultant needs a local object");
    // FP32 prefilter copies: origin at the centre of the initial bounding box
    {
        double lo[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, hi[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
        for (uint32_t i = 0; i < n_; ++i)
            for (int k = 0; k < 3; ++k) {
                lo[k] = std::min(lo[k], host_.pos[3 * i + k]);
                hi[k] = std::max(hi[k], host_.pos[3 * i + k]);
            }
        for (int k = 0; k < 3; ++k) origin_[k] = 0.5 * (lo[k] + hi[k]);
        CK(dalloc(&d_pos32_, n_));
        CK(dalloc(&d_wall32_, n_));
        CK(dalloc(&d_touched_, n_));
        CK(cudaMemset(d_touched_, 0, n_));
        CK(dalloc(&d_nwork_, 1));
        CK(cudaMemset(d_nwork_, 0, sizeof(uint32_t)));
        CK(cudaMemset(d_wall32_, 0, sizeof(float4) * n_));
        std::vector<float> reach((size_t)nm_ * nm_, 0.0f);
        for (size_t q = 0; q < reach.size(); ++q) {
            const double* gq = &tab_.geom[4 * q];   // ra, b0, b1, b2
            double r = 0.0;
            if (tab_.params[q].cd == CD_SS) r = gq[0] + gq[1];
            else if (cd_plane(tab_.params[q].cd) == CD_SP) r = gq[0] + 0.5 * gq[2];
            else if (tab_.params[q].cd == CD_SC) r = gq[0] + gq[1];
            // inside a hollow cylinder: -(R - r), its magnitude rounded down (prefilter.cuh)
            if (tab_.params[q].cd == CD_SIC) reach[q] = (float)(gq[0] - gq[1]) * (1.0f - 1e-6f);
            else reach[q] = (float)r * (1.0f + 1e-6f);
        }
        CK(dalloc(&d_reach_, reach.size()));
        CK(cudaMemcpy(d_reach_, reach.data(), sizeof(float) * reach.size(), cudaMemcpyHostToDevice));
        k_refresh32<<<blocks_for(n_), TPB>>>(n_, d_model_of_, d_models_, d_pos_, d_ox_, d_oz_,
                                             mk(origin_[0], origin_[1], origin_[2]), d_pos32_, d_wall32_);
        CK(cudaGetLastError());
        CK(cudaDeviceSynchronize());
    }
    CK(dalloc(&d_global_, global_ids_.size()));
    if (!global_ids_.empty())
        CK(cudaMemcpy(d_global_, global_ids_.data(), sizeof(uint32_t) * global_ids_.size(), cudaMemcpyHostToDevice));
    // broad-phase scratch
    CK(dalloc(&d_safe_, n_)); CK(dalloc(&d_red_, 8)); CK(dalloc(&d_key_, n_)); CK(dalloc(&d_key_alt_, n_));
    CK(dalloc(&d_cell_key_, n_)); CK(dalloc(&d_sid_, n_)); CK(dalloc(&d_sid_alt_, n_));
    CK(dalloc(&d_cell_start_, (size_t)n_ + 1)); CK(dalloc(&d_cellof_, n_)); CK(dalloc(&d_flag_, n_));
    CK(dalloc(&d_total_, 4));
    CK(dalloc(&d_obs_, (size_t)(blocks_for(n_) + 2) * 16 + 64));
    // IDO records, sorted by key, first of equal keys kept (std::map::insert)
    const HRecords& R = host_.rec;
    if (R.size()) {
        std::vector<uint32_t> ord(R.size());
        for (uint32_t q = 0; q < ord.size(); ++q) ord[q] = q;
        auto key = [&](uint32_t q) { return ((uint64_t)R.first[q] << 32) | R.second[q]; };
        std::stable_sort(ord.begin(), ord.end(), [&](uint32_t a, uint32_t b) { return key(a) < key(b); });
        std::vector<uint64_t> rk;
        std::vector<double4_32a> rh;
        std::vector<double> rv;
        std::vector<uint8_t> rf;
        for (uint32_t q : ord) {
            if (!rk.empty() && rk.back() == key(q)) continue;
            rk.push_back(key(q));
            rh.push_back(make_double4_32a(R.shear[3 * q], R.shear[3 * q + 1], R.shear[3 * q + 2], R.kn[q]));
            rv.push_back(R.v0[q]);
            // default-constructed ImpactStatus + setters (IactRecordTab.cpp:432-530)
            rf.push_back((uint8_t)(ST_DEFAULT | (R.contact[q] ? ST_CONTACT : 0) | (R.bond[q] ? ST_BOND : 0) | PF_NONZERO));
        }
        rc = upload_records(rk, rh, rv, rf);
        if (rc != VEDO_OK) return rc;
    }
    // first candidate list (NBSConsultant constructor) + Initiate
    rc = rebuild(true);
    if (rc != VEDO_OK) return rc;
    CK(cudaStreamSynchronize(stream_));
    backup_pending_ = false;
    if (!out_prefix_.empty()) {
        // SimMediator's constructor (SimMediator.cpp:103-123): the SystemStatus.csv header, then
        // CalculateSystemEnergy with the IactRecordTab read from the file
        std::string dir = out_prefix_;
        const size_t slash = dir.find_last_of('/');
        dir = slash == std::string::npos ? std::string() : dir.substr(0, slash + 1);
        status_ = std::fopen((dir + "SystemStatus.csv").c_str(), "w");
        if (!status_) return fail(VEDO_ERR_IO, "cannot write " + dir + "SystemStatus.csv");
        std::fprintf(status_, "Simulated time, number of elements, number of interactions, Number of contacts, "
                              "System energy, Potential energy, Kinetic energy, Kinetic energy (translation), "
                              "Kinetic energy (rotation), Minimal velocity, Maximal velocity, "
                              "Minimal angular velocity, Maximal angular velocity, Norm of momentum, "
                              "Norm of angular momentum");
        for (uint32_t u = 0; u < 2 * host_.num_udd_impact; ++u) std::fprintf(status_, ", User-defined Value %u", u + 1);
        std::fprintf(status_, "\n");
        uint64_t contacts = 0;
        for (size_t q = 0; q < host_.rec.first.size(); ++q) contacts += host_.rec.contact[q] ? 1u : 0u;
        rc = status_row(host_.rec.first.size(), contacts);
        if (rc != VEDO_OK) return rc;
    }
    return VEDO_OK;
}

// The records the next list takes its history from (sorted by key).
int Engine::upload_records(const std::vector<uint64_t>& rk, const std::vector<double4_32a>& rh,
                           const std::vector<double>& rv, const std::vector<uint8_t>& rf) {
    for (void** p : {(void**)&d_rec_key_, (void**)&d_rec_hist_, (void**)&d_rec_v0_, (void**)&d_rec_flags_}) {
        if (*p) cudaFree(*p);
        *p = nullptr;
    }
    nrec_ = (uint32_t)rk.size();
    if (!nrec_) return VEDO_OK;
    CK(dalloc(&d_rec_key_, nrec_)); CK(dalloc(&d_rec_hist_, nrec_)); CK(dalloc(&d_rec_v0_, nrec_));
    CK(dalloc(&d_rec_flags_, nrec_));
    CK(cudaMemcpy(d_rec_key_, rk.data(), 8 * nrec_, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_rec_hist_, rh.data(), sizeof(double4_32a) * nrec_, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_rec_v0_, rv.data(), 8 * nrec_, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_rec_flags_, rf.data(), nrec_, cudaMemcpyHostToDevice));
    return VEDO_OK;
}

// LeapConsultant::NextStep at a reset (LeapConsultant.cpp:61-68): SyncWorld,
// RebuildIactRecordTab, then Consultant::CleanUp (Consultant.cpp:264-319).  The mobile objects
// outside the zone of interest are erased and the others renumbered (their order kept); the
// records of the interactions active at the current positions -- their statuses as the carry of
// an ordinary reset takes them -- are re-keyed as IactRecordTab::ModifyPair does, and become the
// records the reset's list takes its history from.  Host work, run only when an object leaves.
int Engine::leap_cleanup(bool* erased_any) {
    *erased_any = false;
    int rc = sync_host_state();
    if (rc != VEDO_OK) return rc;
    std::vector<uint32_t> jump;
    const std::vector<uint32_t> erased = zoi_outside(host_, jump);
    if (erased.empty()) return VEDO_OK;
    const uint32_t np = cur_.np;
    std::vector<uint32_t> fa(np), fb(np);
    std::vector<uint8_t> fl(np);
    std::vector<double4_32a> hh(np);
    std::vector<double> vv(np);
    if (np) {
        k_detect_active<<<blocks_for(np), TPB, 0, stream_>>>(np, cur_.sm, cur_.param, d_params_, d_geom_, d_hole_,
                                                             d_reach_, d_pos_, d_ox_, d_oz_, d_pos32_, d_wall32_,
                                                             cur_.flags, tab_.pbc);
        ++launches_;
        CK(cudaMemcpyAsync(fa.data(), cur_.first, 4 * (size_t)np, cudaMemcpyDeviceToHost, stream_));
        CK(cudaMemcpyAsync(fb.data(), cur_.second, 4 * (size_t)np, cudaMemcpyDeviceToHost, stream_));
        CK(cudaMemcpyAsync(fl.data(), cur_.flags, np, cudaMemcpyDeviceToHost, stream_));
        CK(cudaMemcpyAsync(hh.data(), cur_.hist, sizeof(double4_32a) * np, cudaMemcpyDeviceToHost, stream_));
        CK(cudaMemcpyAsync(vv.data(), cur_.v0, 8 * (size_t)np, cudaMemcpyDeviceToHost, stream_));
        CK(cudaStreamSynchronize(stream_));
    }
    std::vector<std::pair<uint32_t, uint32_t>> keys;
    std::vector<uint32_t> src;
    for (uint32_t k = 0; k < np; ++k)
        if (fl[k] & PF_ACTIVE) {
            keys.push_back({fa[k], fb[k]});
            src.push_back(k);
        }
    std::vector<uint64_t> rk;
    std::vector<double4_32a> rh;
    std::vector<double> rv;
    std::vector<uint8_t> rf;
    for (const auto& kv : modify_pair(keys, jump)) {
        const uint32_t k = src[kv.second];
        const bool nz = fl[k] & PF_NONZERO;
        rk.push_back(((uint64_t)kv.first.first << 32) | kv.first.second);
        rh.push_back(nz ? hh[k] : make_double4_32a(0.0, 0.0, 0.0, 0.0));
        rv.push_back(nz ? vv[k] : 0.0);
        rf.push_back((uint8_t)(fl[k] & (PF_STATUS | PF_NONZERO)));
    }
    erase_objects(host_, erased);
    n_ = host_.n;
    // the survivors' state and models (the buffers keep their larger capacity)
    std::vector<double4_32a> tmp;
    double4_32a* dst[] = {d_pos_, d_vel_, d_av_, d_ox_, d_oz_, d_imp_, d_aimp_};
    const std::vector<double>* srcv[] = {&host_.pos, &host_.vel, &host_.av, &host_.ox, &host_.oz, &host_.imp,
                                         &host_.aimp};
    for (int k = 0; k < 7; ++k) {
        upload3(tmp, *srcv[k], n_);
        CK(cudaMemcpy(dst[k], tmp.data(), sizeof(double4_32a) * n_, cudaMemcpyHostToDevice));
    }
    CK(cudaMemcpy(d_model_of_, host_.model_of.data(), sizeof(uint32_t) * n_, cudaMemcpyHostToDevice));
    global_ids_.clear();
    leap_rmax_ = 0.0;                      // LeapConsultant::Reset takes the largest range anew
    for (uint32_t i = 0; i < n_; ++i)
        if (tab_.models[host_.model_of[i]].scope != SCOPE_LOCAL) global_ids_.push_back(i);
        else leap_rmax_ = std::max(leap_rmax_, tab_.models[host_.model_of[i]].range);
    if (global_ids_.size() == n_) return fail(VEDO_ERR_INVALID_SCENE, "the zone of interest erased every local object");
    if (!global_ids_.empty())
        CK(cudaMemcpy(d_global_, global_ids_.data(), sizeof(uint32_t) * global_ids_.size(), cudaMemcpyHostToDevice));
    k_refresh32<<<blocks_for(n_), TPB, 0, stream_>>>(n_, d_model_of_, d_models_, d_pos_, d_ox_, d_oz_,
                                                     mk(origin_[0], origin_[1], origin_[2]), d_pos32_, d_wall32_);
    ++launches_;
    CK(cudaMemsetAsync(d_touched_, 0, n_, stream_));
    CK(cudaStreamSynchronize(stream_));
    rc = upload_records(rk, rh, rv, rf);
    if (rc != VEDO_OK) return rc;
    *erased_any = true;
    return VEDO_OK;
}

// One line of SystemStatus.csv (SimMediator::CalculateSystemEnergy, SimMediator.cpp:46-81):
// time, object count, IactRecordTab size and contact count, then the energies and extrema of
// DOWorld::CalculateSystemEnergy, as the reference's ostream writes them (6 significant
// digits).  The user-defined impact values, which the engine does not carry, are written as 0.
int Engine::status_row(uint64_t records, uint64_t contacts) {
    double o[13];
    const int rc = get_observables(o);
    if (rc != VEDO_OK) return rc;
    std::fprintf(status_, "%g, %u, %llu, %llu, %g, %g, %g, %g, %g, %g, %g, %g, %g, %g, %g", t_, n_,
                 (unsigned long long)records, (unsigned long long)contacts, o[0] + o[1] + o[2], o[0], o[1] + o[2],
                 o[1], o[2], o[3], o[4], o[5], o[6], o[7], o[8]);
    for (uint32_t u = 0; u < 2 * host_.num_udd_impact; ++u) std::fprintf(status_, ", 0");
    std::fprintf(status_, "\n");
    std::fflush(status_);
    return VEDO_OK;
}

// The line SimMediator::Run writes at a reset or record step: the record table rebuilt from the
// interactions that are active at the new positions (NBSConsultant::RebuildIactRecordTab,
// NBSConsultant.cpp:376-389), and among them those whose status holds a contact.
int Engine::status_row_now() {
    uint64_t active = 0, contacts = 0;
    if (cur_.np) {
        k_detect_active<<<blocks_for(cur_.np), TPB, 0, stream_>>>(cur_.np, cur_.sm, cur_.param, d_params_, d_geom_,
                                                                  d_hole_, d_reach_, d_pos_, d_ox_, d_oz_, d_pos32_,
                                                                  d_wall32_, cur_.flags, tab_.pbc);
        std::vector<uint8_t> f(cur_.np);
        CK(cudaMemcpyAsync(f.data(), cur_.flags, cur_.np, cudaMemcpyDeviceToHost, stream_));
        CK(cudaStreamSynchronize(stream_));
        for (uint8_t b : f)
            if (b & PF_ACTIVE) {
                ++active;
                contacts += (b & ST_CONTACT) ? 1u : 0u;
            }
    }
    return status_row(active, contacts);
}

int Engine::rebuild(bool from_records) {
    const uint64_t l0 = g_sort_scan_launches;
    uint64_t own = 0;
    // IsActive() of the current interactions at the current positions
    if (!from_records && cur_.np) {
        k_detect_active<<<blocks_for(cur_.np), TPB, 0, stream_>>>(cur_.np, cur_.sm, cur_.param, d_params_, d_geom_,
                                                                  d_hole_, d_reach_, d_pos_, d_ox_, d_oz_, d_pos32_,
                                                                  d_wall32_, cur_.flags, tab_.pbc);
        ++own;
    }
    std::swap(cur_, old_);
    // 1. safe lengths and bounds (:120-146)
    const double dtu = (double)opts_.up_iact * dt_;
    const double glen = len(mk(g_[0], g_[1], g_[2]));
    unsigned long long red0[8] = {ord_of(DBL_MAX), ord_of(DBL_MIN), ord_of(DBL_MAX), ord_of(DBL_MIN),
                                  ord_of(DBL_MAX), ord_of(DBL_MIN), ord_of(0.0), 0ull};
    CK(cudaMemcpyAsync(d_red_, red0, sizeof(red0), cudaMemcpyHostToDevice, stream_));
    k_safe<<<blocks_for(n_), TPB, 0, stream_>>>(n_, d_model_of_, d_models_, d_pos_, d_vel_, sf_, dtu, glen, d_safe_,
                                                d_red_);
    ++own;
    unsigned long long red[8];
    CK(cudaMemcpyAsync(red, d_red_, sizeof(red), cudaMemcpyDeviceToHost, stream_));
    CK(cudaStreamSynchronize(stream_));
    const double xmin = dbl_of(red[0]), xmax = dbl_of(red[1]), ymin = dbl_of(red[2]), ymax = dbl_of(red[3]);
    const double zmin = dbl_of(red[4]), zmax = dbl_of(red[5]), vmax = dbl_of(red[6]);
    const uint32_t nloc = n_ - (uint32_t)global_ids_.size();
    double rmax = 0.0;
    CellGrid g{};
    g.mode = 0;
    if (leap_) {
        // LeapConsultant::Reset (LeapConsultant.cpp:108-195): the largest range of the local
        // objects, and the comparator from the spans between the 2 % and 98 % quantiles of the
        // local positions per axis (sorted on the device)
        rmax = leap_rmax_;
        const double keep = 1.0 - 0.02, hi_d = keep * nloc - 1, lo_d = 0.02 * nloc;
        const uint32_t ih = hi_d < 0.0 ? 0u : (uint32_t)hi_d, il = (uint32_t)lo_d;
        double span[3];
        for (int a = 0; a < 3; ++a) {
            k_axis_key<<<blocks_for(n_), TPB, 0, stream_>>>(n_, d_model_of_, d_models_, d_pos_, a, d_key_, d_sid_);
            ++own;
            CK(radix_sort_u64(d_key_, d_sid_, d_key_alt_, d_sid_alt_, n_, 0, 64, scratch_, stream_));
            unsigned long long q[2];
            CK(cudaMemcpyAsync(&q[0], d_key_ + ih, 8, cudaMemcpyDeviceToHost, stream_));
            CK(cudaMemcpyAsync(&q[1], d_key_ + il, 8, cudaMemcpyDeviceToHost, stream_));
            CK(cudaStreamSynchronize(stream_));
            span[a] = dbl_of(q[0]) - dbl_of(q[1]);
        }
        g.mode = span[0] >= span[1] ? (span[0] >= span[2] ? 0 : 2) : (span[1] >= span[2] ? 1 : 2);
    } else if (red[7]) {
        rmax = tab_.models[host_.model_of[red[7] - 1]].range;              // the last local DO (:140)
    }
    const double zone = sf_ * (2.0 * rmax + dtu * vmax + 0.5 * dtu * dtu * glen);   // :146, Leap :138
    auto ncel = [&](double lo, double hi) {
        uint32_t c = (uint32_t)std::ceil((hi - lo) / zone);
        return std::max(c, (uint32_t)1);
    };
    const uint32_t ncx = ncel(xmin, xmax), ncy = ncel(ymin, ymax), ncz = ncel(zmin, zmax);
    g.ncel[0] = ncx; g.ncel[1] = ncy; g.ncel[2] = ncz;
    g.leap = leap_ ? 1 : 0;
    // key extents: zone ids reach ncel (a span that is a whole number of zones); Leap visits every
    // zone, so its neighbours reach ncel + 1
    const uint64_t pad = leap_ ? 2 : 1;
    g.dim[0] = (uint64_t)ncx + pad; g.dim[1] = (uint64_t)ncy + pad; g.dim[2] = (uint64_t)ncz + pad;
    if (leap_) {
        const double lo3[3] = {xmin, ymin, zmin}, hi3[3] = {xmax, ymax, zmax};
        for (int a = 0; a < 3; ++a) {                                      // LeapConsultant.h:146-150
            g.pbc[a] = tab_.pbc.sw[a] && (hi3[a] - lo3[a]) >= 0.5 * tab_.pbc.range[a];
            g.has_pbc |= g.pbc[a];
        }
    }
    const uint64_t sentinel = g.dim[0] * g.dim[1] * g.dim[2];
    int bits = 1;
    while (bits < 64 && (sentinel >> bits)) ++bits;
    // 2. cell keys, stable sort (locals by cell in the comparator's order, ids ascending within a cell)
    k_cellkey<<<blocks_for(n_), TPB, 0, stream_>>>(n_, d_model_of_, d_models_, d_pos_, xmin, ymin, zmin, zone, g,
                                                   sentinel, d_key_, d_sid_);
    ++own;
    CK(radix_sort_u64(d_key_, d_sid_, d_key_alt_, d_sid_alt_, n_, 0, bits, scratch_, stream_));
    // 3. cell ranges
    uint32_t np = 0;
    if (nloc) {
        k_cell_flags<<<blocks_for(nloc), TPB, 0, stream_>>>(nloc, d_key_, d_flag_);
        CK(exclusive_scan_u32(d_flag_, d_flag_, nloc, d_total_, scratch_, stream_));
        k_cell_fill<<<blocks_for(nloc), TPB, 0, stream_>>>(nloc, d_key_, d_flag_, d_cell_key_, d_cell_start_,
                                                           d_cellof_, d_total_);
        own += 2;
        // 4. count pass over (object, slot) tasks, scan, fill pass
        const uint64_t ntask = (uint64_t)nloc * NSLOT;
        if (ntask + 1 > task_cap_) {
            if (d_task_) cudaFree(d_task_);
            task_cap_ = (uint32_t)(ntask + 1);
            CK(dalloc(&d_task_, task_cap_));
        }
        CK(cudaMemsetAsync(d_err_, 0, sizeof(int), stream_));
        // dense cell map when the grid is small compared with the object count
        uint32_t* grid = nullptr;
        const uint64_t gcells = sentinel;
        if (gcells <= std::max<uint64_t>(8ull * n_, 1ull << 22) && gcells < (1ull << 31)) {
            if (gcells > grid_cap_) {
                if (d_grid_) cudaFree(d_grid_);
                d_grid_ = nullptr;
                grid_cap_ = gcells + gcells / 4;
                CK(dalloc(&d_grid_, grid_cap_));
            }
            CK(cudaMemsetAsync(d_grid_, 0xff, sizeof(uint32_t) * gcells, stream_));
            k_grid_fill<<<blocks_for(nloc), TPB, 0, stream_>>>(d_total_, d_cell_key_, d_grid_);
            ++own;
            grid = d_grid_;
        }
        k_pairs<false><<<blocks_for(ntask), TPB, 0, stream_>>>(
            nloc, d_sid_, d_cell_key_, d_cell_start_, d_total_, d_cellof_, grid, gcells, d_global_,
            (uint32_t)global_ids_.size(), d_model_of_, d_models_, d_group_iact_, tab_.ngroups, d_pos_, d_ox_, d_oz_,
            d_pos32_, d_wall32_, d_safe_, g, tab_.pbc, d_task_, nullptr, nullptr, d_err_);
        ++own;
        CK(exclusive_scan_u32(d_task_, d_task_, (uint32_t)ntask, d_total_ + 1, scratch_, stream_));
        CK(cudaMemcpyAsync(&np, d_total_ + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream_));
        CK(cudaStreamSynchronize(stream_));
        int rc = ensure_list(cur_, np);
        if (rc != VEDO_OK) return rc;
        k_pairs<true><<<blocks_for(ntask), TPB, 0, stream_>>>(
            nloc, d_sid_, d_cell_key_, d_cell_start_, d_total_, d_cellof_, grid, gcells, d_global_,
            (uint32_t)global_ids_.size(), d_model_of_, d_models_, d_group_iact_, tab_.ngroups, d_pos_, d_ox_, d_oz_,
            d_pos32_, d_wall32_, d_safe_, g, tab_.pbc, d_task_, cur_.first, cur_.second, d_err_);
        ++own;
    } else {
        int rc = ensure_list(cur_, 0);
        if (rc != VEDO_OK) return rc;
    }
    cur_.np = np;
    // 5. interactions: orientation and model selection
    if (np) {
        k_setup<<<blocks_for(np), TPB, 0, stream_>>>(np, cur_.first, cur_.second, d_model_of_, d_models_, d_params_,
                                                     nm_, cur_.sm, cur_.param, d_err_);
        ++own;
        // 6. history
        if (from_records) {
            k_history_rec<<<blocks_for(np), TPB, 0, stream_>>>(np, cur_.first, cur_.second, d_rec_key_, nrec_,
                                                               d_rec_hist_, d_rec_v0_, d_rec_flags_, cur_.hist,
                                                               cur_.v0, cur_.flags);
        } else {
            k_history_old<<<blocks_for(np), TPB, 0, stream_>>>(np, cur_.first, cur_.second, cur_.sm, cur_.param,
                                                               d_params_, d_reach_, d_pos32_, d_wall32_, old_.csr_ptr,
                                                               old_.csr_ent, old_.first, old_.second, old_.flags,
                                                               old_.hist, old_.v0, cur_.hist, cur_.v0, cur_.flags, tab_.pbc);
        }
        ++own;
    }
    // 7. per-object contact entries in ascending pair index (stable radix sort by object)
    const uint32_t m = 2 * np;
    if (m > csr_cap_) {
        for (uint32_t** p : {&d_ck_, &d_ck_alt_, &d_cv_alt_}) {
            if (*p) cudaFree(*p);
            *p = nullptr;
        }
        csr_cap_ = std::max<uint32_t>(m + m / 4, 2048);
        CK(dalloc(&d_ck_, csr_cap_)); CK(dalloc(&d_ck_alt_, csr_cap_)); CK(dalloc(&d_cv_alt_, csr_cap_));
    }
    if (np) {
        k_csr_keys<<<blocks_for(np), TPB, 0, stream_>>>(np, cur_.sm, d_ck_, cur_.csr_ent);
        ++own;
        int obits = 1;
        while (obits < 32 && ((n_ - 1) >> obits)) ++obits;
        CK(radix_sort_u32(d_ck_, cur_.csr_ent, d_ck_alt_, d_cv_alt_, m, 0, obits, scratch_, stream_));
    }
    k_csr_ptr<<<blocks_for((uint64_t)n_ + 1), TPB, 0, stream_>>>(n_, d_ck_, m, cur_.csr_ptr);
    ++own;
    int herr = 0;
    CK(cudaMemcpyAsync(&herr, d_err_, sizeof(int), cudaMemcpyDeviceToHost, stream_));
    CK(cudaStreamSynchronize(stream_));
    CK(cudaGetLastError());
    launches_ += own + (g_sort_scan_launches - l0);
    if (herr & ERR_BAD_SHAPE_PAIR)
        return fail(VEDO_ERR_UNSUPPORTED_MODEL, "broad phase met a shape pair DOMap::CalDistance does not handle");
    if (herr & ERR_UNSUPPORTED_PAIR)
        return fail(VEDO_ERR_UNSUPPORTED_MODEL,
                    "a candidate pair has no detector/solver (the reference would drop it and misalign its "
                    "interaction records)");
    backup_pending_ = false;
    return VEDO_OK;
}

int Engine::step_once(bool write_impulses) {
    const double dt = dt_;
    const bool prof = profiling_;
    // CalculateImpact
    if (prof) CK(cudaEventRecord(ev_[0], stream_));
    if (cur_.np && cur_.np <= FUSED_PAIRS) {
        k_pair_fused<<<blocks_for(cur_.np), TPB, 0, stream_>>>(cur_.np, cur_.sm, cur_.param, d_params_, d_geom_,
                                                               d_hole_, d_reach_, d_pos_, d_vel_, d_av_, d_ox_, d_oz_,
                                                               d_pos32_, d_wall32_, cur_.hist, cur_.v0, cur_.flags,
                                                               cur_.out, dt, backup_pending_ ? 1 : 0, tab_.pbc,
                                                               d_touched_);
        ++launches_;
    } else if (cur_.np) {
        k_pair_pf<<<blocks_for(cur_.np), TPB, 0, stream_>>>(cur_.np, cur_.sm, cur_.param, d_params_, d_reach_,
                                                            d_pos32_, d_wall32_, cur_.hist, cur_.v0, cur_.flags,
                                                            tab_.pbc, cur_.work, d_nwork_);
        if (!pair_grid_) {                         // the exact pass strides with the grid resident at once
            int b = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_pair_exact, TPB, 0) != cudaSuccess || b < 1) b = 1;
            int sms = 1;
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, opts_.device);
            pair_grid_ = (unsigned)(b * std::max(sms, 1));
        }
        k_pair_exact<<<std::min<unsigned>(pair_grid_, blocks_for(cur_.np)), TPB, 0, stream_>>>(
            cur_.work, d_nwork_, cur_.sm, cur_.param, d_params_, d_geom_, d_hole_, d_pos_, d_vel_, d_av_, d_ox_,
            d_oz_, cur_.hist, cur_.v0, cur_.flags, cur_.out, dt, backup_pending_ ? 1 : 0, tab_.pbc, d_touched_);
        launches_ += 2;
    }
    if (prof) CK(cudaEventRecord(ev_[1], stream_));
    // AddFieldImpact + AddConstrainedImpact + Response (+ CheckContactStatus in the next k_pair_exact)
    const d3 fimp = muls(mk(g_[0], g_[1], g_[2]), dt);    // csp->GetFieldAcceleration() * dt (SimMediator.cpp:738)
    const d3 org = mk(origin_[0], origin_[1], origin_[2]);
    k_obj<<<blocks_for(n_), TPB, 0, stream_>>>(n_, d_model_of_, d_models_, d_pos_, d_vel_, d_av_, d_ox_, d_oz_,
                                               d_imp_, d_aimp_, cur_.csr_ptr, cur_.csr_ent, cur_.flags, cur_.out, dt,
                                               fimp, write_impulses ? 1 : 0, org, d_pos32_, d_wall32_, ext_imp_, ext_aimp_,
                                               tab_.pbc, d_touched_, d_nwork_);
    ++launches_;
    if (!global_ids_.empty()) {
        k_obj_global<<<blocks_for((uint64_t)global_ids_.size() * 32), TPB, 0, stream_>>>(
            (uint32_t)global_ids_.size(), d_global_, d_model_of_, d_models_, d_pos_, d_vel_, d_av_, d_ox_, d_oz_,
            d_imp_, d_aimp_, cur_.csr_ptr, cur_.csr_ent, cur_.flags, cur_.out, dt, fimp, write_impulses ? 1 : 0, org,
            d_pos32_, d_wall32_, ext_imp_, ext_aimp_, tab_.pbc, d_touched_);
        ++launches_;
    }
    if (prof) CK(cudaEventRecord(ev_[2], stream_));
    backup_pending_ = true;
    // NBSConsultant::NextStep (NBSConsultant.cpp:35-78)
    ++round_;
    t_ += dt;                                              // SystemParameter::NextStep (SystemParameter.h:113-116)
    if (round_ % opts_.up_iact == 0) {
        if (prof) CK(cudaEventRecord(ev_[3], stream_));
        bool erased = false;
        if (leap_ && zoi_on_) {                            // LeapConsultant.cpp:61-68
            int rc = leap_cleanup(&erased);
            if (rc != VEDO_OK) return rc;
        }
        int rc = rebuild(erased);                          // after an erasure, from the re-keyed records
        if (rc != VEDO_OK) return rc;
        if (prof) {
            CK(cudaEventRecord(ev_[4], stream_));
            CK(cudaEventSynchronize(ev_[4]));
            float ms = 0;
            cudaEventElapsedTime(&ms, ev_[3], ev_[4]);
            prof_ms_[2] += ms;
        }
    }
    if (prof) {
        float a = 0, b = 0;
        CK(cudaEventSynchronize(ev_[2]));
        cudaEventElapsedTime(&a, ev_[0], ev_[1]);
        cudaEventElapsedTime(&b, ev_[1], ev_[2]);
        prof_ms_[0] += a;
        prof_ms_[1] += b;
    }
    if (opts_.record && round_ % opts_.record == 0 && !out_prefix_.empty()) {
        int rc = record_ido();
        if (rc != VEDO_OK) return rc;
    }
    if (status_ && (round_ % opts_.up_iact == 0 || (opts_.record && round_ % opts_.record == 0))) {
        int rc = status_row_now();                         // SimMediator.cpp:784-792
        if (rc != VEDO_OK) return rc;
    }
    if (t_ >= t_stop_ && !out_prefix_.empty()) {         // NBSConsultant.cpp:65-76
        std::string dir = out_prefix_;
        size_t slash = dir.find_last_of('/');
        dir = slash == std::string::npos ? std::string() : dir.substr(0, slash + 1);
        int rc = write_ido((dir + "terminate.ido").c_str());
        if (rc != VEDO_OK) return rc;
    }
    return VEDO_OK;
}

int Engine::run(uint32_t nsteps, int* keep_running) {
    prof_ms_[0] = prof_ms_[1] = prof_ms_[2] = prof_ms_[3] = 0;
    launches_ = 0;
    CK(cudaSetDevice(device_));
    CK(cudaEventRecord(ev_[5], stream_));
    for (uint32_t s = 0; s < nsteps; ++s) {
        int rc = step_once(s + 1 == nsteps);
        if (rc != VEDO_OK) return rc;
    }
    CK(cudaEventRecord(ev_[6], stream_));
    CK(cudaStreamSynchronize(stream_));
    CK(cudaGetLastError());
    float tot = 0;
    cudaEventElapsedTime(&tot, ev_[5], ev_[6]);
    prof_ms_[3] = tot;
    if (keep_running) *keep_running = t_ < t_stop_ ? 1 : 0;   // SimMediator.cpp:839-841
    return VEDO_OK;
}

// One step with per-object external impulses (SimMediator::Run(external impacts),
// SimMediator.cpp:987-1119): host [n][3] arrays, NULL adds zeros as the reference adds them.
int Engine::run_with_impulses(const double* impulse, const double* angular_impulse, int* keep_running) {
    CK(cudaSetDevice(device_));
    if (!d_ext_) CK(cudaMalloc(&d_ext_, 2 * 24 * (size_t)n_));
    const double* src[2] = {impulse, angular_impulse};
    for (int k = 0; k < 2; ++k) {
        double* dst = d_ext_ + (size_t)k * 3 * n_;
        if (src[k]) CK(cudaMemcpyAsync(dst, src[k], 24 * (size_t)n_, cudaMemcpyHostToDevice, stream_));
        else CK(cudaMemsetAsync(dst, 0, 24 * (size_t)n_, stream_));
    }
    ext_imp_ = d_ext_;
    ext_aimp_ = d_ext_ + 3 * (size_t)n_;
    const int rc = run(1, keep_running);
    ext_imp_ = ext_aimp_ = nullptr;
    return rc;
}

uint64_t Engine::last_profile(double out[4]) const {
    for (int k = 0; k < 4; ++k) out[k] = prof_ms_[k];
    return launches_;
}

// ------------------------------------------------------------------------------------
// state I/O: host [n][3] arrays <-> device double4 (x, y, z, pad); the repacking runs on the
// device, the host side is one contiguous copy per array.
namespace {
__global__ void k_pack3(uint32_t n, const double* __restrict__ src, double4_32a* __restrict__ dst) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = make_double4_32a(src[3 * (size_t)i], src[3 * (size_t)i + 1], src[3 * (size_t)i + 2], 0.0);
}
__global__ void k_unpack3(uint32_t n, const double4_32a* __restrict__ src, double* __restrict__ dst) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const double4_32a v = src[i];
        dst[3 * (size_t)i] = v.x;
        dst[3 * (size_t)i + 1] = v.y;
        dst[3 * (size_t)i + 2] = v.z;
    }
}
}  // namespace

int Engine::ensure_stage() {
    if (d_stage_) return VEDO_OK;
    CK(dalloc(&d_stage_, 7 * 3 * (size_t)n_));
    return VEDO_OK;
}

int Engine::get_state(const vedo_state_view& v) {
    int rc = ensure_stage();
    if (rc != VEDO_OK) return rc;
    double* dst[] = {v.position, v.velocity, v.angular_velocity, v.orientation_x, v.orientation_z, v.impact,
                     v.angular_impact};
    const double4_32a* src[] = {d_pos_, d_vel_, d_av_, d_ox_, d_oz_, d_imp_, d_aimp_};
    for (int k = 0; k < 7; ++k) {
        if (!dst[k]) continue;
        double* st = d_stage_ + (size_t)k * 3 * n_;
        k_unpack3<<<blocks_for(n_), TPB, 0, stream_>>>(n_, src[k], st);
        CK(cudaMemcpyAsync(dst[k], st, 24 * (size_t)n_, cudaMemcpyDeviceToHost, stream_));
    }
    CK(cudaStreamSynchronize(stream_));
    CK(cudaGetLastError());
    return VEDO_OK;
}

int Engine::set_state(const vedo_state_view& v) {
    int rc = ensure_stage();
    if (rc != VEDO_OK) return rc;
    const double* srcs[] = {v.position, v.velocity, v.angular_velocity, v.orientation_x, v.orientation_z, v.impact,
                            v.angular_impact};
    double4_32a* dst[] = {d_pos_, d_vel_, d_av_, d_ox_, d_oz_, d_imp_, d_aimp_};
    for (int k = 0; k < 7; ++k) {
        if (!srcs[k]) continue;
        double* st = d_stage_ + (size_t)k * 3 * n_;
        CK(cudaMemcpyAsync(st, srcs[k], 24 * (size_t)n_, cudaMemcpyHostToDevice, stream_));
        k_pack3<<<blocks_for(n_), TPB, 0, stream_>>>(n_, st, dst[k]);
    }
    k_refresh32<<<blocks_for(n_), TPB, 0, stream_>>>(n_, d_model_of_, d_models_, d_pos_, d_ox_, d_oz_,
                                                     mk(origin_[0], origin_[1], origin_[2]), d_pos32_, d_wall32_);
    CK(cudaStreamSynchronize(stream_));
    CK(cudaGetLastError());
    return VEDO_OK;
}

int Engine::num_interactions(uint32_t* n) {
    *n = cur_.np;
    return VEDO_OK;
}

int Engine::get_interactions(const vedo_contact_view& v) {
    const uint32_t np = cur_.np;
    if (!np) return VEDO_OK;
    // ContactInfo::bActive of the last narrow phase = detection at the current positions
    k_detect_active<<<blocks_for(np), TPB, 0, stream_>>>(np, cur_.sm, cur_.param, d_params_, d_geom_, d_hole_, d_reach_,
                                                         d_pos_, d_ox_, d_oz_, d_pos32_, d_wall32_, cur_.flags, tab_.pbc);
    std::vector<uint2> sm(np);
    std::vector<uint8_t> fl(np);
    std::vector<double4_32a> h(np);
    if (v.first) CK(cudaMemcpyAsync(v.first, cur_.first, 4 * np, cudaMemcpyDeviceToHost, stream_));
    if (v.second) CK(cudaMemcpyAsync(v.second, cur_.second, 4 * np, cudaMemcpyDeviceToHost, stream_));
    CK(cudaMemcpyAsync(sm.data(), cur_.sm, sizeof(uint2) * np, cudaMemcpyDeviceToHost, stream_));
    CK(cudaMemcpyAsync(fl.data(), cur_.flags, np, cudaMemcpyDeviceToHost, stream_));
    CK(cudaMemcpyAsync(h.data(), cur_.hist, sizeof(double4_32a) * np, cudaMemcpyDeviceToHost, stream_));
    CK(cudaStreamSynchronize(stream_));
    for (uint32_t k = 0; k < np; ++k) {
        const bool nz = fl[k] & PF_NONZERO;
        if (v.slave) v.slave[k] = sm[k].x;
        if (v.master) v.master[k] = sm[k].y;
        if (v.active) v.active[k] = (fl[k] & PF_ACTIVE) ? 1 : 0;
        if (v.contact) v.contact[k] = (fl[k] & ST_CONTACT) ? 1 : 0;
        if (v.kn) v.kn[k] = nz ? h[k].w : 0.0;
        if (v.shear) {
            v.shear[3 * k] = nz ? h[k].x : 0.0;
            v.shear[3 * k + 1] = nz ? h[k].y : 0.0;
            v.shear[3 * k + 2] = nz ? h[k].z : 0.0;
        }
    }
    return VEDO_OK;
}

int Engine::get_observables(double out[13]) {
    const unsigned nb = std::max(1u, blocks_for(n_));
    double* part = d_obs_;
    double* res = d_obs_ + (size_t)nb * 16 + 16;
    const d3 g = mk(g_[0], g_[1], g_[2]);
    obs::k_obs_a<<<nb, TPB, 0, stream_>>>(n_, d_model_of_, d_models_, d_pos_, d_vel_, d_av_, g, part);
    obs::k_obs_reduce<<<1, 32, 0, stream_>>>(nb, 16, part, res, 12);
    if (cur_.np)
        k_detect_active<<<blocks_for(cur_.np), TPB, 0, stream_>>>(cur_.np, cur_.sm, cur_.param, d_params_, d_geom_,
                                                                  d_hole_, d_reach_, d_pos_, d_ox_, d_oz_, d_pos32_,
                                                                  d_wall32_, cur_.flags, tab_.pbc);
    obs::k_obs_b<<<nb, TPB, 0, stream_>>>(n_, d_model_of_, d_models_, d_pos_, d_vel_, d_av_, res, 0, cur_.flags, cur_.np,
                                     part);
    obs::k_obs_reduce<<<1, 32, 0, stream_>>>(nb, 6, part, res + 16, 6);
    double r[22];
    CK(cudaMemcpyAsync(r, res, sizeof(r), cudaMemcpyDeviceToHost, stream_));
    CK(cudaStreamSynchronize(stream_));
    const bool any = r[9] > 0;
    out[0] = r[0]; out[1] = r[1]; out[2] = r[2];
    out[3] = any ? r[12] : 0.0; out[4] = any ? r[13] : 0.0; out[5] = any ? r[14] : 0.0; out[6] = any ? r[15] : 0.0;
    out[7] = r[16]; out[8] = r[17];
    out[9] = r[21];
    const double msum = r[10];
    out[10] = msum > 0 ? r[18] / msum : 0.0;
    out[11] = msum > 0 ? r[19] / msum : 0.0;
    out[12] = msum > 0 ? r[20] / msum : 0.0;
    return VEDO_OK;
}

int Engine::sync_host_state() {
    vedo_state_view v{host_.pos.data(), host_.vel.data(), host_.av.data(), host_.ox.data(), host_.oz.data(),
                      host_.imp.data(), host_.aimp.data()};
    return get_state(v);
}

int Engine::coordination(uint32_t* below, uint32_t* touching, const double* box, double* average) {
    DeviceObjects d;
    d.n = n_; d.model_of = d_model_of_; d.models = d_models_; d.pos = d_pos_;
    d.stream = stream_; d.scratch = &scratch_; d.scene = &host_; d.launches = &launches_;
    std::string m;
    const int rc = coordination_host(d, below, touching, box, average, m);
    return rc == VEDO_OK ? rc : fail(rc, m);
}

int Engine::write_vtk(const char* path, int with_coordination) {
    DeviceObjects d;
    d.n = n_; d.model_of = d_model_of_; d.models = d_models_; d.pos = d_pos_;
    d.stream = stream_; d.scratch = &scratch_; d.scene = &host_; d.launches = &launches_;
    std::string m;
    const int rc = write_vtk_host(this, d, path, with_coordination, m);
    return rc == VEDO_OK ? rc : fail(rc, m);
}

int Engine::write_ido(const char* path) {
    int rc = sync_host_state();
    if (rc != VEDO_OK) return rc;
    host_.time_current = t_;
    // IactRecordTab = the active interactions (NBSConsultant::RebuildIactRecordTab)
    const uint32_t np = cur_.np;
    std::vector<uint32_t> a(np), b(np);
    std::vector<uint8_t> act(np), con(np);
    std::vector<double> sh(3 * (size_t)np), kn(np);
    vedo_contact_view cv{a.data(), b.data(), nullptr, nullptr, act.data(), sh.data(), kn.data(), con.data()};
    rc = get_interactions(cv);
    if (rc != VEDO_OK) return rc;
    std::vector<double> v0(np);
    if (np) {
        CK(cudaMemcpyAsync(v0.data(), cur_.v0, 8 * np, cudaMemcpyDeviceToHost, stream_));
        CK(cudaStreamSynchronize(stream_));
    }
    HRecords R;
    std::vector<uint32_t> idx;
    for (uint32_t k = 0; k < np; ++k)
        if (act[k]) idx.push_back(k);
    std::sort(idx.begin(), idx.end(), [&](uint32_t x, uint32_t y) {
        return a[x] != a[y] ? a[x] < a[y] : b[x] < b[y];
    });
    for (uint32_t k : idx) {
        R.first.push_back(a[k]); R.second.push_back(b[k]);
        R.contact.push_back(con[k]); R.bond.push_back(0);
        R.kn.push_back(kn[k]); R.v0.push_back(v0[k]);
        for (int q = 0; q < 3; ++q) {
            R.shear.push_back(sh[3 * k + q]);
            R.point.push_back(0.0); R.dirn.push_back(0.0); R.imp.push_back(0.0); R.aimp.push_back(0.0);
        }
        R.overlap.push_back(0.0);
    }
    HScene copy_rec = host_;
    copy_rec.rec = R;
    std::string msg;
    if (!vedo::write_ido(path, copy_rec, msg)) return fail(VEDO_ERR_IO, msg);
    return VEDO_OK;
}

int Engine::record_ido() {                                 // Consultant::RecordIDO (Consultant.cpp:217-230)
    char num[32];
    snprintf(num, sizeof(num), "%d", (int)(10000001 + record_count_));
    std::string file = out_prefix_ + "_" + (record_count_ < 11000001 ? std::string(num + 2) : std::string(num)) + ".ido";
    ++record_count_;
    return write_ido(file.c_str());
}

EngineBase* make_fp64_engine() { return new (std::nothrow) Engine(); }

}  // namespace vedo
