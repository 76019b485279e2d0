// dem_physics.cuh - FP64 narrow phase, impact solvers and integrators of the reference,
// restated as device functions over one candidate pair / one object.
//
// Compiled only into translation units built with -fmad=false: each function keeps the
// reference's operation order, so with IEEE-rounded +,-,*,/ and sqrt the results equal
// the reference's bit for bit (pow, cos and sin are CUDA's and may differ in the last ulp).
#pragma once

#include "dem_common.cuh"

namespace vedo {

// Pair parameters with the geometry the detector needs, copied from the models.
struct PairGeom {
    double ra;               // slave sphere radius
    double b0, b1, b2;       // master attributes (sphere r | cylinder r, h | plate w, h, l)
    double hr, hxo, hyo;     // holed plate: hole radius and offsets (CD_SHP only)
};

struct PairParamFull {
    PairParam p;
    PairGeom g;
};

// ContactDetector::Detect of the three shape pairs: depth, direction, impact point.
// With an active periodic boundary the sphere-sphere detector takes the minimum image of the
// centre difference (CDSphere2Sphere.cpp:19-22); the wall detectors do not.
__device__ __forceinline__ void detect_pair(int cd, const PairGeom& g, d3 Ps, d3 Pm, const double4_32a* __restrict__ ox,
                                            const double4_32a* __restrict__ oz, uint32_t m, const Periodic& pb,
                                            double& depth, d3& n, d3& point) {
    if (cd == CD_SS) {                                        // CDSphere2Sphere.cpp:14-41
        d3 vIm = sub(Pm, Ps);
        if (pb.on) vIm = min_image(pb, vIm);
        depth = g.ra + g.b0 - len(vIm);
        n = dir(vIm);
    } else if (cd == CD_SP) {                                 // CDSphere2QuasiPlate.cpp:15-97
        d3 Oz = ld(oz, m), Ox = ld(ox, m);
        d3 Oy = cross(Oz, Ox);
        d3 Cap = sub(Ps, project_on(sub(Ps, Pm), Oz));
        double hh = 0.5 * g.b1, hw = 0.5 * g.b0, hl = 0.5 * g.b2;
        double dx = dot(sub(Cap, Pm), Ox);
        if (dx < -hw) dx = -hw; else if (dx > hw) dx = hw;
        double dy = dot(sub(Cap, Pm), Oy);
        if (dy < -hl) dy = -hl; else if (dy > hl) dy = hl;
        d3 Caps = add(add(muls(Ox, dx), muls(Oy, dy)), Pm);
        d3 vIm = sub(Caps, Ps);
        depth = g.ra + hh - len(vIm);
        n = dir(vIm);
    } else if (cd == CD_SHP) {                                // CDSphere2QuasiPlateWithCircularHole.cpp:15-133
        d3 Oz = ld(oz, m), Ox = ld(ox, m);
        d3 Oy = cross(Oz, Ox);
        d3 Cap = sub(Ps, project_on(sub(Ps, Pm), Oz));
        double hh = 0.5 * g.b1, hw = 0.5 * g.b0, hl = 0.5 * g.b2;
        // the hole's centre: the offsets are added in world coordinates, as the reference does
        d3 Cha = sub(Ps, add(Pm, mk(g.hxo, g.hyo, 0.0)));
        double dx = dot(sub(Cap, Pm), Ox);
        if (dx < -hw) dx = -hw; else if (dx > hw) dx = hw;
        double dy = dot(sub(Cap, Pm), Oy);
        if (dy < -hl) dy = -hl; else if (dy > hl) dy = hl;
        double dahx = dot(Cha, Ox), dahy = dot(Cha, Oy);
        double dah = sqrt(dahx * dahx + dahy * dahy);
        if (dah < g.hr) {
            if (dah == 0.0) {
                dx = g.hxo;
                dy = g.hyo;
            } else {
                dx = g.hxo + dahx / dah * g.hr;
                dy = g.hyo + dahy / dah * g.hr;
            }
        }
        d3 Caps = add(add(muls(Ox, dx), muls(Oy, dy)), Pm);
        d3 vIm = sub(Caps, Ps);
        if (dah == 0.0) {
            const double lv = len(vIm);
            depth = g.ra + hh - sqrt(lv * lv + g.hr * g.hr);
        } else {
            depth = g.ra + hh - len(vIm);
        }
        n = dir(vIm);
    } else if (cd == CD_SIC) {
        // Engine extension, no reference counterpart: a sphere inside a hollow cylinder of radius
        // b0 and length b1 about its unit OrientationZ (a drum shell).  Within the length the
        // depth is how far the sphere's surface passes the shell, the normal the outward radial
        // direction; beyond an end, the nearest point of that end's rim circle.
        const double hh = 0.5 * g.b1, R = g.b0;
        const d3 ax = ld(oz, m);
        const d3 d = sub(Ps, Pm);
        const double t = dot(d, ax);
        const d3 rp = sub(d, muls(ax, t));
        const d3 u = dir(rp);
        if (t <= hh && t >= -hh) {
            depth = g.ra + len(rp) - R;
            n = u;
        } else {
            const d3 q = add(add(Pm, muls(ax, t > 0.0 ? hh : -hh)), muls(u, R));
            const d3 vIm = sub(q, Ps);
            depth = g.ra - len(vIm);
            n = dir(vIm);
        }
    } else {                                                  // CDSphere2QuasiCylinder.cpp:16-80
        double hh = 0.5 * g.b1;
        d3 ax = ld(oz, m);
        double dap = dot(sub(Ps, Pm), ax);
        if (dap < -hh) dap = -hh; else if (dap > hh) dap = hh;
        d3 Caps = add(Pm, smul(dap, ax));
        d3 vIm = sub(Caps, Ps);
        depth = g.ra + g.b0 - len(vIm);
        n = dir(vIm);
    }
    point = add(Ps, smul(g.ra - 0.5 * depth, n));             // impact point, e.g. CDSphere2Sphere.cpp:47-49
}

// ISwModels helpers (ISwModels.cpp)
__device__ __forceinline__ d3 shear_rotation(d3 F, d3 vs) {        // :263-273
    if (dot(F, vs) <= 0.0) return smul(-len(F), dir(vs));
    return smul(len(F), dir(vs));
}
__device__ __forceinline__ d3 normal_force(double kn, double cn, double depth, d3 n, d3 vn) {   // :134-139
    return sub(smul(-kn * depth, n), smul(cn, vn));
}
__device__ __forceinline__ d3 normal_force_bond(double kn, double cn, double depth, d3 n, d3 vn) {  // :166-180
    if (dot(vn, n) < 0.0) return sub(smul(-kn * depth, n), smul(cn, vn));
    return smul(-cn, vn);
}
__device__ __forceinline__ bool normal_bond(double kn, double bn, double depth) {   // :110-125
    return (depth <= 0.0) && (kn != 0.0) && (bn != 0.0) && (-depth * kn < bn);
}

// Pair status and outputs.
enum : uint8_t { PF_APPLIED = 16, PF_ANGULAR = 32, PF_ACTIVE = 64, PF_NONZERO = 128 };
constexpr uint8_t PF_STATUS = ST_CONTACT | ST_LAST_CONTACT | ST_BOND | ST_LAST_BOND;

struct PairStatus {
    uint8_t f;       // ST_* bits | PF_NONZERO
    d3 shear;
    double kn, v0;
};

// ImpactSolver::NextStep of the five laws for one pair; returns the PF_APPLIED/PF_ANGULAR bits
// and the impulse J on the slave, angular impulses tA (slave) and tB (master).  With an active
// periodic boundary every law takes the minimum image of both lever arms (ISwBSDBF.cpp:69-73,
// ISwBtSDBF.cpp:69-73, ISwBSDB2F.cpp:72-76, ISwHertz.cpp:59-63, ISwH.cpp:69-73).
__device__ __forceinline__ uint8_t solve_pair(int is, const double* __restrict__ c, bool active, double depth, d3 n,
                                              d3 point, d3 Ps, d3 Pm, d3 Va, d3 Vb, d3 AVa, d3 AVb, double dt,
                                              const Periodic& pb, PairStatus& st, d3& J, d3& tA, d3& tB) {
    const d3 Z = mk(0.0, 0.0, 0.0);
    if (is == IS_HERTZ || is == IS_H) {
        if (!active) {                                        // ISwHertz.cpp:26-30, ISwH.cpp:132-136
            st.f = 0; st.shear = Z; st.kn = 0.0; st.v0 = 0.0;  // ImpactStatus::Clean
            return 0;
        }
    } else if (!active && !normal_bond(c[0], c[4], depth)) {  // ISwBSDBF.cpp:32-38
        st.f = 0; st.shear = Z; st.kn = 0.0; st.v0 = 0.0;
        return 0;
    }
    d3 rA = Z, rB = Z, vRel, vRn, vRs;
    d3 Fn = Z, Fs = Z;
    if (depth > 0.0) {
        rA = sub(point, Ps);
        rB = sub(point, Pm);
        if (pb.on) {
            rA = min_image(pb, rA);
            rB = min_image(pb, rB);
        }
        vRel = sub(add(sub(Va, Vb), cross(AVa, rA)), cross(AVb, rB));
        vRn = smul(dot(vRel, n), n);
        vRs = sub(vRel, vRn);
        if (is == IS_BSDBF || is == IS_BSDB2F) {              // ISwBSDBF.cpp:61-112
            const double kn = c[0], ks = c[1], cn = c[2], cs = c[3], bs = c[5], fc = c[6];
            Fn = normal_force(kn, cn, depth, n, vRn);
            Fs = sub(shear_rotation(st.shear, vRs), smul(ks * dt, vRs));
            double fmax = fc * kn * depth;
            bool slide = (bs == 0.0) ? (len(Fs) > fmax) : (len(Fs) > bs);
            if (slide) Fs = smul(fmax, dir(Fs));
            else Fs = sub(Fs, smul(cs, vRs));
            st.shear = Fs;
            st.f |= ST_CONTACT | PF_NONZERO;
        } else if (is == IS_BTSDBF) {                         // ISwBtSDBF.cpp:61-111
            const double kn = c[0], ks = c[1], cn = c[2], cs = c[3], bs = c[5], fc = c[6];
            Fn = normal_force(kn, cn, depth, n, vRn);
            Fs = sub(smul(-ks * dt, vRs), smul(cs, vRs));
            double fmax = fc * kn * depth;
            bool slide = (bs == 0.0) ? (len(Fs) > fmax) : (len(Fs) > bs);
            if (slide) Fs = smul(fmax, dir(Fs));
            else Fs = sub(Fs, smul(cs, vRs));
            st.f |= ST_CONTACT;
        } else if (is == IS_HERTZ) {                          // ISwHertz.cpp:53-78
            const double kn = c[0], cn = c[1];
            if (!(st.f & ST_CONTACT)) {
                st.f |= ST_CONTACT | PF_NONZERO;
                st.v0 = len(vRn);
            }
            Fn = sub(smul(-kn * pow(depth, 1.5), n), smul(cn, vRn));   // ISwModels.cpp:127-132
        } else {                                              // ISwH.cpp:159-231
            const double knH = c[0], Meff = c[1], ksc1 = c[2], ksc2 = c[3], betan = c[4], fk = c[5];
            double kn;
            if (!(st.f & ST_CONTACT)) {
                double vnl = len(vRn);
                if (vnl == 0.0) kn = knH;
                else if (betan < 0.99)
                    kn = 0.957832746294131 / (1.0 - betan * betan) * pow(Meff, 0.2) * pow(knH, 0.8) * pow(vnl, 0.4);
                else
                    kn = 479.155951122633 * pow(Meff, 0.2) * pow(knH, 0.8) * pow(vnl, 0.4);
                st.kn = kn;
                st.f |= ST_CONTACT | PF_NONZERO;
            } else {
                kn = st.kn;
            }
            double ncd = 2.0 * sqrt(Meff * kn);
            double ks = ksc1 * pow(ksc2 * fabs(kn * depth), 1.0 / 3.0);
            Fn = normal_force(kn, ncd * betan, depth, n, vRn);
            double ff = fk * kn * depth;
            Fs = sub(shear_rotation(st.shear, vRs), smul(ks * dt, vRs));
            if (len(Fs) >= ff) Fs = smul(ff, dir(Fs));
            st.shear = Fs;
        }
    } else {
        // reached only with a normal bond (bn != 0) at depth <= 0
        bool clean = true;
        if (is == IS_BSDBF || is == IS_BTSDBF) {              // ISwBSDBF.cpp:113-123
            vRel = sub(Va, Vb);
            vRn = smul(dot(vRel, n), n);
            Fn = (is == IS_BSDBF) ? normal_force_bond(c[0], c[2], depth, n, vRn) : normal_force(c[0], c[2], depth, n, vRn);
        } else if (is == IS_BSDB2F) {                         // ISwBSDB2F.cpp:120-133
            if (st.f & ST_LAST_BOND) {
                vRel = sub(Va, Vb);
                vRn = smul(dot(vRel, n), n);
                Fn = normal_force_bond(c[0], c[2], depth, n, vRn);
            } else {
                clean = false;
            }
        }
        if (clean) {                                          // ImpactStatus::CleanContactStatusAndImpact
            uint8_t nf = (st.f & PF_NONZERO);
            if (st.f & ST_CONTACT) nf |= ST_LAST_CONTACT;
            if (st.f & ST_BOND) nf |= ST_LAST_BOND;
            st.f = nf;
            st.shear = Z;
        }
    }
    if (is == IS_HERTZ) {                                     // ISwHertz.cpp:85-91
        J = muls(Fn, dt);
        tA = Z;
        tB = Z;
        return PF_APPLIED;
    }
    d3 F = add(Fn, Fs);
    J = muls(F, dt);
    tA = smul(dt, cross(rA, F));
    tB = smul(-dt, cross(rB, F));
    return PF_APPLIED | PF_ANGULAR;
}

// DiscreteObject::Response of each shape/behaviour; J, JA are the summed impulses.
__device__ __forceinline__ void respond_object(const ModelDev& m, double dt, d3 J, d3 JA, d3& P, d3& V, d3& AV, d3& Ox,
                                               d3& Oz) {
    if (m.behavior == BEH_FIXED) return;                      // DOFixedQuasiPlate.h:16-19
    if (m.shape == SHAPE_SPHERE) {                            // DOSphere.cpp:21-48
        d3 dv = smul(m.inv_sudo, J);                          // 1.0 / dSudoMass * vImpact
        d3 dav = smul(m.rot_coef, JA);                         // 2.5 / dSudoMass / Radius / Radius * ...
        d3 dp = smul(dt, add(V, smul(0.5, dv)));
        d3 dw = smul(dt, add(AV, smul(0.5, dav)));
        P = add(P, dp);
        const Turn T = turn_of(dw);
        Ox = rotate_by(Ox, T);
        Oz = rotate_by(Oz, T);
        V = add(V, dv);
        AV = add(AV, dav);
    } else if (m.behavior == BEH_ORBITAL) {                   // DOOrbitalQuasiPlate.cpp:18-34
        d3 dp = muls(V, dt);
        d3 dw = muls(AV, dt);
        P = add(P, dp);
        const Turn T = turn_of(dw);
        Ox = rotate_by(Ox, T);
        Oz = rotate_by(Oz, T);
    } else if (m.behavior == BEH_CONSTRAINED) {               // DOConstrainedQuasiPlate.cpp:18-35
        d3 dv = smul(m.inv_sudo, smul(dot(J, Oz), dir(Oz)));
        d3 dp = smul(dt, add(V, smul(0.5, dv)));
        d3 dw = muls(AV, dt);
        P = add(P, dp);
        const Turn T = turn_of(dw);
        Ox = rotate_by(Ox, T);
        Oz = rotate_by(Oz, T);
        V = add(V, dv);
    } else {                                                  // DOQuasiPlate.cpp:20-41, DOQuasiCylinder.cpp
        d3 dv = smul(m.inv_sudo, J);
        d3 dav = mk(dot(JA, Ox) / m.ix, dot(JA, cross(Oz, Ox)) / m.iy, dot(JA, Oz) / m.iz);
        d3 dp = smul(dt, add(V, smul(0.5, dv)));
        d3 dw = smul(dt, add(AV, smul(0.5, dav)));
        P = add(P, dp);
        const Turn T = turn_of(dw);
        Ox = rotate_by(Ox, T);
        Oz = rotate_by(Oz, T);
        V = add(V, dv);
        AV = add(AV, dav);
    }
}

// DOMap::CalDistance (DOMap.cpp:142-414) for the broad phase; i is the primary-cell object.
// Returns a negative value for an unsupported shape pair.
// pb (the Leap consultant): the difference vector takes the boundary's minimum image before its
// length, as DOMap::CalDistance does when given the boundary (DOMap.cpp:152-155, 329-332, 371-374, 402-405).
__device__ __forceinline__ double cal_distance(const ModelDev& mi_, const ModelDev& mj_, uint32_t i_, uint32_t j_,
                                               const double4_32a* __restrict__ pos, const double4_32a* __restrict__ ox,
                                               const double4_32a* __restrict__ oz, const Periodic* pb, bool& ok) {
    const ModelDev* mi = &mi_;
    const ModelDev* mj = &mj_;
    uint32_t i = i_, j = j_;
    if (mi->shape > mj->shape) {
        const ModelDev* t = mi; mi = mj; mj = t;
        uint32_t u = i; i = j; j = u;
    }
    ok = true;
    d3 pi = ld(pos, i), pj = ld(pos, j);
    if (mi->shape == SHAPE_SPHERE && mj->shape == SHAPE_SPHERE) {
        const d3 Im = sub(pi, pj);
        return len(pb ? min_image(*pb, Im) : Im);
    }
    // sphere - plate, and sphere - plate with a hole (DOMap.cpp:336-370: the hole is ignored)
    if (mi->shape == SHAPE_SPHERE && (mj->shape == SHAPE_PLATE || mj->shape == SHAPE_HOLED)) {
        d3 Oz = ld(oz, j), Ox = ld(ox, j);
        d3 Oy = cross(Oz, Ox);
        d3 Cap = sub(pi, project_on(sub(pi, pj), Oz));
        double hw = 0.5 * (mj->a0), hl = 0.5 * (mj->a2);
        double dx = dot(sub(Cap, pj), Ox);
        if (dx < -hw) dx = -hw; else if (dx > hw) dx = hw;
        double dy = dot(sub(Cap, pj), Oy);
        if (dy < -hl) dy = -hl; else if (dy > hl) dy = hl;
        d3 Caps = add(add(muls(Ox, dx), muls(Oy, dy)), pj);
        const d3 Im = sub(Caps, pi);
        return len(pb ? min_image(*pb, Im) : Im);
    }
    if (mi->shape == SHAPE_SPHERE && mj->shape == SHAPE_CYL) {
        double hh = 0.5 * (mj->a1);
        d3 ax = ld(oz, j);
        double dap = dot(sub(pi, pj), ax);
        d3 Cap = add(pj, muls(ax, dap));
        d3 Im;
        if ((dap < hh) && (dap > -hh)) Im = sub(Cap, pi);
        else if (dap >= hh) Im = sub(add(pj, muls(ax, hh)), pi);
        else Im = sub(sub(pj, muls(ax, hh)), pi);
        return len(pb ? min_image(*pb, Im) : Im);
    }
    if (mi->shape == SHAPE_SPHERE && mj->shape == SHAPE_INNER_CYL) {
        // engine extension: centre to the nearest point of the shell (within its length the
        // radial gap, beyond an end the rim circle); the boundary's minimum image is not taken
        const double hh = 0.5 * (mj->a1), R = mj->a0;
        const d3 ax = ld(oz, j);
        const d3 d = sub(pi, pj);
        const double t = dot(d, ax);
        const d3 rp = sub(d, muls(ax, t));
        if (t <= hh && t >= -hh) return fabs(R - len(rp));
        const d3 q = add(add(pj, muls(ax, t > 0.0 ? hh : -hh)), muls(dir(rp), R));
        return len(sub(q, pi));
    }
    ok = false;
    return 0.0;
}

}  // namespace vedo
