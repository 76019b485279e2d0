/*
 * dem_oracle.c - plain-C restatement of the reference DEM time step.
 *
 * TEST INFRASTRUCTURE ONLY (see dem_oracle.h): the checker for the GPU engine
 * and the CPU baseline of bench.py; never linked into the engine.
 *
 * Every routine restates one reference routine and keeps its floating-point
 * operation order, so that with FMA contraction disabled (-ffp-contract=off)
 * this code reproduces the reference's IEEE FP64 results bit for bit.  The
 * reference file:line each routine follows is given beside it; paths are
 * relative to the reference's src/ directory.
 *
 * One deliberate difference: aries::Vector3d<T>::direction() returns an
 * uninitialised vector for a zero-length input (aries/utility/Vector3d.h:
 * 117-126, `Vector3d v;` has an empty default constructor).  Every use in the
 * step multiplies that result by a zero, so the reference's output is zero
 * unless the stack garbage is non-finite; here it is defined as (0,0,0).
 */
#include "dem_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* aries::Vector3d (aries/utility/Vector3d.h)                                */
typedef struct { double x, y, z; } v3;

static v3 V3(double x, double y, double z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
static v3 ld3(const double* p) { return V3(p[0], p[1], p[2]); }
static void st3(double* p, v3 a) { p[0] = a.x; p[1] = a.y; p[2] = a.z; }
static v3 add(v3 a, v3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }          /* :255-259 */
static v3 sub(v3 a, v3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }          /* :261-265 */
static v3 smul(double s, v3 a) { return V3(s * a.x, s * a.y, s * a.z); }           /* :313-317 */
static v3 muls(v3 a, double s) { return V3(a.x * s, a.y * s, a.z * s); }           /* :267-270 */
static v3 neg(v3 a) { return V3(-a.x, -a.y, -a.z); }                               /* :307-311 */
static double dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }        /* :207-210 */
static double len(v3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }        /* :112-115 */
static v3 dir(v3 a) {                                                              /* :117-126 */
    double l = len(a);
    if (l != 0) return V3(a.x / l, a.y / l, a.z / l);
    return V3(0.0, 0.0, 0.0);
}
static v3 cross(v3 a, v3 b) {                                                      /* :222-225 */
    return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static v3 project_on(v3 a, v3 v) { return smul(dot(a, v) / len(v), dir(v)); }      /* :197-200 */
static v3 rotate_around(v3 p, v3 va) {                                             /* :152-178 */
    v3 u = dir(va);
    double a = len(va);
    double s = cos(0.5 * a);
    double t = sin(0.5 * a);
    v3 v = muls(u, t);
    v3 r = add(smul(s * s, p), smul(dot(p, v), v));
    r = add(r, smul(2.0 * s, cross(v, p)));
    return add(r, cross(v, cross(v, p)));
}

/* ------------------------------------------------------------------------ */
enum { CD_NONE = 0, CD_SS = 1, CD_SP = 2, CD_SC = 3, CD_SHP = 4, CD_SIC = 5 };
enum { IS_NONE = 0, IS_BSDBF = 1, IS_BTSDBF = 2, IS_BSDB2F = 3, IS_HERTZ = 4, IS_H = 5 };

typedef struct {
    int shape, behavior, scope, group;
    double density, dfac, range, volume, mass, sudo_model;
    v3 inertia, ext;
    double a[10];
} model_t;

typedef struct {
    int eq;           /* IS_* or IS_NONE when the equation type is unknown */
    double p[8];      /* solver constants as named in the solver constructors */
    int present[8];
} iact_t;

typedef struct {                       /* vedo::ImpactStatus (ImpactStatus.h:208-232) */
    int contact, last_contact, bond, last_bond;
    double kn, v0, overlap;
    v3 shear, point, dirn, imp_master, aimp_master;
} status_t;

typedef struct {                       /* vedo::ContactInfo (ContactDetector.h:12-25) */
    double depth;
    v3 dirn, point;
    int active, unbalance;
} cinfo_t;

typedef struct {
    unsigned slave, master;
    int cd, is;
    double c[8];                       /* solver constants after construction */
    cinfo_t ci;
    status_t st;
} iactn_t;

typedef struct {
    unsigned a, b, ord;
    status_t st;
} record_t;

struct dp_world {
    /* SystemParameter */
    double t_start, t_stop, dt, t;
    v3 g;
    double sf;
    unsigned up_iact;
    int leap;                          /* 1: LeapConsultant's candidate list, 0: NBSConsultant's */
    double zoi_lo[3], zoi_hi[3];       /* the zone of interest after Boundary::Correct */
    int zoi_sw[3], zoi_on;
    unsigned long long round;
    /* periodic boundary after Boundary::Correct: switched axes, bounds, ranges */
    int pbc_on, pbc_sw[3];
    double pbc_lo[3], pbc_hi[3], pbc_r[3];
    /* models */
    int nmodels, ngroups, niact;
    model_t* models;
    iact_t* iacts;
    int* group_iact;                   /* [ngroups*ngroups] -> iact index or -1 */
    /* objects */
    unsigned n;
    unsigned* model_of;
    double *pos, *vel, *av, *ox, *oz, *imp, *aimp;   /* DOStatus */
    double *J, *JA;                                  /* DiscreteObject accumulators */
    double* sudo;                                    /* DiscreteObject dSudoMass */
    /* candidate list (IactPairTab) and interactions (IactContainer) */
    unsigned ncand, capcand;
    unsigned *cfirst, *csecond;
    iactn_t* it;
    /* IactRecordTab */
    unsigned nrec;
    record_t* rec;
};

static void set_err(char* err, size_t len, const char* msg) {
    if (err && len) { strncpy(err, msg, len - 1); err[len - 1] = 0; }
}

static status_t status_default(void) {                     /* ImpactStatus.cpp:8-28 */
    status_t s;
    memset(&s, 0, sizeof(s));
    s.last_contact = 1;
    s.last_bond = 1;
    return s;
}
static void status_clean(status_t* s) {                      /* ImpactStatus.cpp:293-308 */
    s->last_contact = 0; s->contact = 0; s->last_bond = 0; s->bond = 0;
    s->kn = 0.0; s->v0 = 0.0; s->overlap = 0.0;
    s->shear = V3(0, 0, 0); s->point = V3(0, 0, 0); s->dirn = V3(0, 0, 0);
    s->imp_master = V3(0, 0, 0); s->aimp_master = V3(0, 0, 0);
}
static void status_clean_contact(status_t* s) {              /* ImpactStatus.cpp:281-291 */
    s->last_contact = s->contact; s->contact = 0;
    s->last_bond = s->bond; s->bond = 0;
    s->shear = V3(0, 0, 0); s->imp_master = V3(0, 0, 0); s->aimp_master = V3(0, 0, 0);
}

/* ------------------------------------------------------------------------ */
/* Boundary::DifferenceBoundaryConditions (vedo/framework/Boundary.cpp:306-345): the minimum
   image of a difference on every switched axis */
static v3 min_image(const dp_world* w, v3 d) {
    double c[3] = {d.x, d.y, d.z};
    for (int k = 0; k < 3; ++k) {
        if (!w->pbc_sw[k]) continue;
        if (c[k] >= 0.5 * w->pbc_r[k]) c[k] -= w->pbc_r[k];
        if (c[k] < -0.5 * w->pbc_r[k]) c[k] += w->pbc_r[k];
    }
    return V3(c[0], c[1], c[2]);
}

/* Boundary::EnforceBoundaryConditions (Boundary.cpp:225-304): a position on a switched axis
   is brought back into [lower, upper), one range at a time and by fmod beyond that */
static void wrap_position(const dp_world* w, double* p) {
    for (int k = 0; k < 3; ++k) {
        if (!w->pbc_sw[k]) continue;
        const double lo = w->pbc_lo[k], hi = w->pbc_hi[k], r = w->pbc_r[k];
        double x = p[k];
        if (x >= hi) {
            x -= r;
            if (x >= hi) x = lo + fmod(x - lo, r);
        }
        if (x < lo) {
            x += r;
            if (x < lo) x = lo + fmod(x - lo, r) + r;
        }
        p[k] = x;
    }
}

/* ------------------------------------------------------------------------ */
/* DOModel::Analysis (vedo/framework/DOModel.cpp:17-149) */
static int analyse(model_t* m) {
    const double PI = 4.0 * atan(1.0);
    const double FTPI = 4.0 / 3.0 * PI;
    double r, w, h, l, mmi;
    switch (m->shape) {
    case VEDO_SHAPE_SPHERE:
        r = m->a[0];
        m->range = r;
        m->volume = FTPI * r * r * r;
        m->mass = m->density * m->volume;
        m->sudo_model = m->dfac * m->mass;
        mmi = 0.4 * m->mass * r * r;
        m->inertia = V3(mmi, mmi, mmi);
        return 1;
    case VEDO_SHAPE_QUASI_CYLINDER:
        r = m->a[0]; h = m->a[1];
        if (m->scope == VEDO_SCOPE_LOCAL) m->range = (r > 0.5 * h) ? r : 0.5 * h;
        else m->range = r;
        m->volume = PI * r * r * h;
        m->mass = m->density * m->volume;
        m->sudo_model = m->dfac * m->mass;
        mmi = m->mass * (3.0 * r * r + h * h) / 12.0;
        m->inertia = V3(mmi, mmi, 0.5 * m->mass * r * r);
        return 1;
    case VEDO_SHAPE_QUASI_PLATE: {
        w = m->a[0]; h = m->a[1]; l = m->a[2];
        if (m->scope == VEDO_SCOPE_LOCAL) {
            double mx = (w > h) ? w : h;
            mx = (mx > l) ? mx : l;
            m->range = 0.5 * mx;
        } else {
            m->range = 0.5 * h;
        }
        m->volume = w * h * l;
        m->mass = m->density * m->volume;
        m->sudo_model = m->dfac * m->mass;
        double k = m->mass / 12.0;
        m->inertia = smul(k, V3(h * h + l * l, w * w + l * l, h * h + w * w));
        return 1;
    }
    case VEDO_SHAPE_QUASI_PLATE_WITH_CIRCULAR_HOLE: {      /* DOModel.cpp:90-119 */
        w = m->a[0]; h = m->a[1]; l = m->a[2];
        const double hr = m->a[3], hxo = m->a[4], hyo = m->a[5];
        if (m->scope == VEDO_SCOPE_LOCAL) {
            double mx = (w > h) ? w : h;
            mx = (mx > l) ? mx : l;
            m->range = 0.5 * mx;
        } else {
            m->range = 0.5 * h;
        }
        if (!((fabs(hxo) <= (0.5 * w - hr)) && (fabs(hyo) <= (0.5 * l - hr)))) return 0;   /* the reference exits */
        m->volume = w * h * l - hr * hr * PI * h;
        m->mass = m->density * m->volume;
        m->sudo_model = m->dfac * m->mass;
        m->inertia = V3(0.0, 0.0, 0.0);
        return 1;
    }
    case VEDO_SHAPE_INNER_CYLINDER:
        /* No counterpart in the reference (an extension the engine defines): the inside of a
         * hollow cylinder, a shell of no thickness and no mass, global scope only. */
        if (m->scope != VEDO_SCOPE_GLOBAL || !(m->a[0] > 0.0) || !(m->a[1] > 0.0)) return 0;
        m->range = 0.0;
        m->volume = 0.0;
        m->mass = 0.0;
        m->sudo_model = 0.0;
        m->inertia = V3(0.0, 0.0, 0.0);
        return 1;
    default:
        return 0;
    }
}

/* dSudoMass of the DiscreteObject subclass chosen by DOcf<>(shape, behaviour)
 * (ModuleList.h:46-57): DOSphere.cpp:17, DOFixedSphere.cpp, DOFixedQuasiPlate.cpp:14,
 * DOOrbitalQuasiPlate.cpp:14, DOConstrainedQuasiPlate.cpp:14, DOQuasiPlate.cpp:14, and
 * the cylinder counterparts.  Returns -1 when no factory exists. */
static int object_sudo_mass(const model_t* m, double* out) {
    if (m->shape == VEDO_SHAPE_SPHERE) {
        if (m->behavior == VEDO_MOBILE || m->behavior == VEDO_FIXED) { *out = m->sudo_model; return 0; }
        return -1;
    }
    if (m->shape == VEDO_SHAPE_QUASI_PLATE_WITH_CIRCULAR_HOLE) {   /* DOFixedQuasiPlateWithCircularHole.cpp:16-19 */
        if (m->behavior == VEDO_FIXED) { *out = 0.0; return 0; }
        return -1;           /* the mobile one (DOQuasiPlateWithCircularHole) is not restated */
    }
    if (m->shape == VEDO_SHAPE_INNER_CYLINDER) {               /* the engine's extension: fixed or orbital */
        if (m->behavior == VEDO_FIXED || m->behavior == VEDO_ORBITAL) { *out = 0.0; return 0; }
        return -1;
    }
    if (m->shape == VEDO_SHAPE_QUASI_PLATE || m->shape == VEDO_SHAPE_QUASI_CYLINDER) {
        switch (m->behavior) {
        case VEDO_FIXED: case VEDO_ORBITAL: *out = 0.0; return 0;
        case VEDO_CONSTRAINED: *out = m->sudo_model; return 0;
        case VEDO_MOBILE: *out = m->mass; return 0;
        default: return -1;
        }
    }
    return -1;
}

/* ------------------------------------------------------------------------ */
/* Solver constants, as the ISw* constructors read them */
static const char* MECH_NAMES[6][8] = {
    {0},
    {"NormalStiffness", "ShearStiffness", "NormalDampingRatio", "ShearDampingRatio", "NormalBondStrength",
     "ShearBondStrength", "FrictionCoefficient", 0},                                  /* ISwBSDBF.cpp:10-18 */
    {"NormalStiffness", "ShearStiffness", "NormalDampingRatio", "ShearDampingRatio", "NormalBondStrength",
     "ShearBondStrength", "FrictionCoefficient", 0},                                  /* ISwBtSDBF.cpp:10-18 */
    {"NormalStiffness", "ShearStiffness", "NormalDampingRatio", "ShearDampingRatio", "NormalBondStrength",
     "ShearBondStrength", "FrictionCoefficient", 0},                                  /* ISwBSDB2F.cpp */
    {"NormalStiffness", "NormalDampingCoefficient", 0},                               /* ISwHertz.cpp:11-12 */
    {"HertzNormalStiffness", "EquivalentMass", "ShearStiffnessCoefficient1", "ShearStiffnessCoefficient2",
     "DampingRatio", "KineticFrictionCoefficient", 0},                                /* ISwH.cpp:8-19 */
};

static int eq_of(const char* s) {                  /* IScf<IS>("name"), ModuleList.h:59-63 */
    if (!strcmp(s, "ISwBSDBF")) return IS_BSDBF;
    if (!strcmp(s, "ISwBtSDBF")) return IS_BTSDBF;
    if (!strcmp(s, "ISwBSDB2F")) return IS_BSDB2F;
    if (!strcmp(s, "ISwHertz")) return IS_HERTZ;
    if (!strcmp(s, "ISwH")) return IS_H;
    return IS_NONE;
}

/* ------------------------------------------------------------------------ */
/* DOMap::CalDistance (vedo/framework/DOMap.cpp:142-414).  With `periodic` (the Leap consultant
   passes the boundary) the difference vector takes the minimum image before its length. */
static int cal_distance_pbc(const dp_world* w, unsigned i, unsigned j, int periodic, double* out) {
    const model_t* mi = &w->models[w->model_of[i]];
    const model_t* mj = &w->models[w->model_of[j]];
    if (mi->shape > mj->shape) {                    /* :144-147 swap */
        unsigned t = i; i = j; j = t;
        const model_t* tm = mi; mi = mj; mj = tm;
    }
    v3 pi = ld3(w->pos + 3 * i), pj = ld3(w->pos + 3 * j);
    if (mi->shape == VEDO_SHAPE_SPHERE && mj->shape == VEDO_SHAPE_SPHERE) {          /* :149-157 */
        v3 Im = sub(pi, pj);
        if (periodic) Im = min_image(w, Im);
        *out = len(Im);
        return 0;
    }
    if (mi->shape == VEDO_SHAPE_SPHERE && (mj->shape == VEDO_SHAPE_QUASI_PLATE ||
                                           mj->shape == VEDO_SHAPE_QUASI_PLATE_WITH_CIRCULAR_HOLE)) {   /* :294-370 */
        v3 Ca = pi, Cb = pj, Oz = ld3(w->oz + 3 * j), Ox = ld3(w->ox + 3 * j);
        v3 Oy = cross(Oz, Ox);
        v3 Cap = sub(Ca, project_on(sub(Ca, Cb), Oz));
        double hw = 0.5 * (mj->a[0]);
        double hl = 0.5 * (mj->a[2]);
        double dx = dot(sub(Cap, Cb), Ox);
        if (dx < -hw) dx = -hw; else if (dx > hw) dx = hw;
        double dy = dot(sub(Cap, Cb), Oy);
        if (dy < -hl) dy = -hl; else if (dy > hl) dy = hl;
        v3 Caps = add(add(muls(Ox, dx), muls(Oy, dy)), Cb);
        v3 Im = sub(Caps, Ca);
        if (periodic) Im = min_image(w, Im);
        *out = len(Im);
        return 0;
    }
    if (mi->shape == VEDO_SHAPE_SPHERE && mj->shape == VEDO_SHAPE_QUASI_CYLINDER) {  /* :378-408 */
        double hh = 0.5 * (mj->a[1]);
        v3 Ca = pi, Cb = pj, ax = ld3(w->oz + 3 * j);
        double dap = dot(sub(Ca, Cb), ax);
        v3 Cap = add(Cb, muls(ax, dap));
        v3 Im;
        if ((dap < hh) && (dap > -hh)) Im = sub(Cap, Ca);
        else if (dap >= hh) Im = sub(add(Cb, muls(ax, hh)), Ca);
        else Im = sub(sub(Cb, muls(ax, hh)), Ca);
        if (periodic) Im = min_image(w, Im);
        *out = len(Im);
        return 0;
    }
    if (mi->shape == VEDO_SHAPE_SPHERE && mj->shape == VEDO_SHAPE_INNER_CYLINDER) {
        /* the engine's extension: centre to the nearest point of the shell (within its length
         * the radial gap, beyond an end the rim circle); no minimum image */
        const double hh = 0.5 * (mj->a[1]), R = mj->a[0];
        v3 ax = ld3(w->oz + 3 * j);
        v3 d = sub(pi, pj);
        double t = dot(d, ax);
        v3 rp = sub(d, muls(ax, t));
        if (t <= hh && t >= -hh) { *out = fabs(R - len(rp)); return 0; }
        v3 q = add(add(pj, muls(ax, t > 0.0 ? hh : -hh)), muls(dir(rp), R));
        *out = len(sub(q, pi));
        return 0;
    }
    return -1;                                       /* :410-413 exit(-1) in the reference */
}

static int cal_distance(const dp_world* w, unsigned i, unsigned j, double* out) {
    return cal_distance_pbc(w, i, j, 0, out);
}

/* ------------------------------------------------------------------------ */
/* NBSConsultant::Reset + BuildIactTab (vedo/common/NBSConsultant.cpp:85-374) */
typedef struct { unsigned cx, cy, cz, id; } cellent_t;

static int cell_cmp(const void* a, const void* b) {
    const cellent_t* x = (const cellent_t*)a;
    const cellent_t* y = (const cellent_t*)b;
    if (x->cx != y->cx) return x->cx < y->cx ? -1 : 1;
    if (x->cy != y->cy) return x->cy < y->cy ? -1 : 1;
    if (x->cz != y->cz) return x->cz < y->cz ? -1 : 1;
    if (x->id != y->id) return x->id < y->id ? -1 : 1;
    return 0;
}

static int push_cand(dp_world* w, unsigned a, unsigned b) {
    if (w->ncand == w->capcand) {
        unsigned nc = w->capcand ? 2 * w->capcand : 1024;
        unsigned* f = (unsigned*)realloc(w->cfirst, sizeof(unsigned) * nc);
        unsigned* s = (unsigned*)realloc(w->csecond, sizeof(unsigned) * nc);
        if (!f || !s) return -1;
        w->cfirst = f; w->csecond = s; w->capcand = nc;
    }
    w->cfirst[w->ncand] = a < b ? a : b;
    w->csecond[w->ncand] = a < b ? b : a;
    w->ncand++;
    return 0;
}

static int build_tab_pbc(dp_world* w, const unsigned* v1, unsigned n1, const unsigned* v2, unsigned n2,
                         int self, const double* safe, int periodic) {     /* :318-374 */
    for (unsigned i = 0; i < n1; ++i) {
        for (unsigned j = self ? i + 1 : 0; j < n2; ++j) {
            unsigned a = v1[i], b = v2[j];
            int ga = w->models[w->model_of[a]].group, gb = w->models[w->model_of[b]].group;
            if (w->group_iact[ga * w->ngroups + gb] < 0) continue;
            double d;
            if (cal_distance_pbc(w, a, b, periodic, &d) != 0) return -2;
            if (d > (safe[a] + safe[b])) continue;
            if (push_cand(w, a, b) != 0) return -1;
        }
    }
    return 0;
}

static int build_tab(dp_world* w, const unsigned* v1, unsigned n1, const unsigned* v2, unsigned n2,
                     int self, const double* safe) {
    return build_tab_pbc(w, v1, n1, v2, n2, self, safe, 0);
}

static unsigned lookup_cell(const cellent_t* ents, const unsigned* starts, unsigned ncells, unsigned cx,
                            unsigned cy, unsigned cz, unsigned* cnt) {
    /* binary search over the distinct cells (starts[] index into ents) */
    unsigned lo = 0, hi = ncells;
    while (lo < hi) {
        unsigned mid = (lo + hi) / 2;
        const cellent_t* e = &ents[starts[mid]];
        int c;
        if (e->cx != cx) c = e->cx < cx ? -1 : 1;
        else if (e->cy != cy) c = e->cy < cy ? -1 : 1;
        else if (e->cz != cz) c = e->cz < cz ? -1 : 1;
        else c = 0;
        if (c == 0) { *cnt = starts[mid + 1] - starts[mid]; return starts[mid]; }
        if (c < 0) lo = mid + 1; else hi = mid;
    }
    *cnt = 0;
    return 0;
}

static int nbs_reset(dp_world* w) {
    unsigned n = w->n;
    double dtu = (double)w->up_iact * w->dt;                                 /* :99 */
    double glen = len(w->g);
    double* safe = (double*)malloc(sizeof(double) * (n ? n : 1));
    unsigned* glob = (unsigned*)malloc(sizeof(unsigned) * (n ? n : 1));
    cellent_t* ents = (cellent_t*)malloc(sizeof(cellent_t) * (n ? n : 1));
    unsigned* ids = (unsigned*)malloc(sizeof(unsigned) * (n ? n : 1));
    unsigned* starts = (unsigned*)malloc(sizeof(unsigned) * (n + 1));
    if (!safe || !glob || !ents || !ids || !starts) return -1;
    const double DMAX = 1.7976931348623157e308, DMIN = 2.2250738585072014e-308;
    double xmin = DMAX, xmax = DMIN, ymin = DMAX, ymax = DMIN, zmin = DMAX, zmax = DMIN;  /* :106-111 */
    double vmax = 0.0, rmax = 0.0;
    unsigned nglob = 0, nloc = 0;
    for (unsigned u = 0; u < n; ++u) {                                       /* :120-144 */
        const model_t* m = &w->models[w->model_of[u]];
        double vl = len(ld3(w->vel + 3 * u));
        safe[u] = w->sf * (2.0 * m->range + dtu * vl + 0.5 * dtu * dtu * glen);
        if (m->scope == VEDO_SCOPE_LOCAL) {
            const double* p = w->pos + 3 * u;
            xmin = xmin < p[0] ? xmin : p[0]; xmax = xmax > p[0] ? xmax : p[0];
            ymin = ymin < p[1] ? ymin : p[1]; ymax = ymax > p[1] ? ymax : p[1];
            zmin = zmin < p[2] ? zmin : p[2]; zmax = zmax > p[2] ? zmax : p[2];
            vmax = vmax > vl ? vmax : vl;
            rmax = m->range;                                                 /* :140 last local DO */
        }
    }
    double zone = w->sf * (2.0 * rmax + dtu * vmax + 0.5 * dtu * dtu * glen);   /* :146 */
    unsigned ncx = (unsigned)ceil((xmax - xmin) / zone); if (ncx < 1) ncx = 1;  /* :148-153 */
    unsigned ncy = (unsigned)ceil((ymax - ymin) / zone); if (ncy < 1) ncy = 1;
    unsigned ncz = (unsigned)ceil((zmax - zmin) / zone); if (ncz < 1) ncz = 1;
    for (unsigned u = 0; u < n; ++u) {                                       /* :163-183 */
        const model_t* m = &w->models[w->model_of[u]];
        if (m->scope == VEDO_SCOPE_LOCAL) {
            const double* p = w->pos + 3 * u;
            cellent_t e;
            e.cx = (unsigned)((p[0] - xmin) / zone);
            e.cy = (unsigned)((p[1] - ymin) / zone);
            e.cz = (unsigned)((p[2] - zmin) / zone);
            e.id = u;
            ents[nloc++] = e;
        } else {
            glob[nglob++] = u;
        }
    }
    qsort(ents, nloc, sizeof(cellent_t), cell_cmp);
    unsigned ncells = 0;
    for (unsigned k = 0; k < nloc; ++k) {
        ids[k] = ents[k].id;
        if (k == 0 || ents[k].cx != ents[k - 1].cx || ents[k].cy != ents[k - 1].cy || ents[k].cz != ents[k - 1].cz)
            starts[ncells++] = k;
    }
    starts[ncells] = nloc;
    w->ncand = 0;
    /* neighbour visiting order of :202-270 (offsets dx, dy, dz), with 100 = self and 101 = globals */
    static const int ORDER[15][3] = {
        {-1, -1, -1}, {-1, -1, 0}, {-1, -1, 1}, {0, -1, -1}, {0, -1, 0}, {0, -1, 1}, {1, -1, -1}, {1, -1, 0},
        {1, -1, 1}, {-1, 0, -1}, {-1, 0, 0}, {0, 0, -1}, {100, 0, 0}, {101, 0, 0}, {1, 0, -1}};
    int rc = 0;
    for (unsigned c = 0; c < ncells && rc == 0; ++c) {
        const cellent_t* e = &ents[starts[c]];
        if (e->cx >= ncx || e->cy >= ncy || e->cz >= ncz) continue;     /* only cells inside the loops are primary */
        const unsigned* v1 = ids + starts[c];
        unsigned n1 = starts[c + 1] - starts[c];
        for (int s = 0; s < 15 && rc == 0; ++s) {
            if (ORDER[s][0] == 100) { rc = build_tab(w, v1, n1, v1, n1, 1, safe); continue; }
            if (ORDER[s][0] == 101) { rc = build_tab(w, v1, n1, glob, nglob, 0, safe); continue; }
            unsigned cnt;
            unsigned st = lookup_cell(ents, starts, ncells, e->cx + (unsigned)ORDER[s][0],
                                      e->cy + (unsigned)ORDER[s][1], e->cz + (unsigned)ORDER[s][2], &cnt);
            if (cnt) rc = build_tab(w, v1, n1, ids + st, cnt, 0, safe);
        }
    }
    free(safe); free(glob); free(ents); free(ids); free(starts);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* LeapConsultant::Reset + subReset (vedo/common/LeapConsultant.cpp:108-195, LeapConsultant.h:58-446).
   The cell edge comes from the largest range and speed of the local objects; cells are visited
   in the order of a comparator whose first key is the axis with the largest 2 %-98 % spread of
   the local positions (TrirLeX/Y/Z, NBSConsultant.h:62-128); per cell the 13 half-shell
   neighbours (each, when absent, replaced by its periodic image under the rule of
   LeapConsultant.h:195-446), then the cell itself, then the scope-global objects; the candidate
   distance takes the boundary's minimum image. */
static int dcmp(const void* a, const void* b) {
    double x = *(const double*)a, y = *(const double*)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

static int g_leap_mode;                              /* comparator for qsort: 0 X, 1 Y, 2 Z */
static void leap_keys(const cellent_t* e, unsigned k[3]) {
    if (g_leap_mode == 0) { k[0] = e->cx; k[1] = e->cy; k[2] = e->cz; }       /* TrirLeX */
    else if (g_leap_mode == 1) { k[0] = e->cy; k[1] = e->cx; k[2] = e->cz; }  /* TrirLeY */
    else { k[0] = e->cz; k[1] = e->cx; k[2] = e->cy; }                         /* TrirLeZ */
}
static int leap_cmp(const void* a, const void* b) {
    unsigned ka[3], kb[3];
    leap_keys((const cellent_t*)a, ka);
    leap_keys((const cellent_t*)b, kb);
    for (int q = 0; q < 3; ++q)
        if (ka[q] != kb[q]) return ka[q] < kb[q] ? -1 : 1;
    unsigned ia = ((const cellent_t*)a)->id, ib = ((const cellent_t*)b)->id;   /* insertion order */
    return ia < ib ? -1 : (ia > ib ? 1 : 0);
}
static unsigned leap_lookup(const cellent_t* ents, const unsigned* starts, unsigned ncells, unsigned cx, unsigned cy,
                            unsigned cz, unsigned* cnt) {
    cellent_t probe;
    probe.cx = cx; probe.cy = cy; probe.cz = cz; probe.id = 0;
    unsigned kp[3];
    leap_keys(&probe, kp);
    unsigned lo = 0, hi = ncells;
    while (lo < hi) {
        unsigned mid = (lo + hi) / 2;
        unsigned km[3];
        leap_keys(&ents[starts[mid]], km);
        int c = 0;
        for (int q = 0; q < 3 && c == 0; ++q)
            if (km[q] != kp[q]) c = km[q] < kp[q] ? -1 : 1;
        if (c == 0) { *cnt = starts[mid + 1] - starts[mid]; return starts[mid]; }
        if (c < 0) lo = mid + 1; else hi = mid;
    }
    *cnt = 0;
    return 0;
}

static int leap_reset(dp_world* w) {
    unsigned n = w->n;
    unsigned nl = 0;
    for (unsigned u = 0; u < n; ++u) nl += w->models[w->model_of[u]].scope == VEDO_SCOPE_LOCAL;
    if (nl == 0) return -3;                          /* the reference indexes an empty vector */
    double* sx = (double*)malloc(sizeof(double) * nl * 5);
    double* safe = (double*)malloc(sizeof(double) * (n ? n : 1));
    unsigned* glob = (unsigned*)malloc(sizeof(unsigned) * (n ? n : 1));
    cellent_t* ents = (cellent_t*)malloc(sizeof(cellent_t) * nl);
    unsigned* ids = (unsigned*)malloc(sizeof(unsigned) * nl);
    unsigned* starts = (unsigned*)malloc(sizeof(unsigned) * (nl + 1));
    if (!sx || !safe || !glob || !ents || !ids || !starts) return -1;
    double *sy = sx + nl, *sz = sx + 2 * nl, *sv = sx + 3 * nl, *sr = sx + 4 * nl;
    unsigned k = 0;
    for (unsigned u = 0; u < n; ++u) {                                       /* LeapConsultant.cpp:122-136 */
        const model_t* m = &w->models[w->model_of[u]];
        if (m->scope != VEDO_SCOPE_LOCAL) continue;
        sx[k] = w->pos[3 * u]; sy[k] = w->pos[3 * u + 1]; sz[k] = w->pos[3 * u + 2];
        sv[k] = len(ld3(w->vel + 3 * u)); sr[k] = m->range;
        ++k;
    }
    qsort(sx, nl, sizeof(double), dcmp); qsort(sy, nl, sizeof(double), dcmp); qsort(sz, nl, sizeof(double), dcmp);
    qsort(sv, nl, sizeof(double), dcmp); qsort(sr, nl, sizeof(double), dcmp);
    const double xmin = sx[0], xmax = sx[nl - 1], ymin = sy[0], ymax = sy[nl - 1], zmin = sz[0], zmax = sz[nl - 1];
    const double vmax = sv[nl - 1], rmax = sr[nl - 1];
    const double discard = 0.02, keep = 1.0 - discard;                        /* :164-168 */
    const double hi_d = keep * nl - 1, lo_d = discard * nl;
    const size_t ih = hi_d < 0.0 ? 0 : (size_t)hi_d, il = (size_t)lo_d;
    const double xs = sx[ih] - sx[il], ys = sy[ih] - sy[il], zs = sz[ih] - sz[il];
    g_leap_mode = xs >= ys ? (xs >= zs ? 0 : 2) : (ys >= zs ? 1 : 2);         /* :170-193 */
    double dtu = (double)w->up_iact * w->dt;                                  /* LeapConsultant.h:73 */
    double glen = len(w->g);
    for (unsigned u = 0; u < n; ++u) {                                        /* :116-136 */
        const model_t* m = &w->models[w->model_of[u]];
        safe[u] = w->sf * (2.0 * m->range + dtu * len(ld3(w->vel + 3 * u)) + 0.5 * dtu * dtu * glen);
    }
    double zone = w->sf * (2.0 * rmax + dtu * vmax + 0.5 * dtu * dtu * glen); /* :138 */
    unsigned ncx = (unsigned)ceil((xmax - xmin) / zone); if (ncx < 1) ncx = 1;
    unsigned ncy = (unsigned)ceil((ymax - ymin) / zone); if (ncy < 1) ncy = 1;
    unsigned ncz = (unsigned)ceil((zmax - zmin) / zone); if (ncz < 1) ncz = 1;
    const int px = w->pbc_sw[0] && (xmax - xmin) >= 0.5 * w->pbc_r[0];      /* :146-150 */
    const int py = w->pbc_sw[1] && (ymax - ymin) >= 0.5 * w->pbc_r[1];
    const int pz = w->pbc_sw[2] && (zmax - zmin) >= 0.5 * w->pbc_r[2];
    const int has_pbc = px || py || pz;
    const unsigned mx[3] = {ncx - 1, ncy - 1, ncz - 1};
    const int pa[3] = {px, py, pz};
    unsigned nloc = 0, nglob = 0;
    for (unsigned u = 0; u < n; ++u) {                                        /* :160-179 */
        const model_t* m = &w->models[w->model_of[u]];
        if (m->scope == VEDO_SCOPE_LOCAL) {
            const double* p = w->pos + 3 * u;
            cellent_t e;
            e.cx = (unsigned)((p[0] - xmin) / zone);
            e.cy = (unsigned)((p[1] - ymin) / zone);
            e.cz = (unsigned)((p[2] - zmin) / zone);
            e.id = u;
            ents[nloc++] = e;
        } else {
            glob[nglob++] = u;
        }
    }
    qsort(ents, nloc, sizeof(cellent_t), leap_cmp);
    unsigned ncells = 0;
    for (unsigned q = 0; q < nloc; ++q) {
        ids[q] = ents[q].id;
        if (q == 0 || ents[q].cx != ents[q - 1].cx || ents[q].cy != ents[q - 1].cy || ents[q].cz != ents[q - 1].cz)
            starts[ncells++] = q;
    }
    starts[ncells] = nloc;
    w->ncand = 0;
    static const int OFF[13][3] = {                                           /* :195-440 */
        {-1, -1, -1}, {-1, -1, 0}, {-1, -1, 1}, {0, -1, -1}, {0, -1, 0}, {0, -1, 1}, {1, -1, -1}, {1, -1, 0},
        {1, -1, 1}, {-1, 0, -1}, {-1, 0, 0}, {0, 0, -1}, {1, 0, -1}};
    int rc = 0;
    for (unsigned c = 0; c < ncells && rc == 0; ++c) {
        const cellent_t* e = &ents[starts[c]];
        const unsigned ic[3] = {e->cx, e->cy, e->cz};
        const unsigned* v1 = ids + starts[c];
        unsigned n1 = starts[c + 1] - starts[c];
        for (int s = 0; s < 13 && rc == 0; ++s) {
            unsigned nb[3];
            for (int a = 0; a < 3; ++a) nb[a] = ic[a] + (unsigned)OFF[s][a];   /* unsigned, as _uint_t */
            unsigned cnt, st = leap_lookup(ents, starts, ncells, nb[0], nb[1], nb[2], &cnt);
            if (cnt) { rc = build_tab_pbc(w, v1, n1, ids + st, cnt, 0, safe, w->pbc_on); continue; }
            if (!has_pbc) continue;
            /* the periodic image: on an axis stepping down from zone 0 (up from the last zone)
               the neighbour wraps when that axis is periodic; a wrapped id that names the
               opposite neighbour is skipped (:199-216 and the twelve branches that follow) */
            int at_edge = 0, dup = 0;
            unsigned wi[3];
            for (int a = 0; a < 3; ++a) {
                if (OFF[s][a] < 0) {
                    at_edge |= ic[a] == 0;
                    wi[a] = pa[a] ? mx[a] : ic[a] - 1u;
                    dup |= wi[a] == ic[a] + 1u;
                } else if (OFF[s][a] > 0) {
                    at_edge |= ic[a] == mx[a];
                    wi[a] = pa[a] ? 0u : ic[a] + 1u;
                    dup |= wi[a] == ic[a] - 1u;
                } else {
                    wi[a] = ic[a];
                }
            }
            if (!at_edge || dup) continue;
            st = leap_lookup(ents, starts, ncells, wi[0], wi[1], wi[2], &cnt);
            if (cnt) rc = build_tab_pbc(w, v1, n1, ids + st, cnt, 0, safe, w->pbc_on);
        }
        if (rc == 0) rc = build_tab_pbc(w, v1, n1, v1, n1, 1, safe, w->pbc_on);          /* :442-443 */
        if (rc == 0) rc = build_tab_pbc(w, v1, n1, glob, nglob, 0, safe, w->pbc_on);     /* :445-446 */
    }
    free(sx); free(safe); free(glob); free(ents); free(ids); free(starts);
    return rc;
}

static int consultant_reset(dp_world* w) { return w->leap ? leap_reset(w) : nbs_reset(w); }

/* ------------------------------------------------------------------------ */
/* Assembler::CreateInteraction (vedo/framework/Assembler.cpp:15-87) with the
 * CDcf list match (CDFactory.h:66-95; every detector is registered with the list
 * of all five equation types, ModuleList.h:65-69) and the exact IScf match. */
static int create_interaction(const dp_world* w, unsigned p1, unsigned p2, iactn_t* out) {
    const model_t* m1 = &w->models[w->model_of[p1]];
    const model_t* m2 = &w->models[w->model_of[p2]];
    int ia = w->group_iact[m1->group * w->ngroups + m2->group];
    if (ia < 0) return 1;
    if (p1 == p2) return 1;
    if (m2->density < 0.0 || m1->density < 0.0) return 1;
    if (m2->density == 0.0 && m1->density == 0.0) return 1;
    unsigned sl, ma;
    if (m1->shape > m2->shape) { sl = p2; ma = p1; }
    else if (m1->shape < m2->shape) { sl = p1; ma = p2; }
    else if (m1->density == 0.0) { sl = p2; ma = p1; }
    else if (m2->density == 0.0) { sl = p1; ma = p2; }
    else { sl = p1; ma = p2; }
    const model_t* ms = &w->models[w->model_of[sl]];
    const model_t* mm = &w->models[w->model_of[ma]];
    int cd = CD_NONE;
    if (ms->shape == VEDO_SHAPE_SPHERE && mm->shape == VEDO_SHAPE_SPHERE) cd = CD_SS;
    else if (ms->shape == VEDO_SHAPE_SPHERE && mm->shape == VEDO_SHAPE_QUASI_PLATE) cd = CD_SP;
    else if (ms->shape == VEDO_SHAPE_SPHERE && mm->shape == VEDO_SHAPE_QUASI_CYLINDER) cd = CD_SC;
    else if (ms->shape == VEDO_SHAPE_SPHERE && mm->shape == VEDO_SHAPE_QUASI_PLATE_WITH_CIRCULAR_HOLE) cd = CD_SHP;
    else if (ms->shape == VEDO_SHAPE_SPHERE && mm->shape == VEDO_SHAPE_INNER_CYLINDER) cd = CD_SIC;   /* extension */
    const iact_t* im = &w->iacts[ia];
    if (cd == CD_NONE || im->eq == IS_NONE) return 2;
    for (int k = 0; MECH_NAMES[im->eq][k]; ++k)
        if (!im->present[k]) return 3;       /* IactModel::GetIactMechanism exits (IactModel.cpp:69-90) */
    memset(out, 0, sizeof(*out));
    out->slave = sl;
    out->master = ma;
    out->cd = cd;
    out->is = im->eq;
    if (im->eq == IS_BSDBF || im->eq == IS_BTSDBF || im->eq == IS_BSDB2F) {
        /* ISwBSDBF.cpp:7-19 with ISwModels::CriticalDamping (ISwModels.cpp:88-108) */
        double kn = im->p[0], ks = im->p[1];
        double Ma = w->sudo[sl], Mb = w->sudo[ma], Me;
        if (Mb == 0) Me = Ma; else if (Ma == 0) Me = Mb; else Me = 0.5 * (Ma + Mb);
        double c1 = 2.0 * sqrt(Me * kn), c2 = 2.0 * sqrt(Me * ks);
        out->c[0] = kn;
        out->c[1] = ks;
        out->c[2] = (im->p[2]) * c1;   /* cn */
        out->c[3] = (im->p[3]) * c2;   /* cs */
        out->c[4] = im->p[4];          /* bn */
        out->c[5] = im->p[5];          /* bs */
        out->c[6] = im->p[6];          /* fc */
    } else {
        for (int k = 0; k < 8; ++k) out->c[k] = im->p[k];
    }
    out->st = status_default();
    return 0;
}

/* ContactDetector::Detect for the three supported shape pairs */
static void detect(const dp_world* w, iactn_t* I) {
    unsigned s = I->slave, m = I->master;
    const model_t* ms = &w->models[w->model_of[s]];
    const model_t* mm = &w->models[w->model_of[m]];
    v3 Ps = ld3(w->pos + 3 * s), Pm = ld3(w->pos + 3 * m);
    double ra = ms->a[0];
    cinfo_t* ci = &I->ci;
    if (I->cd == CD_SS) {                                    /* CDSphere2Sphere.cpp:14-60 */
        v3 vIm = sub(Pm, Ps);
        if (w->pbc_on) vIm = min_image(w, vIm);              /* :19-22, pBC set when active */
        double rb = mm->a[0];
        ci->depth = ra + rb - len(vIm);
        ci->dirn = dir(vIm);
    } else if (I->cd == CD_SP) {                             /* CDSphere2QuasiPlate.cpp:15-97 */
        v3 Oz = ld3(w->oz + 3 * m), Ox = ld3(w->ox + 3 * m);
        v3 Oy = cross(Oz, Ox);
        v3 Cap = sub(Ps, project_on(sub(Ps, Pm), Oz));
        double hh = 0.5 * mm->a[1], hw = 0.5 * mm->a[0], hl = 0.5 * mm->a[2];
        double dx = dot(sub(Cap, Pm), Ox);
        if (dx < -hw) dx = -hw; else if (dx > hw) dx = hw;
        double dy = dot(sub(Cap, Pm), Oy);
        if (dy < -hl) dy = -hl; else if (dy > hl) dy = hl;
        v3 Caps = add(add(muls(Ox, dx), muls(Oy, dy)), Pm);
        v3 vIm = sub(Caps, Ps);
        ci->depth = ra + hh - len(vIm);
        ci->dirn = dir(vIm);
    } else if (I->cd == CD_SHP) {                            /* CDSphere2QuasiPlateWithCircularHole.cpp:15-133 */
        v3 Oz = ld3(w->oz + 3 * m), Ox = ld3(w->ox + 3 * m);
        v3 Oy = cross(Oz, Ox);
        v3 Cap = sub(Ps, project_on(sub(Ps, Pm), Oz));
        double hh = 0.5 * mm->a[1], hw = 0.5 * mm->a[0], hl = 0.5 * mm->a[2];
        double hr = mm->a[3], hxo = mm->a[4], hyo = mm->a[5];
        v3 Ch = add(Pm, V3(hxo, hyo, 0.0));          /* world-frame offsets, as the reference adds them */
        v3 Cha = sub(Ps, Ch);
        double dx = dot(sub(Cap, Pm), Ox);
        if (dx < -hw) dx = -hw; else if (dx > hw) dx = hw;
        double dy = dot(sub(Cap, Pm), Oy);
        if (dy < -hl) dy = -hl; else if (dy > hl) dy = hl;
        double dahx = dot(Cha, Ox), dahy = dot(Cha, Oy);
        double dah = sqrt(dahx * dahx + dahy * dahy);
        if (dah < hr) {
            if (dah == 0.0) { dx = hxo; dy = hyo; }
            else { dx = hxo + dahx / dah * hr; dy = hyo + dahy / dah * hr; }
        }
        v3 Caps = add(add(muls(Ox, dx), muls(Oy, dy)), Pm);
        v3 vIm = sub(Caps, Ps);
        if (dah == 0.0) ci->depth = ra + hh - sqrt(len(vIm) * len(vIm) + hr * hr);
        else ci->depth = ra + hh - len(vIm);
        ci->dirn = dir(vIm);
    } else if (I->cd == CD_SIC) {
        /* The engine's extension, no reference counterpart: a sphere inside a hollow cylinder
         * of radius a[0] and length a[1] about its unit OrientationZ.  Within the length the
         * depth is how far the sphere passes the shell, the normal the outward radial direction;
         * beyond an end, the nearest point of that end's rim circle. */
        const double hh = 0.5 * mm->a[1], R = mm->a[0];
        v3 ax = ld3(w->oz + 3 * m);
        v3 d = sub(Ps, Pm);
        double t = dot(d, ax);
        v3 rp = sub(d, muls(ax, t));
        v3 u = dir(rp);
        if (t <= hh && t >= -hh) {
            ci->depth = ra + len(rp) - R;
            ci->dirn = u;
        } else {
            v3 q = add(add(Pm, muls(ax, t > 0.0 ? hh : -hh)), muls(u, R));
            v3 vIm = sub(q, Ps);
            ci->depth = ra - len(vIm);
            ci->dirn = dir(vIm);
        }
    } else {                                                 /* CDSphere2QuasiCylinder.cpp:16-80 */
        double hh = 0.5 * mm->a[1];
        v3 ax = ld3(w->oz + 3 * m);
        double dap = dot(sub(Ps, Pm), ax);
        if (dap < -hh) dap = -hh; else if (dap > hh) dap = hh;
        v3 Caps = add(Pm, smul(dap, ax));
        v3 vIm = sub(Caps, Ps);
        double rc = mm->a[0];
        ci->depth = ra + rc - len(vIm);
        ci->dirn = dir(vIm);
    }
    ci->point = add(Ps, smul(ra - 0.5 * ci->depth, ci->dirn));
    if (ci->depth > 0) { ci->unbalance = (ci->active == 0); ci->active = 1; }
    else { ci->active = 0; ci->unbalance = 0; }
}

/* ISwModels::ShearForceRotation (ISwModels.cpp:263-273) */
static v3 shear_rotation(v3 F, v3 vs) {
    if (dot(F, vs) <= 0.0) return smul(-len(F), dir(vs));
    return smul(len(F), dir(vs));
}
/* ISwModels::NormalForce, 5 arguments (ISwModels.cpp:134-139) */
static v3 normal_force(double kn, double cn, double depth, v3 n, v3 vn) {
    return sub(smul(-kn * depth, n), smul(cn, vn));
}
/* ISwModels::NormalForce, bond form (ISwModels.cpp:166-180) */
static v3 normal_force_bond(double kn, double cn, double depth, v3 n, v3 vn) {
    if (dot(vn, n) < 0.0) return sub(smul(-kn * depth, n), smul(cn, vn));
    return smul(-cn, vn);
}
/* ISwModels::NormalBond (ISwModels.cpp:110-125) */
static int normal_bond(double kn, double bn, double depth) {
    return (depth <= 0.0) && (kn != 0.0) && (bn != 0.0) && (-depth * kn < bn);
}

static void add_impact(dp_world* w, unsigned o, v3 J, const v3* JA) {   /* DiscreteObject.cpp:149-158 */
    st3(w->J + 3 * o, add(ld3(w->J + 3 * o), J));
    if (JA) st3(w->JA + 3 * o, add(ld3(w->JA + 3 * o), *JA));
}

/* ImpactSolver::NextStep of the five laws */
static void solve(dp_world* w, iactn_t* I, double dt) {
    const cinfo_t* ci = &I->ci;
    status_t* st = &I->st;
    unsigned A = I->slave, B = I->master;
    const double depth = ci->depth;
    const v3 n = ci->dirn;
    const double* c = I->c;
    v3 Va = ld3(w->vel + 3 * A), Vb = ld3(w->vel + 3 * B);
    v3 AVa = ld3(w->av + 3 * A), AVb = ld3(w->av + 3 * B);
    v3 rA = V3(0, 0, 0), rB = V3(0, 0, 0), vRel, vRn, vRs;
    v3 Fn = V3(0, 0, 0), Fs = V3(0, 0, 0);

    if (I->is == IS_HERTZ || I->is == IS_H) {
        if (!ci->active) { status_clean(st); return; }           /* ISwHertz.cpp:26-30, ISwH.cpp:132-136 */
    } else {
        if (!ci->active && !normal_bond(c[0], c[4], depth)) {    /* ISwBSDBF.cpp:32-38 */
            status_clean(st);
            return;
        }
    }
    st->point = ci->point; st->dirn = ci->dirn; st->overlap = ci->depth;   /* SetContactInformation */

    if (depth > 0.0) {
        rA = sub(ci->point, ld3(w->pos + 3 * A));
        rB = sub(ci->point, ld3(w->pos + 3 * B));
        if (w->pbc_on) {          /* every law: ISwBSDBF.cpp:69-73, ISwBtSDBF.cpp:69-73, ISwBSDB2F.cpp:72-76,
                                     ISwHertz.cpp:59-63, ISwH.cpp:69-73 */
            rA = min_image(w, rA);
            rB = min_image(w, rB);
        }
        vRel = sub(add(sub(Va, Vb), cross(AVa, rA)), cross(AVb, rB));
        vRn = smul(dot(vRel, n), n);
        vRs = sub(vRel, vRn);
        if (I->is == IS_BSDBF || I->is == IS_BSDB2F) {           /* ISwBSDBF.cpp:61-112 */
            double kn = c[0], ks = c[1], cn = c[2], cs = c[3], bs = c[5], fc = c[6];
            Fn = normal_force(kn, cn, depth, n, vRn);
            Fs = sub(shear_rotation(st->shear, vRs), smul(ks * dt, vRs));
            double fmax = fc * kn * depth;
            if (bs == 0.0) {
                if (len(Fs) > fmax) Fs = smul(fmax, dir(Fs));
                else Fs = sub(Fs, smul(cs, vRs));
            } else {
                if (len(Fs) > bs) Fs = smul(fmax, dir(Fs));
                else Fs = sub(Fs, smul(cs, vRs));
            }
            st->shear = Fs;
            st->contact = 1;
        } else if (I->is == IS_BTSDBF) {                         /* ISwBtSDBF.cpp:61-111 */
            double kn = c[0], ks = c[1], cn = c[2], cs = c[3], bs = c[5], fc = c[6];
            Fn = normal_force(kn, cn, depth, n, vRn);
            Fs = sub(smul(-ks * dt, vRs), smul(cs, vRs));
            double fmax = fc * kn * depth;
            if (bs == 0.0) {
                if (len(Fs) > fmax) Fs = smul(fmax, dir(Fs));
                else Fs = sub(Fs, smul(cs, vRs));
            } else {
                if (len(Fs) > bs) Fs = smul(fmax, dir(Fs));
                else Fs = sub(Fs, smul(cs, vRs));
            }
            st->contact = 1;
        } else if (I->is == IS_HERTZ) {                          /* ISwHertz.cpp:53-78 */
            double kn = c[0], cn = c[1];
            if (!st->contact) { st->contact = 1; st->v0 = len(vRn); }
            Fn = sub(smul(-kn * pow(depth, 1.5), n), smul(cn, vRn));   /* ISwModels.cpp:127-132 */
        } else {                                                 /* ISwH.cpp:159-231 */
            double knH = c[0], Meff = c[1], ksc1 = c[2], ksc2 = c[3], betan = c[4], fk = c[5], kn;
            if (!st->contact) {
                if (len(vRn) == 0.0) kn = knH;
                else if (betan < 0.99)
                    kn = 0.957832746294131 / (1.0 - betan * betan) * pow(Meff, 0.2) * pow(knH, 0.8) *
                         pow(len(vRn), 0.4);
                else
                    kn = 479.155951122633 * pow(Meff, 0.2) * pow(knH, 0.8) * pow(len(vRn), 0.4);
                st->kn = kn;
                st->contact = 1;
            } else {
                kn = st->kn;
            }
            double ncd = 2.0 * sqrt(Meff * kn);
            double ks = ksc1 * pow(ksc2 * fabs(kn * depth), 1.0 / 3.0);
            Fn = normal_force(kn, ncd * betan, depth, n, vRn);
            double ff = fk * kn * depth;
            Fs = sub(shear_rotation(st->shear, vRs), smul(ks * dt, vRs));
            if (len(Fs) >= ff) Fs = smul(ff, dir(Fs));
            st->shear = Fs;
        }
    } else {
        if (I->is == IS_BSDBF || I->is == IS_BTSDBF) {           /* ISwBSDBF.cpp:113-123 */
            vRel = sub(Va, Vb);
            vRn = smul(dot(vRel, n), n);
            if (I->is == IS_BSDBF) Fn = normal_force_bond(c[0], c[2], depth, n, vRn);
            else Fn = normal_force(c[0], c[2], depth, n, vRn);   /* ISwBtSDBF.cpp:373 */
            status_clean_contact(st);
        } else if (I->is == IS_BSDB2F) {                         /* ISwBSDB2F.cpp:120-133 */
            if (st->last_bond) {
                vRel = sub(Va, Vb);
                vRn = smul(dot(vRel, n), n);
                Fn = normal_force_bond(c[0], c[2], depth, n, vRn);
                status_clean_contact(st);
            }
        } else {
            status_clean_contact(st);
        }
    }
    if (I->is == IS_HERTZ) {                                     /* ISwHertz.cpp:85-91 */
        v3 J = muls(Fn, dt);
        st->imp_master = neg(J);
        st->aimp_master = V3(0, 0, 0);
        add_impact(w, A, J, 0);
        v3 nJ = neg(J);
        add_impact(w, B, nJ, 0);
        return;
    }
    v3 F = add(Fn, Fs);
    v3 J = muls(F, dt);
    v3 tA = smul(dt, cross(rA, F));
    v3 tB = smul(-dt, cross(rB, F));
    st->imp_master = smul(-1.0, J);
    st->aimp_master = tB;
    add_impact(w, A, J, &tA);
    v3 mJ = smul(-1.0, J);
    add_impact(w, B, mJ, &tB);
}

/* DiscreteObject::Response of each behaviour */
static void respond(dp_world* w, unsigned o, double dt) {
    const model_t* m = &w->models[w->model_of[o]];
    v3 P = ld3(w->pos + 3 * o), Vv = ld3(w->vel + 3 * o), AV = ld3(w->av + 3 * o);
    v3 Ox = ld3(w->ox + 3 * o), Oz = ld3(w->oz + 3 * o);
    v3 J = ld3(w->J + 3 * o), JA = ld3(w->JA + 3 * o);
    double sm = w->sudo[o];
    if (m->behavior == VEDO_FIXED) {
        /* DOFixedQuasiPlate.h:16-19, DOFixedSphere.h: ClearImpact only */
    } else if (m->shape == VEDO_SHAPE_SPHERE) {                  /* DOSphere.cpp:21-48 */
        double R = m->a[0];
        v3 dv = smul(1.0 / sm, J);
        v3 dav = smul(2.5 / sm / R / R, JA);
        v3 dp = smul(dt, add(Vv, smul(0.5, dv)));
        v3 dw = smul(dt, add(AV, smul(0.5, dav)));
        st3(w->pos + 3 * o, add(P, dp));
        st3(w->ox + 3 * o, rotate_around(Ox, dw));
        st3(w->oz + 3 * o, rotate_around(Oz, dw));
        st3(w->vel + 3 * o, add(Vv, dv));
        st3(w->av + 3 * o, add(AV, dav));
    } else if (m->behavior == VEDO_ORBITAL) {                    /* DOOrbitalQuasiPlate.cpp:18-34 */
        v3 dp = muls(Vv, dt);
        v3 dw = muls(AV, dt);
        st3(w->pos + 3 * o, add(P, dp));
        st3(w->ox + 3 * o, rotate_around(Ox, dw));
        st3(w->oz + 3 * o, rotate_around(Oz, dw));
    } else if (m->behavior == VEDO_CONSTRAINED) {                /* DOConstrainedQuasiPlate.cpp:18-35 */
        v3 dv = smul(1.0 / sm, smul(dot(J, Oz), dir(Oz)));
        v3 dp = smul(dt, add(Vv, smul(0.5, dv)));
        v3 dw = muls(AV, dt);
        st3(w->pos + 3 * o, add(P, dp));
        st3(w->ox + 3 * o, rotate_around(Ox, dw));
        st3(w->oz + 3 * o, rotate_around(Oz, dw));
        st3(w->vel + 3 * o, add(Vv, dv));
    } else {                                                     /* DOQuasiPlate.cpp:20-41 */
        v3 dv = smul(1.0 / sm, J);
        v3 dav = V3(dot(JA, Ox) / m->inertia.x, dot(JA, cross(Oz, Ox)) / m->inertia.y, dot(JA, Oz) / m->inertia.z);
        v3 dp = smul(dt, add(Vv, smul(0.5, dv)));
        v3 dw = smul(dt, add(AV, smul(0.5, dav)));
        st3(w->pos + 3 * o, add(P, dp));
        st3(w->ox + 3 * o, rotate_around(Ox, dw));
        st3(w->oz + 3 * o, rotate_around(Oz, dw));
        st3(w->vel + 3 * o, add(Vv, dv));
        st3(w->av + 3 * o, add(AV, dav));
    }
    /* ClearImpact (DiscreteObject.cpp:141-147) */
    st3(w->imp + 3 * o, J);
    st3(w->aimp + 3 * o, JA);
    st3(w->J + 3 * o, V3(0, 0, 0));
    st3(w->JA + 3 * o, V3(0, 0, 0));
}

/* ------------------------------------------------------------------------ */
static int rec_key_cmp(const void* a, const void* b) {
    const record_t* x = (const record_t*)a;
    const record_t* y = (const record_t*)b;
    if (x->a != y->a) return x->a < y->a ? -1 : 1;
    if (x->b != y->b) return x->b < y->b ? -1 : 1;
    return 0;
}
static int rec_cmp(const void* a, const void* b) {
    int c = rec_key_cmp(a, b);
    if (c) return c;
    const record_t* x = (const record_t*)a;
    const record_t* y = (const record_t*)b;
    return x->ord < y->ord ? -1 : (x->ord > y->ord ? 1 : 0);
}
/* sort by key keeping the first inserted of equal keys, as std::map::insert does */
static void sort_records(record_t* r, unsigned* n) {
    for (unsigned k = 0; k < *n; ++k) r[k].ord = k;
    qsort(r, *n, sizeof(record_t), rec_cmp);
    unsigned m = 0;
    for (unsigned k = 0; k < *n; ++k)
        if (m == 0 || rec_key_cmp(&r[k], &r[m - 1]) != 0) r[m++] = r[k];
    *n = m;
}

/* What SimMediator's constructor does once before the first step (SimMediator.cpp:125-134):
   Consultant::CleanUp (Consultant.cpp:264-319) with the zone of interest as Boundary::Correct
   leaves it (Boundary.cpp:79-128: bounds sorted per axis, an axis on where they differ).
   Mobile objects outside the zone are erased; ElementMappingJump holds minus the number erased
   up to and including each object (unsigned); IactRecordTab::ModifyPair (IactRecordTab.cpp:41-69)
   moves every record whose key changes to its new key, in key order, overwriting what is there;
   the survivors keep their order. */
static int zoi_cleanup(dp_world* w) {
    const double* lo = w->zoi_lo;
    const double* hi = w->zoi_hi;
    const int* sw = w->zoi_sw;
    if (!w->zoi_on) return 0;
    const unsigned n = w->n;
    unsigned* jump = (unsigned*)malloc(sizeof(unsigned) * (n ? n : 1));
    char* gone = (char*)calloc(n ? n : 1, 1);
    unsigned dead = 0, nerased = 0;
    for (unsigned u = 0; u < n; ++u) {
        int out = 0;
        for (int k = 0; k < 3; ++k) {
            const double p = w->pos[3 * (size_t)u + k];
            if (sw[k] && (p < lo[k] || p > hi[k])) out = 1;       /* Boundary::InBoundary */
        }
        if (w->models[w->model_of[u]].behavior == VEDO_MOBILE && out) { gone[u] = 1; --dead; ++nerased; }
        jump[u] = dead;
    }
    if (nerased) {
        /* ModifyPair on the records (sorted by key): unchanged keys stay; moved ones take their new
           key, the last moved onto a key (in key order) over earlier ones and over a record there */
        record_t* all = (record_t*)calloc(w->nrec ? w->nrec : 1, sizeof(record_t));
        unsigned moved = 0, total = 0;
        for (unsigned q = 0; q < w->nrec; ++q) {
            record_t r = w->rec[q];
            const unsigned na = r.a + (r.a < n ? jump[r.a] : 0u), nb = r.b + (r.b < n ? jump[r.b] : 0u);
            if (na != r.a || nb != r.b) { r.a = na; r.b = nb; r.ord = w->nrec - 1 - moved; ++moved; }
            else r.ord = w->nrec + q;
            all[total++] = r;
        }
        qsort(all, total, sizeof(record_t), rec_cmp);
        unsigned m = 0;
        for (unsigned k = 0; k < total; ++k)
            if (m == 0 || rec_key_cmp(&all[k], &all[m - 1]) != 0) all[m++] = all[k];
        free(w->rec);
        w->rec = all;
        w->nrec = m;
        /* DOContainer::Erase, DOWorld::EraseDOStatus */
        double* arrs[9] = {w->pos, w->vel, w->av, w->ox, w->oz, w->imp, w->aimp, w->J, w->JA};
        unsigned v = 0;
        for (unsigned u = 0; u < n; ++u) {
            if (gone[u]) continue;
            w->model_of[v] = w->model_of[u];
            w->sudo[v] = w->sudo[u];
            for (int a = 0; a < 9; ++a)
                for (int k = 0; k < 3; ++k) arrs[a][3 * (size_t)v + k] = arrs[a][3 * (size_t)u + k];
            ++v;
        }
        w->n = v;
    }
    free(jump);
    free(gone);
    return (int)nerased;
}

static const record_t* find_record(const dp_world* w, unsigned a, unsigned b) {  /* IactRecordTab.cpp:20-25 */
    record_t key;
    key.a = a; key.b = b;
    return (const record_t*)bsearch(&key, w->rec, w->nrec, sizeof(record_t), rec_key_cmp);
}

/* SimMediator::Initiate (SimMediator.cpp:640-712); with an active periodic boundary the
   detectors and solvers see it (pbc_on) */
static int initiate(dp_world* w) {
    free(w->it);
    w->it = (iactn_t*)calloc(w->ncand ? w->ncand : 1, sizeof(iactn_t));
    if (!w->it) return -1;
    for (unsigned k = 0; k < w->ncand; ++k) {
        int rc = create_interaction(w, w->cfirst[k], w->csecond[k], &w->it[k]);
        if (rc != 0) return -2;   /* the reference would drop it and misalign IactPairTab (NBSConsultant.cpp:386) */
        detect(w, &w->it[k]);
        const record_t* r = find_record(w, w->cfirst[k], w->csecond[k]);
        if (r) w->it[k].st = r->st;
    }
    return 0;
}

/* NBSConsultant::RebuildIactRecordTab (NBSConsultant.cpp:376-395) */
static int rebuild_records(dp_world* w) {
    unsigned na = 0;
    for (unsigned k = 0; k < w->ncand; ++k) na += w->it[k].ci.active ? 1 : 0;
    free(w->rec);
    w->rec = (record_t*)malloc(sizeof(record_t) * (na ? na : 1));
    if (!w->rec) return -1;
    w->nrec = 0;
    for (unsigned k = 0; k < w->ncand; ++k) {
        if (!w->it[k].ci.active) continue;
        w->rec[w->nrec].a = w->cfirst[k];
        w->rec[w->nrec].b = w->csecond[k];
        w->rec[w->nrec].st = w->it[k].st;
        w->nrec++;
    }
    sort_records(w->rec, &w->nrec);
    return 0;
}

/* ------------------------------------------------------------------------ */
dp_world* dp_create(const vedo_scene_desc* sc, unsigned up_iact, int consultant, char* err, size_t errlen) {
    if (!sc || !sc->num_objects) { set_err(err, errlen, "empty scene"); return NULL; }
    dp_world* w = (dp_world*)calloc(1, sizeof(dp_world));
    w->leap = consultant == 1;
    for (int k = 0; k < 3; ++k) {                  /* Boundary::Correct for the zone of interest */
        const double a = sc->zoi_lower[k], b = sc->zoi_upper[k];
        w->zoi_lo[k] = a < b ? a : b;
        w->zoi_hi[k] = a < b ? b : a;
        w->zoi_sw[k] = a != b;
        w->zoi_on |= w->zoi_sw[k];
    }
    /* Boundary::Correct (Boundary.cpp:79-128): an axis is on where its bounds differ */
    for (int k = 0; k < 3; ++k) {
        const double a = sc->pbc_lower[k], b = sc->pbc_upper[k];
        w->pbc_lo[k] = a < b ? a : b;
        w->pbc_hi[k] = a < b ? b : a;
        w->pbc_r[k] = w->pbc_hi[k] - w->pbc_lo[k];
        w->pbc_sw[k] = a != b;
        w->pbc_on |= w->pbc_sw[k];
    }
    w->t_start = sc->time_start; w->t_stop = sc->time_stop; w->dt = sc->time_interval; w->t = sc->time_current;
    w->g = ld3(sc->field_acceleration);
    w->sf = sc->safety_factor;
    w->up_iact = up_iact ? up_iact : 1;
    /* groups: index by first appearance among models and interaction models */
    const char** gnames = (const char**)calloc(2 * sc->num_models + 2 * sc->num_iact_models + 1, sizeof(char*));
    int ng = 0;
#define GROUP_ID(s, out) do { int _f = -1; for (int _g = 0; _g < ng; ++_g) if (!strcmp(gnames[_g], (s))) { _f = _g; break; } \
        if (_f < 0) { gnames[ng] = (s); _f = ng++; } (out) = _f; } while (0)
    w->nmodels = (int)sc->num_models;
    w->models = (model_t*)calloc(w->nmodels, sizeof(model_t));
    for (int k = 0; k < w->nmodels; ++k) {
        const vedo_do_model* dm = &sc->models[k];
        model_t* m = &w->models[k];
        m->shape = (int)dm->shape; m->behavior = (int)dm->behavior; m->scope = (int)dm->scope;
        m->density = dm->density; m->dfac = dm->density_factor;
        m->ext = ld3(dm->external_force);
        memcpy(m->a, dm->attrs, sizeof(m->a));
        GROUP_ID(dm->group, m->group);
        if (!analyse(m)) { set_err(err, errlen, "unsupported shape"); dp_destroy(w); free(gnames); return NULL; }
    }
    w->niact = (int)sc->num_iact_models;
    w->iacts = (iact_t*)calloc(w->niact ? w->niact : 1, sizeof(iact_t));
    int* mg = (int*)calloc(w->niact ? w->niact : 1, sizeof(int));
    int* sg = (int*)calloc(w->niact ? w->niact : 1, sizeof(int));
    for (int k = 0; k < w->niact; ++k) {
        const vedo_iact_model* im = &sc->iact_models[k];
        GROUP_ID(im->master_group, mg[k]);
        GROUP_ID(im->slave_group, sg[k]);
        iact_t* it = &w->iacts[k];
        it->eq = eq_of(im->equation_type);
        if (it->eq != IS_NONE) {
            for (int q = 0; MECH_NAMES[it->eq][q]; ++q) {
                for (unsigned r = 0; r < im->num_mechanisms; ++r) {
                    if (!strcmp(im->mechanism_names[r], MECH_NAMES[it->eq][q])) {
                        it->p[q] = im->mechanism_values[r];
                        it->present[q] = 1;
                        break;
                    }
                }
            }
        }
    }
#undef GROUP_ID
    w->ngroups = ng;
    w->group_iact = (int*)malloc(sizeof(int) * (ng ? ng * ng : 1));
    for (int a = 0; a < ng; ++a)
        for (int b = 0; b < ng; ++b) {
            int f = -1;
            for (int k = 0; k < w->niact; ++k)    /* first match, DOWorld.cpp:297-302 */
                if ((mg[k] == a && sg[k] == b) || (mg[k] == b && sg[k] == a)) { f = k; break; }
            w->group_iact[a * ng + b] = f;
        }
    free(mg); free(sg); free(gnames);
    unsigned n = sc->num_objects;
    w->n = n;
    w->model_of = (unsigned*)malloc(sizeof(unsigned) * n);
    memcpy(w->model_of, sc->object_model, sizeof(unsigned) * n);
    double** arrs[9] = {&w->pos, &w->vel, &w->av, &w->ox, &w->oz, &w->imp, &w->aimp, &w->J, &w->JA};
    for (int k = 0; k < 9; ++k) *arrs[k] = (double*)calloc(3 * (size_t)n, sizeof(double));
    w->sudo = (double*)calloc(n, sizeof(double));
    memcpy(w->pos, sc->position, 24 * (size_t)n);
    memcpy(w->vel, sc->velocity, 24 * (size_t)n);
    memcpy(w->av, sc->angular_velocity, 24 * (size_t)n);
    memcpy(w->ox, sc->orientation_x, 24 * (size_t)n);
    memcpy(w->oz, sc->orientation_z, 24 * (size_t)n);
    if (sc->impact) memcpy(w->imp, sc->impact, 24 * (size_t)n);
    if (sc->angular_impact) memcpy(w->aimp, sc->angular_impact, 24 * (size_t)n);
    for (unsigned u = 0; u < n; ++u) {
        if (w->model_of[u] >= (unsigned)w->nmodels ||
            object_sudo_mass(&w->models[w->model_of[u]], &w->sudo[u]) != 0) {
            set_err(err, errlen, "no discrete-object factory for a model"); dp_destroy(w); return NULL;
        }
    }
    /* IDO records: ImpactStatus built by setters on a default status (IactRecordTab.cpp:432-530) */
    w->nrec = sc->num_records;
    w->rec = (record_t*)calloc(w->nrec ? w->nrec : 1, sizeof(record_t));
    for (unsigned r = 0; r < w->nrec; ++r) {
        record_t* R = &w->rec[r];
        R->a = sc->record_first[r]; R->b = sc->record_second[r];
        R->st = status_default();
        R->st.contact = sc->record_contact ? sc->record_contact[r] != 0 : 0;
        R->st.bond = sc->record_bond ? sc->record_bond[r] != 0 : 0;
        R->st.kn = sc->record_kn ? sc->record_kn[r] : 0.0;
        R->st.v0 = sc->record_initial_velocity ? sc->record_initial_velocity[r] : 0.0;
        if (sc->record_shear) R->st.shear = ld3(sc->record_shear + 3 * r);
    }
    sort_records(w->rec, &w->nrec);
    zoi_cleanup(w);                                /* SimMediator's constructor (SimMediator.cpp:125-134) */
    int rc = consultant_reset(w);
    if (rc == 0) rc = initiate(w);
    if (rc != 0) {
        set_err(err, errlen, rc == -2 ? "unsupported interaction in candidate list"
                             : rc == -3 ? "the Leap consultant needs a local object" : "allocation failed");
        dp_destroy(w);
        return NULL;
    }
    return w;
}

int dp_run(dp_world* w, unsigned nsteps) {
    int cont = 1;
    for (unsigned s = 0; s < nsteps; ++s) {
        double dt = w->dt;
        for (unsigned k = 0; k < w->ncand; ++k) solve(w, &w->it[k], dt);      /* CalculateImpact */
        v3 fimp = muls(w->g, dt);                                              /* SimMediator.cpp:738 */
        for (unsigned o = 0; o < w->n; ++o) {
            add_impact(w, o, muls(fimp, w->sudo[o]), 0);                       /* DOContainer.cpp:25 */
        }
        for (unsigned o = 0; o < w->n; ++o) {                                  /* DiscreteObject.cpp:160-163 */
            add_impact(w, o, smul(dt, w->models[w->model_of[o]].ext), 0);
        }
        for (unsigned o = 0; o < w->n; ++o) respond(w, o, dt);                 /* DOContainer::Response */
        if (w->pbc_on)                                                         /* SimMediator.cpp:746 */
            for (unsigned o = 0; o < w->n; ++o) wrap_position(w, w->pos + 3 * o);
        for (unsigned k = 0; k < w->ncand; ++k) detect(w, &w->it[k]);         /* CheckContactStatus */
        w->round++;                                                            /* NBSConsultant::NextStep */
        w->t += dt;
        int reset = (w->round % w->up_iact) == 0;
        if (reset) {
            rebuild_records(w);
            /* LeapConsultant::NextStep (LeapConsultant.cpp:61-68): SyncWorld, RebuildIactRecordTab,
               CleanUp, Reset -- the Leap consultant erases the mobile objects outside the zone of
               interest at every reset (NBSConsultant::NextStep does not) */
            if (w->leap) zoi_cleanup(w);
            if (consultant_reset(w) != 0) return -1;
        }
        for (unsigned k = 0; k < w->ncand && !reset; ++k) {                   /* BackupImpactStatus */
            w->it[k].st.last_contact = w->it[k].st.contact;
            w->it[k].st.last_bond = w->it[k].st.bond;
        }
        if (reset) initiate(w);                                                /* SimMediator.cpp:776-779 */
        cont = w->t < w->t_stop;
    }
    return cont;
}

unsigned dp_num_objects(const dp_world* w) { return w->n; }

void dp_get_state(const dp_world* w, double* pos, double* vel, double* avel, double* ox, double* oz, double* imp,
                  double* aimp) {
    size_t b = 24 * (size_t)w->n;
    if (pos) memcpy(pos, w->pos, b);
    if (vel) memcpy(vel, w->vel, b);
    if (avel) memcpy(avel, w->av, b);
    if (ox) memcpy(ox, w->ox, b);
    if (oz) memcpy(oz, w->oz, b);
    if (imp) memcpy(imp, w->imp, b);
    if (aimp) memcpy(aimp, w->aimp, b);
}

void dp_set_state(dp_world* w, const double* pos, const double* vel, const double* avel, const double* ox,
                  const double* oz) {
    size_t b = 24 * (size_t)w->n;
    if (pos) memcpy(w->pos, pos, b);
    if (vel) memcpy(w->vel, vel, b);
    if (avel) memcpy(w->av, avel, b);
    if (ox) memcpy(w->ox, ox, b);
    if (oz) memcpy(w->oz, oz, b);
    for (unsigned k = 0; k < w->ncand; ++k) detect(w, &w->it[k]);
}

unsigned dp_num_candidates(const dp_world* w) { return w->ncand; }

void dp_get_candidates(const dp_world* w, unsigned* first, unsigned* second) {
    memcpy(first, w->cfirst, sizeof(unsigned) * w->ncand);
    memcpy(second, w->csecond, sizeof(unsigned) * w->ncand);
}

void dp_get_interactions(const dp_world* w, unsigned* slave, unsigned* master, int* active, double* depth,
                         double* normal, double* shear, double* kn, int* contact) {
    for (unsigned k = 0; k < w->ncand; ++k) {
        const iactn_t* I = &w->it[k];
        if (slave) slave[k] = I->slave;
        if (master) master[k] = I->master;
        if (active) active[k] = I->ci.active;
        if (depth) depth[k] = I->ci.depth;
        if (normal) st3(normal + 3 * k, I->ci.dirn);
        if (shear) st3(shear + 3 * k, I->st.shear);
        if (kn) kn[k] = I->st.kn;
        if (contact) contact[k] = I->st.contact;
    }
}

double dp_time(const dp_world* w) { return w->t; }

/* DOWorld::CalculateSystemEnergy (vedo/framework/DOWorld.cpp:481-660) */
void dp_energy(const dp_world* w, double* out) {
    double Ep = 0, Et = 0, Er = 0, vmax = 0, vmin = 0, avmax = 0, avmin = 0, mn = 0, amn = 0;
    v3 mom = V3(0, 0, 0), amom = V3(0, 0, 0);
    unsigned first = w->n, nm = 0;
    for (unsigned u = 0; u < w->n; ++u)
        if (w->models[w->model_of[u]].behavior == VEDO_MOBILE) { first = u; break; }
    if (first < w->n) {
        for (unsigned u = first; u < w->n; ++u) {
            const model_t* m = &w->models[w->model_of[u]];
            if (m->behavior != VEDO_MOBILE) continue;
            double ms = m->mass;
            v3 mmi = m->inertia, Vv = ld3(w->vel + 3 * u), av = ld3(w->av + 3 * u);
            double v = len(Vv);
            double dav = len(av);
            double ep = -ms * dot(w->g, ld3(w->pos + 3 * u));
            double et = 0.5 * ms * v * v;
            double er = 0.5 * (mmi.x * av.x * av.x + mmi.y * av.y * av.y + mmi.z * av.z * av.z);
            if (u == first) {
                mom = smul(ms, Vv); amom = cross(mmi, av);
                Ep = ep; Et = et; Er = er;
                vmax = vmin = v; avmax = avmin = dav;
                nm = 1;
            } else {
                nm++;
                mom = add(mom, smul(ms, Vv));
                amom = add(amom, cross(mmi, av));
                Ep = Ep - ms * dot(w->g, ld3(w->pos + 3 * u));
                Et += et; Er += er;
                if (v > vmax) vmax = v; else if (v < vmin) vmin = v;
                if (dav > avmax) avmax = dav; else if (dav < avmin) avmin = dav;
            }
        }
        mom = smul(1.0 / nm, mom);
        amom = smul(1.0 / nm, amom);
        for (unsigned u = first; u < w->n; ++u) {
            const model_t* m = &w->models[w->model_of[u]];
            if (m->behavior != VEDO_MOBILE) continue;
            mn += len(sub(smul(m->mass, ld3(w->vel + 3 * u)), mom));
            amn += len(sub(cross(m->inertia, ld3(w->av + 3 * u)), amom));
        }
    }
    out[0] = Ep; out[1] = Et; out[2] = Er; out[3] = vmin; out[4] = vmax; out[5] = avmin; out[6] = avmax;
    out[7] = mn; out[8] = amn;
}

/* CalcCoordinateNum (vedo/knight/CalcCoordinateNum.cpp).  outputCoordinateNumVTK (:79-126) counts
   the pairs i < j of spheres with |p_i - p_j| < r_i + r_j; computeAvgCoordinateNum (:8-77) takes
   the spheres whose centre lies strictly inside the box widened by their radius and counts, for
   each, the other spheres with |p_i - p_j| <= r_i + r_j; the total is an unsigned 32-bit sum. */
double dp_coordination(const dp_world* w, const double* box, unsigned* below, unsigned* touching) {
    for (unsigned i = 0; i < w->n; ++i) { below[i] = 0; touching[i] = 0; }
    for (unsigned i = 0; i < w->n; ++i) {
        const model_t* mi = &w->models[w->model_of[i]];
        if (mi->shape != VEDO_SHAPE_SPHERE) continue;
        for (unsigned j = i + 1; j < w->n; ++j) {
            const model_t* mj = &w->models[w->model_of[j]];
            if (mj->shape != VEDO_SHAPE_SPHERE) continue;
            const double d = len(sub(ld3(w->pos + 3 * i), ld3(w->pos + 3 * j)));
            const double rs = mi->a[0] + mj->a[0];
            if (d < rs) { below[i]++; below[j]++; }
            if (d <= rs) { touching[i]++; touching[j]++; }
        }
    }
    unsigned total = 0, count = 0;
    for (unsigned i = 0; i < w->n; ++i) {
        const model_t* m = &w->models[w->model_of[i]];
        if (m->shape != VEDO_SHAPE_SPHERE) continue;
        const double* p = w->pos + 3 * i;
        const double r = m->a[0];
        if (p[0] < box[1] + r && p[0] > box[0] - r && p[1] < box[3] + r && p[1] > box[2] - r &&
            p[2] < box[5] + r && p[2] > box[4] - r) {
            total += touching[i];
            count++;
        }
    }
    return total / (double)count;
}

void dp_destroy(dp_world* w) {
    if (!w) return;
    free(w->models); free(w->iacts); free(w->group_iact); free(w->model_of);
    free(w->pos); free(w->vel); free(w->av); free(w->ox); free(w->oz); free(w->imp); free(w->aimp);
    free(w->J); free(w->JA); free(w->sudo); free(w->cfirst); free(w->csecond); free(w->it); free(w->rec);
    free(w);
}
