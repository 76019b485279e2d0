// scene_host.cpp - reference .ido reader/writer, scene descriptor import and the
// DOModel / IactModel flattening into device tables.
#include "scene_host.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>

namespace vedo {

namespace {

constexpr int kShapeAttrDoubles = 10;   // sizeof(DOShapeAttributes) / sizeof(double), DOModel.h:36-102
const char* kReleaseDate = "2016-09-23"; // aries::information::_ReleaseDate, Constants.h:42

struct Reader {
    std::vector<char> d;
    size_t p = 0;
    bool ok = true;
    bool raw(void* dst, size_t k) {
        if (!ok || p + k > d.size()) { ok = false; return false; }
        std::memcpy(dst, d.data() + p, k);
        p += k;
        return true;
    }
    uint32_t u32() { uint32_t v = 0; raw(&v, 4); return v; }
    double f64() { double v = 0; raw(&v, 8); return v; }
    std::string str() {
        uint32_t n = u32();
        if (!ok || p + n > d.size()) { ok = false; return std::string(); }
        std::string s(d.data() + p, n);
        p += n;
        return s;
    }
};

struct Writer {
    std::vector<char> d;
    void raw(const void* s, size_t k) { d.insert(d.end(), (const char*)s, (const char*)s + k); }
    void u32(uint32_t v) { raw(&v, 4); }
    void f64(double v) { raw(&v, 8); }
    void str(const std::string& s) { u32((uint32_t)s.size()); raw(s.data(), s.size()); }
};

// DOModel::Analysis (DOModel.cpp:17-149); returns false for shapes the engine lacks.
bool analyse(const HModel& m, ModelDev& o) {
    const double PI = 4.0 * std::atan(1.0);           // aries::math::_PI (Constants.h:22)
    const double FTPI = 4.0 / 3.0 * PI;               // _FourthThirdsPI (Constants.h:32)
    o.shape = (int)m.shape;
    o.behavior = (int)m.behavior;
    o.scope = (int)m.scope;
    o.density = m.density;
    o.a0 = m.attrs[0];
    o.a1 = m.attrs[1];
    o.a2 = m.attrs[2];
    o.ext[0] = m.ext[0]; o.ext[1] = m.ext[1]; o.ext[2] = m.ext[2];
    double vol, mass, sudo_model;
    if (m.shape == SHAPE_SPHERE) {
        double r = m.attrs[0];
        o.range = r;
        vol = FTPI * r * r * r;
        mass = m.density * vol;
        sudo_model = m.density_factor * mass;
        double mmi = 0.4 * mass * r * r;
        o.ix = o.iy = o.iz = mmi;
    } else if (m.shape == SHAPE_CYL) {
        double r = m.attrs[0], h = m.attrs[1];
        o.range = (m.scope == SCOPE_LOCAL) ? std::max(r, 0.5 * h) : r;
        vol = PI * r * r * h;
        mass = m.density * vol;
        sudo_model = m.density_factor * mass;
        double mmi = mass * (3.0 * r * r + h * h) / 12.0;
        o.ix = o.iy = mmi;
        o.iz = 0.5 * mass * r * r;
    } else if (m.shape == SHAPE_HOLED) {                  // DOModel.cpp:90-119
        const double w = m.attrs[0], h = m.attrs[1], l = m.attrs[2], hr = m.attrs[3], hxo = m.attrs[4],
                     hyo = m.attrs[5];
        o.range = (m.scope == SCOPE_LOCAL) ? 0.5 * std::max(std::max(w, h), l) : 0.5 * h;
        if (!((std::abs(hxo) <= (0.5 * w - hr)) && (std::abs(hyo) <= (0.5 * l - hr)))) return false;   // the reference exits
        vol = w * h * l - hr * hr * PI * h;
        mass = m.density * vol;
        sudo_model = m.density_factor * mass;
        o.ix = o.iy = o.iz = 0.0;                        // "Need to be modified."
        // the only factories: fixed and mobile (ModuleList.h:50,56); a mobile one moves as an
        // orbital plate does (DOQuasiPlateWithCircularHole.cpp:22-38), which is not restated
        if (m.behavior != BEH_FIXED) return false;
    } else if (m.shape == SHAPE_INNER_CYL) {
        // engine extension (no reference counterpart): a shell of no thickness and no mass, range
        // 0; only walls (global scope) that are fixed or turn about their own centre
        if (m.scope != SCOPE_GLOBAL || (m.behavior != BEH_FIXED && m.behavior != BEH_ORBITAL)) return false;
        if (!(m.attrs[0] > 0.0) || !(m.attrs[1] > 0.0)) return false;
        o.range = 0.0;
        vol = mass = sudo_model = 0.0;
        o.ix = o.iy = o.iz = 0.0;
    } else if (m.shape == SHAPE_PLATE) {
        double w = m.attrs[0], h = m.attrs[1], l = m.attrs[2];
        o.range = (m.scope == SCOPE_LOCAL) ? 0.5 * std::max(std::max(w, h), l) : 0.5 * h;
        vol = w * h * l;
        mass = m.density * vol;
        sudo_model = m.density_factor * mass;
        double k = mass / 12.0;
        o.ix = k * (h * h + l * l);
        o.iy = k * (w * w + l * l);
        o.iz = k * (h * h + w * w);
    } else {
        return false;
    }
    o.mass = mass;
    // dSudoMass of the DiscreteObject subclass DOcf<>(shape, behaviour) creates (ModuleList.h:46-57)
    if (m.shape == SHAPE_SPHERE) {
        if (m.behavior != BEH_MOBILE && m.behavior != BEH_FIXED) return false;
        o.sudo = sudo_model;                                 // DOSphere.cpp:17, DOFixedSphere.cpp
    } else {
        switch (m.behavior) {
        case BEH_FIXED: case BEH_ORBITAL: o.sudo = 0.0; break;         // DOFixedQuasiPlate.cpp:14
        case BEH_CONSTRAINED: o.sudo = sudo_model; break;               // DOConstrainedQuasiPlate.cpp:14
        case BEH_MOBILE: o.sudo = mass; break;                          // DOQuasiPlate.cpp:14
        default: return false;
        }
    }
    // the per-object divisions of Response depend only on the model: evaluated once here
    // with the same IEEE operations (1.0 / m, then ((2.5 / m) / r) / r)
    o.inv_sudo = 1.0 / o.sudo;
    o.rot_coef = (m.shape == SHAPE_SPHERE) ? 2.5 / o.sudo / o.a0 / o.a0 : 0.0;
    return true;
}

int eq_of(const std::string& s) {                     // IScf<IS>("name"), ModuleList.h:59-63
    if (s == "ISwBSDBF") return IS_BSDBF;
    if (s == "ISwBtSDBF") return IS_BTSDBF;
    if (s == "ISwBSDB2F") return IS_BSDB2F;
    if (s == "ISwHertz") return IS_HERTZ;
    if (s == "ISwH") return IS_H;
    return 0;
}

bool mech(const HIact& im, const char* name, double& v) {   // IactModel::GetIactMechanism, IactModel.cpp:69-90
    for (auto& p : im.mech)
        if (p.first == name) { v = p.second; return true; }
    return false;
}

}  // namespace

// ------------------------------------------------------------------------------------
bool read_ido(const std::string& path, HScene& s, std::string& err) {
    std::ifstream f(path, std::ios::binary);
    if (!f) { err = "cannot open " + path; return false; }
    Reader r;
    r.d.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
    // SystemParameter::operator<< (SystemParameter.cpp:93-140)
    r.str();
    if (r.u32() != 3) { err = "IDO: size of integer data is wrong"; return false; }
    s.num_udd_do = r.u32();
    s.num_udd_impact = r.u32();
    s.max_id_of_do = r.u32();
    if (r.u32() != 1) { err = "IDO: size of float data is wrong"; return false; }
    s.safety_factor = r.f64();
    s.time_start = r.f64(); s.time_stop = r.f64(); s.time_current = r.f64(); s.time_interval = r.f64();
    for (int k = 0; k < 3; ++k) s.g[k] = r.f64();
    r.raw(s.zoi_switch, 3);
    for (int k = 0; k < 3; ++k) s.zoi_lower[k] = r.f64();
    for (int k = 0; k < 3; ++k) s.zoi_upper[k] = r.f64();
    r.raw(s.pbc_switch, 3);
    for (int k = 0; k < 3; ++k) s.pbc_lower[k] = r.f64();
    for (int k = 0; k < 3; ++k) s.pbc_upper[k] = r.f64();
    // DOModel::operator<< (DOModel.cpp:308-347)
    uint32_t nm = r.u32();
    if (!r.ok || nm > (1u << 20)) { err = "IDO: truncated file"; return false; }
    s.models.resize(nm);
    for (auto& m : s.models) {
        m.name = r.str(); m.group = r.str();
        m.behavior = r.u32(); m.scope = r.u32();
        m.density = r.f64(); m.density_factor = r.f64();
        for (int k = 0; k < 3; ++k) m.ext[k] = r.f64();
        m.color = r.u32(); m.shape = r.u32();
        for (int k = 0; k < kShapeAttrDoubles; ++k) m.attrs[k] = r.f64();
        uint32_t nmat = r.u32();
        if (!r.ok || nmat > (1u << 20)) { err = "IDO: truncated file"; return false; }
        for (uint32_t q = 0; q < nmat; ++q) { std::string nmq = r.str(); double v = r.f64(); m.materials.push_back({nmq, v}); }
        if (m.shape == 4) { err = "IDO: polyhedra models are not supported"; return false; }
    }
    // IactModel::operator<< (IactModel.cpp:120-137)
    uint32_t ni = r.u32();
    if (!r.ok || ni > (1u << 24)) { err = "IDO: truncated file"; return false; }
    s.iacts.resize(ni);
    for (auto& im : s.iacts) {
        im.master_group = r.str(); im.slave_group = r.str(); im.equation_type = r.str();
        uint32_t k = r.u32();
        if (!r.ok || k > (1u << 16)) { err = "IDO: truncated file"; return false; }
        for (uint32_t q = 0; q < k; ++q) { std::string nmq = r.str(); double v = r.f64(); im.mech.push_back({nmq, v}); }
    }
    // DOStatus::operator<< (DOStatus.cpp:191-200)
    uint32_t n = r.u32();
    if (!r.ok || (uint64_t)n * 176 > r.d.size()) { err = "IDO: truncated file"; return false; }
    s.n = n;
    s.model_of.resize(n); s.ids.resize(n);
    for (auto* v : {&s.pos, &s.vel, &s.ox, &s.oz, &s.av, &s.imp, &s.aimp}) v->resize(3 * (size_t)n);
    std::map<std::string, uint32_t> by_name;
    for (uint32_t k = 0; k < nm; ++k) by_name.emplace(s.models[k].name, k);   // first match, DOWorld.cpp:290-295
    std::string last;
    uint32_t last_model = 0;
    for (uint32_t i = 0; i < n; ++i) {
        std::string nmq = r.str();
        if (i == 0 || nmq != last) {
            auto it = by_name.find(nmq);
            if (it == by_name.end()) { err = "IDO: unknown model of discrete object " + nmq; return false; }
            last = nmq;
            last_model = it->second;
        }
        s.model_of[i] = last_model;
        s.ids[i] = r.u32();
        double v[21];
        r.raw(v, sizeof(v));
        for (int k = 0; k < 3; ++k) {
            s.pos[3 * i + k] = v[k]; s.vel[3 * i + k] = v[3 + k]; s.ox[3 * i + k] = v[6 + k];
            s.oz[3 * i + k] = v[9 + k]; s.av[3 * i + k] = v[12 + k]; s.imp[3 * i + k] = v[15 + k];
            s.aimp[3 * i + k] = v[18 + k];
        }
    }
    // IactRecordTab::operator<< (IactRecordTab.cpp:432-530)
    uint32_t nr = r.u32();
    if (!r.ok) { err = "IDO: truncated file"; return false; }
    if (nr && s.num_udd_impact) { err = "IDO: user-defined impact values are not supported"; return false; }
    if ((uint64_t)nr * 130 > r.d.size()) { err = "IDO: truncated file"; return false; }
    HRecords& R = s.rec;
    for (uint32_t q = 0; q < nr; ++q) {
        R.first.push_back(r.u32()); R.second.push_back(r.u32());
        uint8_t c = 0, b = 0;
        r.raw(&c, 1); r.raw(&b, 1);
        R.contact.push_back(c); R.bond.push_back(b);
        R.kn.push_back(r.f64()); R.v0.push_back(r.f64());
        for (auto* v : {&R.shear, &R.point, &R.dirn, &R.imp, &R.aimp})
            for (int k = 0; k < 3; ++k) v->push_back(r.f64());
        R.overlap.push_back(r.f64());
    }
    if (!r.ok) { err = "IDO: truncated file"; return false; }
    return true;
}

bool write_ido(const std::string& path, const HScene& s, std::string& err) {
    Writer w;
    w.str(kReleaseDate);                                    // SystemParameter::operator>> (:61-91)
    w.u32(3); w.u32(s.num_udd_do); w.u32(s.num_udd_impact); w.u32(s.max_id_of_do);
    w.u32(1); w.f64(s.safety_factor);
    w.f64(s.time_start); w.f64(s.time_stop); w.f64(s.time_current); w.f64(s.time_interval);
    for (int k = 0; k < 3; ++k) w.f64(s.g[k]);
    w.raw(s.zoi_switch, 3);
    for (int k = 0; k < 3; ++k) w.f64(s.zoi_lower[k]);
    for (int k = 0; k < 3; ++k) w.f64(s.zoi_upper[k]);
    w.raw(s.pbc_switch, 3);
    for (int k = 0; k < 3; ++k) w.f64(s.pbc_lower[k]);
    for (int k = 0; k < 3; ++k) w.f64(s.pbc_upper[k]);
    w.u32((uint32_t)s.models.size());                        // DOModel::operator>> (:267-306)
    for (auto& m : s.models) {
        w.str(m.name); w.str(m.group); w.u32(m.behavior); w.u32(m.scope);
        w.f64(m.density); w.f64(m.density_factor);
        for (int k = 0; k < 3; ++k) w.f64(m.ext[k]);
        w.u32(m.color); w.u32(m.shape);
        for (int k = 0; k < kShapeAttrDoubles; ++k) w.f64(m.attrs[k]);
        w.u32((uint32_t)m.materials.size());
        for (auto& p : m.materials) { w.str(p.first); w.f64(p.second); }
    }
    w.u32((uint32_t)s.iacts.size());                         // IactModel::operator>> (:102-118)
    for (auto& im : s.iacts) {
        w.str(im.master_group); w.str(im.slave_group); w.str(im.equation_type);
        w.u32((uint32_t)im.mech.size());
        for (auto& p : im.mech) { w.str(p.first); w.f64(p.second); }
    }
    w.u32(s.n);                                              // DOStatus::operator>> (:176-189)
    for (uint32_t i = 0; i < s.n; ++i) {
        w.str(s.models[s.model_of[i]].name);
        w.u32(s.ids.empty() ? 0u : s.ids[i]);
        for (auto* v : {&s.pos, &s.vel, &s.ox, &s.oz, &s.av, &s.imp, &s.aimp}) w.raw(v->data() + 3 * (size_t)i, 24);
    }
    const HRecords& R = s.rec;                               // IactRecordTab::operator>> (:346-430)
    w.u32((uint32_t)R.size());
    for (size_t q = 0; q < R.size(); ++q) {
        w.u32(R.first[q]); w.u32(R.second[q]);
        w.raw(&R.contact[q], 1); w.raw(&R.bond[q], 1);
        w.f64(R.kn[q]); w.f64(R.v0[q]);
        for (auto* v : {&R.shear, &R.point, &R.dirn, &R.imp, &R.aimp}) w.raw(v->data() + 3 * q, 24);
        w.f64(R.overlap[q]);
    }
    std::ofstream f(path, std::ios::binary);
    if (!f) { err = "cannot write " + path; return false; }
    f.write(w.d.data(), (std::streamsize)w.d.size());
    if (!f) { err = "cannot write " + path; return false; }
    return true;
}

bool scene_from_desc(const vedo_scene_desc* d, HScene& s, std::string& err) {
    if (!d) { err = "null scene"; return false; }
    s.time_start = d->time_start; s.time_stop = d->time_stop; s.time_interval = d->time_interval;
    s.time_current = d->time_current;
    for (int k = 0; k < 3; ++k) {
        s.g[k] = d->field_acceleration[k];
        s.zoi_switch[k] = d->zoi_switch[k]; s.pbc_switch[k] = d->pbc_switch[k];
        s.zoi_lower[k] = d->zoi_lower[k]; s.zoi_upper[k] = d->zoi_upper[k];
        s.pbc_lower[k] = d->pbc_lower[k]; s.pbc_upper[k] = d->pbc_upper[k];
    }
    s.safety_factor = d->safety_factor;
    s.max_id_of_do = d->max_id_of_do;
    if (d->num_models && !d->models) { err = "models pointer is null"; return false; }
    s.models.resize(d->num_models);
    for (uint32_t k = 0; k < d->num_models; ++k) {
        const vedo_do_model& m = d->models[k];
        HModel& h = s.models[k];
        h.name = m.name ? m.name : "";
        h.group = m.group ? m.group : "";
        h.behavior = m.behavior; h.scope = m.scope; h.shape = m.shape;
        h.density = m.density; h.density_factor = m.density_factor;
        for (int q = 0; q < 3; ++q) h.ext[q] = m.external_force[q];
        for (int q = 0; q < 10; ++q) h.attrs[q] = m.attrs[q];
    }
    if (d->num_iact_models && !d->iact_models) { err = "iact_models pointer is null"; return false; }
    s.iacts.resize(d->num_iact_models);
    for (uint32_t k = 0; k < d->num_iact_models; ++k) {
        const vedo_iact_model& m = d->iact_models[k];
        HIact& h = s.iacts[k];
        h.master_group = m.master_group ? m.master_group : "";
        h.slave_group = m.slave_group ? m.slave_group : "";
        h.equation_type = m.equation_type ? m.equation_type : "";
        for (uint32_t q = 0; q < m.num_mechanisms; ++q) h.mech.push_back({m.mechanism_names[q], m.mechanism_values[q]});
    }
    uint32_t n = d->num_objects;
    s.n = n;
    if (n && (!d->object_model || !d->position || !d->velocity || !d->orientation_x || !d->orientation_z ||
              !d->angular_velocity)) {
        err = "object arrays must not be null";
        return false;
    }
    s.model_of.assign(d->object_model, d->object_model + n);
    if (d->object_id) s.ids.assign(d->object_id, d->object_id + n); else s.ids.assign(n, 0u);
    auto cp = [n](const double* p, std::vector<double>& v) {
        if (p) v.assign(p, p + 3 * (size_t)n); else v.assign(3 * (size_t)n, 0.0);
    };
    cp(d->position, s.pos); cp(d->velocity, s.vel); cp(d->orientation_x, s.ox); cp(d->orientation_z, s.oz);
    cp(d->angular_velocity, s.av); cp(d->impact, s.imp); cp(d->angular_impact, s.aimp);
    for (uint32_t i = 0; i < n; ++i)
        if (s.model_of[i] >= s.models.size()) { err = "object model index out of range"; return false; }
    HRecords& R = s.rec;
    uint32_t nr = d->num_records;
    if (nr && (!d->record_first || !d->record_second)) { err = "record pointers must not be null"; return false; }
    for (uint32_t q = 0; q < nr; ++q) {
        R.first.push_back(d->record_first[q]); R.second.push_back(d->record_second[q]);
        R.contact.push_back(d->record_contact ? d->record_contact[q] : 0);
        R.bond.push_back(d->record_bond ? d->record_bond[q] : 0);
        R.kn.push_back(d->record_kn ? d->record_kn[q] : 0.0);
        R.v0.push_back(d->record_initial_velocity ? d->record_initial_velocity[q] : 0.0);
        for (int k = 0; k < 3; ++k) {
            R.shear.push_back(d->record_shear ? d->record_shear[3 * q + k] : 0.0);
            R.point.push_back(0.0); R.dirn.push_back(0.0); R.imp.push_back(0.0); R.aimp.push_back(0.0);
        }
        R.overlap.push_back(0.0);
    }
    return true;
}

// ------------------------------------------------------------------------------------
namespace {
void correct_boundary(uint8_t sw[3], double lo[3], double hi[3]) {
    for (int k = 0; k < 3; ++k) {
        const double a = std::min(lo[k], hi[k]), b = std::max(lo[k], hi[k]);
        lo[k] = a;
        hi[k] = b;
        sw[k] = a != b ? 1 : 0;
    }
}
}  // namespace

std::vector<uint32_t> zoi_outside(const HScene& s, std::vector<uint32_t>& jump) {
    std::vector<uint32_t> erased;
    jump.assign(s.n, 0u);
    if (!(s.zoi_switch[0] || s.zoi_switch[1] || s.zoi_switch[2])) return erased;
    // Boundary::InBoundary (Boundary.cpp:161-190): outside when below or above a switched axis
    auto inside = [&](uint32_t i) {
        for (int k = 0; k < 3; ++k) {
            const double p = s.pos[3 * (size_t)i + k];
            if (s.zoi_switch[k] && (p < s.zoi_lower[k] || p > s.zoi_upper[k])) return false;
        }
        return true;
    };
    // ElementMappingJump: minus the number of erased objects up to and including this one
    // (unsigned, as the reference's _uint_t arithmetic)
    uint32_t dead = 0;
    for (uint32_t i = 0; i < s.n; ++i) {
        const uint32_t m = s.model_of[i];
        if (m < s.models.size() && s.models[m].behavior == VEDO_MOBILE && !inside(i)) {
            erased.push_back(i);
            --dead;
        }
        jump[i] = dead;
    }
    return erased;
}

std::vector<std::pair<std::pair<uint32_t, uint32_t>, size_t>> modify_pair(
    const std::vector<std::pair<uint32_t, uint32_t>>& keys, const std::vector<uint32_t>& jump) {
    // every record whose key changes is moved to its new key, overwriting whatever is there (in
    // key order); records of erased objects are re-keyed the same way
    using Key = std::pair<uint32_t, uint32_t>;
    const uint32_t n = (uint32_t)jump.size();
    std::map<Key, size_t> tab;
    for (size_t q = 0; q < keys.size(); ++q) tab[keys[q]] = q;
    auto j = [&](uint32_t id) { return id < n ? jump[id] : 0u; };   // std::map::operator[] default
    std::vector<Key> gone;
    std::map<Key, size_t> extra;
    for (const auto& kv : tab) {
        const Key nk(kv.first.first + j(kv.first.first), kv.first.second + j(kv.first.second));
        if (nk != kv.first) {
            gone.push_back(kv.first);
            extra[nk] = kv.second;
        }
    }
    for (const Key& k : gone) tab.erase(k);
    for (const auto& kv : extra) tab[kv.first] = kv.second;
    return std::vector<std::pair<Key, size_t>>(tab.begin(), tab.end());
}

void erase_objects(HScene& s, const std::vector<uint32_t>& erased) {
    std::vector<uint8_t> keep(s.n, 1);
    for (uint32_t i : erased) keep[i] = 0;
    uint32_t w = 0;
    for (uint32_t i = 0; i < s.n; ++i) {
        if (!keep[i]) continue;
        s.model_of[w] = s.model_of[i];
        if (i < s.ids.size() && w < s.ids.size()) s.ids[w] = s.ids[i];
        for (std::vector<double>* v : {&s.pos, &s.vel, &s.ox, &s.oz, &s.av, &s.imp, &s.aimp})
            for (int k = 0; k < 3; ++k) (*v)[3 * (size_t)w + k] = (*v)[3 * (size_t)i + k];
        ++w;
    }
    s.n = w;
    s.model_of.resize(w);
    if (s.ids.size() > w) s.ids.resize(w);
    for (std::vector<double>* v : {&s.pos, &s.vel, &s.ox, &s.oz, &s.av, &s.imp, &s.aimp}) v->resize(3 * (size_t)w);
}

uint32_t prepare_scene(HScene& s) {
    correct_boundary(s.zoi_switch, s.zoi_lower, s.zoi_upper);
    correct_boundary(s.pbc_switch, s.pbc_lower, s.pbc_upper);
    std::vector<uint32_t> jump;
    const std::vector<uint32_t> erased = zoi_outside(s, jump);
    if (erased.empty()) return 0;
    HRecords& R = s.rec;
    std::vector<std::pair<uint32_t, uint32_t>> keys(R.size());
    for (size_t q = 0; q < R.size(); ++q) keys[q] = {R.first[q], R.second[q]};
    HRecords N;
    for (const auto& kv : modify_pair(keys, jump)) {
        const size_t q = kv.second;
        N.first.push_back(kv.first.first);
        N.second.push_back(kv.first.second);
        N.contact.push_back(R.contact[q]);
        N.bond.push_back(R.bond[q]);
        N.kn.push_back(R.kn[q]);
        N.v0.push_back(R.v0[q]);
        N.overlap.push_back(R.overlap[q]);
        for (int k = 0; k < 3; ++k) {
            N.shear.push_back(R.shear[3 * q + k]);
            N.point.push_back(R.point[3 * q + k]);
            N.dirn.push_back(R.dirn[3 * q + k]);
            N.imp.push_back(R.imp[3 * q + k]);
            N.aimp.push_back(R.aimp[3 * q + k]);
        }
    }
    R = std::move(N);
    erase_objects(s, erased);
    return (uint32_t)erased.size();
}

int build_tables(const HScene& s, Tables& t, std::string& err) {
    // Boundary::Correct (Boundary.cpp:79-128) as prepare_scene applied it: switched where the
    // bounds differ; range = upper - lower
    t.pbc = Periodic{};
    for (int k = 0; k < 3; ++k) {
        const double a = std::min(s.pbc_lower[k], s.pbc_upper[k]), b = std::max(s.pbc_lower[k], s.pbc_upper[k]);
        t.pbc.lo[k] = a;
        t.pbc.hi[k] = b;
        t.pbc.range[k] = b - a;
        t.pbc.sw[k] = a != b ? 1 : 0;
        t.pbc.range32[k] = a != b ? (float)(b - a) : 0.0f;
        t.pbc.on |= t.pbc.sw[k];
    }
    if (s.n == 0) { err = "empty world"; return VEDO_ERR_INVALID_SCENE; }
    const size_t nm = s.models.size();
    std::map<std::string, int> gid;
    auto group_of = [&](const std::string& g) {
        auto it = gid.find(g);
        if (it != gid.end()) return it->second;
        int id = (int)gid.size();
        gid.emplace(g, id);
        return id;
    };
    t.models.assign(nm, ModelDev{});
    for (size_t k = 0; k < nm; ++k) {
        if (!analyse(s.models[k], t.models[k])) {
            err = "model " + s.models[k].name + ": no discrete-object factory for its shape/behaviour";
            return VEDO_ERR_UNSUPPORTED_MODEL;
        }
        t.models[k].group = group_of(s.models[k].group);
    }
    std::vector<int> mg(s.iacts.size()), sg(s.iacts.size());
    for (size_t k = 0; k < s.iacts.size(); ++k) {
        mg[k] = group_of(s.iacts[k].master_group);
        sg[k] = group_of(s.iacts[k].slave_group);
    }
    const int G = (int)gid.size();
    t.ngroups = G;
    t.group_iact.assign((size_t)G * G, -1);
    for (int a = 0; a < G; ++a)
        for (int b = 0; b < G; ++b)
            for (size_t k = 0; k < s.iacts.size(); ++k)             // first match, DOWorld.cpp:297-302
                if ((mg[k] == a && sg[k] == b) || (mg[k] == b && sg[k] == a)) {
                    t.group_iact[(size_t)a * G + b] = (int)k;
                    break;
                }
    t.params.assign(nm * nm, PairParam{});
    t.geom.assign(nm * nm * 4, 0.0);
    t.hole.assign(nm * nm * 4, 0.0);
    for (size_t ms = 0; ms < nm; ++ms) {
        for (size_t mm = 0; mm < nm; ++mm) {
            const ModelDev& S = t.models[ms];
            const ModelDev& M = t.models[mm];
            PairParam& P = t.params[ms * nm + mm];
            int ia = t.group_iact[(size_t)S.group * G + M.group];
            if (ia < 0 || S.shape != SHAPE_SPHERE) continue;
            int cd = M.shape == SHAPE_SPHERE ? CD_SS : M.shape == SHAPE_PLATE ? CD_SP : M.shape == SHAPE_CYL ? CD_SC
                     : M.shape == SHAPE_HOLED ? CD_SHP : M.shape == SHAPE_INNER_CYL ? CD_SIC : 0;
            const HIact& im = s.iacts[ia];
            int is = eq_of(im.equation_type);
            if (!cd || !is) continue;                      // the factories return null (Assembler.cpp:72-85)
            P.cd = cd;
            P.is = is;
            P.iact = ia;
            double* geo = &t.geom[(ms * nm + mm) * 4];
            geo[0] = S.a0; geo[1] = M.a0; geo[2] = M.a1; geo[3] = M.a2;
            if (cd == CD_SHP)
                for (int k = 0; k < 3; ++k) t.hole[(ms * nm + mm) * 4 + k] = s.models[mm].attrs[3 + k];
            auto need = [&](const char* name, double& v) {
                if (!mech(im, name, v)) {
                    err = "interaction " + im.master_group + "/" + im.slave_group + " has no mechanism " + name;
                    return false;
                }
                return true;
            };
            if (is == IS_BSDBF || is == IS_BTSDBF || is == IS_BSDB2F) {
                // ISwBSDBF.cpp:7-19 with ISwModels::CriticalDamping (ISwModels.cpp:88-108)
                double kn, ks, ndr, sdr, bn, bs, fc;
                if (!need("NormalStiffness", kn) || !need("ShearStiffness", ks) || !need("NormalDampingRatio", ndr) ||
                    !need("ShearDampingRatio", sdr) || !need("NormalBondStrength", bn) ||
                    !need("ShearBondStrength", bs) || !need("FrictionCoefficient", fc))
                    return VEDO_ERR_INVALID_SCENE;
                double Ma = S.sudo, Mb = M.sudo, Me;
                if (Mb == 0) Me = Ma; else if (Ma == 0) Me = Mb; else Me = 0.5 * (Ma + Mb);
                double c1 = 2.0 * std::sqrt(Me * kn), c2 = 2.0 * std::sqrt(Me * ks);
                P.c[0] = kn; P.c[1] = ks; P.c[2] = ndr * c1; P.c[3] = sdr * c2; P.c[4] = bn; P.c[5] = bs; P.c[6] = fc;
            } else if (is == IS_HERTZ) {                   // ISwHertz.cpp:8-13
                if (!need("NormalStiffness", P.c[0]) || !need("NormalDampingCoefficient", P.c[1]))
                    return VEDO_ERR_INVALID_SCENE;
            } else {                                       // ISwH.cpp:8-19
                if (!need("HertzNormalStiffness", P.c[0]) || !need("EquivalentMass", P.c[1]) ||
                    !need("ShearStiffnessCoefficient1", P.c[2]) || !need("ShearStiffnessCoefficient2", P.c[3]) ||
                    !need("DampingRatio", P.c[4]) || !need("KineticFrictionCoefficient", P.c[5]))
                    return VEDO_ERR_INVALID_SCENE;
            }
        }
    }
    return VEDO_OK;
}

}  // namespace vedo
