// xml_io.cpp - DOWorldSchema XML scenes: a small XML reader (elements, attributes, comments,
// processing instructions; character data is skipped) and the mapping of DOWorld_ReadXML.cpp
// (the reference reads XML through boost::property_tree, absent here), plus a writer in the
// layout of DOWorld_WriteXML.cpp with full precision.
#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

#include "scene_host.h"

namespace vedo {
namespace {

struct XNode {
    std::string name;
    std::vector<std::pair<std::string, std::string>> attrs;
    std::vector<XNode> kids;
    const std::string* attr(const char* k) const {
        for (auto& a : attrs)
            if (a.first == k) return &a.second;
        return nullptr;
    }
    const XNode* child(const char* k) const {
        for (auto& c : kids)
            if (c.name == k) return &c;
        return nullptr;
    }
};

class XParser {
public:
    explicit XParser(const std::string& t) : s_(t) {}
    bool parse(XNode& root, std::string& err) {
        skip_misc();
        if (!element(root)) {
            err = "XML: " + msg_ + " near byte " + std::to_string(p_);
            return false;
        }
        return true;
    }

private:
    const std::string& s_;
    size_t p_ = 0;
    std::string msg_;
    bool fail(const char* m) {
        msg_ = m;
        return false;
    }
    void ws() {
        while (p_ < s_.size() && (s_[p_] == ' ' || s_[p_] == '\t' || s_[p_] == '\n' || s_[p_] == '\r')) ++p_;
    }
    bool starts(const char* t) const { return s_.compare(p_, std::strlen(t), t) == 0; }
    bool skip_to(const char* t) {
        const size_t q = s_.find(t, p_);
        if (q == std::string::npos) return false;
        p_ = q + std::strlen(t);
        return true;
    }
    // declarations, processing instructions, comments, doctype
    void skip_misc() {
        for (;;) {
            ws();
            if (starts("<?")) { if (!skip_to("?>")) return; }
            else if (starts("<!--")) { if (!skip_to("-->")) return; }
            else if (starts("<!")) { if (!skip_to(">")) return; }
            else return;
        }
    }
    static bool name_char(char c) {
        return std::isalnum((unsigned char)c) || c == '_' || c == '-' || c == '.' || c == ':';
    }
    bool name(std::string& out) {
        const size_t b = p_;
        while (p_ < s_.size() && name_char(s_[p_])) ++p_;
        if (p_ == b) return fail("a name was expected");
        out.assign(s_, b, p_ - b);
        return true;
    }
    static std::string decode(const std::string& v) {
        std::string o;
        for (size_t i = 0; i < v.size(); ++i) {
            if (v[i] != '&') { o += v[i]; continue; }
            const size_t e = v.find(';', i);
            const std::string ent = e == std::string::npos ? std::string() : v.substr(i + 1, e - i - 1);
            if (ent == "amp") o += '&';
            else if (ent == "lt") o += '<';
            else if (ent == "gt") o += '>';
            else if (ent == "quot") o += '"';
            else if (ent == "apos") o += '\'';
            else if (!ent.empty() && ent[0] == '#') o += (char)std::strtol(ent.c_str() + (ent[1] == 'x' ? 2 : 1), nullptr, ent[1] == 'x' ? 16 : 10);
            else { o += '&'; continue; }
            i = e;
        }
        return o;
    }
    bool element(XNode& n) {
        if (p_ >= s_.size() || s_[p_] != '<') return fail("'<' expected");
        ++p_;
        if (!name(n.name)) return false;
        for (;;) {
            ws();
            if (p_ >= s_.size()) return fail("unterminated tag");
            if (starts("/>")) { p_ += 2; return true; }
            if (s_[p_] == '>') { ++p_; break; }
            std::string k;
            if (!name(k)) return false;
            ws();
            if (p_ >= s_.size() || s_[p_] != '=') return fail("'=' expected");
            ++p_;
            ws();
            if (p_ >= s_.size() || (s_[p_] != '"' && s_[p_] != '\'')) return fail("quoted value expected");
            const char q = s_[p_++];
            const size_t e = s_.find(q, p_);
            if (e == std::string::npos) return fail("unterminated value");
            n.attrs.emplace_back(k, decode(s_.substr(p_, e - p_)));
            p_ = e + 1;
        }
        for (;;) {                                   // content: children, comments, text
            const size_t lt = s_.find('<', p_);
            if (lt == std::string::npos) return fail("missing closing tag");
            p_ = lt;
            if (starts("</")) {
                p_ += 2;
                std::string k;
                if (!name(k)) return false;
                if (k != n.name) return fail("mismatched closing tag");
                ws();
                if (p_ >= s_.size() || s_[p_] != '>') return fail("'>' expected");
                ++p_;
                return true;
            }
            if (starts("<!--")) { if (!skip_to("-->")) return fail("unterminated comment"); continue; }
            if (starts("<![CDATA[")) { if (!skip_to("]]>")) return fail("unterminated CDATA"); continue; }
            if (starts("<?")) { if (!skip_to("?>")) return fail("unterminated instruction"); continue; }
            n.kids.emplace_back();
            if (!element(n.kids.back())) return false;
        }
    }
};

struct Mapper {
    std::string err;
    bool num(const XNode& n, const char* k, double& v, bool required = true, double dflt = 0.0) {
        const std::string* a = n.attr(k);
        if (!a) {
            if (required) {
                err = "XML: <" + n.name + "> has no attribute " + k;
                return false;
            }
            v = dflt;
            return true;
        }
        char* end = nullptr;
        errno = 0;
        v = std::strtod(a->c_str(), &end);
        while (end && (*end == ' ' || *end == '\t')) ++end;
        if (end == a->c_str() || (end && *end) || errno == ERANGE) {
            err = "XML: <" + n.name + "> attribute " + k + " is not a number: " + *a;
            return false;
        }
        return true;
    }
    bool u32(const XNode& n, const char* k, uint32_t& v) {
        double d;
        if (!num(n, k, d)) return false;
        v = (uint32_t)d;
        return true;
    }
    bool vec(const XNode* n, const char* what, double* out) {     // Node2Vector3d
        if (!n) {
            err = std::string("XML: <") + what + "> missing";
            return false;
        }
        return num(*n, "x", out[0]) && num(*n, "y", out[1]) && num(*n, "z", out[2]);
    }
    bool vec_opt(const XNode* parent, const char* what, double* out) {
        const XNode* n = parent->child(what);
        if (!n) { out[0] = out[1] = out[2] = 0.0; return true; }
        return vec(n, what, out);
    }
};

// DOWorld_ReadXML.cpp:216-299 (Node2SystemParameter)
bool sim_parameter(Mapper& M, const XNode& sp, HScene& s) {
    s.safety_factor = 1.1;
    if (const XNode* sc = sp.child("SimConstant"))
        for (const XNode& c : sc->kids) {
            const std::string* nm = c.attr("Name");
            if (nm && *nm == "SafetyFactor") {                 // ContactDetectSafetyFactor is not read
                double v;
                if (!M.num(c, "Value", v)) return false;
                s.safety_factor = std::max(1.0, v);
            }
        }
    if (!M.vec(sp.child("FieldAcceleration"), "FieldAcceleration", s.g)) return false;
    const XNode* tc = sp.child("TimeControl");
    if (!tc) { M.err = "XML: <TimeControl> missing"; return false; }
    if (!M.num(*tc, "Start", s.time_start) || !M.num(*tc, "Stop", s.time_stop) ||
        !M.num(*tc, "Interval", s.time_interval) || !M.num(*tc, "Current", s.time_current))
        return false;
    auto boundary = [&](const char* tag, double* lo, double* hi, uint8_t* sw) -> bool {
        double a[3] = {0, 0, 0}, b[3] = {0, 0, 0};
        if (const XNode* z = sp.child(tag)) {
            const char* kl[3] = {"XMin", "YMin", "ZMin"};
            const char* ku[3] = {"XMax", "YMax", "ZMax"};
            for (int k = 0; k < 3; ++k)
                if (!M.num(*z, kl[k], a[k], false) || !M.num(*z, ku[k], b[k], false)) return false;
        }
        for (int k = 0; k < 3; ++k) {                  // Boundary::Correct (Boundary.cpp:79-120)
            lo[k] = std::min(a[k], b[k]);
            hi[k] = std::max(a[k], b[k]);
            sw[k] = lo[k] == hi[k] ? 0 : 1;
        }
        return true;
    };
    return boundary("ZOI", s.zoi_lower, s.zoi_upper, s.zoi_switch) &&
           boundary("PBC", s.pbc_lower, s.pbc_upper, s.pbc_switch);
}

// DOWorld_ReadXML.cpp:84-214 (Node2DOShapeTypeAndAttributes), 407-468 (Node2DOModel)
bool do_model(Mapper& M, const XNode& n, HModel& m) {
    const std::string* nm = n.attr("DOName");
    const std::string* gr = n.attr("DOGroup");
    const std::string* be = n.attr("Behavior");
    if (!nm || !gr || !be) { M.err = "XML: <DOModel> needs DOName, DOGroup and Behavior"; return false; }
    m.name = *nm;
    m.group = *gr;
    if (!M.num(n, "Density", m.density) || !M.num(n, "DensityFactor", m.density_factor, false, 1.0)) return false;
    if (*be == "constrained") m.behavior = 1;
    else if (*be == "fixed") m.behavior = 2;
    else if (*be == "mobile") m.behavior = 3;
    else if (*be == "orbital") m.behavior = 4;
    else { M.err = "XML: Behavior \"" + *be + "\" is illegal"; return false; }
    const std::string* co = n.attr("Color");
    const std::string c = co ? *co : "bylayer";
    m.color = c == "red" ? 1 : c == "yellow" ? 2 : c == "green" ? 3 : c == "cyan" ? 4 : c == "blue" ? 5
            : c == "magenta" ? 6 : 256;
    const std::string* sc = n.attr("Scope");
    const std::string sv = sc ? *sc : "undefined";
    if (sv == "local") m.scope = 2;
    else if (sv == "global") m.scope = 1;
    else if (sv == "undefined") m.scope = m.behavior == 3 ? 2 : 1;
    else { M.err = "XML: Scope \"" + sv + "\" is illegal"; return false; }
    if (!M.vec_opt(&n, "ExternalForce", m.ext)) return false;
    for (double& a : m.attrs) a = 0.0;
    const XNode* sh = n.child("Shape");
    const XNode* x = nullptr;
    if (sh && (x = sh->child("Sphere"))) {
        m.shape = 1;
        if (!M.num(*x, "Radius", m.attrs[0], false)) return false;
        if (m.attrs[0] <= 0.0) { M.err = "XML: sphere radius must be positive"; return false; }
    } else if (sh && (x = sh->child("Triangle"))) {
        m.shape = 9;
        const char* k[9] = {"Point0X", "Point0Y", "Point0Z", "Point1X", "Point1Y", "Point1Z", "Point2X", "Point2Y", "Point2Z"};
        for (int q = 0; q < 9; ++q)
            if (!M.num(*x, k[q], m.attrs[1 + q], false)) return false;
    } else if (sh && (x = sh->child("QuasiPlate"))) {
        m.shape = 7;
        if (!M.num(*x, "Width", m.attrs[0], false) || !M.num(*x, "Height", m.attrs[1], false) ||
            !M.num(*x, "Length", m.attrs[2], false))
            return false;
    } else if (sh && (x = sh->child("QuasiPlateWithCircularHole"))) {
        m.shape = 8;
        const char* k[6] = {"Width", "Height", "Length", "HoleRadius", "HoleXOffset", "HoleYOffset"};
        for (int q = 0; q < 6; ++q)
            if (!M.num(*x, k[q], m.attrs[q], false)) return false;
    } else if (sh && (x = sh->child("QuasiCylinder"))) {
        m.shape = 6;
        if (!M.num(*x, "Radius", m.attrs[0], false) || !M.num(*x, "Height", m.attrs[1], false)) return false;
    } else if (sh && (x = sh->child("Ellipsoid"))) {
        m.shape = 3;
        if (!M.num(*x, "XLength", m.attrs[0], false) || !M.num(*x, "YLength", m.attrs[1], false) ||
            !M.num(*x, "ZLength", m.attrs[2], false))
            return false;
    } else if (sh && (sh->child("Polyhedra") || sh->child("DMSphere") || sh->child("polyhedrabrep"))) {
        M.err = "XML: polyhedra and DM spheres are not supported";
        return false;
    } else {
        M.err = "XML: <DOModel " + m.name + "> has no supported <Shape>";
        return false;
    }
    m.materials.clear();
    if (const XNode* mo = n.child("MaterialOption"))
        for (const XNode& o : mo->kids) {
            const std::string* on = o.attr("Name");
            double v;
            if (!on || !M.num(o, "Value", v)) { M.err = "XML: <MaterialOption> entry needs Name and Value"; return false; }
            m.materials.push_back({*on, v});
        }
    return true;
}

// DOWorld_ReadXML.cpp:470-498 (Node2IactModel): every child but the attributes is a mechanism
bool iact_model(Mapper& M, const XNode& n, HIact& im) {
    const std::string* ma = n.attr("MasterGroup");
    const std::string* sl = n.attr("SlaveGroup");
    const std::string* eq = n.attr("EquationType");
    if (!ma || !sl || !eq) { M.err = "XML: <IactModel> needs MasterGroup, SlaveGroup and EquationType"; return false; }
    im.master_group = *ma;
    im.slave_group = *sl;
    im.equation_type = *eq;
    for (const XNode& c : n.kids) {
        const std::string* nm = c.attr("Name");
        double v;
        if (!nm || !M.num(c, "Value", v)) { M.err = "XML: <" + c.name + "> in <IactModel> needs Name and Value"; return false; }
        im.mech.push_back({*nm, v});
    }
    return true;
}

}  // namespace

// DOWorld::ReadXML (DOWorld_ReadXML.cpp:592-660) with the IactRecordTab
bool read_xml(const std::string& path, HScene& s, std::string& err) {
    std::ifstream f(path, std::ios::binary);
    if (!f) { err = "cannot open " + path; return false; }
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string text = ss.str();
    XNode root;
    XParser P(text);
    if (!P.parse(root, err)) return false;
    if (root.name != "DOWorld") { err = "XML: the root element is not <DOWorld>"; return false; }
    Mapper M;
    s = HScene();
    const XNode* sp = root.child("SimParameter");
    if (!sp) { err = "XML: <SimParameter> missing"; return false; }
    if (!sim_parameter(M, *sp, s)) { err = M.err; return false; }
    if (const XNode* t = root.child("DOModelTab"))
        for (const XNode& c : t->kids) {
            HModel m;
            if (!do_model(M, c, m)) { err = M.err; return false; }
            s.models.push_back(m);
        }
    if (const XNode* t = root.child("IactModelTab"))
        for (const XNode& c : t->kids) {
            HIact im;
            if (!iact_model(M, c, im)) { err = M.err; return false; }
            s.iacts.push_back(im);
        }
    if (const XNode* t = root.child("DOStatusTab"))
        for (const XNode& c : t->kids) {                // Node2DOStatus (DOWorld_ReadXML.cpp:500-534)
            const std::string* dn = c.attr("DOName");
            if (!dn) { err = "XML: <DOStatus> needs DOName"; return false; }
            uint32_t mi = 0;
            while (mi < s.models.size() && s.models[mi].name != *dn) ++mi;
            if (mi == s.models.size()) { err = "XML: DOStatus of unknown DOModel " + *dn; return false; }
            double v[7][3];
            const char* tags[5] = {"Position", "Velocity", "OrientationX", "OrientationZ", "AngularVelocity"};
            for (int k = 0; k < 5; ++k)
                if (!M.vec(c.child(tags[k]), tags[k], v[k])) { err = M.err; return false; }
            if (!M.vec_opt(&c, "Impact", v[5]) || !M.vec_opt(&c, "AngularImpact", v[6])) { err = M.err; return false; }
            std::vector<double>* dst[7] = {&s.pos, &s.vel, &s.ox, &s.oz, &s.av, &s.imp, &s.aimp};
            for (int k = 0; k < 7; ++k) dst[k]->insert(dst[k]->end(), v[k], v[k] + 3);
            s.model_of.push_back(mi);
            s.ids.push_back(s.n);
            ++s.n;
        }
    s.max_id_of_do = s.n;
    if (const XNode* t = root.child("IactStatusTab"))
        for (const XNode& c : t->kids) {                // Node2IactStatus (DOWorld_ReadXML.cpp:536-590)
            uint32_t a = 0, b = 0, con = 0, bond = 0;
            double kn = 0, v0 = 0, ov = 0, sh[3], pt[3], dr[3], im[3], am[3];
            if (!M.u32(c, "MasterDOStatusSN", a) || !M.u32(c, "SlaveDOStatusSN", b) || !M.u32(c, "Contact", con) ||
                !M.u32(c, "Bond", bond) || !M.num(c, "NormalStiffness", kn) || !M.num(c, "InitialVelocity", v0) ||
                !M.num(c, "Overlap", ov) || !M.vec(c.child("ShearForce"), "ShearForce", sh) ||
                !M.vec(c.child("ImpactPoint"), "ImpactPoint", pt) ||
                !M.vec(c.child("ImpactDirection"), "ImpactDirection", dr) ||
                !M.vec(c.child("ImpactToMaster"), "ImpactToMaster", im) ||
                !M.vec(c.child("AngularImpactToMaster"), "AngularImpactToMaster", am)) {
                err = M.err;
                return false;
            }
            HRecords& R = s.rec;
            R.first.push_back(a);
            R.second.push_back(b);
            R.contact.push_back(con ? 1 : 0);
            R.bond.push_back(bond ? 1 : 0);
            R.kn.push_back(kn);
            R.v0.push_back(v0);
            R.overlap.push_back(ov);
            R.shear.insert(R.shear.end(), sh, sh + 3);
            R.point.insert(R.point.end(), pt, pt + 3);
            R.dirn.insert(R.dirn.end(), dr, dr + 3);
            R.imp.insert(R.imp.end(), im, im + 3);
            R.aimp.insert(R.aimp.end(), am, am + 3);
        }
    return true;
}

// DOWorld::WriteXML (DOWorld_WriteXML.cpp:17-498) layout, every value with 17 significant digits
bool write_xml(const std::string& path, const HScene& s, std::string& err) {
    std::ofstream o(path);
    if (!o) { err = "cannot write " + path; return false; }
    char b[64];
    auto f = [&](double v) {
        std::snprintf(b, sizeof(b), "%.17g", v);
        return std::string(b);
    };
    auto vec = [&](const char* tag, const double* v, const char* ind) {
        o << ind << "<" << tag << " x=\"" << f(v[0]) << "\" y=\"" << f(v[1]) << "\" z=\"" << f(v[2]) << "\"/>\n";
    };
    o << "<?xml version=\"1.0\" encoding=\"UTF-8\"?>\n<DOWorld>\n\t<SimParameter>\n\t\t<SimConstant>\n"
      << "\t\t\t<Constant Name=\"SafetyFactor\" Value=\"" << f(s.safety_factor) << "\"/>\n"
      << "\t\t\t<Constant Name=\"MaxIDofDOStatus\" Value=\"" << s.max_id_of_do << "\"/>\n\t\t</SimConstant>\n"
      << "\t\t<TimeControl Start=\"" << f(s.time_start) << "\" Stop=\"" << f(s.time_stop) << "\" Interval=\""
      << f(s.time_interval) << "\" Current=\"" << f(s.time_current) << "\"/>\n";
    vec("FieldAcceleration", s.g, "\t\t");
    auto boundary = [&](const char* tag, const double* lo, const double* hi, const uint8_t* sw) {
        if (!sw[0] && !sw[1] && !sw[2]) return;
        o << "\t\t<" << tag << " XMin=\"" << f(lo[0]) << "\" YMin=\"" << f(lo[1]) << "\" ZMin=\"" << f(lo[2])
          << "\" XMax=\"" << f(hi[0]) << "\" YMax=\"" << f(hi[1]) << "\" ZMax=\"" << f(hi[2]) << "\"/>\n";
    };
    boundary("ZOI", s.zoi_lower, s.zoi_upper, s.zoi_switch);
    boundary("PBC", s.pbc_lower, s.pbc_upper, s.pbc_switch);
    o << "\t</SimParameter>\n\t<DOModelTab>\n";
    const char* beh[5] = {"", "constrained", "fixed", "mobile", "orbital"};
    for (const HModel& m : s.models) {
        const char* col = m.color == 1 ? "red" : m.color == 2 ? "yellow" : m.color == 3 ? "green" : m.color == 4 ? "cyan"
                        : m.color == 5 ? "blue" : m.color == 6 ? "magenta" : "bylayer";
        o << "\t\t<DOModel DOName=\"" << m.name << "\" DOGroup=\"" << m.group << "\" Behavior=\""
          << (m.behavior < 5 ? beh[m.behavior] : "") << "\" Scope=\"" << (m.scope == 2 ? "local" : "global")
          << "\" Color=\"" << col << "\" Density=\"" << f(m.density) << "\" DensityFactor=\"" << f(m.density_factor)
          << "\">\n";
        vec("ExternalForce", m.ext, "\t\t\t");
        o << "\t\t\t<Shape>";
        const double* a = m.attrs;
        switch (m.shape) {
        case 1: o << "<Sphere Radius=\"" << f(a[0]) << "\"/>"; break;
        case 3: o << "<Ellipsoid XLength=\"" << f(a[0]) << "\" YLength=\"" << f(a[1]) << "\" ZLength=\"" << f(a[2]) << "\"/>"; break;
        case 6: o << "<QuasiCylinder Radius=\"" << f(a[0]) << "\" Height=\"" << f(a[1]) << "\"/>"; break;
        case 7: o << "<QuasiPlate Width=\"" << f(a[0]) << "\" Length=\"" << f(a[2]) << "\" Height=\"" << f(a[1]) << "\"/>"; break;
        case 8:
            o << "<QuasiPlateWithCircularHole Width=\"" << f(a[0]) << "\" Length=\"" << f(a[2]) << "\" Height=\"" << f(a[1])
              << "\" HoleRadius=\"" << f(a[3]) << "\" HoleXOffset=\"" << f(a[4]) << "\" HoleYOffset=\"" << f(a[5]) << "\"/>";
            break;
        case 9:
            o << "<Triangle Point0X=\"" << f(a[1]) << "\" Point0Y=\"" << f(a[2]) << "\" Point0Z=\"" << f(a[3]) << "\" Point1X=\""
              << f(a[4]) << "\" Point1Y=\"" << f(a[5]) << "\" Point1Z=\"" << f(a[6]) << "\" Point2X=\"" << f(a[7])
              << "\" Point2Y=\"" << f(a[8]) << "\" Point2Z=\"" << f(a[9]) << "\"/>";
            break;
        default: err = "XML: shape " + std::to_string(m.shape) + " cannot be written"; return false;
        }
        o << "</Shape>\n";
        if (!m.materials.empty()) {
            o << "\t\t\t<MaterialOption>\n";
            for (auto& p : m.materials) o << "\t\t\t\t<Option Name=\"" << p.first << "\" Value=\"" << f(p.second) << "\"/>\n";
            o << "\t\t\t</MaterialOption>\n";
        }
        o << "\t\t</DOModel>\n";
    }
    o << "\t</DOModelTab>\n\t<IactModelTab>\n";
    for (const HIact& im : s.iacts) {
        o << "\t\t<IactModel MasterGroup=\"" << im.master_group << "\" SlaveGroup=\"" << im.slave_group
          << "\" EquationType=\"" << im.equation_type << "\">\n";
        for (auto& p : im.mech) o << "\t\t\t<Mechanism Name=\"" << p.first << "\" Value=\"" << f(p.second) << "\"/>\n";
        o << "\t\t</IactModel>\n";
    }
    o << "\t</IactModelTab>\n\t<DOStatusTab>\n";
    for (uint32_t i = 0; i < s.n; ++i) {
        o << "\t\t<DOStatus DOName=\"" << s.models[s.model_of[i]].name << "\">\n";
        vec("Position", &s.pos[3 * (size_t)i], "\t\t\t");
        vec("Velocity", &s.vel[3 * (size_t)i], "\t\t\t");
        vec("OrientationX", &s.ox[3 * (size_t)i], "\t\t\t");
        vec("OrientationZ", &s.oz[3 * (size_t)i], "\t\t\t");
        vec("AngularVelocity", &s.av[3 * (size_t)i], "\t\t\t");
        vec("Impact", &s.imp[3 * (size_t)i], "\t\t\t");
        vec("AngularImpact", &s.aimp[3 * (size_t)i], "\t\t\t");
        o << "\t\t</DOStatus>\n";
    }
    o << "\t</DOStatusTab>\n";
    const HRecords& R = s.rec;
    if (R.size()) {
        o << "\t<IactStatusTab>\n";
        for (size_t k = 0; k < R.size(); ++k) {
            o << "\t\t<IactStatus MasterDOStatusSN=\"" << R.first[k] << "\" SlaveDOStatusSN=\"" << R.second[k]
              << "\" Contact=\"" << (int)R.contact[k] << "\" Bond=\"" << (int)R.bond[k] << "\" NormalStiffness=\""
              << f(R.kn[k]) << "\" InitialVelocity=\"" << f(R.v0[k]) << "\" Overlap=\"" << f(R.overlap[k]) << "\">\n";
            vec("ShearForce", &R.shear[3 * k], "\t\t\t");
            vec("ImpactPoint", &R.point[3 * k], "\t\t\t");
            vec("ImpactDirection", &R.dirn[3 * k], "\t\t\t");
            vec("ImpactToMaster", &R.imp[3 * k], "\t\t\t");
            vec("AngularImpactToMaster", &R.aimp[3 * k], "\t\t\t");
            o << "\t\t</IactStatus>\n";
        }
        o << "\t</IactStatusTab>\n";
    }
    o << "</DOWorld>\n";
    if (!o) { err = "write failed: " + path; return false; }
    return true;
}

}  // namespace vedo
