// VXA/VXD reading, material derivation and topology construction.
//
// The reading rules follow the reference's reader chain: CVX_Sim::ReadXML
// (Voxelyze3/src/VXA/VX_Sim.cpp:185-258), CVX_Environment::ReadXML
// (Voxelyze3/src/old/VX_Environment.cpp:101-175), the VXC palette and structure
// readers (Voxelyze3/src/VXA/VX_Object.cpp:446-500, 1373-1460, 1760-1860) and
// CVX_Sim::Import (VX_Sim.cpp:59-153), including its quirks: gravity is always
// GravAcc (SetGravityAccel runs after the GravEnabled switch), and Poisson's
// ratio is forced to zero unless Features/VolumeEffectsEnabled is set.
// Numbers are converted with strtod exactly like the reference's atof, then
// narrowed to float where the reference stores float.
#include "world.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdlib>
#include <charconv>
#include <cstring>
#include <deque>
#include <unordered_map>

namespace gvx {

// atof of the field starting at p (raw text ends at e).  A plain decimal field is read
// with std::from_chars, which rounds correctly like strtod and so gives the same double,
// several times faster on long digit strings; any other form (leading blanks or '+',
// hexadecimal, out of range, trailing text) goes to atof itself.
double field_atof(const char* p, const char* e) {
    double v;
    const auto r = std::from_chars(p, e, v);
    if (r.ec == std::errc() && (r.ptr == e || *r.ptr == ',')) return v;
    return atof(p);
}

namespace {

double atof_s(const std::string& s) { return atof(s.c_str()); }

// Start of every comma-separated field of raw, in order.  atof of a field's start reads
// the same number as atof of the field cut out: a number never runs on through a comma.
void comma_fields(const std::string& raw, std::vector<const char*>* out) {
    const char* p = raw.c_str();
    const char* e = p + raw.size();
    for (;;) {
        out->push_back(p);
        const char* c = (const char*)memchr(p, ',', (size_t)(e - p));
        if (!c) break;
        p = c + 1;
    }
}
int atoi_s(const std::string& s) { return atoi(s.c_str()); }

bool load_d(const XmlNode* el, const char* tag, double* out) {
    if (!el) return false;
    const XmlNode* c = el->child(tag);
    if (!c) return false;
    *out = atof_s(c->text);
    return true;
}
bool load_i(const XmlNode* el, const char* tag, int* out) {
    if (!el) return false;
    const XmlNode* c = el->child(tag);
    if (!c) return false;
    *out = atoi_s(c->text);
    return true;
}
double get_d(const XmlNode* el, const char* tag, double def) { double v; return load_d(el, tag, &v) ? v : def; }
float get_f(const XmlNode* el, const char* tag, double def) { double v; return load_d(el, tag, &v) ? (float)v : (float)def; }
int get_i(const XmlNode* el, const char* tag, int def) { int v; return load_i(el, tag, &v) ? v : def; }
bool get_b(const XmlNode* el, const char* tag, bool def) { int v; return load_i(el, tag, &v) ? v != 0 : def; }

std::string trim(const std::string& s) {
    size_t b = 0, e = s.size();
    while (b < e && isspace((unsigned char)s[b])) b++;
    while (e > b && isspace((unsigned char)s[e - 1])) e--;
    return s.substr(b, e - b);
}
// boost::property_tree get<bool>/get<double> with a default
bool ptree_bool(const XmlNode& root, const char* path, bool def) {
    const XmlNode* n = root.path(path);
    if (!n) return def;
    std::string t = trim(n->text);
    if (t == "1" || t == "true") return true;
    if (t == "0" || t == "false") return false;
    return def;
}
double ptree_num(const XmlNode& root, const char* path, double def) {
    const XmlNode* n = root.path(path);
    if (!n) return def;
    std::string t = trim(n->text);
    char* end = nullptr;
    double v = strtod(t.c_str(), &end);
    if (t.empty() || (end && *end)) return def;
    return v;
}

std::string b64decode(const std::string& in) {
    static const std::string chars = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";
    std::string out;
    int val = 0, bits = -8;
    for (unsigned char c : in) {
        if (c == '=') break;
        size_t p = chars.find(c);
        if (p == std::string::npos) continue;
        val = (val << 6) + (int)p;
        bits += 6;
        if (bits >= 0) { out.push_back(char((val >> bits) & 0xFF)); bits -= 8; }
    }
    return out;
}

// ParseMathTree: breadth-first walk, reversed, with mtEND last.
void parse_mathtree(const XmlNode* node, MathTree* m) {
    m->n = 0;
    m->valid = 1;
    if (!node) return;
    std::vector<std::pair<std::string, std::string>> bfs;
    std::deque<const XmlNode*> frontier{node};
    while (!frontier.empty()) {
        const XmlNode* t = frontier.front();
        frontier.pop_front();
        for (auto& c : t->children) {
            std::string v = c->text;
            while (!v.empty() && isspace((unsigned char)v.back())) v.pop_back();
            bfs.emplace_back(c->tag, v);
            frontier.push_back(c.get());
        }
    }
    if ((int)bfs.size() + 1 > kMaxMathTokens) { m->valid = 0; return; }
    static const char* names[] = {"mtEND", "mtCONST", "mtE", "mtPI", "mtVAR", "mtADD", "mtSUB", "mtMUL", "mtDIV",
                                  "mtPOW", "mtSQRT", "mtSIN", "mtCOS", "mtTAN", "mtATAN", "mtLOG", "mtINT", "mtABS",
                                  "mtNOT", "mtGREATERTHAN", "mtLESSTHAN", "mtAND", "mtOR", "mtNORMALCDF"};
    static const char* vars[] = {"x", "y", "z", "hit", "t", "angle", "targetCloseness", "numClosePairs", "num_voxel"};
    int k = 0;
    for (int i = (int)bfs.size() - 1; i >= 0; i--) {
        MathToken& t = m->tok[k++];
        t.op = -1;
        t.pad = 0;
        t.value = 0;
        for (int o = 0; o < (int)(sizeof(names) / sizeof(names[0])); o++)
            if (bfs[i].first == names[o]) t.op = o;
        if (t.op < 0) { m->valid = 0; t.op = mtEND; }
        if (t.op == mtVAR) {
            int vi = -1;
            for (int q = 0; q < 9; q++) if (trim(bfs[i].second) == vars[q]) vi = q;
            if (vi < 0) m->valid = 0;
            t.value = vi;
        } else if (t.op == mtCONST) {
            char* end = nullptr;
            std::string s = trim(bfs[i].second);
            t.value = strtod(s.c_str(), &end);
            if (s.empty()) m->valid = 0;
        }
    }
    m->tok[k].op = mtEND;
    m->tok[k].value = 0;
    m->n = k + 1;
}

// ------------------------------------------------------------ boundary conditions
// A region of the environment (CVX_FRegion, Voxelyze3/src/old/VX_FRegion.h:40-120) in
// workspace-relative units, with what it does to the voxels it touches.
struct BCRegion {
    int prim = 0;                                  // PRIM_BOX 0, PRIM_CYLINDER 1, PRIM_SPHERE 2 (VX_FRegion.h:25-28)
    double X = 0, Y = 0, Z = 0, dX = 0, dY = 0, dZ = 0, radius = 0;
    int dof = 0;                                   // DOF_X 0x01 .. DOF_TZ 0x20
    double force[3] = {0, 0, 0}, torque[3] = {0, 0, 0}, disp[3] = {0, 0, 0}, ang[3] = {0, 0, 0};
};

// CVX_FRegion::ReadXML (VX_FRegion.cpp:165-216)
bool read_region(const XmlNode* fr, BCRegion* r, std::string* err) {
    int prim;
    if (!load_i(fr, "PrimType", &prim)) { *err = "boundary condition region without PrimType"; return false; }
    if (prim == 3) { *err = "mesh boundary-condition regions are not supported"; return false; }
    if (prim < 0 || prim > 3) { *err = "unknown boundary-condition PrimType"; return false; }
    r->prim = prim;
    r->X = get_d(fr, "X", 0); r->Y = get_d(fr, "Y", 0); r->Z = get_d(fr, "Z", 0);
    r->dX = get_d(fr, "dX", 0); r->dY = get_d(fr, "dY", 0); r->dZ = get_d(fr, "dZ", 0);
    r->radius = get_d(fr, "Radius", 0);
    int dof;
    if (load_i(fr, "DofFixed", &dof)) r->dof = (int)(char)dof;
    else r->dof = get_b(fr, "Fixed", false) ? 0x3F : 0;   // older files: a binary Fixed tag
    const char* f[3] = {"ForceX", "ForceY", "ForceZ"}, *t[3] = {"TorqueX", "TorqueY", "TorqueZ"};
    const char* dd[3] = {"DisplaceX", "DisplaceY", "DisplaceZ"}, *a[3] = {"AngDisplaceX", "AngDisplaceY", "AngDisplaceZ"};
    for (int k = 0; k < 3; k++) {
        r->force[k] = get_d(fr, f[k], 0); r->torque[k] = get_d(fr, t[k], 0);
        r->disp[k] = get_d(fr, dd[k], 0); r->ang[k] = get_d(fr, a[k], 0);
    }
    return true;
}

// CPrimitive::IsTouching(P, Dist vector, Envelope) for box, cylinder and sphere
// (VX_FRegion.cpp:420-429, 495-534, 591-604); P and Dist in meters, Env = workspace size.
bool region_touching(const BCRegion& r, const double P[3], const double D[3], const double E[3]) {
    if (r.prim == 0) {
        const double ps[3] = {P[0] / E[0], P[1] / E[1], P[2] / E[2]}, ds[3] = {D[0] / E[0], D[1] / E[1], D[2] / E[2]};
        return ps[0] + ds[0] > r.X && ps[0] - ds[0] < r.X + r.dX && ps[1] + ds[1] > r.Y && ps[1] - ds[1] < r.Y + r.dY &&
               ps[2] + ds[2] > r.Z && ps[2] - ds[2] < r.Z + r.dZ;
    }
    const double pos[3] = {r.X * E[0], r.Y * E[1], r.Z * E[2]};
    const double size[3] = {r.dX * E[0], r.dY * E[1], r.dZ * E[2]};
    const double emax = std::max(E[0], std::max(E[1], E[2]));
    const double rad = r.radius * emax;
    if (r.prim == 1) {   // cylinder: IsIn only, along the first nonzero axis
        if (r.dX != 0)
            return P[0] > pos[0] && P[0] < pos[0] + size[0] && sqrt((P[1] - pos[1]) * (P[1] - pos[1]) + (P[2] - pos[2]) * (P[2] - pos[2])) < rad;
        if (r.dY != 0)
            return P[1] > pos[1] && P[1] < pos[1] + size[1] && sqrt((P[0] - pos[0]) * (P[0] - pos[0]) + (P[2] - pos[2]) * (P[2] - pos[2])) < rad;
        if (r.dZ != 0)
            return P[2] > pos[2] && P[2] < pos[2] + size[2] && sqrt((P[0] - pos[0]) * (P[0] - pos[0]) + (P[1] - pos[1]) * (P[1] - pos[1])) < rad;
        return false;
    }
    // sphere: against |Dist| around the point
    const double dist = sqrt(D[0] * D[0] + D[1] * D[1] + D[2] * D[2]);
    return sqrt((P[0] - pos[0]) * (P[0] - pos[0]) + (P[1] - pos[1]) * (P[1] - pos[1]) + (P[2] - pos[2]) * (P[2] - pos[2])) < rad + dist;
}

// Boundary conditions of <Environment>: regions that fix, displace, force or torque the voxels
// they touch (CVX_Environment::ReadXML, VX_Environment.cpp:101-146), applied as CVX_Sim::Import
// does (VXA/VX_Sim.cpp:109-144): a region's force and torque are split over the number of
// structure cells it touches (CVX_Environment::GetNumTouching, VX_Environment.cpp:215-232, which
// tests the cell centres with CVX_Object::GetXYZ's 1e-6 lattice-unit offset), and each touched
// voxel's external force becomes f + (float)(f + F/n) as Import writes it.
bool apply_boundary_conditions(const XmlNode* root, const XmlNode* vxc, int NX, int NY, int NZ, const std::vector<uint8_t>& cells,
                               SimDesc* d, std::string* err) {
    std::vector<BCRegion> regions;
    const XmlNode* env = root->child("Environment");
    auto read_list = [&](const XmlNode* parent, const char* count_tag) {
        int n = get_i(parent, count_tag, 0);
        std::vector<const XmlNode*> frs = parent->children_named("FRegion");
        if (n > (int)frs.size()) { *err = std::string("fewer FRegion elements than ") + count_tag; return false; }
        for (int i = 0; i < n; i++) {
            BCRegion r;
            if (!read_region(frs[i], &r, err)) return false;
            regions.push_back(r);
        }
        return true;
    };
    if (env) {
        if (const XmlNode* bc = env->child("Boundary_Conditions")) {
            if (!read_list(bc, "NumBCs")) return false;
        } else {
            if (const XmlNode* fx = env->child("Fixed_Regions"))
                if (!read_list(fx, "NumFixed")) return false;
            if (const XmlNode* fo = env->child("Forced_Regions"))
                if (!read_list(fo, "NumForced")) return false;
        }
    }
    if (regions.empty()) return true;
    const XmlNode* lat = vxc->child("Lattice");
    const double ld = get_d(lat, "Lattice_Dim", 0.001);
    const double adj[3] = {get_d(lat, "X_Dim_Adj", 1.0), get_d(lat, "Y_Dim_Adj", 1.0), get_d(lat, "Z_Dim_Adj", 1.0)};
    if (get_d(lat, "X_Line_Offset", 0) != 0 || get_d(lat, "Y_Line_Offset", 0) != 0 || get_d(lat, "X_Layer_Offset", 0) != 0 ||
        get_d(lat, "Y_Layer_Offset", 0) != 0) {
        *err = "boundary conditions on offset lattices are not supported";
        return false;
    }
    const double latenv[3] = {ld * adj[0], ld * adj[1], ld * adj[2]};                    // GetLatDimEnv
    const double ws[3] = {ld * adj[0] * NX, ld * adj[1] * NY, ld * adj[2] * NZ};         // GetWorkSpace
    const double half[3] = {latenv[0] / 2.0, latenv[1] / 2.0, latenv[2] / 2.0};
    // cells touched per region (GetXYZ with its offset hack: Eps = 1e-6 lattice units in x and y)
    const double eps = 0.000001;
    std::vector<int> touching(regions.size(), 0);
    for (long i = 0; i < (long)NX * NY * NZ; i++) {
        if (cells[i] == 0) continue;
        const int ix = (int)(i % NX), iy = (int)((i / NX) % NY), iz = (int)(i / ((long)NX * NY));
        const double offx = eps - (int)(eps / adj[0]) * adj[0], offy = eps - (int)(eps / adj[1]) * adj[1];
        const double p[3] = {ld * (adj[0] * (0.5 + ix) + offx), ld * (adj[1] * (0.5 + iy) + offy), ld * adj[2] * (0.5 + iz)};
        for (size_t j = 0; j < regions.size(); j++)
            if (region_touching(regions[j], p, half, ws)) touching[j]++;
    }
    // apply to the voxels in list order
    const int nv = (int)d->voxels.size() / 4;
    std::vector<int> ext_of(nv, -1);
    for (size_t k = 0; k < d->externals.size(); k++) ext_of[d->externals[k].voxel] = (int)k;
    const double s = d->vox_size;                                                        // CVX_Voxel::originalPosition
    for (int v = 0; v < nv; v++) {
        const double p[3] = {d->voxels[4 * v] * s + latenv[0] / 2, d->voxels[4 * v + 1] * s + latenv[1] / 2,
                             d->voxels[4 * v + 2] * s + latenv[2] / 2};
        for (size_t j = 0; j < regions.size(); j++) {
            const BCRegion& r = regions[j];
            if (!region_touching(r, p, half, ws)) continue;
            if (ext_of[v] < 0) {
                External e;
                e.voxel = v;
                ext_of[v] = (int)d->externals.size();
                d->externals.push_back(e);
            }
            External& e = d->externals[ext_of[v]];
            // CVX_External::setDisplacement: fixes the DOF, sets the value when nonzero (VX_External.cpp:53-66)
            const double vals[6] = {r.disp[0], r.disp[1], r.disp[2], r.ang[0], r.ang[1], r.ang[2]};
            for (int k = 0; k < 6; k++) {
                if (!(r.dof & (1 << k))) continue;
                e.dof_fixed |= 1 << k;
                if (vals[k] != 0.0f) (k < 3 ? e.translate[k] : e.rotate[k - 3]) = vals[k];
            }
            for (int k = 0; k < 3; k++) {
                e.force[k] += (float)(e.force[k] + r.force[k] / touching[j]);
                e.moment[k] += (float)(e.moment[k] + r.torque[k] / touching[j]);
            }
        }
    }
    return true;
}

}  // namespace

void merge_vxd(XmlNode* base, const XmlNode& vxd) {
    const XmlNode* src = vxd.tag == "VXD" ? &vxd : vxd.child("VXD");
    if (!src) return;
    for (auto& c : src->children) {
        const char* rep = c->attr("replace");
        if (!rep || !*rep) continue;
        std::string path(rep);
        std::vector<std::string> parts;
        size_t s = 0;
        for (;;) {
            size_t d = path.find('.', s);
            parts.push_back(path.substr(s, d == std::string::npos ? std::string::npos : d - s));
            if (d == std::string::npos) break;
            s = d + 1;
        }
        if (parts.empty() || parts[0] != base->tag) continue;
        XmlNode* node = base;
        for (size_t i = 1; i + 1 < parts.size(); i++) {
            XmlNode* nx = node->child(parts[i]);
            if (!nx) {
                node->children.push_back(std::make_unique<XmlNode>());
                nx = node->children.back().get();
                nx->tag = parts[i];
            }
            node = nx;
        }
        auto nn = c->clone();
        nn->tag = parts.back();
        bool replaced = false;
        for (auto& ch : node->children)
            if (ch->tag == parts.back()) { ch = std::move(nn); replaced = true; break; }
        if (!replaced) node->children.push_back(std::move(nn));
    }
}

bool parse_vxa(const std::string& base_xml, const char* vxd_xml, SimDesc* d, std::string* err) {
    std::string perr;
    auto root = xml_parse(base_xml, &perr);
    if (!root) { *err = "base VXA: " + perr; return false; }
    if (vxd_xml && *vxd_xml) {
        auto vxd = xml_parse(vxd_xml, &perr);
        if (!vxd) { *err = "VXD: " + perr; return false; }
        merge_vxd(root.get(), *vxd);
    }
    if (root->tag != "VXA") { *err = "root element is not <VXA>"; return false; }
    const XmlNode* sim = root->child("Simulator");
    *d = SimDesc();
    if (sim) {
        if (const XmlNode* in = sim->child("Integration")) d->dt_frac = get_d(in, "DtFrac", 0.9);
        if (const XmlNode* dm = sim->child("Damping")) {
            d->zeta_internal = get_f(dm, "BondDampingZ", 0.1);
            d->zeta_collision = get_f(dm, "ColDampingZ", 1.0);
            d->zeta_global = get_f(dm, "SlowDampingZ", 1.0);
        }
        if (const XmlNode* f = sim->child("Features")) d->volume_effects = get_b(f, "VolumeEffectsEnabled", false);
    }
    double grav_acc = -9.81;
    if (const XmlNode* env = root->child("Environment")) {
        if (const XmlNode* g = env->child("Gravity")) {
            grav_acc = get_d(g, "GravAcc", -9.81);
            d->floor = get_b(g, "FloorEnabled", false);
        }
        if (const XmlNode* th = env->child("Thermal")) {
            d->temp_enabled = get_b(th, "TempEnabled", false);
            d->temp_base = get_d(th, "TempBase", 25);
            double v;
            if (load_d(th, "TempAmplitude", &v)) d->temp_amplitude = v;
            else if (load_d(th, "TempAmp", &v)) d->temp_amplitude = v - d->temp_base;
            else d->temp_amplitude = 0;
            d->vary_temp = get_b(th, "VaryTempEnabled", false);
            d->temp_period = get_d(th, "TempPeriod", 0.1);
        }
    }
    /* CVX_Sim::SetGravityAccel(float) -> CVoxelyze::setGravity(float) (VX_Sim.cpp:485) */
    float ga = (float)grav_acc;
    d->gravity_mult = (float)(-ga / 9.80665);
    /* initial temperature: CVX_Sim::UpdateMatTemps with CVX_Environment::UpdateCurTemp at t=0
       (VX_Sim.cpp:467-483, VX_Environment.cpp:327-346) */
    if (d->temp_enabled) {
        float cur;
        if (d->vary_temp) cur = d->temp_period == 0 ? 0.0f : (float)(d->temp_base + d->temp_amplitude * sin(0.0));
        else cur = (float)(d->temp_base + d->temp_amplitude);
        d->initial_temp = (float)(cur - d->temp_base);
    }
    const XmlNode* vxc = root->child("VXC");
    if (!vxc) { *err = "missing <VXC>"; return false; }
    if (const XmlNode* lat = vxc->child("Lattice")) d->vox_size = get_d(lat, "Lattice_Dim", 0.001) * get_d(lat, "X_Dim_Adj", 1.0);
    else d->vox_size = 0.001;
    if (const XmlNode* pal = vxc->child("Palette")) {
        for (auto* m : pal->children_named("Material")) {
            PaletteMaterial pm;
            int mt = get_i(m, "MatType", 0);
            if (mt != 0) { *err = "only basic (SINGLE) materials are supported"; return false; }
            pm.name = m->child("Name") ? m->child("Name")->text : "Default";
            // Display colour, 0..1 floats, defaults as CVXC_Material::ReadXML (VXA/VX_Object.cpp:1385-1390)
            if (const XmlNode* disp = m->child("Display")) {
                pm.rgba[0] = (float)get_d(disp, "Red", 0.5);
                pm.rgba[1] = (float)get_d(disp, "Green", 0.5);
                pm.rgba[2] = (float)get_d(disp, "Blue", 0.5);
                pm.rgba[3] = (float)get_d(disp, "Alpha", 1.0);
            }
            const XmlNode* mech = m->child("Mechanical");
            pm.model = get_i(mech, "MatModel", 0);
            pm.E = get_d(mech, "Elastic_Mod", 0);
            pm.plastic_mod = get_d(mech, "Plastic_Mod", 0);
            pm.yield_stress = get_d(mech, "Yield_Stress", 0);
            pm.fail_stress = get_d(mech, "Fail_Stress", 0);
            pm.rho = get_d(mech, "Density", 0);
            pm.nu = get_d(mech, "Poissons_Ratio", 0);
            pm.cte = get_d(mech, "CTE", 0);
            pm.mu_static = get_d(mech, "uStatic", 0);
            pm.mu_kinetic = get_d(mech, "uDynamic", 0);
            pm.is_measured = get_i(mech, "isMeasured", 1);
            pm.cilia = get_d(mech, "Cilia", 0);
            pm.cilia_on_after = get_d(mech, "TurnOnCiliaAfterThisManySeconds", 0);
            pm.thermal_on_after = get_d(mech, "TurnOnThermalExpansionAfterThisManySeconds", 0);
            pm.is_pacemaker = get_i(mech, "isPaceMaker", 0) != 0;
            pm.pacemaker_period = get_d(mech, "PaceMakerPeriod", 0);
            pm.signal_decay = get_d(mech, "signalValueDecay", 0.9);
            pm.signal_delay = get_d(mech, "signalTimeDelay", 0.03);
            pm.inactive_period = get_d(mech, "inactivePeriod", 0.03);
            pm.is_target = get_i(mech, "isTarget", 0) != 0;
            pm.remove_after = get_d(mech, "RemoveFromSimulationAfterThisManySeconds", 0);
            pm.fixed = get_i(mech, "Fixed", 0) != 0;
            pm.sticky = get_i(mech, "Sticky", 0) != 0;
            if (const XmlNode* ss = mech ? mech->child("SSData") : nullptr) {
                if (const XmlNode* se = ss->child("StrainData"))
                    for (auto* c : se->children_named("Strain")) pm.strain_data.push_back(atof_s(c->text));
                if (const XmlNode* st = ss->child("StressData"))
                    for (auto* c : st->children_named("Stress")) pm.stress_data.push_back(atof_s(c->text));
            }
            if (pm.model == 3 && (pm.strain_data.size() != pm.stress_data.size() || pm.strain_data.size() > (size_t)kMaxModelPoints)) {
                *err = "material stress/strain data malformed or longer than 16 points";
                return false;
            }
            d->mats.push_back(pm);
        }
    }
    if (!d->volume_effects) for (auto& m : d->mats) m.nu = 0;   /* CVX_Sim::EnableVolumeEffects(false), VX_Sim.cpp:445-458 */
    const XmlNode* st = vxc->child("Structure");
    if (!st) { *err = "missing <Structure>"; return false; }
    int X = get_i(st, "X_Voxels", 1), Y = get_i(st, "Y_Voxels", 1), Z = get_i(st, "Z_Voxels", 1);
    if (X <= 0 || Y <= 0 || Z <= 0 || (long)X * Y * Z > (1L << 31) / 8) { *err = "bad structure dimensions"; return false; }
    const char* compa = st->attr("Compression");
    std::string comp = compa ? compa : "";
    const XmlNode* data = st->child("Data");
    std::vector<const XmlNode*> layers = data ? data->children_named("Layer") : std::vector<const XmlNode*>();
    std::vector<uint8_t> cells((size_t)X * Y * Z, 0);
    for (int k = 0; k < Z; k++) {
        std::string raw = k < (int)layers.size() ? layers[k]->text : std::string();
        std::string vals;
        if (comp == "ASCII_READABLE") { vals.resize(raw.size()); for (size_t i = 0; i < raw.size(); i++) vals[i] = raw[i] - 48; }
        else if (comp == "RAW_DATA") vals = raw;
        else if (comp == "ZLIB" || comp == "QT_ZLIB") { *err = "compressed structure data is not supported"; return false; }
        else vals = b64decode(raw);
        if ((long)vals.size() != (long)X * Y) { *err = "voxel layer data does not match X_Voxels*Y_Voxels"; return false; }
        memcpy(&cells[(size_t)k * X * Y], vals.data(), vals.size());
    }
    std::vector<double> phase_by_voxel;
    bool have_phase = false;
    if (const XmlNode* po = st->child("PhaseOffset")) {
        have_phase = true;
        auto pl = po->children_named("Layer");
        for (int k = 0; k < Z; k++) {
            // the comma-separated fields read in place, one pass; cells past the last field read 0
            const char* p = k < (int)pl.size() ? pl[k]->text.c_str() : nullptr;
            const char* end = p ? p + pl[k]->text.size() : nullptr;
            for (int j = 0; j < X * Y; j++) {
                if (cells[(size_t)k * X * Y + j] > 0) phase_by_voxel.push_back(p ? field_atof(p, end) : 0.0);
                if (p) {
                    const char* c = (const char*)memchr(p, ',', (size_t)(end - p));
                    p = c ? c + 1 : nullptr;
                }
            }
        }
    }
    /* BaseCiliaForce and ShiftCiliaForce: per filled cell an x,y,z triple, layer by layer; a
       short layer pads with zeros (VXA/VX_Object.cpp:1886-1958) */
    auto read_triples = [&](const XmlNode* node, std::vector<double>* out) {
        auto pl = node->children_named("Layer");
        for (int k = 0; k < Z; k++) {
            std::vector<const char*> arr;   // start of each comma-separated field, read in place
            const char* end = nullptr;
            if (k < (int)pl.size()) { comma_fields(pl[k]->text, &arr); end = pl[k]->text.c_str() + pl[k]->text.size(); }
            for (int j = 0; j < X * Y; j++) {
                if (cells[(size_t)k * X * Y + j] == 0) continue;
                for (int c = 0; c < 3; c++)
                    out->push_back(arr.size() > (size_t)(3 * j + c) && arr.size() > (size_t)(3 * j) ? field_atof(arr[3 * j + c], end) : 0.0);
            }
        }
    };
    if (const XmlNode* bcf = st->child("BaseCiliaForce")) read_triples(bcf, &d->base_cilia);
    if (const XmlNode* scf = st->child("ShiftCiliaForce")) read_triples(scf, &d->shift_cilia);
    // voxels in structure order (x fastest), with their lattice indices and material
    size_t filled = 0;
    for (uint8_t c : cells) filled += (signed char)c > 0;
    d->voxels.resize(4 * filled);
    d->phase.resize(filled);
    {
        const int nm = (int)d->mats.size();
        size_t n = 0, i = 0;
        for (int z = 0; z < Z; z++)
            for (int y = 0; y < Y; y++)
                for (int x = 0; x < X; x++, i++) {
                    const int mi = (int)(signed char)cells[i] - 1;
                    if (mi < 0) continue;
                    if (mi >= nm) { *err = "voxel references a material missing from the palette"; return false; }
                    int32_t* v = &d->voxels[4 * n];
                    v[0] = x; v[1] = y; v[2] = z; v[3] = mi;
                    d->phase[n] = have_phase ? phase_by_voxel[n] : 0.0;
                    n++;
                }
    }
    if (!apply_boundary_conditions(root.get(), vxc, X, Y, Z, cells, d, err)) return false;
    /* VX3 keys, Voxelyze3/src/VX3/VX3_SimulationManager.cu:326-367 */
    d->collisions = ptree_bool(*root, "VXA.Simulator.AttachDetach.EnableCollision", true);
    d->bounding_radius = (float)ptree_num(*root, "VXA.Simulator.AttachDetach.boundingRadius", 0.75);
    d->watch_distance = (float)ptree_num(*root, "VXA.Simulator.AttachDetach.watchDistance", 1.0);
    d->enable_expansion = (int)ptree_num(*root, "VXA.Simulator.EnableExpansion", 0);
    d->save_all_positions = (int)ptree_num(*root, "VXA.Simulator.SavePositionOfAllVoxels", 0);
    d->max_dist_pairs = ptree_num(*root, "VXA.Simulator.MaxDistInVoxelLengthsToCountAsPair", 0);
    d->record_step_size = (int)ptree_num(*root, "VXA.Simulator.RecordHistory.RecordStepSize", 0);
    d->record_voxel = (int)ptree_num(*root, "VXA.Simulator.RecordHistory.RecordVoxel", 1);
    d->record_link = (int)ptree_num(*root, "VXA.Simulator.RecordHistory.RecordLink", 0);
    /* VX3 extras: cilia switch and force field; an absent force-field component is the constant 0
       (VX3_ForceField's default, Utils/VX3_ForceField.h:10-19) */
    d->enable_cilia = (int)ptree_num(*root, "VXA.Simulator.EnableCilia", 0);
    d->enable_signals = (int)ptree_num(*root, "VXA.Simulator.EnableSignals", 0);
    d->enable_detach = ptree_bool(*root, "VXA.Simulator.AttachDetach.EnableDetach", false);
    d->secondary_experiment = (int)ptree_num(*root, "VXA.Simulator.SecondaryExperiment", 0);
    d->reinit_initial_after = ptree_num(*root, "VXA.Simulator.ReinitializeInitialPositionAfterThisManySeconds", 0.0);
    d->enable_attach = ptree_bool(*root, "VXA.Simulator.AttachDetach.EnableAttach", false);
    d->safety_guard = (int)ptree_num(*root, "VXA.Simulator.AttachDetach.SafetyGuard", 500);
    d->attach_cond_mask = 0;
    for (int k = 0; k < 5; k++) {
        const std::string path = "VXA.Simulator.AttachDetach.AttachCondition.Condition_" + std::to_string(k);
        if (const XmlNode* n = root->path(path.c_str())) {
            parse_mathtree(n, &d->attach_cond[k]);
            if (!d->attach_cond[k].valid) { *err = "invalid attach condition formula"; return false; }
            d->attach_cond_mask |= 1 << k;
        }
    }
    const char* ff_paths[3] = {"VXA.Simulator.ForceField.x_forcefield", "VXA.Simulator.ForceField.y_forcefield",
                               "VXA.Simulator.ForceField.z_forcefield"};
    for (int k = 0; k < 3; k++) {
        MathTree& m = d->force_field[k];
        if (const XmlNode* n = root->path(ff_paths[k])) {
            parse_mathtree(n, &m);
            if (!m.valid) { *err = "invalid force-field formula"; return false; }
            const bool zero = m.n == 2 && m.tok[0].op == mtCONST && m.tok[0].value == 0.0;
            if (!zero) d->has_force_field = true;
        } else {
            m.n = 2; m.valid = 1;
            m.tok[0].op = mtCONST; m.tok[0].value = 0.0;
            m.tok[1].op = mtEND; m.tok[1].value = 0.0;
        }
    }
    parse_mathtree(root->path("VXA.Simulator.StopCondition.StopConditionFormula"), &d->stop_formula);
    parse_mathtree(root->path("VXA.Simulator.FitnessFunction"), &d->fitness);
    // a formula the evaluator cannot take (an unknown token or variable, or more than
    // kMaxMathTokens - 1 tokens) is refused rather than evaluated to NaN
    if (!d->stop_formula.valid) { *err = "invalid or too long stop condition formula (at most 63 tokens)"; return false; }
    if (!d->fitness.valid) { *err = "invalid or too long fitness formula (at most 63 tokens)"; return false; }
    return true;
}

/* ------------------------------------------------------------------------ */
/* Material derivation: CVX_Material / CVX_MaterialVoxel / CVX_MaterialLink
 * (Voxelyze3/src/old/VX_Material.cpp:15-549, VX_MaterialVoxel.cpp:31-86,
 * VX_MaterialLink.cpp:16-141).  Float arithmetic in the reference's order. */
namespace {

void update_derived(VoxelMaterial* m) {
    m->eHat = m->E / ((1 - 2 * m->nu) * (1 + m->nu));
    double volume = m->nom * m->nom * m->nom;
    m->mass = (float)(volume * m->rho);
    m->I = (float)(m->mass * m->nom * m->nom / 6.0f);
    if (volume == 0 || m->mass == 0 || m->I == 0) { m->massInv = m->sqrtMass = m->Iinv = m->c2m = m->c2i = 0.0f; return; }
    m->massInv = 1.0f / m->mass;
    m->sqrtMass = sqrtf(m->mass);
    m->Iinv = 1.0f / m->I;
    m->c2m = (float)(2.0f * sqrt(m->mass * m->E * m->nom));
    m->c2i = (float)(2.0f * sqrt(m->I * m->E * m->nom * m->nom * m->nom));
}
void update_link_derived(LinkMaterial* m) {
    update_derived(m);
    float L = (float)m->nom;
    m->a1 = m->E * L;
    m->a2 = m->E * L * L * L / (12.0f * (1 + m->nu));
    m->b1 = m->E * L;
    m->b2 = m->E * L * L / 2.0f;
    m->b3 = m->E * L * L * L / 6.0f;
    m->sqA1 = sqrtf(m->a1);
    m->sqA2xIp = sqrtf(m->a2 * L * L / 6.0f);
    m->sqB1 = sqrtf(m->b1);
    m->sqB2xFMp = sqrtf(m->b2 * L / 2.0f);
    m->sqB3xIp = sqrtf(m->b3 * L * L / 6.0f);
}
void set_linear(VoxelMaterial* m, float E, float fail) {
    if (E <= 0) return;
    if (fail != -1.0f && fail <= 0) return;
    float tf = fail;
    if (tf == -1) tf = 1000000;
    float tfs = tf / E;
    m->n = 2;
    m->strain[0] = 0; m->stress[0] = 0; m->strain[1] = tfs; m->stress[1] = tf;
    m->linear = 1;
    m->E = E;
    m->sigmaYield = fail; m->sigmaFail = fail;
    m->epsYield = (fail == -1) ? -1 : tfs;
    m->epsFail = (fail == -1) ? -1 : tfs;
}
void yield_from_data(VoxelMaterial* m, float pct) {
    m->sigmaYield = -1.0f; m->epsYield = -1.0f;
    float oM = m->E, oB = (-pct / 100 * oM);
    int dp = m->n - 1;
    for (int i = 1; i < dp - 1; i++) {
        float x1 = m->strain[i], x2 = m->strain[i + 1], y1 = m->stress[i], y2 = m->stress[i + 1];
        float tM = (y2 - y1) / (x2 - x1), tB = y1 - tM * x1;
        if (oM != tM) {
            float xi = (tB - oB) / (oM - tM);
            if (xi > x1 && xi < x2) {
                float p = (xi - x1) / (x2 - x1);
                m->sigmaYield = y1 + p * (y2 - y1);
                m->epsYield = xi;
                return;
            }
        }
    }
    m->sigmaYield = m->sigmaFail; m->epsYield = m->epsFail;
}
bool set_model(VoxelMaterial* m, int count, const float* se, const float* ss) {
    if (*se == 0 && *ss == 0) { se++; ss++; count--; }
    if (count <= 0 || count > kMaxModelPoints) return false;
    if (*se <= 0 || *ss <= 0) return false;
    float ts[kMaxModelPoints + 2], tt[kMaxModelPoints + 2];
    ts[0] = 0; tt[0] = 0;
    float sE = 0.0f, sS = 0.0f;
    for (int i = 0; i < count; i++) {
        float e = se[i], s = ss[i];
        if (e <= sE) return false;
        if (i > 0 && (s - sS) / (e - sE) > tt[0] / ts[0]) return false;
        sE = e; sS = s;
        ts[i + 1] = e; tt[i + 1] = s;
    }
    m->n = count + 1;
    for (int i = 0; i < m->n; i++) { m->strain[i] = ts[i]; m->stress[i] = tt[i]; }
    m->E = m->stress[1] / m->strain[1];
    m->sigmaFail = m->stress[m->n - 1];
    m->epsFail = m->strain[m->n - 1];
    m->linear = (count == 1);
    if (count == 1 || count == 2) { m->sigmaYield = m->stress[1]; m->epsYield = m->strain[1]; }
    else yield_from_data(m, 0.2f);
    return true;
}
void set_bilinear(VoxelMaterial* m, float E, float pE, float ys, float fs) {
    if (E <= 0 || pE <= 0 || pE >= E || ys <= 0) return;
    if (fs != -1.0f && fs <= ys) return;
    float yS = ys / E, tfs = fs;
    if (tfs == -1) tfs = 3 * ys;
    float tM = pE, tB = ys - tM * yS, tfst = (tfs - tB) / tM;
    m->n = 3;
    m->strain[0] = 0; m->strain[1] = yS; m->strain[2] = tfst;
    m->stress[0] = 0; m->stress[1] = ys; m->stress[2] = tfs;
    m->linear = 0;
    m->E = E;
    m->sigmaYield = ys; m->sigmaFail = fs; m->epsYield = yS;
    m->epsFail = fs == -1.0f ? -1.0f : tfst;
}
bool is_failed(const VoxelMaterial* m, float s) { return m->epsFail != -1.0f && s > m->epsFail; }
float modulus(const VoxelMaterial* m, float s) {
    if (is_failed(m, s)) return 0.0f;
    if (s <= m->strain[1] || m->linear) return m->E;
    for (int i = 2; i < m->n; i++)
        if (s <= m->strain[i] || i == m->n - 1) return (m->stress[i] - m->stress[i - 1]) / (m->strain[i] - m->strain[i - 1]);
    return 0.0f;
}
float strain_of(const VoxelMaterial* m, float stress) {
    if (stress <= m->stress[1] || m->linear) return stress / m->E;
    for (int i = 2; i < m->n; i++)
        if (stress <= m->stress[i] || i == m->n - 1) {
            float p = (stress - m->stress[i - 1]) / (m->stress[i] - m->stress[i - 1]);
            return m->strain[i - 1] + p * (m->strain[i] - m->strain[i - 1]);
        }
    return 0.0f;
}

VoxelMaterial make_voxel_material(const PaletteMaterial& p, const SimDesc& d) {
    VoxelMaterial m;
    m.nu = 0.0f; m.rho = 1.0f; m.cte = 0.0f; m.mus = 0.0f; m.muk = 0.0f; m.zi = 1.0f; m.zg = 0.0f; m.zc = 0.0f;
    // CVoxelyze::addMaterial() starts from CVX_MaterialVoxel(1e6, 1e3); a model setter that rejects
    // its arguments (e.g. bilinear with Fail_Stress <= Yield_Stress) leaves this linear model in place.
    set_linear(&m, 1e6f, -1.0f);
    switch (p.model) {
    case 0: set_linear(&m, (float)p.E, -1.0f); break;
    case 1: set_linear(&m, (float)p.E, (float)p.fail_stress); break;
    case 2: set_bilinear(&m, (float)p.E, (float)p.plastic_mod, (float)p.yield_stress, (float)p.fail_stress); break;
    case 3: {
        float se[kMaxModelPoints], ss[kMaxModelPoints];
        int n = (int)p.strain_data.size();
        for (int i = 0; i < n; i++) { se[i] = (float)p.strain_data[i]; ss[i] = (float)p.stress_data[i]; }
        if (n > 0) set_model(&m, n, se, ss);
        break;
    }
    default: break;
    }
    float nu = (float)p.nu;
    if (nu < 0) nu = 0;
    if (nu >= 0.5) nu = (float)(0.5 - FLT_EPSILON * 2);
    m.nu = nu;
    float rho = (float)p.rho;
    if (rho <= 0) rho = FLT_MIN;
    m.rho = rho;
    m.cte = (float)p.cte;
    float mus = (float)p.mu_static, muk = (float)p.mu_kinetic;
    m.mus = mus <= 0 ? 0 : mus;
    m.muk = muk <= 0 ? 0 : muk;
    m.zi = d.zeta_internal <= 0 ? 0 : d.zeta_internal;
    m.zg = d.zeta_global <= 0 ? 0 : d.zeta_global;
    m.zc = d.zeta_collision <= 0 ? 0 : d.zeta_collision;
    m.nom = d.vox_size;
    m.grav = d.gravity_mult;
    m.is_measured = p.is_measured;
    update_derived(&m);
    return m;
}

LinkMaterial make_link_material(const VoxelMaterial& a, const VoxelMaterial& b, int ia, int ib) {
    LinkMaterial m;
    m.vox1 = ia; m.vox2 = ib;
    m.nom = 0.5 * (a.nom + b.nom);
    m.rho = 0.5f * (a.rho + b.rho);
    m.cte = 0.5f * (a.cte + b.cte);
    m.mus = 0.5f * (a.mus + b.mus);
    m.muk = 0.5f * (a.muk + b.muk);
    m.zi = 0.5f * (a.zi + b.zi);
    m.zg = 0.5f * (a.zg + b.zg);
    m.zc = 0.5f * (a.zc + b.zc);
    float f1 = a.sigmaFail, f2 = b.sigmaFail, sf;
    if (f1 == -1.0f) sf = f2;
    else if (f2 == -1.0f) sf = f1;
    else sf = f1 < f2 ? f1 : f2;
    if (a.linear && b.linear) {
        set_linear(&m, 2.0f * a.E * b.E / (a.E + b.E), sf);
    } else {
        float ns[2 * kMaxModelPoints + 4], ne[2 * kMaxModelPoints + 4];
        int cnt = 1;
        ns[0] = 0.0f; ne[0] = 0.0f;
        int i1 = 1, i2 = 1;
        while (i1 < a.n && i2 < b.n && cnt < 2 * kMaxModelPoints + 3) {
            float s = FLT_MAX;
            if (i1 < a.n) s = a.strain[i1];
            if (i2 < b.n && b.strain[i2] < s) s = b.strain[i2];
            if (s == a.strain[i1]) i1++;
            if (s == b.strain[i2]) i2++;
            float m1 = modulus(&a, s - FLT_EPSILON), m2 = modulus(&b, s - FLT_EPSILON);
            float tm = 2.0f * m1 * m2 / (m1 + m2);
            int last = cnt - 1;
            ne[cnt] = s;
            ns[cnt] = ns[last] + tm * (s - ne[last]);
            cnt++;
        }
        set_model(&m, cnt, ne, ns);
        m.sigmaFail = sf;
        m.epsFail = sf == -1.0f ? -1.0f : strain_of(&m, sf);
    }
    if (a.nu == 0 && b.nu == 0) m.nu = 0;
    else {
        float tmpEHat = 2 * a.eHat * b.eHat / (a.eHat + b.eHat);
        float tmpE = m.E;
        float c2 = (float)((tmpEHat - tmpE) / (2 * tmpEHat) + 0.0625);
        m.nu = (float)(sqrtf(c2) - 0.25);
    }
    update_link_derived(&m);
    return m;
}

}  // namespace

/* Topology: CVoxelyze::addVoxel / addLink (Voxelyze3/src/old/Voxelyze.cpp:439-539)
 * and the CVX_Link constructor (VX_Link.cpp:21-54).  Voxels are added in structure
 * order; each voxel links to the already-present neighbours in direction order
 * 0..5, so the link list order and negative/positive ends match the reference. */
bool build_world(const SimDesc& d, SimWorld* w, std::string* err) {
    w->desc = d;
    w->vmats.clear();
    w->lmats.clear();
    for (auto& p : d.mats) w->vmats.push_back(make_voxel_material(p, d));
    int nv = (int)d.voxels.size() / 4;
    w->nv = nv;
    if (nv == 0) { *err = "no voxels"; return false; }
    int mn[3] = {1 << 30, 1 << 30, 1 << 30}, mx[3] = {-(1 << 30), -(1 << 30), -(1 << 30)};
    for (int i = 0; i < nv; i++)
        for (int k = 0; k < 3; k++) { mn[k] = std::min(mn[k], d.voxels[4 * i + k]); mx[k] = std::max(mx[k], d.voxels[4 * i + k]); }
    const long dx = mx[0] - mn[0] + 1, dy = mx[1] - mn[1] + 1, dz = mx[2] - mn[2] + 1;
    // lattice sites with a border of one empty site, so the six neighbour reads need no bounds test
    const long px = dx + 2, pxy = (dx + 2) * (dy + 2);
    std::vector<int32_t> grid((size_t)(pxy * (dz + 2)), -1);
    const long step[6] = {1, -1, px, -px, pxy, -pxy};   // direction order X+,X-,Y+,Y-,Z+,Z-
    const int nm = (int)w->vmats.size();
    std::vector<int> pair_lmat((size_t)nm * nm, -1);    // link material of a material pair, either order
    w->vox_links.assign((size_t)nv * 6, -1);
    w->link_neg.clear(); w->link_pos.clear(); w->link_axis.clear(); w->link_mat.clear();
    w->link_neg.reserve((size_t)nv * 3); w->link_pos.reserve((size_t)nv * 3);
    w->link_axis.reserve((size_t)nv * 3); w->link_mat.reserve((size_t)nv * 3);
    for (int i = 0; i < nv; i++) {
        const int* v = &d.voxels[4 * (size_t)i];
        if (v[3] < 0 || v[3] >= nm) { *err = "voxel references a material missing from the palette"; return false; }
        const long site = ((v[2] - mn[2] + 1) * (dy + 2) + (v[1] - mn[1] + 1)) * px + (v[0] - mn[0] + 1);
        if (grid[(size_t)site] >= 0) { *err = "two voxels at the same lattice site"; return false; }
        grid[(size_t)site] = i;
        // a link is made when the second of its two voxels (in structure order) is placed
        for (int dir = 0; dir < 6; dir++) {
            const int b = grid[(size_t)(site + step[dir])];
            if (b < 0 || w->vox_links[(size_t)i * 6 + dir] >= 0) continue;
            const int ma = v[3], mb = d.voxels[4 * (size_t)b + 3];
            int lmi = pair_lmat[(size_t)ma * nm + mb];
            if (lmi < 0) {
                lmi = (int)w->lmats.size();
                pair_lmat[(size_t)ma * nm + mb] = pair_lmat[(size_t)mb * nm + ma] = lmi;
                w->lmats.push_back(make_link_material(w->vmats[ma], w->vmats[mb], ma, mb));
            }
            const int li = (int)w->link_neg.size();
            const bool rev = dir % 2 == 1;
            w->link_neg.push_back(rev ? b : i);
            w->link_pos.push_back(rev ? i : b);
            w->link_axis.push_back((uint8_t)(dir / 2));
            w->link_mat.push_back((uint8_t)lmi);
            w->vox_links[(size_t)i * 6 + dir] = li;
            w->vox_links[(size_t)b * 6 + (dir ^ 1)] = li;
        }
    }
    // VX3 attachment: a new link between two voxels of one sticky material takes the combined
    // material of that material with itself (VX3_VoxelyzeKernel::combinedMaterial, :516-528)
    w->loaded_lmats = (int)w->lmats.size();
    w->attach_lmat.assign(w->vmats.size(), -1);
    if (d.enable_attach) {
        for (int m = 0; m < (int)d.mats.size(); m++) {
            if (!d.mats[m].sticky) continue;
            int& lmi = pair_lmat[(size_t)m * nm + m];
            if (lmi < 0) {
                lmi = (int)w->lmats.size();
                w->lmats.push_back(make_link_material(w->vmats[m], w->vmats[m], m, m));
            }
            w->attach_lmat[m] = lmi;
        }
    }
    if (w->lmats.size() > 255 || w->vmats.size() > 255) { *err = "too many materials"; return false; }
    w->nl = (int)w->link_neg.size();
    w->vox_interior.assign(nv, 0);
    w->surface_count = 0;
    for (int i = 0; i < nv; i++) {
        bool in = true;
        for (int k = 0; k < 6; k++) if (w->vox_links[(size_t)i * 6 + k] < 0) in = false;
        w->vox_interior[i] = in;
        if (!in) w->surface_count++;
    }
    w->vox_ext.assign(nv, -1);
    for (size_t k = 0; k < d.externals.size(); k++) {
        int v = d.externals[k].voxel;
        if (v < 0 || v >= nv) { *err = "external refers to a missing voxel"; return false; }
        w->vox_ext[v] = (int)k;
    }
    return true;
}

std::vector<int8_t> l1_ball_offsets(int depth) {
    std::vector<int8_t> o;
    for (int z = -depth; z <= depth; z++)
        for (int y = -depth; y <= depth; y++)
            for (int x = -depth; x <= depth; x++)
                if (abs(x) + abs(y) + abs(z) <= depth) { o.push_back((int8_t)x); o.push_back((int8_t)y); o.push_back((int8_t)z); }
    return o;
}

std::vector<uint32_t> reach_masks(const SimWorld& w, int depth, int words) {
    std::vector<int8_t> offs = l1_ball_offsets(depth);
    int n_off = (int)offs.size() / 3;
    int side = 2 * depth + 1;
    std::vector<int> off_index((size_t)side * side * side, -1);
    for (int k = 0; k < n_off; k++)
        off_index[(size_t)((offs[3 * k + 2] + depth) * side + (offs[3 * k + 1] + depth)) * side + (offs[3 * k] + depth)] = k;
    std::vector<uint32_t> masks((size_t)w.nv * words, 0);
    std::vector<int> dist(w.nv, -1);
    std::vector<int> touched;
    for (int s = 0; s < w.nv; s++) {
        if (w.vox_interior[s]) continue;
        touched.clear();
        std::deque<int> q{s};
        dist[s] = 0;
        touched.push_back(s);
        while (!q.empty()) {
            int v = q.front();
            q.pop_front();
            if (dist[v] == depth) continue;
            for (int k = 0; k < 6; k++) {
                int li = w.vox_links[(size_t)v * 6 + k];
                if (li < 0) continue;
                int o = w.link_neg[li] == v ? w.link_pos[li] : w.link_neg[li];
                if (dist[o] >= 0) continue;
                dist[o] = dist[v] + 1;
                touched.push_back(o);
                q.push_back(o);
            }
        }
        for (int v : touched) {
            if (v != s) {
                int ox = w.desc.voxels[4 * v] - w.desc.voxels[4 * s], oy = w.desc.voxels[4 * v + 1] - w.desc.voxels[4 * s + 1],
                    oz = w.desc.voxels[4 * v + 2] - w.desc.voxels[4 * s + 2];
                int k = off_index[(size_t)((oz + depth) * side + (oy + depth)) * side + (ox + depth)];
                if (k >= 0 && k < 32 * words) masks[(size_t)s * words + k / 32] |= 1u << (k % 32);
            }
            dist[v] = -1;
        }
    }
    return masks;
}

}  // namespace gvx
