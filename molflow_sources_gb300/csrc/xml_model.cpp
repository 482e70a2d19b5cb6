// xml_model.cpp — MolFlow+ XML files into a model descriptor and a results view, on the C++ host.
//
// Reads the `<SimulationEnvironment>` documents the reference writes (src/IO/WriterXML.cpp:72-903)
// and reads (src/IO/LoaderXML.cpp:31-1130): the geometry (vertices, facet polygons), the facet
// settings the tracer uses (LoaderXML.cpp:831-1120), the simulation settings (gas, time settings and
// user moments, time-dependent parameters, scattering, motion, force measurement, low-flux mode,
// histograms) and the stored results (LoaderXML.cpp:366-760).  Time-dependent parameters: the
// file's own, followed by those of a parameter catalog folder when one is given.
#include "xml_model.h"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <numeric>

namespace mfgx {

namespace {

double to_d(const char* s) { return std::strtod(s, nullptr); }
// integer attribute: "true"/"false", or a number truncated toward zero
long long to_i(const char* s) {
    if (std::strcmp(s, "true") == 0) return 1;
    if (std::strcmp(s, "false") == 0) return 0;
    const double v = std::strtod(s, nullptr);
    if (!(v == v)) return 0;   // not a number
    if (v >= 9.2e18) return 9200000000000000000LL;   // out of range: clamped, not undefined
    if (v <= -9.2e18) return -9200000000000000000LL;
    return (long long)v;
}
double fa(const XNode* n, const char* a, double def = 0.0) {
    const char* v = n ? n->attr(a) : nullptr;
    return v ? to_d(v) : def;
}
long long ia(const XNode* n, const char* a, long long def = 0) {
    const char* v = n ? n->attr(a) : nullptr;
    return v ? to_i(v) : def;
}
// integer attribute clamped to the 32-bit range of the descriptor's fields
int32_t ia32(const XNode* n, const char* a, long long def = 0) {
    return int32_t(std::min<long long>(std::max<long long>(ia(n, a, def), INT32_MIN), INT32_MAX));
}
// count stored as a number: not a number or negative -> 0, past 2^64 -> 2^64-1
uint64_t to_u64(double v) {
    if (!(v > 0)) return 0;
    if (v >= 18446744073709551615.0) return UINT64_MAX;
    return uint64_t(v);
}
const XNode* kid(const XNode* n, const char* tag) { return n ? n->child(tag) : nullptr; }

// whitespace-separated numbers of an element's text
void numbers(const std::string& t, std::vector<double>& out) {
    const char* p = t.c_str();
    char* e = nullptr;
    while (true) {
        while (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r') ++p;
        if (!*p) break;
        const double v = std::strtod(p, &e);
        if (e == p) break;
        out.push_back(v);
        p = e;
    }
}

// HistogramParams of a <Histograms> / <Global_histograms> settings node (LoaderXML.cpp:179-203)
mfg_histogram_params hist_params(const XNode* n) {
    mfg_histogram_params h{};
    h.record = 0;
    h.bounce_binsize = 1;
    h.bounce_max = 0;
    h.distance_binsize = 1.0;
    h.distance_max = 0.0;
    h.time_binsize = 1.0;
    h.time_max = 0.0;
    if (!n) return h;
    if (const XNode* b = n->child("Bounces")) {
        h.record |= MFG_HIST_BOUNCE;
        h.bounce_binsize = uint64_t(ia(b, "binSize", 1));
        h.bounce_max = uint64_t(ia(b, "max", 0));
    }
    if (const XNode* d = n->child("Distance")) {
        h.record |= MFG_HIST_DISTANCE;
        h.distance_binsize = fa(d, "binSize");
        h.distance_max = fa(d, "max");
    }
    if (const XNode* t = n->child("Time")) {
        h.record |= MFG_HIST_TIME;
        h.time_binsize = fa(t, "binSize");
        h.time_max = fa(t, "max");
    }
    return h;
}

// UserMoments entries (TimeMoments::ParseUserMoment, TimeMoments.cpp:58-83): "begin,spacing,end"
// ranges enumerated by repeated addition while time <= end, or single times
void user_moments(const XNode* um, std::vector<double>& times, std::vector<double>& windows) {
    if (!um) return;
    for (const XNode* u : um->children("UserEntry")) {
        const char* c = u->attr("content");
        const double win = fa(u, "window", 0.0);
        std::string s = c ? c : "";
        s.erase(std::remove(s.begin(), s.end(), ' '), s.end());
        std::vector<double> parts;
        size_t pos = 0;
        for (int k = 0; k < 3 && pos <= s.size(); ++k) {
            size_t q = s.find(',', pos);
            const std::string tok = s.substr(pos, q == std::string::npos ? std::string::npos : q - pos);
            char* e = nullptr;
            const double v = std::strtod(tok.c_str(), &e);
            if (tok.empty() || e != tok.c_str() + tok.size()) break;
            parts.push_back(v);
            if (q == std::string::npos) break;
            pos = q + 1;
        }
        if (parts.size() == 1 && parts[0] >= 0.0) {
            times.push_back(parts[0]);
            windows.push_back(win);
        } else if (parts.size() == 3) {
            const double b = parts[0], sp = parts[1], e = parts[2];
            if (b >= 0.0 && e > b && sp < e - b && !(sp < win)) {
                for (double t = b; t <= e; t += sp) {
                    times.push_back(t);
                    windows.push_back(win);
                }
            }
        }
    }
}

}  // namespace

namespace {
// Parameter catalog (TimeDependentParameters::LoadParameterCatalog, MolflowSimGeom.cpp:1250-1319):
// one parameter per .csv file of "t,value" rows in file-name order, named "[catalog] <file name>",
// pairs sorted by t, linear interpolation
bool load_catalog(const std::string& dir, std::vector<std::string>& names,
                  std::vector<std::vector<std::pair<double, double>>>& tables, std::string& err) {
    std::error_code ec;
    if (!std::filesystem::is_directory(dir, ec)) { err = "parameter catalog " + dir + " is not a folder"; return false; }
    std::vector<std::string> files;
    for (const auto& e : std::filesystem::directory_iterator(dir, ec)) {
        const std::string fn = e.path().filename().string();
        if (fn.size() >= 4 && fn.compare(fn.size() - 4, 4, ".csv") == 0) files.push_back(fn);
    }
    std::sort(files.begin(), files.end());
    for (const std::string& fn : files) {
        FILE* f = std::fopen((std::filesystem::path(dir) / fn).string().c_str(), "rb");
        if (!f) { err = "cannot open " + fn; return false; }
        std::string text;
        char buf[1 << 14];
        size_t k;
        while ((k = std::fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, k);
        std::fclose(f);
        if (text.compare(0, 3, "\xEF\xBB\xBF") == 0) text.erase(0, 3);   // UTF-8 byte-order mark
        std::vector<std::pair<double, double>> pairs;
        size_t pos = 0;
        while (pos < text.size()) {
            size_t q = text.find('\n', pos);
            if (q == std::string::npos) q = text.size();
            std::string line = text.substr(pos, q - pos);
            pos = q + 1;
            auto trim = [](std::string x) {
                const size_t a = x.find_first_not_of(" \t\r"), b = x.find_last_not_of(" \t\r");
                return a == std::string::npos ? std::string() : x.substr(a, b - a + 1);
            };
            line = trim(line);
            if (line.empty()) continue;
            const size_t c1 = line.find(',');
            if (c1 == std::string::npos || line.find(',', c1 + 1) != std::string::npos) break;   // not two columns
            const std::string a = trim(line.substr(0, c1)), b = trim(line.substr(c1 + 1));
            char* e1 = nullptr;
            char* e2 = nullptr;
            const double t = std::strtod(a.c_str(), &e1), v = std::strtod(b.c_str(), &e2);
            if (a.empty() || b.empty() || *e1 || *e2) { err = "parameter catalog " + fn + ": bad row \"" + line + "\""; return false; }
            pairs.emplace_back(t, v);
        }
        std::stable_sort(pairs.begin(), pairs.end(), [](const auto& x, const auto& y) { return x.first < y.first; });
        names.push_back("[catalog] " + fn);
        tables.push_back(std::move(pairs));
    }
    return true;
}
}  // namespace

bool XmlModel::load(const std::string& path, std::string& err, const char* catalog_dir) {
    std::string text;
    if (!read_document(path, text, err)) return false;
    if (!doc.parse(text, err)) return false;
    const XNode* r = doc.root();
    const XNode* g = r->child("Geometry");
    if (!g) { err = "no <Geometry> element"; return false; }
    const XNode* vn = g->child("Vertices");
    const XNode* fn = g->child("Facets");
    if (!vn || !fn) { err = "no <Vertices> or <Facets> element"; return false; }
    for (const XNode* v : vn->children("Vertex")) {
        vertices.push_back(fa(v, "x"));
        vertices.push_back(fa(v, "y"));
        vertices.push_back(fa(v, "z"));
    }
    const std::vector<const XNode*> facets = fn->children("Facet");
    const int nf = int(facets.size());
    fv_start.assign(1, 0);
    for (const XNode* f : facets) {
        const XNode* ind = f->child("Indices");
        if (ind)
            for (const XNode* i : ind->children("Indice")) fv_index.push_back(ia32(i, "vertex"));
        fv_start.push_back(int32_t(fv_index.size()));
    }
    // reference defaults (MolflowSimulationModel / facet settings)
    sticking.assign(nf, 0.0); opacity.assign(nf, 1.0); outgassing.assign(nf, 0.0); temperature.assign(nf, 293.15);
    accommodation.assign(nf, 1.0); desorb_type.assign(nf, MFG_DES_NONE); desorb_exponent.assign(nf, 0.0);
    refl_diffuse.assign(nf, 1.0); refl_specular.assign(nf, 0.0); refl_cos_exponent.assign(nf, 0.0);
    is_2sided.assign(nf, 0); structure.assign(nf, 0); link_dest.assign(nf, 0); teleport_dest.assign(nf, 0);
    tex_width.assign(nf, 0.0); tex_height.assign(nf, 0.0); count_flags.assign(nf, 0u); profile_type.assign(nf, MFG_PROFILE_NONE);
    max_speed.assign(nf, 0.0); am_phi_width.assign(nf, 0); am_theta_limit.assign(nf, 1.570796326);
    am_lower.assign(nf, 0); am_higher.assign(nf, 0); am_record.assign(nf, 0);
    sticking_param.assign(nf, -1); opacity_param.assign(nf, -1); outgassing_param.assign(nf, -1); temperature_param.assign(nf, -1);
    enable_sojourn.assign(nf, 0); sojourn_freq.assign(nf, 0.0); sojourn_e.assign(nf, 0.0); is_moving.assign(nf, 0);
    facet_hist.assign(nf, hist_params(nullptr));
    og_w.assign(nf, 0); og_h.assign(nf, 0); og_ru.assign(nf, 0.0); og_rv.assign(nf, 0.0);

    // time-dependent parameters (LoaderXML.cpp:69-100)
    const XNode* sims = r->child("MolflowSimuSettings");
    param_start.assign(1, 0);
    if (const XNode* pn = kid(sims, "Parameters")) {
        for (const XNode* p : pn->children("Parameter")) {
            for (const XNode* m : p->children("Moment")) {
                param_t.push_back(fa(m, "t"));
                param_v.push_back(fa(m, "value"));
            }
            param_start.push_back(int32_t(param_t.size()));
            param_log_x.push_back(uint8_t(ia(p, "logXinterp")));
            param_log_y.push_back(uint8_t(ia(p, "logYinterp")));
            const char* nm = p->attr("name");
            param_names.push_back(nm ? nm : "");
        }
    }
    if (catalog_dir && *catalog_dir) {   // catalog parameters follow the file's own
        std::vector<std::string> names;
        std::vector<std::vector<std::pair<double, double>>> tables;
        if (!load_catalog(catalog_dir, names, tables, err)) return false;
        for (size_t i = 0; i < names.size(); ++i) {
            for (const auto& tv : tables[i]) {
                param_t.push_back(tv.first);
                param_v.push_back(tv.second);
            }
            param_start.push_back(int32_t(param_t.size()));
            param_log_x.push_back(0);
            param_log_y.push_back(0);
            param_names.push_back(names[i]);
        }
    }
    // a facet's parameter: by name (newer files), else by index (LoaderXML.cpp:847-925)
    auto param_ref = [&](const XNode* n, const char* name_attr, int32_t& out) {
        if (!n) return true;
        const char* nm = n->attr(name_attr);
        if (nm && *nm) {
            auto it = std::find(param_names.begin(), param_names.end(), std::string(nm));
            if (it == param_names.end()) {
                err = std::string("parameter \"") + nm + "\" not found";
                return false;
            }
            out = int32_t(it - param_names.begin());
            return true;
        }
        out = ia32(n, "parameterId", -1);
        return true;
    };

    std::vector<std::vector<double>> am_maps(nf);
    std::vector<std::vector<double>> og_maps(nf);
    for (int k = 0; k < nf; ++k) {
        const XNode* f = facets[k];
        const XNode* st = f->child("Sticking");
        const XNode* op = f->child("Opacity");
        const XNode* og = f->child("Outgassing");
        const XNode* te = f->child("Temperature");
        const XNode* rf = f->child("Reflection");
        const XNode* su = f->child("Structure");
        const XNode* rec = f->child("Recordings");
        const XNode* tx = kid(rec, "Texture");
        sticking[k] = fa(st, "constValue");
        if (!param_ref(st, "stickingParam", sticking_param[k])) return false;
        opacity[k] = fa(op, "constValue", 1.0);
        if (!param_ref(op, "opacityParam", opacity_param[k])) return false;
        is_2sided[k] = uint8_t(ia(op, "is2sided"));
        outgassing[k] = fa(og, "constValue");
        if (!param_ref(og, "OutgassingParam", outgassing_param[k])) return false;
        desorb_type[k] = ia32(og, "desType");
        desorb_exponent[k] = fa(og, "desExponent");
        temperature[k] = fa(te, "value", 293.15);
        if (!param_ref(te, "tempParam", temperature_param[k])) return false;
        accommodation[k] = fa(te, "accFactor", 1.0);
        if (rf && rf->attr("diffusePart")) {
            refl_diffuse[k] = fa(rf, "diffusePart", 1.0);
            refl_specular[k] = fa(rf, "specularPart", 0.0);
            refl_cos_exponent[k] = fa(rf, "cosineExponent", 0.0);
        } else if (rf) {   // older files: reflection type 0 diffuse, 1 specular, else neither
            const long long t = ia(rf, "type");
            refl_diffuse[k] = t == 0 ? 1.0 : 0.0;
            refl_specular[k] = t == 1 ? 1.0 : 0.0;
        }
        enable_sojourn[k] = uint8_t(ia(rf, "enableSojournTime"));
        sojourn_freq[k] = fa(rf, "sojournFreq");
        sojourn_e[k] = fa(rf, "sojournE");
        structure[k] = ia32(su, "inStructure");
        link_dest[k] = ia32(su, "linksTo");
        teleport_dest[k] = ia32(f->child("Teleport"), "target");
        is_moving[k] = uint8_t(ia(f->child("Motion"), "isMoving"));
        if (rec) {
            profile_type[k] = ia32(rec->child("Profile"), "type");
            if (const XNode* am = rec->child("IncidentAngleMap")) {
                am_record[k] = uint8_t(ia(am, "record"));
                am_phi_width[k] = ia32(am, "phiWidth");
                am_theta_limit[k] = fa(am, "thetaLimit", 1.570796326);
                am_lower[k] = ia32(am, "thetaLowerRes");
                am_higher[k] = ia32(am, "thetaHigherRes");
            }
        }
        // a recorded angle map in the facet node sets the map parameters and is the source of
        // angle-map desorption; without one, angle-map desorption falls back to none
        // (LoaderXML.cpp:1043-1073)
        const XNode* gam = f->child("IncidentAngleMap");
        if (gam && gam->child("map") && gam->attr("angleMapThetaLimit")) {
            am_phi_width[k] = ia32(gam, "angleMapPhiWidth");
            am_theta_limit[k] = fa(gam, "angleMapThetaLimit");
            am_lower[k] = ia32(gam, "angleMapThetaLowerRes");
            am_higher[k] = ia32(gam, "angleMapThetaHigherRes");
            if (desorb_type[k] == MFG_DES_ANGLEMAP) numbers(gam->child("map")->text, am_maps[k]);
        } else if (desorb_type[k] == MFG_DES_ANGLEMAP) {
            desorb_type[k] = MFG_DES_NONE;
        }
        // outgassing map (MolflowFacet.cpp:249-285): used when the Outgassing node asks for it and
        // the DynamicOutgassing node has a map; the old format has one square ratio
        const XNode* dyn = f->child("DynamicOutgassing");
        if (ia(og, "useOutgassingFile") && dyn && dyn->child("map")) {
            const int w = int(ia(dyn, "width")), h = int(ia(dyn, "height"));
            const double ru = fa(dyn, "ratioU", fa(dyn, "ratio")), rv = fa(dyn, "ratioV", fa(dyn, "ratio"));
            std::vector<double> vals;
            numbers(dyn->child("map")->text, vals);
            if (w > 0 && h > 0 && vals.size() >= size_t(w) * size_t(h)) {
                og_w[k] = w; og_h[k] = h; og_ru[k] = ru; og_rv[k] = rv;
                vals.resize(size_t(w) * size_t(h));
                og_maps[k] = std::move(vals);
            }
        }
        facet_hist[k] = hist_params(f->child("Histograms"));
        if (tx) {
            tex_width[k] = fa(tx, "texDimX");
            tex_height[k] = fa(tx, "texDimY");
            uint32_t fl = 0;
            if (ia(tx, "countDes")) fl |= MFG_COUNT_DES;
            if (ia(tx, "countAbs")) fl |= MFG_COUNT_ABS;
            if (ia(tx, "countRefl")) fl |= MFG_COUNT_REFL;
            if (ia(tx, "countTrans")) fl |= MFG_COUNT_TRANS;
            if (ia(tx, "countDir")) fl |= MFG_COUNT_DIR;
            count_flags[k] = fl;
        }
    }
    // angle maps of the facets that desorb by angle map, in facet order, each cut or padded to
    // phiWidth x (lowerRes + higherRes) counts
    for (int k = 0; k < nf; ++k) {
        if (desorb_type[k] != MFG_DES_ANGLEMAP) continue;
        const int64_t n = int64_t(std::max(am_phi_width[k], 0)) * std::max<int64_t>(int64_t(am_lower[k]) + am_higher[k], 0);
        if (n > int64_t(INT32_MAX)) {
            err = "facet " + std::to_string(k + 1) + ": angle map of more than 2^31-1 cells";
            return false;
        }
        for (int64_t i = 0; i < n; ++i)
            desorb_anglemap.push_back(size_t(i) < am_maps[k].size() ? to_u64(am_maps[k][size_t(i)]) : 0ull);
    }
    bool any_og = false;
    for (int k = 0; k < nf; ++k)
        if (og_w[k] > 0) { any_og = true; og_cells.insert(og_cells.end(), og_maps[k].begin(), og_maps[k].end()); }
    bool any_hist = false;
    for (int k = 0; k < nf; ++k) any_hist = any_hist || facet_hist[k].record != 0;

    std::memset(&desc, 0, sizeof desc);
    desc.abi_version = MFG_ABI_VERSION;
    desc.n_vertices = int32_t(vertices.size() / 3);
    desc.vertices = vertices.data();
    desc.n_facets = nf;
    desc.facet_vertex_start = fv_start.data();
    desc.facet_vertex_index = fv_index.data();
    desc.sticking = sticking.data(); desc.opacity = opacity.data(); desc.outgassing = outgassing.data();
    desc.temperature = temperature.data(); desc.accommodation = accommodation.data(); desc.desorb_type = desorb_type.data();
    desc.desorb_exponent = desorb_exponent.data(); desc.refl_diffuse = refl_diffuse.data(); desc.refl_specular = refl_specular.data();
    desc.refl_cos_exponent = refl_cos_exponent.data(); desc.is_2sided = is_2sided.data(); desc.structure = structure.data();
    desc.link_dest = link_dest.data(); desc.teleport_dest = teleport_dest.data(); desc.tex_width = tex_width.data();
    desc.tex_height = tex_height.data(); desc.count_flags = count_flags.data(); desc.profile_type = profile_type.data();
    desc.max_speed = max_speed.data(); desc.anglemap_phi_width = am_phi_width.data(); desc.anglemap_theta_limit = am_theta_limit.data();
    desc.anglemap_theta_lower_res = am_lower.data(); desc.anglemap_theta_higher_res = am_higher.data();
    desc.anglemap_record = am_record.data(); desc.sticking_param = sticking_param.data(); desc.opacity_param = opacity_param.data();
    desc.outgassing_param = outgassing_param.data(); desc.temperature_param = temperature_param.data();
    desc.enable_sojourn = enable_sojourn.data(); desc.sojourn_freq = sojourn_freq.data(); desc.sojourn_e = sojourn_e.data();
    desc.is_moving = is_moving.data();

    // simulation settings
    desc.gas_mass = 28.0; desc.use_maxwell = 1; desc.constant_flow = 1; desc.time_window = 1e-10;
    desc.enable_decay = 0; desc.half_life = 1.0; desc.low_flux_mode = 0; desc.low_flux_cutoff = 1e-7;
    desc.scatter_mass_ratio = 1.0; desc.scatter_mean_free_path_cm = 1e30; desc.scatter_rho = 1e-8;
    desc.log_facet = -1; desc.log_limit = 0;
    desc.n_structures = int32_t(std::max<long long>(1, ia(g->child("Structures"), "nb", 1)));
    desc.global_histogram = hist_params(nullptr);
    std::vector<double> mt, mw;
    if (sims) {
        const XNode* gas = sims->child("Gas");
        desc.gas_mass = fa(gas, "mass", 28.0);
        if (const XNode* sc = kid(gas, "Scattering")) {   // LoaderXML.cpp:106-116 (rho is not in the file)
            desc.scatter_enabled = ia32(sc, "enabled");
            desc.scatter_mass_ratio = fa(sc, "massRatio", 1.0);
            desc.scatter_mean_free_path_cm = fa(sc, "meanFreePath_cm", 1e30);
            if (const XNode* co = sc->child("LowSpeedCutoff")) {
                desc.scatter_cutoff_enabled = ia32(co, "enabled");
                desc.scatter_cutoff_speed = fa(co, "speed");
            }
        }
        if (const XNode* mo = sims->child("Motion")) {   // LoaderXML.cpp:144-160
            desc.motion_type = ia32(mo, "type");
            if (desc.motion_type == 1) {
                const XNode* v = mo->child("VelocityVector");
                desc.motion_vector2[0] = fa(v, "vx"); desc.motion_vector2[1] = fa(v, "vy"); desc.motion_vector2[2] = fa(v, "vz");
            } else if (desc.motion_type == 2) {
                const XNode* b = mo->child("AxisBasePoint");
                const XNode* rv = mo->child("RotationVector");
                desc.motion_vector1[0] = fa(b, "x"); desc.motion_vector1[1] = fa(b, "y"); desc.motion_vector1[2] = fa(b, "z");
                desc.motion_vector2[0] = fa(rv, "x"); desc.motion_vector2[1] = fa(rv, "y"); desc.motion_vector2[2] = fa(rv, "z");
            }
        }
        desc.enable_decay = ia32(gas, "enableDecay");
        desc.half_life = fa(gas, "halfLife", 1.0);
        if (const XNode* fm = sims->child("MeasureForces")) {   // LoaderXML.cpp:163-177
            desc.enable_force_measurement = ia32(fm, "enabled");
            if (const XNode* rp = kid(fm->child("Torque"), "refPoint")) {
                desc.torque_ref_point[0] = fa(rp, "x"); desc.torque_ref_point[1] = fa(rp, "y"); desc.torque_ref_point[2] = fa(rp, "z");
            }
        }
        const XNode* lf = sims->child("LowFluxMode");
        desc.low_flux_mode = ia32(lf, "enabled");
        desc.low_flux_cutoff = fa(lf, "cutoff", 1e-7);
        desc.global_histogram = hist_params(sims->child("Global_histograms"));
        const XNode* ts = sims->child("TimeSettings");
        desc.time_window = fa(ts, "timeWindow", 1e-10);
        desc.use_maxwell = ia32(ts, "useMaxwellDistr", 1);
        desc.constant_flow = ia32(ts, "calcConstFlow", 1);
        user_moments(kid(ts, "UserMoments"), mt, mw);
    }
    {   // moments sorted by time (stable)
        std::vector<size_t> order(mt.size());
        std::iota(order.begin(), order.end(), size_t(0));
        std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return mt[a] < mt[b]; });
        for (size_t i : order) { moment_time.push_back(mt[i]); moment_window.push_back(mw[i]); }
    }
    desc.n_moments = int32_t(moment_time.size());
    desc.moment_time = moment_time.data();
    desc.moment_window = moment_window.data();
    desc.n_params = int32_t(param_names.size());
    desc.param_start = param_start.data();
    desc.param_t = param_t.data();
    desc.param_v = param_v.data();
    desc.param_log_x = param_log_x.data();
    desc.param_log_y = param_log_y.data();
    desc.facet_histogram = any_hist ? facet_hist.data() : nullptr;
    desc.desorb_anglemap = desorb_anglemap.empty() ? nullptr : desorb_anglemap.data();
    if (any_og) {
        desc.outgassing_map_width = og_w.data();
        desc.outgassing_map_height = og_h.data();
        desc.outgassing_map_ratio_u = og_ru.data();
        desc.outgassing_map_ratio_v = og_rv.data();
        desc.outgassing_map = og_cells.data();
    }
    return true;
}

namespace {
// stored histogram bins of a results <Histograms> node: bounce, distance, time, those recorded
void hist_values(const XNode* n, const int32_t sizes[3], double* out) {
    static const char* tags[3] = {"Bounces", "Distance", "Time"};
    size_t o = 0;
    for (int t = 0; t < 3; ++t) {
        const int32_t sz = sizes[t];
        if (sz <= 0) continue;
        const XNode* h = kid(n, tags[t]);
        if (h && ia(h, "size") == sz) {
            int32_t b = 0;
            for (const XNode* bin : h->children("Bin")) {
                if (b >= sz) break;
                out[o + size_t(b++)] = fa(bin, "count");
            }
        }
        o += size_t(sz);
    }
}
}  // namespace

int read_results(const XNode* r, const mfg::HostModel& h, mfg_state_view* v, std::string& err) {
    const XNode* res = r->child("MolflowResults");
    if (!res) { err = "the file holds no results"; return MFG_ERR_INVALID_ARGUMENT; }
    const mfg_state_layout& L = h.layout;
    const int64_t F = L.n_facets, B = 1 + L.n_moments;
    const std::vector<const XNode*> moments = kid(res, "Moments") ? res->child("Moments")->children("Moment")
                                                                   : std::vector<const XNode*>();
    if (v->global)
        for (int64_t i = 0; i < L.n_global; ++i) v->global[i] = 0;
    auto zero = [](auto* p, int64_t n) { if (p) std::fill(p, p + n, 0); };
    zero(v->facet_counts, L.n_facet_counts); zero(v->facet_sums, L.n_facet_sums); zero(v->texture, L.n_texture);
    zero(v->profile, L.n_profile); zero(v->direction, L.n_direction); zero(v->anglemap, L.n_anglemap);
    zero(v->histogram, L.n_histogram);
    const int32_t gsz[3] = {h.ghist.nb, h.ghist.nd, h.ghist.nt};
    for (size_t mi = 0; mi < moments.size() && int64_t(mi) < B; ++mi) {
        const XNode* mom = moments[mi];
        if (mi == 0 && v->global) {
            const XNode* gh = kid(kid(mom, "Global"), "Hits");
            v->global[MFG_G_NBMCHIT] = fa(gh, "totalHit");
            v->global[MFG_G_NBHITEQUIV] = fa(gh, "totalHitEquiv");
            v->global[MFG_G_NBDESORBED] = fa(gh, "totalDes");
            v->global[MFG_G_NBABSEQUIV] = fa(gh, "totalAbsEquiv");
            v->global[MFG_G_NBLEAK] = fa(gh, "totalLeak");
            v->global[MFG_G_DIST_TOTAL] = fa(gh, "totalDist_total");
            v->global[MFG_G_DIST_FULLHITS] = fa(gh, "totalDist_fullHitsOnly");
        }
        if (v->histogram && L.histogram_bins > 0 && gsz[0] + gsz[1] + gsz[2] > 0)
            hist_values(mom->child("Histograms"), gsz, v->histogram + int64_t(mi) * L.histogram_bins + h.ghist.off);
        const XNode* frs = mom->child("FacetResults");
        if (!frs) continue;
        for (const XNode* fr : frs->children("Facet")) {
            const int64_t k = ia(fr, "id", -1);
            if (k < 0 || k >= F) continue;
            if (v->histogram && L.histogram_bins > 0 && !h.fhist.empty() && h.fhist[size_t(k)].off >= 0) {
                const HistDev& hd = h.fhist[size_t(k)];
                const int32_t sz[3] = {hd.nb, hd.nd, hd.nt};
                hist_values(fr->child("Histograms"), sz, v->histogram + int64_t(mi) * L.histogram_bins + hd.off);
            }
            const XNode* hh = fr->child("Hits");
            const size_t fo = size_t(mi * F + k);
            if (v->facet_counts && hh) {
                v->facet_counts[fo * MFG_FC_N + MFG_FC_NBMCHIT] = uint64_t(ia(hh, "nbHit"));
                v->facet_counts[fo * MFG_FC_N + MFG_FC_NBDESORBED] = uint64_t(ia(hh, "nbDes"));
                v->facet_counts[fo * MFG_FC_N + MFG_FC_NBABSORBED] = to_u64(std::nearbyint(fa(hh, "nbAbsEquiv")));
            }
            if (v->facet_sums && hh) {
                double* s = v->facet_sums + fo * MFG_FS_N;
                s[MFG_FS_NBHITEQUIV] = fa(hh, "nbHitEquiv");
                s[MFG_FS_NBABSEQUIV] = fa(hh, "nbAbsEquiv");
                s[MFG_FS_SUM_V_ORT] = fa(hh, "sum_v_ort");
                s[MFG_FS_SUM_1_PER_ORT_VEL] = fa(hh, "sum_1_per_v");
                s[MFG_FS_SUM_1_PER_VELOCITY] = fa(hh, "sum_v");
            }
            const XNode* pr = fr->child("Profile");
            if (v->profile && pr && h.prof_idx[size_t(k)] >= 0) {
                double* p = v->profile + (int64_t(mi) * L.profile_facets + h.prof_idx[size_t(k)]) * MFG_PROFILE_SIZE * 3;
                for (const XNode* s : pr->children("Slice")) {
                    const long long j = ia(s, "id", -1);
                    if (j < 0 || j >= MFG_PROFILE_SIZE) continue;
                    p[j * 3 + 0] = fa(s, "countEquiv");
                    p[j * 3 + 1] = fa(s, "sum_v_ort");
                    p[j * 3 + 2] = fa(s, "sum_1_per_v");
                }
            }
            const XNode* tx = fr->child("Texture");
            if (v->texture && tx && h.tex_off[size_t(k)] >= 0) {
                const int64_t w = h.tex_w[size_t(k)], hgt = h.tex_h[size_t(k)];
                const int64_t fw = ia(tx, "width"), fh = ia(tx, "height");
                static const char* tags[3] = {"count", "sum_v_ort", "sum_1_per_v"};
                for (int field = 0; field < 3; ++field) {
                    const XNode* c = tx->child(tags[field]);
                    if (!c) continue;
                    std::vector<double> vals;
                    numbers(c->text, vals);
                    const int64_t nv = int64_t(vals.size());
                    if (fw <= 0 || fh <= 0 || fw > nv || fh > nv / fw) continue;   // fewer than fw*fh numbers
                    double* t = v->texture + (int64_t(mi) * L.texture_cells + h.tex_off[size_t(k)]) * 3;
                    for (int64_t y = 0; y < std::min(hgt, fh); ++y)
                        for (int64_t x = 0; x < std::min(w, fw); ++x) t[(y * w + x) * 3 + field] = vals[size_t(y * fw + x)];
                }
            }
            const XNode* dn = fr->child("Directions");
            if (v->direction && dn && h.dir_off[size_t(k)] >= 0) {
                const int64_t cells = int64_t(h.tex_w[size_t(k)]) * h.tex_h[size_t(k)];
                double* d = v->direction + (int64_t(mi) * L.direction_cells + h.dir_off[size_t(k)]) * 4;
                if (const XNode* vv = dn->child("vel.vectors")) {   // "x,y,z" items separated by tabs or newlines
                    const std::string& s = vv->text;
                    int64_t c = 0;
                    size_t pos = 0;
                    while (c < cells && pos < s.size()) {
                        size_t q = s.find_first_of("\t\n", pos);
                        if (q == std::string::npos) q = s.size();
                        const std::string item = s.substr(pos, q - pos);
                        pos = q + 1;
                        if (item.find_first_not_of(" \r") == std::string::npos) continue;
                        const char* ip = item.c_str();
                        char* e = nullptr;
                        for (int a = 0; a < 3; ++a) {
                            d[c * 4 + a] = std::strtod(ip, &e);
                            ip = (*e == ',') ? e + 1 : e;
                        }
                        ++c;
                    }
                }
                if (const XNode* cn = dn->child("count")) {
                    std::vector<double> vals;
                    numbers(cn->text, vals);
                    for (int64_t c = 0; c < std::min<int64_t>(cells, int64_t(vals.size())); ++c) d[c * 4 + 3] = vals[size_t(c)];
                }
            }
        }
    }
    // recorded incident-angle maps sit in the geometry's facet nodes (LoaderXML.cpp:1043-1070)
    if (v->anglemap) {
        const XNode* fn = kid(r->child("Geometry"), "Facets");
        const std::vector<const XNode*> facets = fn ? fn->children("Facet") : std::vector<const XNode*>();
        for (size_t k = 0; k < facets.size() && int64_t(k) < F; ++k) {
            const XNode* am = facets[k]->child("IncidentAngleMap");
            if (!am || !am->child("map") || !am->attr("angleMapThetaLimit") || h.ang_off[k] < 0) continue;
            std::vector<double> vals;
            numbers(am->child("map")->text, vals);
            const int64_t o = h.ang_off[k];
            const int64_t n = std::min<int64_t>(int64_t(vals.size()), L.n_anglemap - o);
            for (int64_t i = 0; i < n; ++i) v->anglemap[o + i] = to_u64(vals[size_t(i)]);
        }
    }
    return MFG_OK;
}

}  // namespace mfgx
