// xml_writer.cpp — a model and its results as a MolFlow+ file, on the C++ host.
//
// The `<SimulationEnvironment type="molflow">` document of src/IO/WriterXML.cpp (SaveGeometry
// :72-365, SaveFacet :684-903, SaveSimulationState :367-682): vertices; facets with their settings,
// outgassing maps, angle-map settings and maps, histogram settings; the simulation settings (gas,
// decay, scattering, low-flux mode, time settings with the moments, motion, forces, parameters,
// global histograms); and per moment the global counters, facet hit buffers, forces, profiles,
// textures, direction cells and histograms.  The GUI's interface settings and the hit/leak display
// caches are not part of a result and are written empty.  Numbers are written in their shortest
// round-trip decimal form; a path ending in ".zip" gets one stored (uncompressed) XML entry.
#include "xml_writer.h"

#include <algorithm>
#include <charconv>
#include <cstdio>
#include <cstring>
#include <type_traits>

#include "xml_file.h"

namespace mfgx {

namespace {

const char* profile_name(int t) {
    static const char* n[] = {"none", "pressure u", "pressure v", "angular", "speed", "ortho.v", "tang.v."};
    return (t >= 0 && t <= 6) ? n[t] : "none";
}

std::string num(double x) {
    char b[64];
    auto r = std::to_chars(b, b + sizeof b, x);   // shortest representation that reads back exactly
    return std::string(b, r.ptr);
}
template <class T, typename std::enable_if<std::is_integral<T>::value, int>::type = 0>
std::string num(T x) {
    return std::to_string(x);
}
// a count held as a double, written as an integer: not a number -> 0, clamped to the 64-bit range
std::string count(double x) {
    if (!(x == x)) return "0";
    if (x >= 9.2e18) return num(9200000000000000000LL);
    if (x <= -9.2e18) return num(-9200000000000000000LL);
    return num((long long)x);
}

std::string esc(const std::string& s) {
    std::string o;
    for (char c : s) {
        if (c == '&') o += "&amp;";
        else if (c == '<') o += "&lt;";
        else if (c == '>') o += "&gt;";
        else if (c == '"') o += "&quot;";
        else o += c;
    }
    return o;
}

// streaming element writer
class W {
public:
    std::string out;
    void open(const char* tag, std::initializer_list<std::pair<const char*, std::string>> attrs, bool empty = false) {
        out += '<';
        out += tag;
        for (const auto& a : attrs) {
            out += ' ';
            out += a.first;
            out += "=\"";
            out += esc(a.second);
            out += '"';
        }
        out += empty ? " />" : ">";
    }
    void leaf(const char* tag, std::initializer_list<std::pair<const char*, std::string>> attrs) { open(tag, attrs, true); }
    void close(const char* tag) {
        out += "</";
        out += tag;
        out += '>';
    }
    void text(const char* tag, const std::string& t) {
        out += '<';
        out += tag;
        out += '>';
        out += t;
        close(tag);
    }
};

// rows of a w x h grid, tab separated, one line per row
template <class F>
std::string grid(int64_t w, int64_t h, F value) {
    std::string s = "\n";
    for (int64_t y = 0; y < h; ++y) {
        for (int64_t x = 0; x < w; ++x) {
            s += value(y * w + x);
            s += '\t';
        }
        s += '\n';
    }
    return s;
}

void hist_settings(W& w, const mfg_histogram_params& p) {
    if (p.record & MFG_HIST_BOUNCE)
        w.leaf("Bounces", {{"binSize", num((unsigned long long)p.bounce_binsize)}, {"max", num((unsigned long long)p.bounce_max)}});
    if (p.record & MFG_HIST_DISTANCE) w.leaf("Distance", {{"binSize", num(p.distance_binsize)}, {"max", num(p.distance_max)}});
    if (p.record & MFG_HIST_TIME) w.leaf("Time", {{"binSize", num(p.time_binsize)}, {"max", num(p.time_max)}});
}

void hist_results(W& w, const mfg_histogram_params& p, const int32_t sizes[3], const double* v) {
    static const char* tags[3] = {"Bounces", "Distance", "Time"};
    const uint32_t rec[3] = {MFG_HIST_BOUNCE, MFG_HIST_DISTANCE, MFG_HIST_TIME};
    const double bs[3] = {double(p.bounce_binsize), p.distance_binsize, p.time_binsize};
    const std::string bss[3] = {num((unsigned long long)p.bounce_binsize), num(p.distance_binsize), num(p.time_binsize)};
    const std::string mxs[3] = {num((unsigned long long)p.bounce_max), num(p.distance_max), num(p.time_max)};
    size_t o = 0;
    for (int t = 0; t < 3; ++t) {
        const int32_t n = sizes[t];
        if (!(p.record & rec[t]) || n <= 0) continue;
        w.open(tags[t], {{"size", num(n)}, {"binSize", bss[t]}, {"max", mxs[t]}});
        for (int32_t k = 0; k < n; ++k)
            w.leaf("Bin", {{"start", k == n - 1 ? std::string("overRange") : (t == 0 ? num(uint64_t(k) * p.bounce_binsize) : num(k * bs[t]))},
                           {"count", num(v[o + size_t(k)])}});
        w.close(tags[t]);
        o += size_t(n);
    }
}

bool write_stored_zip(const std::string& path, const std::string& inner, const std::string& data, std::string& err) {
    // one stored entry: local header, data, central directory, end record (PKWARE APPNOTE)
    const uint32_t crc = crc32(reinterpret_cast<const uint8_t*>(data.data()), data.size());
    if (data.size() + 2 * inner.size() + 128 >= 0xffffffffull || inner.size() > 0xffff) {   // offsets and sizes are 32-bit
        err = "the document is too large for a ZIP archive without ZIP64";
        return false;
    }
    std::string z;
    auto u16 = [&](uint32_t v) { z += char(v & 0xff); z += char((v >> 8) & 0xff); };
    auto u32 = [&](uint32_t v) { u16(v & 0xffff); u16(v >> 16); };
    const uint32_t size = uint32_t(data.size());
    u32(0x04034b50u); u16(20); u16(0); u16(0); u16(0); u16(0x21);   // version, flags, stored, time, date (1980-01-01)
    u32(crc); u32(size); u32(size); u16(uint32_t(inner.size())); u16(0);
    z += inner;
    z += data;
    const uint32_t cd = uint32_t(z.size());
    u32(0x02014b50u); u16(20); u16(20); u16(0); u16(0); u16(0); u16(0x21);
    u32(crc); u32(size); u32(size); u16(uint32_t(inner.size())); u16(0); u16(0); u16(0); u16(0); u32(0); u32(0);
    z += inner;
    const uint32_t cdsize = uint32_t(z.size()) - cd;
    u32(0x06054b50u); u16(0); u16(0); u16(1); u16(1); u32(cdsize); u32(cd); u16(0);
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) { err = "cannot write " + path; return false; }
    const bool ok = std::fwrite(z.data(), 1, z.size(), f) == z.size();
    return (std::fclose(f) == 0) && ok ? true : (err = "write error on " + path, false);
}

}  // namespace

bool write_file(const std::string& path, const mfg_model_desc& d, const mfg::HostModel& h, const mfg_state_view* st,
                const std::vector<std::string>& param_names, std::string& err) {
    const int nf = d.n_facets;
    const mfg_state_layout& L = h.layout;
    const int nm = d.n_moments;
    auto pname = [&](int p) { return p < int(param_names.size()) && !param_names[size_t(p)].empty() ? param_names[size_t(p)] : "param" + std::to_string(p); };
    auto fd = [&](const double* a, int i, double def) { return a ? a[i] : def; };
    auto fi = [&](const int32_t* a, int i, int def) { return a ? int(a[i]) : def; };
    auto fu8 = [&](const uint8_t* a, int i) { return a ? int(a[i]) : 0; };
    W w;
    w.out = "<?xml version='1.0' encoding='utf-8'?>\n";
    w.open("SimulationEnvironment", {{"type", "molflow"}, {"version", "2.9.25"}});
    // ---- geometry (SaveGeometry / SaveFacet) ----
    w.open("Geometry", {});
    w.open("Vertices", {{"nb", num(d.n_vertices)}});
    for (int i = 0; i < d.n_vertices; ++i)
        w.leaf("Vertex", {{"id", num(i)}, {"x", num(d.vertices[3 * i])}, {"y", num(d.vertices[3 * i + 1])}, {"z", num(d.vertices[3 * i + 2])}});
    w.close("Vertices");
    w.open("Facets", {{"nb", num(nf)}});
    size_t og_cell = 0, am_src = 0;
    for (int i = 0; i < nf; ++i) {
        w.open("Facet", {{"id", num(i)}});
        const int two = fu8(d.is_2sided, i);
        auto const_or_param = [&](const char* tag, const char* pattr, double value, int p, double def, bool close_now) {
            if (p >= 0) w.out += std::string("<") + tag + " " + pattr + "=\"" + esc(pname(p)) + "\" parameterId=\"" + num(p) +
                                 "\" constValue=\"" + num(def) + "\"";
            else w.out += std::string("<") + tag + " constValue=\"" + num(value) + "\" parameterId=\"-1\"";
            if (close_now) w.out += " />";
        };
        const_or_param("Sticking", "stickingParam", fd(d.sticking, i, 0.0), fi(d.sticking_param, i, -1), 0.0, true);
        const_or_param("Opacity", "opacityParam", fd(d.opacity, i, 1.0), fi(d.opacity_param, i, -1), 1.0, false);
        w.out += " is2sided=\"" + num(two) + "\" />";
        const bool has_map = d.outgassing_map_width && d.outgassing_map_width[i] > 0;
        const_or_param("Outgassing", "outgassingParam", fd(d.outgassing, i, 0.0), fi(d.outgassing_param, i, -1), 0.0, false);
        w.out += " is2sided=\"" + num(two) + "\" desType=\"" + num(fi(d.desorb_type, i, MFG_DES_NONE)) + "\" desExponent=\"" +
                 num(fd(d.desorb_exponent, i, 0.0)) + "\" hasOutgassingFile=\"" + num(int(has_map)) + "\" useOutgassingFile=\"" +
                 num(int(has_map)) + "\" />";
        if (fi(d.temperature_param, i, -1) >= 0)
            w.leaf("Temperature", {{"tempParam", pname(fi(d.temperature_param, i, -1))}, {"accFactor", num(fd(d.accommodation, i, 1.0))}});
        else
            w.leaf("Temperature", {{"value", num(fd(d.temperature, i, 293.15))}, {"accFactor", num(fd(d.accommodation, i, 1.0))}});
        w.leaf("Area", {{"m2", num(h.facets[size_t(i)].area * 1e-4)}});
        const double df = fd(d.refl_diffuse, i, 1.0), sp = fd(d.refl_specular, i, 0.0);
        w.leaf("Reflection", {{"diffusePart", num(df)}, {"specularPart", num(sp)}, {"cosineExponent", num(fd(d.refl_cos_exponent, i, 0.0))},
                              {"type", num(df > 0.99 ? 0 : (sp > 0.99 ? 1 : 2))}, {"enableSojournTime", num(fu8(d.enable_sojourn, i))},
                              {"sojournFreq", num(fd(d.sojourn_freq, i, 0.0))}, {"sojournE", num(fd(d.sojourn_e, i, 0.0))}});
        w.leaf("Structure", {{"inStructure", num(fi(d.structure, i, 0))}, {"linksTo", num(fi(d.link_dest, i, 0))}});
        w.leaf("Teleport", {{"target", num(fi(d.teleport_dest, i, 0))}});
        w.leaf("Motion", {{"isMoving", num(fu8(d.is_moving, i))}});
        w.open("Recordings", {});
        const int pt = fi(d.profile_type, i, MFG_PROFILE_NONE);
        w.leaf("Profile", {{"type", num(pt)}, {"name", profile_name(pt)}});
        const uint32_t cf = d.count_flags ? d.count_flags[i] : 0u;
        w.leaf("Texture", {{"hasMesh", num(int((cf & (MFG_COUNT_DES | MFG_COUNT_ABS | MFG_COUNT_REFL | MFG_COUNT_TRANS)) != 0))},
                           {"texDimX", num(fd(d.tex_width, i, 0.0))}, {"texDimY", num(fd(d.tex_height, i, 0.0))},
                           {"countDes", num(int((cf & MFG_COUNT_DES) != 0))}, {"countAbs", num(int((cf & MFG_COUNT_ABS) != 0))},
                           {"countRefl", num(int((cf & MFG_COUNT_REFL) != 0))}, {"countTrans", num(int((cf & MFG_COUNT_TRANS) != 0))},
                           {"countDir", num(int((cf & MFG_COUNT_DIR) != 0))}, {"countAC", "0"}});
        const int amw = fi(d.anglemap_phi_width, i, 0);
        const int amrows = fi(d.anglemap_theta_lower_res, i, 0) + fi(d.anglemap_theta_higher_res, i, 0);
        const double amlim = fd(d.anglemap_theta_limit, i, 1.570796326);
        if (fu8(d.anglemap_record, i))
            w.leaf("IncidentAngleMap", {{"record", num(fu8(d.anglemap_record, i))}, {"phiWidth", num(amw)}, {"thetaLimit", num(amlim)},
                                        {"thetaLowerRes", num(fi(d.anglemap_theta_lower_res, i, 0))},
                                        {"thetaHigherRes", num(fi(d.anglemap_theta_higher_res, i, 0))}});
        w.close("Recordings");
        const int nv = d.facet_vertex_start[i + 1] - d.facet_vertex_start[i];
        w.open("Indices", {{"nb", num(nv)}});
        for (int k = 0; k < nv; ++k) w.leaf("Indice", {{"id", num(k)}, {"vertex", num(d.facet_vertex_index[d.facet_vertex_start[i] + k])}});
        w.close("Indices");
        if (has_map) {
            const int mw = d.outgassing_map_width[i], mh = d.outgassing_map_height[i];
            const double* cells = d.outgassing_map + og_cell;
            double tot = 0;
            for (int k = 0; k < mw * mh; ++k) tot += cells[k];
            w.open("DynamicOutgassing", {{"width", num(mw)}, {"height", num(mh)}, {"ratioU", num(d.outgassing_map_ratio_u[i])},
                                         {"ratioV", num(d.outgassing_map_ratio_v[i])}, {"totalDose", "0"}, {"totalOutgassing", num(tot)},
                                         {"totalFlux", "0"}});
            w.text("map", grid(mw, mh, [&](int64_t k) { return num(cells[k]); }));
            w.close("DynamicOutgassing");
            og_cell += size_t(mw) * size_t(mh);
        }
        // angle map: the recorded one of the result, else the map the facet desorbs by
        const uint64_t* pdf = nullptr;
        if (st && st->anglemap && h.ang_off[size_t(i)] >= 0) pdf = st->anglemap + h.ang_off[size_t(i)];
        const bool desorbs_am = fi(d.desorb_type, i, 0) == MFG_DES_ANGLEMAP && d.desorb_anglemap;
        if (!pdf && desorbs_am) pdf = d.desorb_anglemap + am_src;
        if (desorbs_am) am_src += size_t(std::max(amw, 0)) * size_t(std::max(amrows, 0));
        if (pdf && amw > 0 && amrows > 0) {
            w.open("IncidentAngleMap", {{"angleMapPhiWidth", num(amw)}, {"angleMapThetaLimit", num(amlim)},
                                        {"angleMapThetaLowerRes", num(fi(d.anglemap_theta_lower_res, i, 0))},
                                        {"angleMapThetaHigherRes", num(fi(d.anglemap_theta_higher_res, i, 0))}});
            w.text("map", grid(amw, amrows, [&](int64_t k) { return num((unsigned long long)pdf[k]); }));
            w.close("IncidentAngleMap");
        }
        w.open("Histograms", {});
        if (d.facet_histogram) hist_settings(w, d.facet_histogram[i]);
        w.close("Histograms");
        w.close("Facet");
    }
    w.close("Facets");
    w.open("Structures", {{"nb", num(std::max(1, d.n_structures))}});
    for (int s = 0; s < std::max(1, d.n_structures); ++s) w.leaf("Structure", {{"id", num(s)}, {"name", "structure " + std::to_string(s + 1)}});
    w.close("Structures");
    w.close("Geometry");

    // ---- simulation settings ----
    w.open("MolflowSimuSettings", {});
    w.open("Gas", {{"mass", num(d.gas_mass)}, {"enableDecay", num(d.enable_decay)}, {"halfLife", num(d.half_life)}});
    w.open("Scattering", {{"enabled", num(d.scatter_enabled)}, {"massRatio", num(d.scatter_mass_ratio)},
                          {"meanFreePath_cm", num(d.scatter_mean_free_path_cm)}});
    w.leaf("LowSpeedCutoff", {{"enabled", num(d.scatter_cutoff_enabled)}, {"speed", num(d.scatter_cutoff_speed)}});
    w.close("Scattering");
    w.leaf("Outgassing_info", {{"final_rate_molecules_per_s", num(h.final_outgassing_rate)},
                               {"total_desorbed_molecules", num(h.total_desorbed_molecules)}});
    w.close("Gas");
    w.leaf("LowFluxMode", {{"enabled", num(d.low_flux_mode)}, {"cutoff", num(d.low_flux_cutoff)}});
    w.open("TimeSettings", {{"timeWindow", num(d.time_window)}, {"useMaxwellDistr", num(d.use_maxwell)}, {"calcConstFlow", num(d.constant_flow)}});
    w.open("UserMoments", {{"nb", num(nm)}});
    for (int k = 0; k < nm; ++k) w.leaf("UserEntry", {{"id", num(k)}, {"content", num(d.moment_time[k])}, {"window", num(d.moment_window[k])}});
    w.close("UserMoments");
    const double latest = nm ? d.moment_time[nm - 1] + 0.5 * d.moment_window[nm - 1] : 0.5 * d.time_window;
    w.leaf("Info", {{"latest_moment_s", num(latest)}});
    w.close("TimeSettings");
    w.open("Motion", {{"type", num(d.motion_type)}});
    if (d.motion_type == 1)
        w.leaf("VelocityVector", {{"vx", num(d.motion_vector2[0])}, {"vy", num(d.motion_vector2[1])}, {"vz", num(d.motion_vector2[2])}});
    else if (d.motion_type == 2) {
        w.leaf("AxisBasePoint", {{"x", num(d.motion_vector1[0])}, {"y", num(d.motion_vector1[1])}, {"z", num(d.motion_vector1[2])}});
        w.leaf("RotationVector", {{"x", num(d.motion_vector2[0])}, {"y", num(d.motion_vector2[1])}, {"z", num(d.motion_vector2[2])}});
    }
    w.close("Motion");
    w.open("MeasureForces", {{"enabled", num(d.enable_force_measurement)}});
    w.open("Torque", {});
    w.leaf("refPoint", {{"x", num(d.torque_ref_point[0])}, {"y", num(d.torque_ref_point[1])}, {"z", num(d.torque_ref_point[2])}});
    w.close("Torque");
    w.close("MeasureForces");
    w.open("Parameters", {{"nb", num(d.n_params)}});
    for (int p = 0; p < d.n_params; ++p) {
        const int s0 = d.param_start[p], s1 = d.param_start[p + 1];
        w.open("Parameter", {{"id", num(p)}, {"name", pname(p)}, {"nbMoments", num(s1 - s0)},
                             {"logXinterp", num(d.param_log_x ? int(d.param_log_x[p]) : 0)},
                             {"logYinterp", num(d.param_log_y ? int(d.param_log_y[p]) : 0)}});
        for (int j = s0; j < s1; ++j) w.leaf("Moment", {{"id", num(j - s0)}, {"t", num(d.param_t[j])}, {"value", num(d.param_v[j])}});
        w.close("Parameter");
    }
    w.close("Parameters");
    w.open("Global_histograms", {});
    hist_settings(w, d.global_histogram);
    w.close("Global_histograms");
    w.close("MolflowSimuSettings");
    w.leaf("Interface", {});

    // ---- results (SaveSimulationState) ----
    if (st) {
        const int64_t F = nf;
        w.open("MolflowResults", {});
        w.open("Moments", {{"nb", num(nm + 1)}});
        const double ndes = st->global ? st->global[MFG_G_NBDESORBED] : 0.0;
        const int32_t gsz[3] = {h.ghist.nb, h.ghist.nd, h.ghist.nt};
        for (int m = 0; m <= nm; ++m) {
            std::string mpt;
            if (ndes > 0)
                mpt = num(m == 0 ? h.final_outgassing_rate / ndes : h.total_desorbed_molecules / d.moment_window[m - 1] / ndes);
            if (m == 0) {
                if (ndes > 0) w.open("Moment", {{"id", "0"}, {"time", "Constant flow"}, {"timeWindow", "0"}, {"molecules_per_TP", mpt}});
                else w.open("Moment", {{"id", "0"}, {"time", "Constant flow"}, {"timeWindow", "0"}});
                const double* g = st->global;
                auto gv = [&](int k) { return g ? g[k] : 0.0; };
                w.open("Global", {});
                w.leaf("Hits", {{"totalHit", count(gv(MFG_G_NBMCHIT))}, {"totalHitEquiv", num(gv(MFG_G_NBHITEQUIV))},
                                {"totalDes", count(gv(MFG_G_NBDESORBED))}, {"totalAbsEquiv", num(gv(MFG_G_NBABSEQUIV))},
                                {"totalDist_total", num(gv(MFG_G_DIST_TOTAL))}, {"totalDist_fullHitsOnly", num(gv(MFG_G_DIST_FULLHITS))},
                                {"totalLeak", count(gv(MFG_G_NBLEAK))}, {"maxDesorption", "0"}});
                w.leaf("Hit_Cache", {{"nb", "0"}});
                w.leaf("Leak_Cache", {{"nb", "0"}});
                w.close("Global");
            } else {
                if (ndes > 0)
                    w.open("Moment", {{"id", num(m)}, {"time", num(d.moment_time[m - 1])}, {"timeWindow", num(d.moment_window[m - 1])},
                                      {"molecules_per_TP", mpt}});
                else
                    w.open("Moment", {{"id", num(m)}, {"time", num(d.moment_time[m - 1])}, {"timeWindow", num(d.moment_window[m - 1])}});
            }
            if (st->histogram && d.global_histogram.record && gsz[0] + gsz[1] + gsz[2] > 0) {
                w.open("Histograms", {});
                hist_results(w, d.global_histogram, gsz, st->histogram + int64_t(m) * L.histogram_bins + std::max(h.ghist.off, 0));
                w.close("Histograms");
            }
            w.open("FacetResults", {});
            for (int i = 0; i < nf; ++i) {
                w.open("Facet", {{"id", num(i)}});
                const size_t fo = size_t(int64_t(m) * F + i);
                const uint64_t* c = st->facet_counts ? st->facet_counts + fo * MFG_FC_N : nullptr;
                const double* s = st->facet_sums ? st->facet_sums + fo * MFG_FS_N : nullptr;
                auto cv = [&](int k) { return c ? (unsigned long long)c[k] : 0ull; };
                auto sv = [&](int k) { return s ? s[k] : 0.0; };
                w.leaf("Hits", {{"nbHit", num(cv(MFG_FC_NBMCHIT))}, {"nbHitEquiv", num(sv(MFG_FS_NBHITEQUIV))},
                                {"nbDes", num(cv(MFG_FC_NBDESORBED))}, {"nbAbsEquiv", num(sv(MFG_FS_NBABSEQUIV))},
                                {"sum_v_ort", num(sv(MFG_FS_SUM_V_ORT))}, {"sum_1_per_v", num(sv(MFG_FS_SUM_1_PER_ORT_VEL))},
                                {"sum_v", num(sv(MFG_FS_SUM_1_PER_VELOCITY))}});
                if (d.enable_force_measurement && st->force && L.n_force > 0) {
                    const double* q = st->force + fo * 9;
                    w.open("Forces", {});
                    w.leaf("Impulse", {{"x", num(q[0])}, {"y", num(q[1])}, {"z", num(q[2])}});
                    w.leaf("Impulse_square", {{"x", num(q[3])}, {"y", num(q[4])}, {"z", num(q[5])}});
                    w.leaf("Impulse_momentum", {{"x", num(q[6])}, {"y", num(q[7])}, {"z", num(q[8])}});
                    w.close("Forces");
                }
                const int64_t pk = h.prof_idx[size_t(i)];
                if (pk >= 0 && st->profile) {
                    w.open("Profile", {{"size", num(MFG_PROFILE_SIZE)}});
                    const double* p = st->profile + (int64_t(m) * L.profile_facets + pk) * MFG_PROFILE_SIZE * 3;
                    for (int j = 0; j < MFG_PROFILE_SIZE; ++j)
                        w.leaf("Slice", {{"id", num(j)}, {"countEquiv", num(p[j * 3])}, {"sum_1_per_v", num(p[j * 3 + 2])},
                                         {"sum_v_ort", num(p[j * 3 + 1])}});
                    w.close("Profile");
                }
                const int64_t to = h.tex_off[size_t(i)];
                if (to >= 0 && st->texture) {
                    const int64_t tw = h.tex_w[size_t(i)], th = h.tex_h[size_t(i)];
                    const double* t = st->texture + (int64_t(m) * L.texture_cells + to) * 3;
                    w.open("Texture", {{"width", num(tw)}, {"height", num(th)}});
                    w.text("count", grid(tw, th, [&](int64_t k) { return num(t[k * 3]); }));
                    w.text("sum_1_per_v", grid(tw, th, [&](int64_t k) { return num(t[k * 3 + 2]); }));
                    w.text("sum_v_ort", grid(tw, th, [&](int64_t k) { return num(t[k * 3 + 1]); }));
                    w.close("Texture");
                }
                const int64_t dof = h.dir_off[size_t(i)];
                if (dof >= 0 && st->direction) {
                    const int64_t tw = h.tex_w[size_t(i)], th = h.tex_h[size_t(i)];
                    const double* dv = st->direction + (int64_t(m) * L.direction_cells + dof) * 4;
                    w.open("Directions", {{"width", num(tw)}, {"height", num(th)}});
                    std::string rows = "\n";
                    for (int64_t y = 0; y < th; ++y) {
                        for (int64_t x = 0; x < tw; ++x) {
                            const double* a = dv + (y * tw + x) * 4;
                            rows += num(a[0]) + "," + num(a[1]) + "," + num(a[2]) + "\t";
                        }
                        rows += "\n";
                    }
                    w.text("vel.vectors", rows);
                    w.text("count", grid(tw, th, [&](int64_t k) { return count(dv[k * 4 + 3]); }));
                    w.close("Directions");
                }
                if (st->histogram && !h.fhist.empty() && h.fhist[size_t(i)].off >= 0 && d.facet_histogram) {
                    const HistDev& hd = h.fhist[size_t(i)];
                    const int32_t sz[3] = {hd.nb, hd.nd, hd.nt};
                    w.open("Histograms", {});
                    hist_results(w, d.facet_histogram[i], sz, st->histogram + int64_t(m) * L.histogram_bins + hd.off);
                    w.close("Histograms");
                }
                w.close("Facet");
            }
            w.close("FacetResults");
            w.close("Moment");
        }
        w.close("Moments");
        w.close("MolflowResults");
    }
    w.close("SimulationEnvironment");

    std::string low = path;
    for (char& ch : low) ch = char(ch >= 'A' && ch <= 'Z' ? ch - 'A' + 'a' : ch);
    if (low.size() >= 4 && low.compare(low.size() - 4, 4, ".zip") == 0) {
        std::string base = path.substr(path.find_last_of("/\\") == std::string::npos ? 0 : path.find_last_of("/\\") + 1);
        base = base.substr(0, base.size() - 4) + ".xml";
        return write_stored_zip(path, base, w.out, err);
    }
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) { err = "cannot write " + path; return false; }
    const bool ok = std::fwrite(w.out.data(), 1, w.out.size(), f) == w.out.size();
    if (std::fclose(f) != 0 || !ok) { err = "write error on " + path; return false; }
    return true;
}

}  // namespace mfgx
