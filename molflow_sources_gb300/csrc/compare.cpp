// compare.cpp — two GlobalSimuState-shaped results compared with the rule of MolFlow+'s test suite,
// on the C++ host: GlobalSimuState::Compare (src/Simulation/MolflowSimGeom.cpp:559-1148), which the
// suite calls with a 0.9 % global and a 7 % local threshold (tests/testsuite.cpp:460).
//
// Three error counts, (global, facet, fine), as the reference returns them; a run passes the suite
// when the first two are 0.  The reference's sample-size cut-offs (6400 counts for histogram bins
// and facet counters, 40000 Monte Carlo hits per facet and moment, 100 for a smoothed profile bin,
// 640 for a texture cell), the per-moment threshold max(local, 1/sqrt(hits)), the 40x looser
// velocity thresholds and the scales are kept.  IsEqual lives in the reference's absent shared
// math code; it is taken as relative, |a - b| < tol * max(|a|, |b|) (a zero pair is equal).
#include "compare.h"

#include <algorithm>
#include <charconv>
#include <cmath>

namespace mfgx {

namespace {
constexpr double kVel = 40.0;   // velocity thresholds are this much looser
bool is_equal(double a, double b, double tol) {
    return std::fabs(a - b) < std::max(1e-99, tol * std::max(std::fabs(a), std::fabs(b))) || a == b;
}
bool too_few(double a, double b, double cut) { return std::max(1.0, std::min(a, b)) < cut; }
std::string num(double x) {
    char b[64];
    auto r = std::to_chars(b, b + sizeof b, x);
    return std::string(b, r.ptr);
}
}  // namespace

CompareResult compare_states(const mfg::HostModel& h, const mfg_state_view& l, const mfg_state_view& r,
                             double glob, double loc_threshold) {
    CompareResult out;
    std::vector<std::string> fine;
    const mfg_state_layout& L = h.layout;
    const double des_l = l.global[MFG_G_NBDESORBED], des_r = r.global[MFG_G_NBDESORBED];
    if (des_l == 0 || des_r == 0) {
        out.global = 1;
        out.facet = out.fine = -1;
        out.messages.push_back(des_l == 0 && des_r == 0 ? "[Global][desorp] Neither state has recorded desorptions"
                               : des_l == 0 ? "[Global][desorp] First state has no recorded desorptions"
                                            : "[Global][desorp] Second state has no recorded desorptions");
        return out;
    }
    auto msg = [&](std::vector<std::string>& v, const std::string& tag, double x, double y) {
        v.push_back(tag + " has large difference: " + num(x) + " vs " + num(y));
    };
    const double a_l = l.global[MFG_G_NBABSEQUIV] / des_l, a_r = r.global[MFG_G_NBABSEQUIV] / des_r;
    if (!is_equal(a_l, a_r, glob)) { msg(out.messages, "[Global][absRatio abs/des]", a_l, a_r); ++out.global; }
    const double h_l = l.global[MFG_G_NBMCHIT] / des_l, h_r = r.global[MFG_G_NBMCHIT] / des_r;
    if (!is_equal(h_l, h_r, glob)) { msg(out.messages, "[Global][hits/des]", h_l, h_r); ++out.global; }
    const double hits_l = l.global[MFG_G_NBMCHIT], hits_r = r.global[MFG_G_NBMCHIT];
    const int64_t B = 1 + L.n_moments, F = L.n_facets;
    // global histograms, every moment block
    const int32_t gsz[3] = {h.ghist.nb, h.ghist.nd, h.ghist.nt};
    if (L.histogram_bins > 0 && gsz[0] + gsz[1] + gsz[2] > 0 && l.histogram && r.histogram) {
        static const char* names[3] = {"Bounces/global hits", "Dist", "Time"};
        for (int64_t m = 0; m < B; ++m) {
            int64_t o = std::max(h.ghist.off, 0);
            for (int kind = 0; kind < 3; ++kind) {
                for (int32_t i = 0; i < gsz[kind]; ++i) {
                    const double x = l.histogram[m * L.histogram_bins + o + i], y = r.histogram[m * L.histogram_bins + o + i];
                    if (too_few(x, y, 6400.0)) continue;
                    if (!is_equal(x / hits_l, y / hits_r, loc_threshold)) {
                        msg(out.messages, std::string("[Global][Hist][") + names[kind] + "][" + std::to_string(i) + "]",
                            x / hits_l, y / hits_r);
                        ++out.global;
                    }
                }
                o += gsz[kind];
            }
        }
    }
    // facets
    const double hitq_l = l.global[MFG_G_NBHITEQUIV], hitq_r = r.global[MFG_G_NBHITEQUIV];
    const double scale_l = 1.0 / hitq_l, scale_r = 1.0 / hitq_r;
    const double full_l = 1.0 / (hitq_l + l.global[MFG_G_NBABSEQUIV] + des_l);
    const double full_r = 1.0 / (hitq_r + r.global[MFG_G_NBABSEQUIV] + des_r);
    for (int64_t f = 0; f < F; ++f) {
        for (int64_t m = 0; m < B; ++m) {
            const size_t fo = size_t(m * F + f);
            const uint64_t* cl = l.facet_counts + fo * MFG_FC_N;
            const uint64_t* cr = r.facet_counts + fo * MFG_FC_N;
            const double* sl = l.facet_sums + fo * MFG_FS_N;
            const double* sr = r.facet_sums + fo * MFG_FS_N;
            const long long mc_l = (long long)cl[MFG_FC_NBMCHIT], mc_r = (long long)cr[MFG_FC_NBMCHIT];
            if ((mc_l == 0 && mc_r == 0) || mc_l < 40000 || mc_r < 40000) continue;
            const double loc = std::max(loc_threshold, 1.0 / std::sqrt(double(std::min(mc_l, mc_r))));
            const double sum_hd_l = sl[MFG_FS_NBHITEQUIV] + double(cl[MFG_FC_NBDESORBED]);
            const double sum_hd_r = sr[MFG_FS_NBHITEQUIV] + double(cr[MFG_FC_NBDESORBED]);
            const std::string tag = "[Facet][" + std::to_string(f) + "]";
            const std::string mo = "[moment" + std::to_string(m) + "]";
            if (!too_few(sl[MFG_FS_NBHITEQUIV], sr[MFG_FS_NBHITEQUIV], 6400.0)) {
                struct Check { const char* name; double x, y, t; };
                const Check checks[4] = {
                    {"facet_hits / global_hits", sl[MFG_FS_NBHITEQUIV] * scale_l, sr[MFG_FS_NBHITEQUIV] * scale_r, loc},
                    {"sum_v_ort", sl[MFG_FS_SUM_V_ORT] * scale_l, sr[MFG_FS_SUM_V_ORT] * scale_r, loc},
                    {"sum_1_per_velocity", sl[MFG_FS_SUM_1_PER_VELOCITY] * full_l, sr[MFG_FS_SUM_1_PER_VELOCITY] * full_r, loc * kVel},
                    {"sum_1_per_ort_velocity", sl[MFG_FS_SUM_1_PER_ORT_VEL] * full_l, sr[MFG_FS_SUM_1_PER_ORT_VEL] * full_r, loc * kVel}};
                for (const Check& c : checks)
                    if (!is_equal(c.x, c.y, c.t)) { msg(out.messages, tag + "[" + c.name + "]" + mo, c.x, c.y); ++out.facet; }
            }
            if (!too_few(sl[MFG_FS_NBABSEQUIV], sr[MFG_FS_NBABSEQUIV], 6400.0)) {
                const double x = sl[MFG_FS_NBABSEQUIV] / double(mc_l), y = sr[MFG_FS_NBABSEQUIV] / double(mc_r);
                if (!is_equal(x, y, loc)) { msg(out.messages, tag + "[abs/hits ratio]" + mo, x, y); ++out.facet; }
            }
            if (!too_few(double(cl[MFG_FC_NBDESORBED]), double(cr[MFG_FC_NBDESORBED]), 6400.0)) {
                const double x = double(cl[MFG_FC_NBDESORBED]) / double(mc_l), y = double(cr[MFG_FC_NBDESORBED]) / double(mc_r);
                if (!is_equal(x, y, loc)) { msg(out.messages, tag + "[desRatio]" + mo, x, y); ++out.facet; }
            }
            const std::string mm = "[" + std::to_string(m) + "]";
            // profile: 1-4-6-4-1 smoothed counts (MolflowSimGeom.cpp:865-903 smooths countEquiv for
            // the velocity-sum checks too)
            const int64_t k = h.prof_idx[size_t(f)];
            if (k >= 0 && l.profile && r.profile) {
                const double* pl = l.profile + (m * L.profile_facets + k) * MFG_PROFILE_SIZE * 3;
                const double* pr = r.profile + (m * L.profile_facets + k) * MFG_PROFILE_SIZE * 3;
                auto sm = [](const double* p, int i) {
                    return (p[(i - 2) * 3] + 4 * p[(i - 1) * 3] + 6 * p[i * 3] + 4 * p[(i + 1) * 3] + p[(i + 2) * 3]) / 16.0;
                };
                for (int i = 2; i < MFG_PROFILE_SIZE - 2; ++i) {
                    const double wl = sm(pl, i), wr = sm(pr, i);
                    if (std::max(1.0, std::min(wl, wr)) < 100) continue;
                    const std::string pt = tag + "[Profile][" + std::to_string(i) + "]";
                    if (!is_equal(wl / sum_hd_l, wr / sum_hd_r, loc)) { fine.push_back(pt + "[countEquiv]" + mm); ++out.fine; }
                    for (const char* name : {"sum_1_per_ort_velocity", "sum_v_ort"})
                        if (!is_equal(wl * scale_l, wr * scale_r, loc * kVel)) {
                            fine.push_back(pt + "[" + name + "]" + mm);
                            ++out.fine;
                        }
                }
            }
            // texture cells
            const int64_t to = h.tex_off[size_t(f)];
            if (to >= 0 && l.texture && r.texture) {
                const int64_t n = int64_t(h.tex_w[size_t(f)]) * h.tex_h[size_t(f)];
                const double* tl = l.texture + (m * L.texture_cells + to) * 3;
                const double* tr = r.texture + (m * L.texture_cells + to) * 3;
                for (int64_t c = 0; c < n; ++c) {
                    if (std::max(1.0, std::min(tl[c * 3], tr[c * 3])) < 640) continue;
                    const std::string tt = tag + "[Texture][" + std::to_string(c) + "]";
                    if (!is_equal(tl[c * 3] / sum_hd_l, tr[c * 3] / sum_hd_r, loc)) { fine.push_back(tt + "[countEquiv]" + mm); ++out.fine; }
                    if (!is_equal(tl[c * 3 + 2] * full_l, tr[c * 3 + 2] * full_r, loc * kVel)) {
                        fine.push_back(tt + "[sum_1_per_ort_velocity]" + mm);
                        ++out.fine;
                    }
                    if (!is_equal(tl[c * 3 + 1] * scale_l, tr[c * 3 + 1] * scale_r, loc * kVel)) {
                        fine.push_back(tt + "[sum_v_ort_per_area]" + mm);
                        ++out.fine;
                    }
                }
            }
            // direction cells
            const int64_t dof = h.dir_off[size_t(f)];
            if (dof >= 0 && l.direction && r.direction) {
                const int64_t n = int64_t(h.tex_w[size_t(f)]) * h.tex_h[size_t(f)];
                const double* dl = l.direction + (m * L.direction_cells + dof) * 4;
                const double* dr = r.direction + (m * L.direction_cells + dof) * 4;
                static const int order[4] = {3, 0, 1, 2};
                static const char* names[4] = {"count", "dir.x", "dir.y", "dir.z"};
                for (int64_t c = 0; c < n; ++c) {
                    if (too_few(dl[c * 4 + 3], dr[c * 4 + 3], 6400.0)) continue;
                    for (int j = 0; j < 4; ++j)
                        if (!is_equal(dl[c * 4 + order[j]], dr[c * 4 + order[j]], loc)) {
                            fine.push_back(tag + "[dirs][" + std::to_string(c) + "][" + names[j] + "]" + mm);
                            ++out.fine;
                        }
                }
            }
            // facet histograms
            if (!h.fhist.empty() && h.fhist[size_t(f)].off >= 0 && l.histogram && r.histogram) {
                const HistDev& hd = h.fhist[size_t(f)];
                int64_t o = hd.off;
                for (int32_t n : {hd.nb, hd.nd, hd.nt}) {
                    for (int32_t i = 0; i < n; ++i) {
                        const double x = l.histogram[m * L.histogram_bins + o + i], y = r.histogram[m * L.histogram_bins + o + i];
                        if (too_few(x, y, 6400.0)) continue;
                        if (!is_equal(x / double(mc_l), y / double(mc_r), loc)) {
                            fine.push_back(tag + "[Hist][" + std::to_string(i) + "]" + mm);
                            ++out.fine;
                        }
                    }
                    o += n;
                }
            }
        }
    }
    out.messages.insert(out.messages.end(), fine.begin(), fine.end());
    return out;
}

}  // namespace mfgx
