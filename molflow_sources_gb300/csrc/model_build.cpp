// model_build.cpp — host preparation of a model (geometry, tables, BVH, device records).
#include "model_build.h"

#include <algorithm>
#include <climits>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <functional>
#include <numeric>

namespace mfg {
namespace {

constexpr double kKb = 1.38E-23;   // Boltzmann constant as used by the reference (Particle.cpp:428)

struct V3 {
    double x, y, z;
};
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 mul(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double len(V3 a) { return std::sqrt(dot(a, a)); }
inline void put(double* d, V3 a) { d[0] = a.x; d[1] = a.y; d[2] = a.z; }

template <class T>
T opt(const T* p, int i, T def) { return p ? p[i] : def; }

// Facet basis from the polygon: normal by the right-hand rule on the first
// non-degenerate pair of consecutive edges, U along the first edge, V = N x U,
// (u,v) normalised to the bounding rectangle, N and V flipped when the signed
// area in (U,V) is negative (concave polygons whose first turn is reflex).
bool facet_geometry(const double* vert, const int32_t* idx, int n, HostFacet& F, double* v2) {
    auto P = [&](int k) { const double* p = vert + 3 * idx[k]; return V3{p[0], p[1], p[2]}; };
    V3 N{0, 0, 0};
    bool ok = false;
    for (int k = 0; k + 2 < n && !ok; ++k) {
        N = cross(sub(P(k + 1), P(k)), sub(P(k + 2), P(k + 1)));
        ok = len(N) >= 1e-11;
    }
    if (!ok) return false;
    N = mul(N, 1.0 / len(N));
    V3 p0 = P(0);
    V3 U = sub(P(1), p0);
    double ul = len(U);
    if (!(ul > 0)) return false;
    U = mul(U, 1.0 / ul);
    V3 V = cross(N, U);
    double umin = 0, umax = 0, vmin = 0, vmax = 0;
    for (int j = 0; j < n; ++j) {
        V3 d = sub(P(j), p0);
        double u = j ? dot(U, d) : 0.0, v = j ? dot(V, d) : 0.0;
        v2[2 * j] = u;
        v2[2 * j + 1] = v;
        umin = std::min(umin, u); umax = std::max(umax, u);
        vmin = std::min(vmin, v); vmax = std::max(vmax, v);
    }
    double a2 = 0;
    for (int j = 0; j < n; ++j) {
        int k = (j + 1) % n;
        a2 += v2[2 * j] * v2[2 * k + 1] - v2[2 * k] * v2[2 * j + 1];
    }
    if (a2 < 0) {
        N = mul(N, -1.0);
        V = mul(V, -1.0);
        vmin = vmax = 0;
        for (int j = 0; j < n; ++j) {
            v2[2 * j + 1] = -v2[2 * j + 1];
            vmin = std::min(vmin, v2[2 * j + 1]);
            vmax = std::max(vmax, v2[2 * j + 1]);
        }
    }
    double uD = umax - umin, vD = vmax - vmin;
    if (!(uD > 0) || !(vD > 0)) return false;
    F.area = std::fabs(0.5 * a2);
    put(F.N, N);
    put(F.nU, U);
    put(F.nV, V);
    put(F.O, add(p0, add(mul(U, umin), mul(V, vmin))));
    put(F.U, mul(U, uD));
    put(F.V, mul(V, vD));
    for (int j = 0; j < n; ++j) {
        v2[2 * j] = (v2[2 * j] - umin) / uD;
        v2[2 * j + 1] = (v2[2 * j + 1] - vmin) / vD;
    }
    for (int a = 0; a < 3; ++a) { F.bbmin[a] = DBL_MAX; F.bbmax[a] = -DBL_MAX; }
    for (int j = 0; j < n; ++j) {
        const double* p = vert + 3 * idx[j];
        for (int a = 0; a < 3; ++a) {
            F.bbmin[a] = std::min(F.bbmin[a], p[a]);
            F.bbmax[a] = std::max(F.bbmax[a], p[a]);
        }
    }
    for (int a = 0; a < 3; ++a) F.center[a] = 0.5 * (F.bbmin[a] + F.bbmax[a]);
    return true;
}

// even-odd crossing test in (u,v)
bool inside_poly(const double* v2, int n, double u, double v) {
    bool in = false;
    for (int i = 0, j = n - 1; i < n; j = i++) {
        double ui = v2[2 * i], vi = v2[2 * i + 1], uj = v2[2 * j], vj = v2[2 * j + 1];
        if ((vi > v) != (vj > v)) {
            double cr = (uj - ui) * (v - vi) - (u - ui) * (vj - vi);
            if ((cr > 0) == (vj > vi)) in = !in;
        }
    }
    return in;
}

// polygon area inside an axis-aligned rectangle (Sutherland-Hodgman clipping)
double clipped_area(const std::vector<double>& poly, double x0, double y0, double x1, double y1) {
    std::vector<double> in = poly, out;
    for (int e = 0; e < 4; ++e) {
        out.clear();
        size_t m = in.size() / 2;
        for (size_t i = 0; i < m; ++i) {
            const double* P = &in[2 * i];
            const double* Q = &in[2 * ((i + 1) % m)];
            auto side = [&](const double* X) {
                switch (e) {
                    case 0: return X[0] - x0;
                    case 1: return x1 - X[0];
                    case 2: return X[1] - y0;
                    default: return y1 - X[1];
                }
            };
            double dp = side(P), dq = side(Q);
            if (dp >= 0) { out.push_back(P[0]); out.push_back(P[1]); }
            if ((dp >= 0) != (dq >= 0)) {
                double t = dp / (dp - dq);
                out.push_back(P[0] + t * (Q[0] - P[0]));
                out.push_back(P[1] + t * (Q[1] - P[1]));
            }
        }
        in.swap(out);
        if (in.empty()) return 0.0;
    }
    double a = 0;
    size_t m = in.size() / 2;
    for (size_t i = 0; i < m; ++i) {
        size_t j = (i + 1) % m;
        a += in[2 * i] * in[2 * j + 1] - in[2 * j] * in[2 * i + 1];
    }
    return std::fabs(0.5 * a);
}

// ---- table interpolation (InterpolateX / InterpolateY contracts) ----
int last_le(double key, const double* tab, int n) {
    return int(std::upper_bound(tab, tab + n, key) - tab) - 1;
}
double interp_y(double x, const double* xs, const double* ys, int n, bool lx, bool ly, bool ex) {
    if (n == 1) return ys[0];
    int i = last_le(x, xs, n);
    if (i < 0) { if (!ex) return ys[0]; i = 0; }
    else if (i >= n - 1) { if (!ex) return ys[n - 1]; i = n - 2; }
    double w = lx ? (std::log10(x) - std::log10(xs[i])) / (std::log10(xs[i + 1]) - std::log10(xs[i]))
                  : (x - xs[i]) / (xs[i + 1] - xs[i]);
    if (ly) return std::pow(10.0, std::log10(ys[i]) + (std::log10(ys[i + 1]) - std::log10(ys[i])) * w);
    return ys[i] + (ys[i + 1] - ys[i]) * w;
}

// Integrated desorption of one time-dependent outgassing parameter, from t=0 to
// latestMoment, in Pa*m3 (IDGeneration.cpp:45-207): constant extrapolation before
// the first point, truncation at latestMoment, non-constant sections split in 10.
void integrated_desorption(const double* t, const double* v, int n, bool lx, bool ly, double latest,
                           std::vector<double>& it, std::vector<double>& ic) {
    std::vector<double> ot, ov;
    int ia = 0;
    while (ia < n && t[ia] < latest) ++ia;
    bool all_before = ia >= n;
    if (all_before) ia = n - 1;
    it.assign(1, 0.0);
    ic.assign(1, 0.0);
    if (t[0] > 0.0) { ot.push_back(0.0); ov.push_back(v[0]); }
    if (all_before) {
        for (int i = 0; i < n; ++i) { ot.push_back(t[i]); ov.push_back(v[i]); }
        ot.push_back(latest); ov.push_back(ov.back());
    } else {
        for (int i = 0; i < ia; ++i) { ot.push_back(t[i]); ov.push_back(v[i]); }
        if (ot.empty() || !(std::fabs(ot.back() - latest) < 1e-10)) {
            ot.push_back(latest);
            ov.push_back(interp_y(latest, t, v, n, lx, ly, true));
        }
    }
    const double k_mbarls = 0.1;   // mbar*l/s -> Pa*m3/s
    for (size_t i = 1; i < ot.size(); ++i) {
        if (std::fabs(ov[i] - ov[i - 1]) < 1e-10) {
            it.push_back(ot[i]);
            ic.push_back(ic.back() + (ot[i] - ot[i - 1]) * ov[i] * k_mbarls);
            continue;
        }
        const int steps = 10;
        double t0 = ot[i - 1], t1 = ot[i], delta = 1.0 / steps;
        double lt0 = 0, ldt = 0, sub_dt = (t1 - t0) * delta, sub_ldt = 0;
        if (lx) { lt0 = (t0 == 0) ? -99 : std::log10(t0); ldt = std::log10(t1) - lt0; sub_ldt = ldt * delta; }
        double pv = ov[i - 1], pt = t0;
        for (double f = delta; f < 1.0001; f += delta) {
            double et = lx ? std::pow(10.0, lt0 + f * ldt) : t0 + f * (t1 - t0);
            double ev = interp_y(et, ot.data(), ov.data(), int(ot.size()), lx, ly, true);
            double g;
            if (!lx && !ly) g = sub_dt * 0.5 * (pv + ev);
            else if (lx && !ly) g = (ev - pv) * (pt - et) / std::log(et / pt) - pt * pv + et * ev;
            else if (!lx && ly) {
                double le = ev > 0 ? std::log10(ev) : -99, lp = pt > 0 ? std::log10(pv) : -99;
                g = sub_dt * (ev - pv) * std::log10(std::exp(1.0)) / (le - lp);
            } else {
                double le = ev > 0 ? std::log10(ev) : -99, lp = pt > 0 ? std::log10(pv) : -99;
                double m = (le - lp) / sub_ldt;
                g = (m != -1.0) ? pv / std::pow(pt, m) / (m + 1.0) * (std::pow(et, m + 1.0) - std::pow(pt, m + 1.0))
                                : pt * pv * sub_ldt;
            }
            it.push_back(et);
            ic.push_back(ic.back() + g * k_mbarls);
            pv = ev;
            pt = et;
        }
    }
}

// ---- BVH (binned SAH over facet bounding boxes) ----
struct BuildNode {
    double lo[3], hi[3];
    int left = -1, right = -1, first = 0, count = 0, axis = 0;
};

constexpr int kMaxBvhDepth = 48;

// Binned SAH build.  With per-facet weights W (the share of the hits a prior run recorded on each
// facet, RebuildAccelStructure with ProbSplit, MolflowSimGeom.cpp:155-169) the chance that a ray
// enters a child is taken as the mean of its surface-area fraction and its share of the node's
// weight, so often-hit facets end up in shallow, tight subtrees.
int build_rec(std::vector<BuildNode>& out, std::vector<int>& ids, int begin, int end,
              const std::vector<HostFacet>& F, int leaf_max, int depth, int64_t& max_depth,
              const double* W = nullptr) {
    BuildNode nd;
    for (int a = 0; a < 3; ++a) { nd.lo[a] = DBL_MAX; nd.hi[a] = -DBL_MAX; }
    double cmin[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, cmax[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
    for (int k = begin; k < end; ++k) {
        const HostFacet& f = F[ids[k]];
        for (int a = 0; a < 3; ++a) {
            nd.lo[a] = std::min(nd.lo[a], f.bbmin[a]);
            nd.hi[a] = std::max(nd.hi[a], f.bbmax[a]);
            cmin[a] = std::min(cmin[a], f.center[a]);
            cmax[a] = std::max(cmax[a], f.center[a]);
        }
    }
    max_depth = std::max<int64_t>(max_depth, depth);
    int me = int(out.size());
    out.push_back(nd);
    int n = end - begin;
    // a node at the depth cap becomes a leaf whatever its size, so that the traversal stacks (64
    // entries, one far child per level) cannot overflow on any model
    if (n <= leaf_max || depth >= kMaxBvhDepth) {
        out[me].first = begin;
        out[me].count = n;
        return me;
    }
    constexpr int NB = 32;
    auto area = [](const double* lo, const double* hi) {
        double dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        return dx * dy + dy * dz + dz * dx;
    };
    const double parea = area(nd.lo, nd.hi);
    double wtot = 0;
    if (W)
        for (int k = begin; k < end; ++k) wtot += W[ids[k]];
    const bool weighted = W && wtot > 0 && parea > 0;
    double best = DBL_MAX;
    int bax = -1;
    double bsplit = 0;
    for (int ax = 0; ax < 3; ++ax) {
        double ext = cmax[ax] - cmin[ax];
        if (!(ext > 0)) continue;
        int cnt[NB] = {0};
        double bw[NB] = {0};
        double bl[NB][3], bh[NB][3];
        for (int b = 0; b < NB; ++b)
            for (int a = 0; a < 3; ++a) { bl[b][a] = DBL_MAX; bh[b][a] = -DBL_MAX; }
        for (int k = begin; k < end; ++k) {
            const HostFacet& f = F[ids[k]];
            int b = std::min(NB - 1, std::max(0, int((f.center[ax] - cmin[ax]) / ext * NB)));
            cnt[b]++;
            if (weighted) bw[b] += W[ids[k]];
            for (int a = 0; a < 3; ++a) { bl[b][a] = std::min(bl[b][a], f.bbmin[a]); bh[b][a] = std::max(bh[b][a], f.bbmax[a]); }
        }
        double rl[NB][3], rh[NB][3], rw[NB];
        int rc[NB];
        for (int b = NB - 1; b >= 0; --b) {
            rw[b] = bw[b] + (b == NB - 1 ? 0.0 : rw[b + 1]);
            for (int a = 0; a < 3; ++a) {
                rl[b][a] = (b == NB - 1) ? bl[b][a] : std::min(bl[b][a], rl[b + 1][a]);
                rh[b][a] = (b == NB - 1) ? bh[b][a] : std::max(bh[b][a], rh[b + 1][a]);
            }
            rc[b] = cnt[b] + (b == NB - 1 ? 0 : rc[b + 1]);
        }
        double ll[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, lh[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
        int lc = 0;
        double lw = 0;
        for (int s = 1; s < NB; ++s) {
            lc += cnt[s - 1];
            lw += bw[s - 1];
            for (int a = 0; a < 3; ++a) { ll[a] = std::min(ll[a], bl[s - 1][a]); lh[a] = std::max(lh[a], bh[s - 1][a]); }
            if (!lc || !rc[s]) continue;
            double c;
            if (weighted)
                c = (0.5 * area(ll, lh) / parea + 0.5 * lw / wtot) * lc + (0.5 * area(rl[s], rh[s]) / parea + 0.5 * rw[s] / wtot) * rc[s];
            else
                c = area(ll, lh) * lc + area(rl[s], rh[s]) * rc[s];
            if (c < best) { best = c; bax = ax; bsplit = cmin[ax] + ext * double(s) / NB; }
        }
    }
    int mid;
    if (bax < 0) {
        mid = begin + n / 2;
    } else {
        auto it = std::partition(ids.begin() + begin, ids.begin() + end,
                                 [&](int i) { return F[i].center[bax] < bsplit; });
        mid = int(it - ids.begin());
        if (mid == begin || mid == end) mid = begin + n / 2;
    }
    out[me].axis = std::max(bax, 0);
    int l = build_rec(out, ids, begin, mid, F, leaf_max, depth + 1, max_depth, W);
    int r = build_rec(out, ids, mid, end, F, leaf_max, depth + 1, max_depth, W);
    out[me].left = l;
    out[me].right = r;
    return me;
}

// Guide to the moment search: over log2(t) from one octave below the smallest positive window
// start to one above the largest, 1024 buckets, each holding the number of starts <= its own start
// time.  The device search then starts at the guide entry one bucket below the one log2f(t) names
// (a lower bound whatever the rounding of log2f) and steps forward: the same answer as the binary
// search, in about one step for log-spaced moments.  Only for non-decreasing starts.
void build_moment_guide(HostModel& m) {
    m.mguide.clear();
    if (m.nm < 8) return;
    double lo = DBL_MAX, hi = 0;
    for (int k = 0; k < m.nm; ++k) {
        if (k > 0 && m.mstart[k] < m.mstart[k - 1]) return;
        if (m.mstart[k] > 0) { lo = std::min(lo, m.mstart[k]); hi = std::max(hi, m.mstart[k]); }
    }
    if (!(hi > 0)) return;
    const int G = 1024;
    const double l0 = std::floor(std::log2(lo)) - 1.0, l1 = std::ceil(std::log2(hi)) + 1.0;
    m.mg_l0 = float(l0);
    m.mg_scale = float(G / (l1 - l0));
    m.mg_t0 = std::exp2(l0);
    m.mguide.resize(G);
    for (int b = 0; b < G; ++b) {
        const double tb = std::exp2(l0 + double(b) / double(m.mg_scale));
        int c = 0;
        while (c < m.nm && m.mstart[c] <= tb) ++c;
        m.mguide[b] = c;
    }
}

float round_down(double x) {
    float f = float(x);
    return (double(f) > x) ? std::nextafter(f, -FLT_MAX) : f;
}
float round_up(double x) {
    float f = float(x);
    return (double(f) < x) ? std::nextafter(f, FLT_MAX) : f;
}

}  // namespace

int build_host_model(const mfg_model_desc* d, HostModel& m, std::string& err, int leaf_max) {
    if (!d) { err = "null descriptor"; return MFG_ERR_INVALID_ARGUMENT; }
    if (d->abi_version != MFG_ABI_VERSION) { err = "descriptor ABI version mismatch"; return MFG_ERR_INVALID_MODEL; }
    if (d->n_facets <= 0 || d->n_vertices <= 0 || !d->vertices || !d->facet_vertex_start || !d->facet_vertex_index) {
        err = "empty geometry";
        return MFG_ERR_INVALID_MODEL;
    }
    const int nf = d->n_facets;
    m.nf = nf;
    m.nstruct = d->n_structures > 0 ? d->n_structures : 1;
    if (m.nstruct > MFG_MAX_STRUCTURES) { err = "more than " + std::to_string(MFG_MAX_STRUCTURES) + " structures"; return MFG_ERR_LIMIT; }
    m.facets.resize(nf);
    const int32_t* fs = d->facet_vertex_start;
    if (fs[0] != 0) { err = "facet_vertex_start[0] must be 0"; return MFG_ERR_INVALID_MODEL; }
    for (int i = 0; i < nf; ++i)
        if (int64_t(fs[i + 1]) - fs[i] < 3) { err = "facet " + std::to_string(i + 1) + " has fewer than 3 vertices"; return MFG_ERR_INVALID_MODEL; }
    for (int64_t k = 0; k < 3 * int64_t(d->n_vertices); ++k)
        if (!std::isfinite(d->vertices[k])) { err = "vertex " + std::to_string(k / 3 + 1) + " is not a finite point"; return MFG_ERR_INVALID_MODEL; }
    m.v2.assign(2 * size_t(fs[nf]), 0.0);
    for (int i = 0; i < nf; ++i) {
        HostFacet& F = m.facets[i];
        F.vstart = fs[i];
        F.nv = fs[i + 1] - fs[i];
        for (int k = 0; k < F.nv; ++k) {
            int vi = d->facet_vertex_index[F.vstart + k];
            if (vi < 0 || vi >= d->n_vertices) { err = "vertex index out of range on facet " + std::to_string(i + 1); return MFG_ERR_INVALID_MODEL; }
        }
        if (!facet_geometry(d->vertices, d->facet_vertex_index + F.vstart, F.nv, F, &m.v2[2 * size_t(F.vstart)])) {
            err = "facet " + std::to_string(i + 1) + " is degenerate";
            return MFG_ERR_INVALID_MODEL;
        }
    }
    auto cp = [&](std::vector<double>& dst, const double* src, double def) {
        dst.resize(nf);
        for (int i = 0; i < nf; ++i) dst[i] = opt(src, i, def);
    };
    auto cpi = [&](std::vector<int32_t>& dst, const int32_t* src, int32_t def) {
        dst.resize(nf);
        for (int i = 0; i < nf; ++i) dst[i] = opt(src, i, def);
    };
    auto cpb = [&](std::vector<uint8_t>& dst, const uint8_t* src) {
        dst.resize(nf);
        for (int i = 0; i < nf; ++i) dst[i] = opt<uint8_t>(src, i, 0);
    };
    cp(m.sticking, d->sticking, 0.0);
    cp(m.opacity, d->opacity, 1.0);
    for (auto& o : m.opacity) o = std::clamp(o, 0.0, 1.0);   // MolflowSimGeom.cpp:148-150
    cp(m.outgassing, d->outgassing, 0.0);
    cp(m.temperature, d->temperature, 293.15);
    cp(m.accommodation, d->accommodation, 1.0);
    cp(m.desorb_exp, d->desorb_exponent, 0.0);
    cp(m.diffuse, d->refl_diffuse, 1.0);
    cp(m.specular, d->refl_specular, 0.0);
    cp(m.cos_exp, d->refl_cos_exponent, 0.0);
    cp(m.texw_p, d->tex_width, 0.0);
    cp(m.texh_p, d->tex_height, 0.0);
    cp(m.max_speed, d->max_speed, 0.0);
    cp(m.am_limit, d->anglemap_theta_limit, 1.570796326);
    cp(m.soj_freq, d->sojourn_freq, 0.0);
    cp(m.soj_e, d->sojourn_e, 0.0);
    cpi(m.desorb_type, d->desorb_type, MFG_DES_NONE);
    cpi(m.structure, d->structure, 0);
    cpi(m.link, d->link_dest, 0);
    cpi(m.teleport, d->teleport_dest, 0);
    cpi(m.profile_type, d->profile_type, MFG_PROFILE_NONE);
    cpi(m.am_phi, d->anglemap_phi_width, 0);
    cpi(m.am_lo, d->anglemap_theta_lower_res, 0);
    cpi(m.am_hi, d->anglemap_theta_higher_res, 0);
    cpi(m.p_stick, d->sticking_param, -1);
    cpi(m.p_opac, d->opacity_param, -1);
    cpi(m.p_outg, d->outgassing_param, -1);
    cpi(m.p_temp, d->temperature_param, -1);
    cpb(m.two_sided, d->is_2sided);
    cpb(m.am_record, d->anglemap_record);
    cpb(m.sojourn, d->enable_sojourn);
    cpb(m.moving, d->is_moving);
    cpi(m.og_w, d->outgassing_map_width, 0);
    cpi(m.og_h, d->outgassing_map_height, 0);
    cp(m.og_ru, d->outgassing_map_ratio_u, 0.0);
    cp(m.og_rv, d->outgassing_map_ratio_v, 0.0);
    m.count.resize(nf);
    for (int i = 0; i < nf; ++i) m.count[i] = opt<uint32_t>(d->count_flags, i, 0u);
    m.gas_mass = d->gas_mass;
    m.use_maxwell = d->use_maxwell;
    m.constant_flow = d->constant_flow;
    m.time_window = d->time_window;
    m.enable_decay = d->enable_decay;
    m.half_life = d->half_life;
    m.low_flux = d->low_flux_mode;
    m.low_flux_cutoff = d->low_flux_cutoff;
    m.motion_type = d->motion_type;
    for (int k = 0; k < 3; ++k) { m.mv1[k] = d->motion_vector1[k]; m.mv2[k] = d->motion_vector2[k]; }
    m.scatter = d->scatter_enabled;
    m.scatter_cutoff = d->scatter_cutoff_enabled;
    m.sc_mass_ratio = d->scatter_mass_ratio;
    m.sc_mfp = d->scatter_mean_free_path_cm;
    m.sc_rho = d->scatter_rho;
    m.sc_cutoff_speed = d->scatter_cutoff_speed;
    m.log_facet = (d->log_facet >= 0 && d->log_facet < nf && d->log_limit > 0) ? d->log_facet : -1;
    m.log_cap = m.log_facet >= 0 ? d->log_limit : 0;
    m.force = d->enable_force_measurement != 0;
    for (int k = 0; k < 3; ++k) m.torque_ref[k] = d->torque_ref_point[k];
    if (m.motion_type < 0 || m.motion_type > 2) { err = "motion type must be 0, 1 or 2"; return MFG_ERR_INVALID_MODEL; }
    if (m.scatter && !(m.sc_mfp > 0 && m.sc_rho > 0 && m.sc_mass_ratio > 0)) {
        err = "scattering needs a positive mean free path, collision radius and mass ratio";
        return MFG_ERR_INVALID_MODEL;
    }
    if (!(m.gas_mass > 0)) { err = "gas mass must be positive"; return MFG_ERR_INVALID_MODEL; }
    {
        const mfg_histogram_params& hp = d->global_histogram;
        if (((hp.record & MFG_HIST_DISTANCE) && !(hp.distance_binsize > 0 && hp.distance_max >= 0 && hp.distance_max / hp.distance_binsize < 1e8)) ||
            ((hp.record & MFG_HIST_TIME) && !(hp.time_binsize > 0 && hp.time_max >= 0 && hp.time_max / hp.time_binsize < 1e8)) ||
            ((hp.record & MFG_HIST_BOUNCE) && hp.bounce_max / (hp.bounce_binsize ? hp.bounce_binsize : 1) > 100000000ull)) {
            err = "bad global histogram settings";
            return MFG_ERR_INVALID_MODEL;
        }
    }
    for (int i = 0; i < nf; ++i) {
        if (m.structure[i] < -1 || m.structure[i] >= m.nstruct) { err = "structure index out of range on facet " + std::to_string(i + 1); return MFG_ERR_INVALID_MODEL; }
        if (m.link[i] < 0 || m.link[i] > m.nstruct) { err = "structure link destination out of range on facet " + std::to_string(i + 1); return MFG_ERR_INVALID_MODEL; }
        if (d->facet_histogram) {
            const mfg_histogram_params& hp = d->facet_histogram[i];
            if (((hp.record & MFG_HIST_DISTANCE) && !(hp.distance_binsize > 0 && hp.distance_max >= 0 && hp.distance_max / hp.distance_binsize < 1e8)) ||
                ((hp.record & MFG_HIST_TIME) && !(hp.time_binsize > 0 && hp.time_max >= 0 && hp.time_max / hp.time_binsize < 1e8)) ||
                ((hp.record & MFG_HIST_BOUNCE) && hp.bounce_max / (hp.bounce_binsize ? hp.bounce_binsize : 1) > 100000000ull)) {
                err = "bad histogram settings on facet " + std::to_string(i + 1);
                return MFG_ERR_INVALID_MODEL;
            }
        }
        if (!(m.temperature[i] > 0)) { err = "temperature must be positive on facet " + std::to_string(i + 1); return MFG_ERR_INVALID_MODEL; }
    }

    // time-dependent parameters
    const int np = d->n_params;
    m.par_start.assign(1, 0);
    for (int p = 0; p < np; ++p) {
        int s = d->param_start[p], e = d->param_start[p + 1];
        if (e - s < 1) { err = "empty time-dependent parameter"; return MFG_ERR_INVALID_MODEL; }
        for (int k = s; k < e; ++k) { m.par_t.push_back(d->param_t[k]); m.par_v.push_back(d->param_v[k]); }
        m.par_start.push_back(int32_t(m.par_t.size()));
        m.par_logx.push_back(opt<uint8_t>(d->param_log_x, p, 0));
        m.par_logy.push_back(opt<uint8_t>(d->param_log_y, p, 0));
    }
    for (int i = 0; i < nf; ++i)
        if (m.p_stick[i] >= np || m.p_opac[i] >= np || m.p_outg[i] >= np || m.p_temp[i] >= np) {
            err = "facet " + std::to_string(i + 1) + " refers to a missing time-dependent parameter";
            return MFG_ERR_INVALID_MODEL;
        }

    // moments, latest moment (PrepareToRun) and interval cache
    m.nm = d->n_moments;
    for (int k = 0; k < m.nm; ++k) {
        if (k > 0 && d->moment_time[k] < d->moment_time[k - 1]) { err = "moments must be sorted by time"; return MFG_ERR_INVALID_MODEL; }
        m.mstart.push_back(d->moment_time[k] - 0.5 * d->moment_window[k]);
        m.mend.push_back(d->moment_time[k] + 0.5 * d->moment_window[k]);
        m.maxwin = std::max(m.maxwin, d->moment_window[k]);
    }
    m.latest = m.nm ? d->moment_time[m.nm - 1] + 0.5 * d->moment_window[m.nm - 1] : m.time_window * 0.5;
    build_moment_guide(m);

    // Maxwell CDF at 1 K on 100 points up to 4x the most probable speed (CDFGeneration.cpp:54-83)
    {
        const double kb = 1.38E-23, R = 8.3144621;
        double a = std::sqrt(kb / (m.gas_mass * 1.67E-27));
        double vp = std::sqrt(2.0 * R / (m.gas_mass / 1000.0));
        double bin = 4.0 * vp / double(MFG_MAXWELL_N);
        for (int i = 0; i < MFG_MAXWELL_N; ++i) {
            double x = double(i) * bin;
            double y = (x * x) / (2.0 * a * a);
            m.cdf_v[i] = x;
            m.cdf_p[i] = 1.0 - std::exp(-y) * (y + 1.0);
        }
    }

    // integrated desorption tables, one per outgassing parameter
    m.facet_id.assign(nf, -1);
    m.id_start.assign(1, 0);
    {
        std::vector<int> par2id(np, -1);
        for (int i = 0; i < nf; ++i) {
            int p = m.p_outg[i];
            if (p < 0) continue;
            if (par2id[p] < 0) {
                std::vector<double> it, ic;
                int s = m.par_start[p], e = m.par_start[p + 1];
                integrated_desorption(&m.par_t[s], &m.par_v[s], e - s, m.par_logx[p], m.par_logy[p], m.latest, it, ic);
                m.id_t.insert(m.id_t.end(), it.begin(), it.end());
                m.id_cum.insert(m.id_cum.end(), ic.begin(), ic.end());
                m.id_start.push_back(int32_t(m.id_t.size()));
                par2id[p] = int(m.id_start.size()) - 2;
            }
            m.facet_id[i] = par2id[p];
        }
    }

    // source table (StartFromSource weights, Particle.cpp:421-464; CalcTotalOutgassing,
    // MolflowSimGeom.cpp:297-328).  A facet with an outgassing map gets one entry per cell of
    // non-zero rate, so that one search picks the facet and the cell (Particle.cpp:425-446:
    // the first cell whose cumulative rate exceeds the remainder).
    m.src_cdf.clear();
    m.src_facet.clear();
    m.src_id.clear();
    m.src_cell.clear();
    m.og.clear();
    bool any_map = false;
    for (int i = 0; i < nf; ++i) any_map = any_map || (m.og_w[i] > 0 && m.og_h[i] > 0);
    if (any_map && !d->outgassing_map) { err = "outgassing_map_width is set but outgassing_map is NULL"; return MFG_ERR_INVALID_MODEL; }
    if (any_map) {
        m.og.assign(nf, OgDev{0, 0, 0.0, 0.0});
        for (int i = 0; i < nf; ++i) {
            if (!(m.og_w[i] > 0 && m.og_h[i] > 0)) continue;
            const HostFacet& F = m.facets[i];
            const double nu = std::sqrt(F.U[0] * F.U[0] + F.U[1] * F.U[1] + F.U[2] * F.U[2]);
            const double nv = std::sqrt(F.V[0] * F.V[0] + F.V[1] * F.V[1] + F.V[2] * F.V[2]);
            m.og[i] = OgDev{m.og_w[i], m.og_h[i], nu * m.og_ru[i], nv * m.og_rv[i]};
            if (!(m.og[i].wp > m.og_w[i] - 1.0 && m.og[i].hp > m.og_h[i] - 1.0)) {
                err = "facet " + std::to_string(i + 1) + ": the outgassing map has more cells than its ratio puts on the facet";
                return MFG_ERR_INVALID_MODEL;
            }
        }
    }
    double sum = 0;
    size_t cursor = 0;
    for (int i = 0; i < nf; ++i) {
        const bool map = m.og_w[i] > 0 && m.og_h[i] > 0;
        const double* cells = map ? d->outgassing_map + cursor : nullptr;
        const int ncell = map ? m.og_w[i] * m.og_h[i] : 0;
        cursor += size_t(ncell);
        if (m.desorb_type[i] == MFG_DES_NONE) continue;
        if (map) {
            double tot = 0;
            for (int c = 0; c < ncell; ++c) {
                if (!(cells[c] >= 0)) { err = "facet " + std::to_string(i + 1) + ": negative outgassing-map cell"; return MFG_ERR_INVALID_MODEL; }
                tot += cells[c];
            }
            m.final_outgassing_rate += tot / (kKb * m.temperature[i]);
            m.final_outgassing_rate_pa += tot;
            if (!(tot > 0)) continue;
            if (m.structure[i] == -1) { err = "facet " + std::to_string(i + 1) + " is in all structures, it cannot desorb"; return MFG_ERR_INVALID_MODEL; }
            for (int c = 0; c < ncell; ++c) {
                if (!(cells[c] > 0)) continue;
                sum += m.latest * cells[c] / (kKb * m.temperature[i]);
                m.src_cdf.push_back(sum);
                m.src_facet.push_back(i);
                m.src_id.push_back(-1);
                m.src_cell.push_back(c);
            }
            continue;
        }
        double w;
        if (m.facet_id[i] >= 0) {
            w = m.id_cum[m.id_start[m.facet_id[i] + 1] - 1];
            const int p = m.p_outg[i];
            const double last = m.par_v[m.par_start[p + 1] - 1] * 0.1;   // mbar*l/s -> Pa*m3/s
            m.final_outgassing_rate += last / (kKb * m.temperature[i]);
            m.final_outgassing_rate_pa += last;
        } else {
            w = m.latest * m.outgassing[i];
            m.final_outgassing_rate += m.outgassing[i] / (kKb * m.temperature[i]);
            m.final_outgassing_rate_pa += m.outgassing[i];
        }
        w /= (kKb * m.temperature[i]);
        if (!(w > 0)) continue;
        if (m.structure[i] == -1) { err = "facet " + std::to_string(i + 1) + " is in all structures, it cannot desorb"; return MFG_ERR_INVALID_MODEL; }
        sum += w;
        m.src_cdf.push_back(sum);
        m.src_facet.push_back(i);
        m.src_id.push_back(m.facet_id[i]);
        if (any_map) m.src_cell.push_back(-1);
    }
    m.src_total = sum;
    m.total_desorbed_molecules = sum;

    // unsupported-on-GPU features
    auto unsupported = [&](const std::string& why) {
        if (m.gpu_supported) { m.gpu_supported = false; m.gpu_unsupported_reason = why; }
    };
    (void)unsupported;
    for (int i = 0; i < nf; ++i) {   // teleport destinations (PerformTeleport, Particle.cpp:83-121)
        const int t = m.teleport[i];
        if (t < -1) { err = "facet " + std::to_string(i + 1) + ": teleport destination out of range"; return MFG_ERR_INVALID_MODEL; }
        if (t > 0 && t <= nf && m.structure[t - 1] == -1) {
            err = "facet " + std::to_string(i + 1) + ": teleport destination is in all structures";
            return MFG_ERR_INVALID_MODEL;
        }
    }

    // layout + texture increments (Initializer.cpp:433-456)
    mfg_state_layout& L = m.layout;
    L = mfg_state_layout{};
    L.n_facets = nf;
    L.n_moments = m.nm;
    m.tex_off.assign(nf, -1); m.dir_off.assign(nf, -1); m.ang_off.assign(nf, -1); m.prof_idx.assign(nf, -1);
    m.tex_w.assign(nf, 0); m.tex_h.assign(nf, 0);
    // the device addresses texture, direction and angle-map cells with 32-bit offsets
    constexpr int64_t kMaxCells = 2147483647;
    for (int i = 0; i < nf; ++i) {
        if (!(m.texw_p[i] >= 0 && m.texh_p[i] >= 0 && m.texw_p[i] < double(kMaxCells) && m.texh_p[i] < double(kMaxCells))) {
            err = "texture size out of range on facet " + std::to_string(i + 1);
            return MFG_ERR_INVALID_MODEL;
        }
        if (m.texw_p[i] * m.texh_p[i] > 0) {
            m.tex_w[i] = std::max(1, int(std::ceil(m.texw_p[i] - 1e-9)));
            m.tex_h[i] = std::max(1, int(std::ceil(m.texh_p[i] - 1e-9)));
            m.tex_off[i] = L.texture_cells;
            L.texture_cells += int64_t(m.tex_w[i]) * m.tex_h[i];
            if (m.count[i] & MFG_COUNT_DIR) { m.dir_off[i] = L.direction_cells; L.direction_cells += int64_t(m.tex_w[i]) * m.tex_h[i]; }
        } else {
            m.count[i] = 0;
        }
        if (m.profile_type[i] != MFG_PROFILE_NONE) m.prof_idx[i] = L.profile_facets++;
        if (m.am_record[i] && m.am_phi[i] > 0 && m.am_lo[i] >= 0 && m.am_hi[i] >= 0 && m.am_lo[i] + m.am_hi[i] > 0) {
            m.ang_off[i] = L.anglemap_cells;
            L.anglemap_cells += int64_t(m.am_phi[i]) * (int64_t(m.am_lo[i]) + m.am_hi[i]);
        }
        if (L.texture_cells > kMaxCells || L.direction_cells > kMaxCells || L.anglemap_cells > kMaxCells) {
            err = "more than 2^31-1 texture, direction or angle-map cells (at facet " + std::to_string(i + 1) + ")";
            return MFG_ERR_LIMIT;
        }
    }
    const int64_t B = 1 + m.nm;
    L.n_global = MFG_G_N;
    L.n_facet_counts = B * nf * MFG_FC_N;
    L.n_facet_sums = B * nf * MFG_FS_N;
    L.n_texture = B * L.texture_cells * 3;
    L.n_profile = B * L.profile_facets * MFG_PROFILE_SIZE * 3;
    L.n_direction = B * L.direction_cells * 4;
    L.n_anglemap = L.anglemap_cells;
    // angle-map desorption: midpoint CDFs and normalised phi pdfs of each source facet's recorded
    // map (MolflowSimFacet::InitializeAngleMap, MolflowSimFacet.cpp:90-215)
    m.am_of_facet.clear();
    m.am_dev.clear();
    m.am_pool.clear();
    {
        size_t cursor = 0;
        for (int i = 0; i < nf; ++i) {
            if (m.desorb_type[i] != MFG_DES_ANGLEMAP) continue;
            if (m.am_of_facet.empty()) m.am_of_facet.assign(nf, -1);
            const int w = m.am_phi[i], lo = m.am_lo[i], hi = m.am_hi[i];
            if (!(w > 0 && lo >= 0 && hi >= 0 && int64_t(lo) + hi > 0) || !d->desorb_anglemap) {
                err = "facet " + std::to_string(i + 1) + " desorbs by angle map but has no recorded angle map";
                return MFG_ERR_INVALID_MODEL;
            }
            if (2 * int64_t(w) * (int64_t(lo) + hi) + (int64_t(lo) + hi) + 8 + int64_t(m.am_pool.size()) > kMaxCells) {
                err = "facet " + std::to_string(i + 1) + ": angle-map desorption tables past 2^31-1 entries";
                return MFG_ERR_LIMIT;
            }
            const uint64_t* pdf = d->desorb_anglemap + cursor;
            cursor += size_t(w) * (lo + hi);
            AmDev a{};
            a.w = w; a.lo = lo; a.hi = hi; a.limit = m.am_limit[i];
            std::vector<double> sum_lo(lo), sum_hi(hi);
            double slo = 0, sall = 0;
            for (int t = 0; t < lo; ++t) { for (int k = 0; k < w; ++k) sum_lo[t] += double(pdf[size_t(t) * w + k]); slo += sum_lo[t]; }
            sall = slo;
            for (int t = 0; t < hi; ++t) { for (int k = 0; k < w; ++k) sum_hi[t] += double(pdf[size_t(lo + t) * w + k]); sall += sum_hi[t]; }
            if (sall == 0) {
                err = "facet " + std::to_string(i + 1) + " has an all-zero recorded angle map but desorbs by it";
                return MFG_ERR_INVALID_MODEL;
            }
            a.total = sall;
            a.lower_ratio = slo / sall;
            auto put = [&](const std::vector<double>& v) { int32_t o = int32_t(m.am_pool.size()); m.am_pool.insert(m.am_pool.end(), v.begin(), v.end()); m.am_pool.push_back(0.0); return o; };
            std::vector<double> tcdf_lo(lo), tcdf_hi(hi), pcdf_lo(size_t(w) * lo), pcdf_hi(size_t(w) * hi),
                ppdf_lo(size_t(w) * lo), ppdf_hi(size_t(w) * hi);
            const double tn = 1.0 / sall;
            for (int part = 0; part < 2; ++part) {
                const int n = part ? hi : lo, base = part ? lo : 0;
                std::vector<double>& tcdf = part ? tcdf_hi : tcdf_lo;
                const std::vector<double>& sum = part ? sum_hi : sum_lo;
                std::vector<double>& pcdf = part ? pcdf_hi : pcdf_lo;
                std::vector<double>& ppdf = part ? ppdf_hi : ppdf_lo;
                for (int t = 0; t < n; ++t) {
                    tcdf[t] = t == 0 ? (part ? a.lower_ratio : 0.0) + 0.5 * sum[0] * tn : tcdf[t - 1] + (sum[t - 1] + sum[t]) * 0.5 * tn;
                    const double pn = 1.0 / sum[t];
                    const uint64_t* line = pdf + size_t(base + t) * w;
                    for (int k = 0; k < w; ++k) {
                        const size_t q = size_t(t) * w + k;
                        if (sum[t] == 0) {   // empty line: uniform phi
                            pcdf[q] = (0.5 + k) / double(w);
                            ppdf[q] = 1.0 / double(w);
                        } else {
                            pcdf[q] = k == 0 ? 0.5 * double(line[0]) * pn : pcdf[q - 1] + double(line[k - 1] + line[k]) * 0.5 * pn;
                            ppdf[q] = double(line[k]) * pn;
                        }
                    }
                }
            }
            a.tcdf_lo = put(tcdf_lo); a.tcdf_hi = put(tcdf_hi);
            a.sum_lo = put(sum_lo); a.sum_hi = put(sum_hi);
            a.pcdf_lo = put(pcdf_lo); a.pcdf_hi = put(pcdf_hi);
            a.ppdf_lo = put(ppdf_lo); a.ppdf_hi = put(ppdf_hi);
            m.am_of_facet[i] = int32_t(m.am_dev.size());
            m.am_dev.push_back(a);
        }
    }
    // histograms: global set at offset 0, then each recording facet's (bounce, distance, time);
    // bin counts restated from the sizes the reference stores with its histograms
    // (false for a bin size that is not positive or a bin count past 2^30)
    auto hist_of = [](const mfg_histogram_params& p, HistDev& h) -> bool {
        h = HistDev{};
        h.off = -1;
        h.record = p.record;
        if (!p.record) return true;
        constexpr double kMaxBins = 1073741824.0;
        h.bounce_bin = p.bounce_binsize ? p.bounce_binsize : 1;
        h.dist_bin = p.distance_binsize;
        h.time_bin = p.time_binsize;
        if (p.record & MFG_HIST_BOUNCE) {
            if (double(p.bounce_max / h.bounce_bin) >= kMaxBins) return false;
            h.nb = int32_t(p.bounce_max / h.bounce_bin + 2);
        }
        if (p.record & MFG_HIST_DISTANCE) {
            const double n = p.distance_max / p.distance_binsize;
            if (!(p.distance_binsize > 0 && p.distance_max >= 0 && n < kMaxBins)) return false;
            h.nd = int32_t(size_t(n) + 1);
        }
        if (p.record & MFG_HIST_TIME) {
            const double n = p.time_max / p.time_binsize;
            if (!(p.time_binsize > 0 && p.time_max >= 0 && n < kMaxBins)) return false;
            h.nt = int32_t(size_t(n) + 1);
        }
        return true;
    };
    int64_t hb = 0;
    if (!hist_of(d->global_histogram, m.ghist)) { err = "global histogram: bin size or range out of range"; return MFG_ERR_INVALID_MODEL; }
    if (m.ghist.record) { m.ghist.off = 0; hb = int64_t(m.ghist.nb) + m.ghist.nd + m.ghist.nt; }
    m.fhist.clear();
    if (d->facet_histogram) {
        m.fhist.resize(nf);
        for (int i = 0; i < nf; ++i) {
            if (!hist_of(d->facet_histogram[i], m.fhist[i])) {
                err = "histogram of facet " + std::to_string(i + 1) + ": bin size or range out of range";
                return MFG_ERR_INVALID_MODEL;
            }
            if (m.fhist[i].record) {
                m.fhist[i].off = int32_t(hb);
                hb += int64_t(m.fhist[i].nb) + m.fhist[i].nd + m.fhist[i].nt;
                if (hb > kMaxCells) { err = "more than 2^31-1 histogram bins (at facet " + std::to_string(i + 1) + ")"; return MFG_ERR_LIMIT; }
            }
        }
    }
    L.histogram_bins = hb;
    L.n_histogram = B * hb;
    L.n_force = m.force ? B * int64_t(nf) * 9 : 0;
    m.tex_inc.assign(size_t(L.texture_cells), 0.0);
    for (int i = 0; i < nf; ++i) {
        if (m.tex_off[i] < 0) continue;
        const HostFacet& F = m.facets[i];
        double lu = std::sqrt(F.U[0] * F.U[0] + F.U[1] * F.U[1] + F.U[2] * F.U[2]);
        double lv = std::sqrt(F.V[0] * F.V[0] + F.V[1] * F.V[1] + F.V[2] * F.V[2]);
        double rw = lu / m.texw_p[i], rh = lv / m.texh_p[i];
        double sides = m.two_sided[i] ? 2.0 : 1.0;
        std::vector<double> poly(2 * F.nv);
        for (int k = 0; k < F.nv; ++k) {
            poly[2 * k] = m.v2[2 * (F.vstart + k)] * lu;
            poly[2 * k + 1] = m.v2[2 * (F.vstart + k) + 1] * lv;
        }
        for (int y = 0; y < m.tex_h[i]; ++y)
            for (int x = 0; x < m.tex_w[i]; ++x) {
                double a = clipped_area(poly, x * rw, y * rh, (x + 1) * rw, (y + 1) * rh);
                m.tex_inc[m.tex_off[i] + int64_t(y) * m.tex_w[i] + x] = (a > 1e-12 * rw * rh) ? 1.0 / (a * sides) : 0.0;
            }
    }

    // scene scale
    double sc = 0;
    for (int k = 0; k < 3 * d->n_vertices; ++k) sc = std::max(sc, std::fabs(d->vertices[k]));
    m.scene_scale = std::max(sc, 1e-30);

    // BVH per structure, breadth-first
    m.roots.clear();
    m.prims.clear();
    m.nodes_d.clear();
    m.nodes_c.clear();
    m.roots_c.clear();
    m.prims_c.clear();
    m.bvh_depth = 0;
    m.bvh_leaves = 0;
    const double pad64 = 1e-9 * m.scene_scale, pad32 = 2e-6 * m.scene_scale;
    for (int s = 0; s < m.nstruct; ++s) {
        std::vector<int> ids;
        for (int i = 0; i < nf; ++i)
            if (m.structure[i] == -1 || m.structure[i] == s) ids.push_back(i);
        m.roots.push_back(int32_t(m.nodes_d.size()));
        // root NodeC of the structure: child 0 = the whole tree (filled below), child 1 = an
        // empty leaf whose box is a point far outside any scene
        m.roots_c.push_back(int32_t(m.nodes_c.size()));
        {
            NodeC r{};
            for (int a = 0; a < 3; ++a) { r.lo0[a] = r.hi0[a] = r.lo1[a] = r.hi1[a] = 1e30f; }
            r.c0 = r.c1 = -1 - int32_t(m.prims_c.size());
            m.prims_c.push_back(-1);
            m.nodes_c.push_back(r);
        }
        if (ids.empty()) {   // empty structure: one leaf with no facets and an empty box
            NodeD e{};
            for (int a = 0; a < 3; ++a) { e.lo[a] = 1; e.hi[a] = -1; }
            e.a = int32_t(m.prims.size());
            e.b = -1;
            m.nodes_d.push_back(e);
            continue;
        }
        std::vector<BuildNode> tree;
        int64_t depth = 0;
        build_rec(tree, ids, 0, int(ids.size()), m.facets, std::max(1, leaf_max), 0, depth, d->bvh_facet_weight);
        m.bvh_depth = std::max(m.bvh_depth, depth);
        // breadth-first relabel
        std::vector<int> order;
        order.push_back(0);
        std::vector<int> newidx(tree.size(), -1);
        newidx[0] = 0;
        int base = int(m.nodes_d.size());
        for (size_t q = 0; q < order.size(); ++q) {
            const BuildNode& b = tree[order[q]];
            if (b.left >= 0) {
                newidx[b.left] = int(order.size());
                order.push_back(b.left);
                newidx[b.right] = int(order.size());
                order.push_back(b.right);
            }
        }
        int pbase = int(m.prims.size());
        for (size_t q = 0; q < order.size(); ++q) {
            const BuildNode& b = tree[order[q]];
            NodeD nd{};
            for (int a = 0; a < 3; ++a) {
                nd.lo[a] = b.lo[a] - pad64;
                nd.hi[a] = b.hi[a] + pad64;
            }
            if (b.left >= 0) {
                nd.a = base + newidx[b.left];
                nd.b = b.axis;
            } else {
                nd.a = pbase + b.first;
                nd.b = -1 - b.count;
                m.bvh_leaves++;
            }
            m.nodes_d.push_back(nd);
        }
        for (int i : ids) m.prims.push_back(i);
        // two-child FP32 layout, breadth-first over the internal nodes
        {
            const int croot = m.roots_c.back();
            auto box32 = [&](const BuildNode& b, float* lo, float* hi) {
                for (int a = 0; a < 3; ++a) { lo[a] = round_down(b.lo[a] - pad32); hi[a] = round_up(b.hi[a] + pad32); }
            };
            auto leaf_ref = [&](const BuildNode& b) {
                const int32_t ref = -1 - int32_t(m.prims_c.size());
                for (int k = 0; k < b.count; ++k) m.prims_c.push_back(ids[b.first + k]);
                m.prims_c.push_back(-1);
                return ref;
            };
            std::vector<int> inner;                 // tree indices of internal nodes, BFS order
            std::vector<int32_t> cidx(tree.size(), -1);
            if (tree[0].left >= 0) {
                inner.push_back(0);
                for (size_t q = 0; q < inner.size(); ++q) {
                    const BuildNode& b = tree[inner[q]];
                    for (int c : {b.left, b.right})
                        if (tree[c].left >= 0) inner.push_back(c);
                }
            }
            const int32_t cbase = int32_t(m.nodes_c.size());
            for (size_t q = 0; q < inner.size(); ++q) cidx[inner[q]] = cbase + int32_t(q);
            {
                NodeC& r = m.nodes_c[croot];
                box32(tree[0], r.lo0, r.hi0);
                r.c0 = tree[0].left >= 0 ? cidx[0] : leaf_ref(tree[0]);
            }
            for (size_t q = 0; q < inner.size(); ++q) {
                const BuildNode& b = tree[inner[q]];
                NodeC nc{};
                box32(tree[b.left], nc.lo0, nc.hi0);
                box32(tree[b.right], nc.lo1, nc.hi1);
                nc.c0 = tree[b.left].left >= 0 ? cidx[b.left] : leaf_ref(tree[b.left]);
                nc.c1 = tree[b.right].left >= 0 ? cidx[b.right] : leaf_ref(tree[b.right]);
                m.nodes_c.push_back(nc);
            }
        }
    }

    // device records
    m.isect_d.resize(nf);
    m.isect_f.resize(nf);
    m.poly_d.resize(nf);
    m.poly_f.resize(nf);
    m.tri_f.assign(nf, TriF{});
    m.phys_d.resize(nf);
    m.phys_f.resize(nf);
    m.info.resize(nf);
    m.info2.resize(nf);
    m.centers.resize(3 * size_t(nf));
    m.v2_d.resize(m.v2.size() / 2);
    m.v2_f.resize(m.v2.size() / 2);
    for (size_t k = 0; k < m.v2_d.size(); ++k) {
        m.v2_d[k] = make_double2(m.v2[2 * k], m.v2[2 * k + 1]);
        m.v2_f[k] = make_float2(float(m.v2[2 * k]), float(m.v2[2 * k + 1]));
    }
    for (int i = 0; i < nf; ++i) {
        const HostFacet& F = m.facets[i];
        double u2 = F.U[0] * F.U[0] + F.U[1] * F.U[1] + F.U[2] * F.U[2];
        double v2 = F.V[0] * F.V[0] + F.V[1] * F.V[1] + F.V[2] * F.V[2];
        double* r = m.isect_d[i].v;
        std::memset(r, 0, sizeof(double) * 16);
        for (int a = 0; a < 3; ++a) {
            r[a] = F.N[a];
            r[4 + a] = F.O[a];
            r[8 + a] = F.U[a] / u2;
            r[12 + a] = F.V[a] / v2;
        }
        r[3] = F.N[0] * F.O[0] + F.N[1] * F.O[1] + F.N[2] * F.O[2];
        // flags in the record's padding: bit 0 two-sided, bits 1-2 opacity class
        const long long opac_class = (m.p_opac[i] >= 0 || (m.opacity[i] > 0.0 && m.opacity[i] < 1.0)) ? 2
                                   : (m.opacity[i] <= 0.0 ? 1 : 0);
        const long long flags = (m.two_sided[i] ? 1 : 0) | (opac_class << 1);
        std::memcpy(&r[7], &flags, sizeof flags);
        if (opac_class) m.has_transparent = 1;
        // FP32 copy: [N | O hi/lo split | U/|U|^2 | V/|V|^2] (origin-relative FP32 facet test)
        float* q = m.isect_f[i].v;
        for (int k = 0; k < 16; ++k) q[k] = 0.0f;
        for (int a = 0; a < 3; ++a) {
            q[a] = float(r[a]);
            q[8 + a] = float(r[8 + a]);
            q[12 + a] = float(r[12 + a]);
            q[4 + a] = float(F.O[a]);
        }
        q[3] = float(F.O[0] - double(q[4]));
        q[7] = float(F.O[1] - double(q[5]));
        q[11] = float(F.O[2] - double(q[6]));
        q[15] = float(flags);
        // circle shortcut for the point-in-polygon test
        double su = std::sqrt(u2), sv = std::sqrt(v2);
        const double* pv = &m.v2[2 * size_t(F.vstart)];
        bool rect = false;
        if (F.nv == 4) {
            int corners = 0;
            for (int k = 0; k < 4; ++k) {
                double u = pv[2 * k], v = pv[2 * k + 1];
                bool cu = std::fabs(u) < 1e-12 || std::fabs(u - 1) < 1e-12;
                bool cv = std::fabs(v) < 1e-12 || std::fabs(v - 1) < 1e-12;
                corners += (cu && cv);
            }
            rect = corners == 4;
        }
        double cx = 0, cy = 0;
        for (int k = 0; k < F.nv; ++k) { cx += pv[2 * k] * su; cy += pv[2 * k + 1] * sv; }
        cx /= F.nv;
        cy /= F.nv;
        double rin = 0, rout = 0;
        bool cin = inside_poly(pv, F.nv, cx / su, cy / sv);
        for (int k = 0; k < F.nv; ++k) {
            int j = (k + 1) % F.nv;
            double ax = pv[2 * k] * su, ay = pv[2 * k + 1] * sv, bx = pv[2 * j] * su, by = pv[2 * j + 1] * sv;
            rout = std::max(rout, std::hypot(ax - cx, ay - cy));
            double ex = bx - ax, ey = by - ay, l2 = ex * ex + ey * ey;
            double t = l2 > 0 ? std::clamp(((cx - ax) * ex + (cy - ay) * ey) / l2, 0.0, 1.0) : 0.0;
            double dd = std::hypot(ax + t * ex - cx, ay + t * ey - cy);
            rin = (k == 0) ? dd : std::min(rin, dd);
        }
        if (!cin) rin = 0;
        PolyD& P = m.poly_d[i];
        P.cu = cx / su;
        P.cv = cy / sv;
        P.su = su;
        P.sv = sv;
        P.rin2 = rect ? 1e300 : (rin * (1 - 1e-9)) * (rin * (1 - 1e-9));
        P.rout2 = (rout * (1 + 1e-9)) * (rout * (1 + 1e-9));
        P.vstart = F.vstart;
        P.nv = F.nv;
        PolyF& Q = m.poly_f[i];
        Q.cu = float(P.cu);
        Q.cv = float(P.cv);
        Q.su = float(su);
        Q.sv = float(sv);
        Q.rin2 = rect ? 1e30f : float(P.rin2 * (1 - 1e-5));
        Q.rout2 = float(P.rout2 * (1 + 1e-5));
        Q.vstart = F.vstart;
        Q.nv = F.nv;
        if (F.nv == 3) {   // edge lines in cm, oriented so that the inside is positive
            double px[3], py[3];
            for (int k = 0; k < 3; ++k) { px[k] = pv[2 * k] * su; py[k] = pv[2 * k + 1] * sv; }
            const double area2 = (px[1] - px[0]) * (py[2] - py[0]) - (px[2] - px[0]) * (py[1] - py[0]);
            if (area2 != 0) {
                const double sg = area2 > 0 ? 1.0 : -1.0;
                for (int k = 0; k < 3; ++k) {
                    const int j = (k + 1) % 3;
                    const double ex = px[j] - px[k], ey = py[j] - py[k], len = std::hypot(ex, ey);
                    // distance of (x, y) = (u su, v sv): sg (ex (y - py_k) - (x - px_k) ey) / len
                    const double a = -sg * ey * su / len, b = sg * ex * sv / len, c = sg * (px[k] * ey - py[k] * ex) / len;
                    float* e = m.tri_f[i].e[k];
                    e[0] = float(a); e[1] = float(b); e[2] = float(c); e[3] = 0.0f;
                }
            }
        }
        FacetPhysD& ph = m.phys_d[i];
        for (int a = 0; a < 3; ++a) { ph.nU[a] = F.nU[a]; ph.nV[a] = F.nV[a]; }
        ph.sticking = m.sticking[i];
        ph.sqrtT = std::sqrt(m.temperature[i]);
        ph.accommodation = m.accommodation[i];
        ph.diffuse = m.diffuse[i];
        ph.specular = m.specular[i];
        ph.cos_exp = m.cos_exp[i];
        ph.texw_p = m.texw_p[i];
        ph.texh_p = m.texh_p[i];
        ph.soj_freq = m.soj_freq[i];
        ph.soj_e = m.soj_e[i];
        FacetPhysF& pf = m.phys_f[i];
        for (int a = 0; a < 3; ++a) { pf.nU[a] = float(F.nU[a]); pf.nV[a] = float(F.nV[a]); pf.N[a] = float(F.N[a]); }
        pf.sticking = float(m.sticking[i]);
        pf.sqrtT = float(ph.sqrtT);
        pf.accommodation = float(m.accommodation[i]);
        pf.diffuse = float(m.diffuse[i]);
        pf.specular = float(m.specular[i]);
        pf.cos_exp = float(m.cos_exp[i]);
        pf.texw_p = float(m.texw_p[i]);
        pf.texh_p = float(m.texh_p[i]);
        pf.pad = 0;
        FacetInfo& in = m.info[i];
        in.flags = (m.two_sided[i] ? FF_TWO_SIDED : 0) | (m.tex_off[i] >= 0 ? FF_TEXTURED : 0) |
                   (m.p_stick[i] >= 0 ? FF_STICK_PARAM : 0) | (m.p_temp[i] >= 0 ? FF_TEMP_PARAM : 0) |
                   (m.sojourn[i] ? FF_SOJOURN : 0) | (m.ang_off[i] >= 0 ? FF_ANGLEMAP : 0) |
                   (m.prof_idx[i] >= 0 ? FF_PROFILE : 0) | (m.diffuse[i] > 0.999999 ? FF_DIFFUSE_ONLY : 0) |
                   (m.link[i] ? FF_LINK : 0) | (m.teleport[i] ? FF_TELEPORT : 0);
        if (m.diffuse[i] > 0.999999 && m.accommodation[i] > 0.9999 && m.use_maxwell && !m.sojourn[i] && m.p_temp[i] < 0 &&
            !m.moving[i])
            in.flags |= FF_FAST_REFL;
        if (m.moving[i]) in.flags |= FF_MOVING;
        in.count = m.count[i];
        in.tex_off = int32_t(m.tex_off[i]);
        in.tex_w = m.tex_w[i];
        in.tex_h = m.tex_h[i];
        in.prof_idx = int32_t(m.prof_idx[i]);
        in.ang_off = int32_t(m.ang_off[i]);
        in.profile_type = m.profile_type[i];
        FacetInfo2& i2 = m.info2[i];
        i2.structure = m.structure[i];
        i2.desorb_type = m.desorb_type[i];
        i2.stick_param = m.p_stick[i];
        i2.temp_param = m.p_temp[i];
        i2.am_phi = m.am_phi[i];
        i2.am_lo = m.am_lo[i];
        i2.am_hi = m.am_hi[i];
        i2.dir_off = int32_t(m.dir_off[i]);
        i2.opacity = m.opacity[i];
        i2.opac_param = m.p_opac[i];
        i2.link = m.link[i] ? m.link[i] - 1 : -1;
        i2.teleport = m.teleport[i];
        i2.am_limit = m.am_limit[i];
        i2.max_speed = m.max_speed[i];
        i2.desorb_exp = m.desorb_exp[i];
        i2.temperature = m.temperature[i];
        for (int a = 0; a < 3; ++a) m.centers[3 * i + a] = F.center[a];
    }
    HostModel::Instance inst;
    inst.nf = nf;
    inst.nstruct = m.nstruct;
    inst.nsrc = int(m.src_facet.size());
    inst.src_total = m.src_total;
    inst.layout = m.layout;
    m.instances.assign(1, inst);
    bool any_moving = false;
    for (int i = 0; i < nf; ++i) any_moving = any_moving || m.moving[i];
    m.has_ext = m.has_transparent || m.layout.histogram_bins > 0 || m.low_flux || m.scatter || any_moving || !m.am_dev.empty() || m.force || m.log_facet >= 0 ||
                std::any_of(m.teleport.begin(), m.teleport.end(), [](int32_t t) { return t != 0; });
    return MFG_OK;
}

int merge_host_models(const std::vector<const HostModel*>& parts, HostModel& out, std::string& err) {
    if (parts.empty()) { err = "no models to merge"; return MFG_ERR_INVALID_ARGUMENT; }
    const HostModel& p0 = *parts[0];
    for (const HostModel* p : parts) {
        if (p->instances.size() != 1) { err = "merged models cannot be merged again"; return MFG_ERR_INVALID_ARGUMENT; }
        if (p->gas_mass != p0.gas_mass || p->use_maxwell != p0.use_maxwell || p->constant_flow != p0.constant_flow ||
            p->enable_decay != p0.enable_decay || p->half_life != p0.half_life || p->time_window != p0.time_window ||
            p->mstart != p0.mstart || p->mend != p0.mend || p->low_flux != p0.low_flux) {
            err = "batched models must share gas, speed law, flow mode, decay and moments";
            return MFG_ERR_INVALID_ARGUMENT;
        }
    }
    for (const HostModel* p : parts) {
        if (p->layout.histogram_bins > 0) { err = "histograms are not recorded in batched instances"; return MFG_ERR_UNSUPPORTED_FEATURE; }
        if (p->low_flux) { err = "low-flux mode is not traced in batched instances"; return MFG_ERR_UNSUPPORTED_FEATURE; }
        if (p->scatter || p->motion_type || !p->am_dev.empty() || !p->og.empty() || p->force || p->log_facet >= 0 ||
            std::any_of(p->teleport.begin(), p->teleport.end(), [](int32_t t) { return t != 0; })) {
            err = "scattering, moving facets, angle-map desorption, outgassing maps, teleports, force measurement and the particle logger are not traced in batched instances";
            return MFG_ERR_UNSUPPORTED_FEATURE;
        }
    }
    out = HostModel();
    out.nm = p0.nm;
    out.gas_mass = p0.gas_mass; out.time_window = p0.time_window; out.half_life = p0.half_life;
    out.low_flux_cutoff = p0.low_flux_cutoff; out.use_maxwell = p0.use_maxwell;
    out.constant_flow = p0.constant_flow; out.enable_decay = p0.enable_decay; out.low_flux = p0.low_flux;
    out.latest = p0.latest; out.mstart = p0.mstart; out.mend = p0.mend; out.maxwin = p0.maxwin;
    out.mguide = p0.mguide; out.mg_t0 = p0.mg_t0; out.mg_l0 = p0.mg_l0; out.mg_scale = p0.mg_scale;
    std::copy(p0.cdf_v, p0.cdf_v + MFG_MAXWELL_N, out.cdf_v);
    std::copy(p0.cdf_p, p0.cdf_p + MFG_MAXWELL_N, out.cdf_p);
    out.par_start.assign(1, 0);
    out.id_start.assign(1, 0);
    out.layout = mfg_state_layout{};
    out.layout.n_moments = p0.nm;
    out.nstruct = 0;
    out.bvh_depth = 0;
    out.scene_scale = 0;
    int inst = 0;
    for (const HostModel* pp : parts) {
        const HostModel& p = *pp;
        ++inst;
        // the merged arrays are addressed with 32-bit offsets on the device
        auto fits = [](int64_t have, int64_t add) { return have + add <= int64_t(INT32_MAX); };
        if (!fits(out.nf, p.nf) || !fits(out.nstruct, p.nstruct) || !fits(out.layout.texture_cells, p.layout.texture_cells) ||
            !fits(out.layout.direction_cells, p.layout.direction_cells) || !fits(out.layout.anglemap_cells, p.layout.anglemap_cells) ||
            !fits(out.layout.profile_facets, p.layout.profile_facets) || !fits(int64_t(out.nodes_d.size()), int64_t(p.nodes_d.size())) ||
            !fits(int64_t(out.nodes_c.size()), int64_t(p.nodes_c.size())) || !fits(int64_t(out.prims.size()), int64_t(p.prims.size())) ||
            !fits(int64_t(out.prims_c.size()), int64_t(p.prims_c.size())) || !fits(int64_t(out.v2_d.size()), int64_t(p.v2_d.size())) ||
            !fits(int64_t(out.src_facet.size()), int64_t(p.src_facet.size())) || !fits(int64_t(out.id_t.size()), int64_t(p.id_t.size())) ||
            !fits(int64_t(out.par_t.size()), int64_t(p.par_t.size()))) {
            err = "the merged model passes 2^31-1 facets, structures, cells, BVH nodes or table entries at instance " +
                  std::to_string(inst);
            return MFG_ERR_LIMIT;
        }
        HostModel::Instance in = p.instances[0];
        in.facet_base = out.nf;
        in.struct_base = out.nstruct;
        in.src_base = int(out.src_facet.size());
        in.tex_base = out.layout.texture_cells;
        in.prof_base = out.layout.profile_facets;
        in.ang_base = out.layout.anglemap_cells;
        in.dir_base = out.layout.direction_cells;
        const int node_base = int(out.nodes_d.size()), prim_base = int(out.prims.size());
        const int v2_base = int(out.v2_d.size()), par_base = int(out.par_logx.size()), id_base = int(out.id_start.size()) - 1;
        if (!p.gpu_supported && out.gpu_supported) { out.gpu_supported = false; out.gpu_unsupported_reason = p.gpu_unsupported_reason; }
        for (NodeD nd : p.nodes_d) {
            if (nd.b >= 0) nd.a += node_base; else nd.a += prim_base;
            out.nodes_d.push_back(nd);
        }
        for (int r : p.roots) out.roots.push_back(r + node_base);
        const int32_t cbase = int32_t(out.nodes_c.size()), pcbase = int32_t(out.prims_c.size());
        for (NodeC nc : p.nodes_c) {
            nc.c0 = nc.c0 >= 0 ? nc.c0 + cbase : nc.c0 - pcbase;
            nc.c1 = nc.c1 >= 0 ? nc.c1 + cbase : nc.c1 - pcbase;
            out.nodes_c.push_back(nc);
        }
        for (int r : p.roots_c) out.roots_c.push_back(r + cbase);
        for (int f : p.prims_c) out.prims_c.push_back(f >= 0 ? f + in.facet_base : -1);
        for (int f : p.prims) out.prims.push_back(f + in.facet_base);
        out.isect_d.insert(out.isect_d.end(), p.isect_d.begin(), p.isect_d.end());
        out.isect_f.insert(out.isect_f.end(), p.isect_f.begin(), p.isect_f.end());
        for (PolyD q : p.poly_d) { q.vstart += v2_base; out.poly_d.push_back(q); }
        for (PolyF q : p.poly_f) { q.vstart += v2_base; out.poly_f.push_back(q); }
        out.tri_f.insert(out.tri_f.end(), p.tri_f.begin(), p.tri_f.end());
        out.v2_d.insert(out.v2_d.end(), p.v2_d.begin(), p.v2_d.end());
        out.v2_f.insert(out.v2_f.end(), p.v2_f.begin(), p.v2_f.end());
        out.phys_d.insert(out.phys_d.end(), p.phys_d.begin(), p.phys_d.end());
        out.phys_f.insert(out.phys_f.end(), p.phys_f.begin(), p.phys_f.end());
        for (FacetInfo fi : p.info) {
            if (fi.tex_off >= 0) fi.tex_off += int32_t(in.tex_base);
            if (fi.prof_idx >= 0) fi.prof_idx += int32_t(in.prof_base);
            if (fi.ang_off >= 0) fi.ang_off += int32_t(in.ang_base);
            out.info.push_back(fi);
        }
        for (FacetInfo2 f2 : p.info2) {
            if (f2.structure >= 0) f2.structure += in.struct_base;
            if (f2.dir_off >= 0) f2.dir_off += int32_t(in.dir_base);
            if (f2.stick_param >= 0) f2.stick_param += par_base;
            if (f2.temp_param >= 0) f2.temp_param += par_base;
            if (f2.opac_param >= 0) f2.opac_param += par_base;
            if (f2.link >= 0) f2.link += in.struct_base;
            out.info2.push_back(f2);
        }
        out.centers.insert(out.centers.end(), p.centers.begin(), p.centers.end());
        out.src_cdf.insert(out.src_cdf.end(), p.src_cdf.begin(), p.src_cdf.end());
        for (int f : p.src_facet) out.src_facet.push_back(f + in.facet_base);
        for (int k : p.src_id) out.src_id.push_back(k >= 0 ? k + id_base : -1);
        for (size_t k = 1; k < p.id_start.size(); ++k) out.id_start.push_back(p.id_start[k] + int32_t(out.id_t.size()));
        out.id_t.insert(out.id_t.end(), p.id_t.begin(), p.id_t.end());
        out.id_cum.insert(out.id_cum.end(), p.id_cum.begin(), p.id_cum.end());
        for (size_t k = 1; k < p.par_start.size(); ++k) out.par_start.push_back(p.par_start[k] + int32_t(out.par_t.size()));
        out.par_t.insert(out.par_t.end(), p.par_t.begin(), p.par_t.end());
        out.par_v.insert(out.par_v.end(), p.par_v.begin(), p.par_v.end());
        out.par_logx.insert(out.par_logx.end(), p.par_logx.begin(), p.par_logx.end());
        out.par_logy.insert(out.par_logy.end(), p.par_logy.begin(), p.par_logy.end());
        out.tex_inc.insert(out.tex_inc.end(), p.tex_inc.begin(), p.tex_inc.end());
        for (int i = 0; i < p.nf; ++i) {
            out.tex_off.push_back(p.tex_off[i] >= 0 ? p.tex_off[i] + in.tex_base : -1);
            out.dir_off.push_back(p.dir_off[i] >= 0 ? p.dir_off[i] + in.dir_base : -1);
            out.ang_off.push_back(p.ang_off[i] >= 0 ? p.ang_off[i] + in.ang_base : -1);
            out.prof_idx.push_back(p.prof_idx[i] >= 0 ? p.prof_idx[i] + in.prof_base : -1);
            out.tex_w.push_back(p.tex_w[i]);
            out.tex_h.push_back(p.tex_h[i]);
        }
        out.facets.insert(out.facets.end(), p.facets.begin(), p.facets.end());
        out.nf += p.nf;
        out.nstruct += p.nstruct;
        out.layout.texture_cells += p.layout.texture_cells;
        out.layout.profile_facets += p.layout.profile_facets;
        out.layout.anglemap_cells += p.layout.anglemap_cells;
        out.layout.direction_cells += p.layout.direction_cells;
        out.bvh_depth = std::max(out.bvh_depth, p.bvh_depth);
        out.bvh_leaves += p.bvh_leaves;
        out.scene_scale = std::max(out.scene_scale, p.scene_scale);
        out.has_transparent |= p.has_transparent;
        out.has_ext |= p.has_ext;
        out.instances.push_back(in);
    }
    mfg_state_layout& L = out.layout;
    const int64_t B = 1 + out.nm;
    L.n_facets = out.nf;
    L.n_global = MFG_G_N;
    L.n_facet_counts = B * out.nf * MFG_FC_N;
    L.n_facet_sums = B * out.nf * MFG_FS_N;
    L.n_texture = B * L.texture_cells * 3;
    L.n_profile = B * L.profile_facets * MFG_PROFILE_SIZE * 3;
    L.n_direction = B * L.direction_cells * 4;
    L.n_anglemap = L.anglemap_cells;
    out.src_total = 0;
    return MFG_OK;
}

}  // namespace mfg
