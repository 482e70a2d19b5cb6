// trace_kernels.cuh — persistent test-particle tracer for sm_103a.
//
// One thread carries one particle (origin FP64, direction, speed, time) through
// desorb -> BVH trace -> stick/reflect -> tally, and takes a new particle from
// its warp's pool when the old one is absorbed or leaks (the loop of
// MFSim::ParticleTracer::SimulationMCStep, src/Simulation/Particle.cpp:207-396).
// Two precisions share the code:
//   FP64   — plain double traversal, polygon tests and physics; random numbers and
//            their order are those of the CPU oracle, so per-particle trajectories
//            coincide with it;
//   FP32R  — FP32 traversal and facet tests with error bounds; a ray whose result
//            is ambiguous within those bounds is re-traced in FP64; the new origin
//            is computed in FP64 against the FP64 plane of the hit facet.
// Tallies are 64-bit fixed point: per-block shared-memory partials (facet
// counters, global counters) flushed to 128-bit global accumulators.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "device_model.h"
#include "philox.cuh"

namespace mfgk {

constexpr double kPi = 3.14159265358979323846;

// double stream: two uniforms per Philox block (the CPU oracle's order)
// counter = (particle id lo, hi, draw index, instance)
struct RngD {
    uint32_t p0, p1, ctr, k0, k1, inst;
    bool have;
    double cache;
    __device__ void start(uint64_t pid, uint32_t instance) {
        p0 = (uint32_t)pid; p1 = (uint32_t)(pid >> 32); ctr = 0; inst = instance; have = false;
    }
    __device__ double next() {
        if (have) { have = false; return cache; }
        uint32_t c0 = p0, c1 = p1, c2 = ctr++, c3 = inst;
        philox4x32_10(c0, c1, c2, c3, k0, k1);
        cache = u01d(c2, c3);
        have = true;
        return u01d(c0, c1);
    }
};
// float stream: four uniforms per Philox block, kept in registers (a buffer indexed at run time
// would live in local memory; +0.5 % hits/s on the tube)
struct RngF {
    uint32_t p0, p1, ctr, k0, k1, inst;
    uint32_t w0, w1, w2, w3;
    int n;
    __device__ void start(uint64_t pid, uint32_t instance) {
        p0 = (uint32_t)pid; p1 = (uint32_t)(pid >> 32); ctr = 0; inst = instance; n = 0;
    }
    __device__ float next() {
        if (n == 0) {
            uint32_t c0 = p0, c1 = p1, c2 = ctr++, c3 = inst;
            philox4x32_10(c0, c1, c2, c3, k0, k1);
            w0 = c0; w1 = c1; w2 = c2; w3 = c3;
            n = 4;
        }
        --n;
        const uint32_t r = w3;   // the words in the order w3, w2, w1, w0
        w3 = w2; w2 = w1; w1 = w0;
        return u01f(r);
    }
};

// ------------------------------------------------------------ tallies ----
__device__ __forceinline__ void add128(unsigned long long* lo, unsigned long long v) {
    if (v == 0ull) return;
    unsigned long long old = atomicAdd(lo, v);
    if (old + v < old) atomicAdd(lo + 1, 1ull);
}
// shared partial; moves to the 128-bit global accumulator before it can overflow
__device__ __forceinline__ void sadd(unsigned long long* s, unsigned long long v, unsigned long long* g) {
    if (v == 0ull) return;
    unsigned long long old = atomicAdd(s, v);
    if (old + v >= MFG_SMEM_FLUSH) {
        unsigned long long x = atomicExch(s, 0ull);
        add128(g, x);
    }
}
__device__ __forceinline__ unsigned long long qd(double x, double scale) {
    double y = x * scale;
    y = fmin(y, MFG_Q_MAX);
    return (unsigned long long)__double2ll_rn(y);
}
__device__ __forceinline__ unsigned long long qf(float x, float scale) {
    float y = fminf(x * scale, 1.125899907e15f);
    return (unsigned long long)__float2ll_rn(y);
}

// ------------------------------------------------------- moment lookup --
// Calls f(m) for every moment block m>=1 whose window [start,end) holds t.
template <class F>
__device__ __forceinline__ void for_moments(const DevModel& M, double t, F f) {
    if (M.nm == 0) return;
    int lo = 0;   // first start > t
    if (M.mguide) {   // guide entry one bucket low (a lower bound), then forward steps
        if (t > M.mg_t0) {
            int b = (int)((log2f((float)t) - M.mg_l0) * M.mg_scale) - 1;
            b = min(max(b, 0), M.mg_n - 1);
            lo = M.mguide[b];
        }
        while (lo < M.nm && M.mstart[lo] <= t) ++lo;
    } else {
        int hi = M.nm;
        while (lo < hi) { int mid = (lo + hi) >> 1; if (M.mstart[mid] <= t) lo = mid + 1; else hi = mid; }
    }
    for (int k = lo - 1; k >= 0 && M.mstart[k] > t - M.maxwin - 1e-300; --k)
        if (M.mstart[k] <= t && t < M.mend[k]) f(k + 1);
}

// ------------------------------------------------------ interpolation ---
// InterpolateX over an increasing table (value at y), extrapolating the end segments
__device__ __forceinline__ double interp_x_d(double y, const double* xs, const double* ys, int n) {
    if (n == 1) return xs[0];
    int lo = 0, hi = n;
    while (lo < hi) { int mid = (lo + hi) >> 1; if (ys[mid] <= y) lo = mid + 1; else hi = mid; }
    int i = lo - 1;
    if (i < 0) i = 0;
    if (i > n - 2) i = n - 2;
    double y0 = ys[i], y1 = ys[i + 1];
    double w = (y - y0) / (y1 - y0);
    return xs[i] + (xs[i + 1] - xs[i]) * w;
}
// The same interval search started from a guide table: g[b] = number of ys <= b / MFG_GUIDE_N,
// so that y in bucket b starts next to its interval and one or two steps find the index the
// binary search finds (any start gives the same index, as ys is non-decreasing).
#define MFG_GUIDE_N 128
__device__ __forceinline__ float interp_x_guided(float y, const float* xs, const float* ys, const unsigned char* g, int n) {
    int b = (int)(y * (float)MFG_GUIDE_N);
    b = min(max(b, 0), MFG_GUIDE_N - 1);
    int lo = g[b];
    while (lo > 0 && ys[lo - 1] > y) --lo;
    while (lo < n && ys[lo] <= y) ++lo;
    int i = lo - 1;
    if (i < 0) i = 0;
    if (i > n - 2) i = n - 2;
    float w = (y - ys[i]) / (ys[i + 1] - ys[i]);
    return xs[i] + (xs[i + 1] - xs[i]) * w;
}
__device__ __forceinline__ float interp_x_f(float y, const float* xs, const float* ys, int n) {
    int lo = 0, hi = n;
    while (lo < hi) { int mid = (lo + hi) >> 1; if (ys[mid] <= y) lo = mid + 1; else hi = mid; }
    int i = lo - 1;
    if (i < 0) i = 0;
    if (i > n - 2) i = n - 2;
    float w = (y - ys[i]) / (ys[i + 1] - ys[i]);
    return xs[i] + (xs[i + 1] - xs[i]) * w;
}
}  // namespace mfgk

#include "traversal.cuh"
#include "anglemap_gen.cuh"

namespace mfgk {

// ------------------------------------------------------- block tallies --
struct BlockTally {
    unsigned long long* sfac;   // shared [nf*SF_N] or nullptr
    unsigned long long* sglob;  // shared [TG_N]
};


// facet counter for moment block 0 (shared when available) and time moments (global)
__device__ __forceinline__ void facet_add(const DevModel& M, const DevTally& T, const BlockTally& B, int f, int m,
                                          unsigned long long hits, unsigned long long des, unsigned long long abs_,
                                          unsigned long long s1ov, unsigned long long svort, unsigned long long s1v) {
    unsigned long long* g = T.facet + ((size_t)m * M.nf + f) * TF_N;
    if (m == 0 && B.sfac) {
        unsigned long long* s = B.sfac + (size_t)f * SF_N;
        if (hits) atomicAdd(s + SF_HITS, hits);
        if (des) atomicAdd(s + SF_DES, des);
        if (abs_) atomicAdd(s + SF_ABS, abs_);
        sadd(s + SF_S1OV, s1ov, g + TF_S1OV);
        sadd(s + SF_SVORT, svort, g + TF_SVORT);
        sadd(s + SF_S1V, s1v, g + TF_S1V);
    } else {
        if (hits) atomicAdd(g + TF_HITS, hits);
        if (des) atomicAdd(g + TF_DES, des);
        if (abs_) atomicAdd(g + TF_ABS, abs_);
        add128(g + TF_S1OV, s1ov);
        add128(g + TF_SVORT, svort);
        add128(g + TF_S1V, s1v);
    }
}
__device__ __forceinline__ void cell_add(unsigned long long* g, unsigned long long cnt, unsigned long long s1ov,
                                         unsigned long long svort) {
    if (cnt) atomicAdd(g + TT_COUNT, cnt);
    add128(g + TT_S1OV, s1ov);
    add128(g + TT_SVORT, svort);
}

// ------------------------------------------------ the persistent kernel --
template <bool kFP32>
struct Real_ {
    typedef double T;
};
template <>
struct Real_<true> {
    typedef float T;
};

struct ParticleState {
    double ox, oy, oz;
    double time, decay_at;
    uint64_t bounces;      // trace steps since desorption (reflections and link passes)
    int last, structure;
    // extended variants: flight distance (cm), desorption time and reflections since desorption,
    // and the low-flux weight (oriRatio)
    double dist, gen_time;
    uint64_t refl;
    double ori;
    double scat_at;        // flight distance (cm) of the next background-gas collision
    int tele_from;         // teleportedFrom: destination of the last teleport, -1 none
};

// ProfileFacet (Particle.cpp:1026-1085); profiles are tallied in global memory
// profile bin of a hit: -1 when outside; `full` for U/V profiles, which also take the sums
__device__ __forceinline__ int profile_bin(const DevModel& M, int f, bool count_hit, double cosn, double vel, double u,
                                           double v, bool& full) {
    const int pt = M.info[f].profile_type;
    full = false;
    if (count_hit && pt == MFG_PROFILE_ANGULAR) {
        double th = acos(fmin(cosn, 1.0));
        int pos = (int)(th / (kPi / 2) * (double)MFG_PROFILE_SIZE);
        return min(max(pos, 0), MFG_PROFILE_SIZE - 1);
    } else if (pt == MFG_PROFILE_U || pt == MFG_PROFILE_V) {
        double x = (pt == MFG_PROFILE_U ? u : v) * (double)MFG_PROFILE_SIZE;
        if (!(x >= 0.0) || x >= (double)MFG_PROFILE_SIZE) return -1;
        full = true;
        return (int)x;
    } else if (count_hit && pt >= MFG_PROFILE_VELOCITY && pt <= MFG_PROFILE_TAN_VELOCITY) {
        double dd = (pt == MFG_PROFILE_VELOCITY) ? 1.0 : (pt == MFG_PROFILE_ORT_VELOCITY ? cosn : sqrt(fmax(0.0, 1.0 - cosn * cosn)));
        double x = dd * vel / M.info2[f].max_speed * (double)MFG_PROFILE_SIZE;
        if (!(x >= 0.0) || x >= (double)MFG_PROFILE_SIZE) return -1;
        return (int)x;
    }
    return -1;
}
// Profile tally: inlined at the moment-0 call sites of the kernel (+4 % on the tube, +5 % on the
// 100-moment tube), a called function inside the moment loop (inlined there too, the 100-moment
// tube ran 17 % slower)
__device__ __forceinline__ void profile_add_i(const DevModel& M, const DevTally& T, int f, int m, bool count_hit,
                                            unsigned long long vfac, unsigned long long ofac, double cosn, double vel,
                                            double u, double v, unsigned long long q1, unsigned long long q2) {
    bool full;
    const int pos = profile_bin(M, f, count_hit, cosn, vel, u, v, full);
    if (pos < 0) return;
    unsigned long long* g = T.profile + (((size_t)m * M.profile_facets + M.info[f].prof_idx) * MFG_PROFILE_SIZE + pos) * TT_N;
    if (count_hit) atomicAdd(g + TT_COUNT, 1ull);
    if (full) {
        add128(g + TT_S1OV, vfac * q1);
        add128(g + TT_SVORT, ofac * q2);
    }
}
__device__ __noinline__ void profile_add(const DevModel& M, const DevTally& T, int f, int m, bool count_hit,
                                            unsigned long long vfac, unsigned long long ofac, double cosn, double vel,
                                            double u, double v, unsigned long long q1, unsigned long long q2) {
    profile_add_i(M, T, f, m, count_hit, vfac, ofac, cosn, vel, u, v, q1, q2);
}

// Low-flux mode (Particle.cpp:338-356): the counters keep Monte Carlo counts; the weighted
// ("equivalent") counts of one tally event go to FP64 arrays, in moment 0 and every window
// holding `time`: facet nbHitEquiv/nbAbsEquiv (he, ae), texture countEquiv (cell, cw), profile
// countEquiv (pw), and the global nbHitEquiv/nbAbsEquiv (ghe, gae)
__device__ __noinline__ void lf_counts(const DevModel& M, const DevTally& T, int f, double time, double he, double ae,
                                       int cell, double cw, double pw, double cosn, double vel, double u, double v,
                                       double ghe, double gae) {
    if (ghe != 0.0) atomicAdd(T.lf_glob, ghe);
    if (gae != 0.0) atomicAdd(T.lf_glob + 1, gae);
    bool full = false;
    const int pos = (pw != 0.0 && (M.info[f].flags & FF_PROFILE)) ? profile_bin(M, f, true, cosn, vel, u, v, full) : -1;
    auto add = [&](int m) {
        double* fc = T.lf_facet + ((size_t)m * M.nf + f) * 2;
        if (he != 0.0) atomicAdd(fc, he);
        if (ae != 0.0) atomicAdd(fc + 1, ae);
        if (cell >= 0 && cw != 0.0) atomicAdd(T.lf_tex + (size_t)m * M.texture_cells + cell, cw);
        if (pos >= 0)
            atomicAdd(T.lf_prof + ((size_t)m * M.profile_facets + M.info[f].prof_idx) * MFG_PROFILE_SIZE + pos, pw);
    };
    add(0);
    for_moments(M, time, add);
}

// RecordAngleMap (Particle.cpp:1104-1136): incident (theta, phi) histogram, not time resolved
__device__ __forceinline__ void anglemap_add(const DevModel& M, const DevTally& T, int f, double dx, double dy, double dz) {
    const FacetInfo& In = M.info[f];
    const FacetInfo2& I2 = M.info2[f];
    const FacetIsectD& R = M.isect_d[f];
    const FacetPhysD& Ph = M.phys_d[f];
    double dn = dx * R.v[0] + dy * R.v[1] + dz * R.v[2];
    double th = acos(fmin(fmax(dn, -1.0), 1.0));
    double ph = atan2(dx * Ph.nV[0] + dy * Ph.nV[1] + dz * Ph.nV[2], dx * Ph.nU[0] + dy * Ph.nU[1] + dz * Ph.nU[2]);
    if (th > kPi / 2.0) th = fabs(kPi - th);
    int ti;
    if (th < I2.am_limit) {
        if (I2.am_lo <= 0) return;
        ti = (int)(th / I2.am_limit * (double)I2.am_lo);
    } else {
        if (I2.am_hi <= 0) return;
        ti = I2.am_lo + (int)((th - I2.am_limit) / (kPi / 2.0 - I2.am_limit) * (double)I2.am_hi);
    }
    int pi = (int)((ph + 3.1415926) / (2.0 * kPi) * (double)I2.am_phi);
    ti = min(ti, I2.am_lo + I2.am_hi - 1);
    pi = min(max(pi, 0), I2.am_phi - 1);
    atomicAdd(T.anglemap + In.ang_off + (size_t)ti * I2.am_phi + pi, 1ull);
}

// Direction from the polar angles in the facet basis (PolarToCartesian contract):
// d = sin(th)cos(ph) nU + sin(th)sin(ph) nV + cos(th) N, N reversed when `flip`.
// FP64 evaluates theta = acos(ct) and sin/cos as the reference does; FP32 uses
// sin(th) = sqrt(1 - ct^2) and sincospi.
template <bool kFP32, class R>
__device__ __forceinline__ void polar_dir(const DevModel& M, int f, R ct, R r2, bool flip, R& dx, R& dy, R& dz) {
    R st, cp, sp;
    if (kFP32) {
        float c = (float)ct;
        st = (R)sqrtf(fmaxf(0.0f, 1.0f - c * c));
        float sf, cf;
        sincospif(2.0f * (float)r2, &sf, &cf);
        cp = (R)cf;
        sp = (R)sf;
        if (flip) ct = -ct;
        const FacetPhysF& Pf = M.phys_f[f];
        R u = st * cp, v = st * sp;
        dx = u * Pf.nU[0] + v * Pf.nV[0] + ct * Pf.N[0];
        dy = u * Pf.nU[1] + v * Pf.nV[1] + ct * Pf.N[1];
        dz = u * Pf.nU[2] + v * Pf.nV[2] + ct * Pf.N[2];
    } else {
        double th = acos((double)ct);
        double ph = (double)r2 * 2.0 * kPi;
        double s = sin(th), c = cos(th), sd, cd;
        sincos(ph, &sd, &cd);
        if (flip) c = -c;
        const FacetPhysD& Ph = M.phys_d[f];
        const FacetIsectD& Rr = M.isect_d[f];
        double u = s * cd, v = s * sd;
        dx = (R)(u * Ph.nU[0] + v * Ph.nV[0] + c * Rr.v[0]);
        dy = (R)(u * Ph.nU[1] + v * Ph.nV[1] + c * Rr.v[1]);
        dz = (R)(u * Ph.nU[2] + v * Ph.nV[2] + c * Rr.v[2]);
    }
}

// Desorption time from a facet's integrated desorption table (Physics.cpp:11-19)
__device__ __forceinline__ double desorption_time(const DevModel& M, int idt, double r) {
    int s = M.id_start[idt], e = M.id_start[idt + 1];
    return interp_x_d(r * M.id_cum[e - 1], M.id_t + s, M.id_cum + s, e - s);
}

// point-in-polygon in FP32 for start points (FP32R kernel).  A point within rounding distance of
// an edge is decided in FP64: a start point just outside its polygon would, on a source whose rim
// lies on the walls (a tube's inlet disk), start the particle outside the walls.
__device__ __forceinline__ bool in_facet_f(const DevModel& M, int f, float u, float v) {
    const PolyF P = M.poly_f[f];
    if (P.rin2 > 1e29f) return true;
    float du = (u - P.cu) * P.su, dv = (v - P.cv) * P.sv;
    float r2 = du * du + dv * dv;
    if (r2 < P.rin2) return true;
    if (r2 > P.rout2) return false;
    bool amb = false;
    const bool in = edge_inside_f(M, P, u, v, 4e-7f * fmaxf(P.su, P.sv), amb);
    return amb ? in_facet_d(M, f, (double)u, (double)v) : in;
}

// Start point of a desorption: uniform (u,v) in the bounding rectangle until inside the polygon,
// at most 1000 tries, else the facet centre (Particle.cpp:513-570).  With an outgassing map,
// (u,v) is uniform in the chosen cell (the last row and column of the grid may be partial) and
// the fallback is the cell's centre.  The point is formed in FP64.
template <bool kFP32, class Rng, class R>
__device__ __forceinline__ void start_point(const DevModel& M, int fo, int cell, Rng& rng, double& ox, double& oy,
                                         double& oz, R& pu, R& pv) {
    const FacetIsectD& Rr = M.isect_d[fo];
    const PolyD& PP = M.poly_d[fo];
    bool found = false;
    double su = 0.5, sv = 0.5;
    int cw = 0, ch = 0;
    double wp = 1.0, hp = 1.0, lu = 1.0, lv = 1.0;
    if (cell >= 0) {
        const OgDev g = M.og[fo];
        ch = cell / g.w;
        cw = cell - ch * g.w;
        wp = g.wp;
        hp = g.hp;
        lu = cw < g.w - 1 ? 1.0 : g.wp - (g.w - 1.0);
        lv = ch < g.h - 1 ? 1.0 : g.hp - (g.h - 1.0);
        su = (cw + 0.5) / wp;
        sv = (ch + 0.5) / hp;
    }
    for (int tr = 0; tr < 1000 && !found; ++tr) {
        R u, v;
        if (cell >= 0) {
            const double ru = (double)rng.next(), rv = (double)rng.next();
            u = (R)((cw + ru * lu) / wp);
            v = (R)((ch + rv * lv) / hp);
        } else {
            u = (R)rng.next();
            v = (R)rng.next();
        }
        bool in = kFP32 ? in_facet_f(M, fo, (float)u, (float)v) : in_facet_d(M, fo, (double)u, (double)v);
        if (in) { su = (double)u; sv = (double)v; found = true; }
    }
    if (found || cell >= 0) {
        double a = su * PP.su * PP.su, b = sv * PP.sv * PP.sv;   // O + u*U + v*V (record keeps U/|U|^2)
        ox = Rr.v[4] + a * Rr.v[8] + b * Rr.v[12];
        oy = Rr.v[5] + a * Rr.v[9] + b * Rr.v[13];
        oz = Rr.v[6] + a * Rr.v[10] + b * Rr.v[14];
    } else {
        ox = M.center[3 * fo];
        oy = M.center[3 * fo + 1];
        oz = M.center[3 * fo + 2];
    }
    pu = (R)su;
    pv = (R)sv;
}

// texture cell index floor(u*w) + floor(v*h)*width of a facet (RecordHitOnTexture, Particle.cpp:981-983)
template <bool kFP32, class R>
__device__ __forceinline__ int texture_cell(const DevModel& M, int f, R u, R v) {
    const FacetInfo& In = M.info[f];
    if (In.tex_off < 0) return -1;
    int tu, tv;
    if (kFP32) { tu = (int)((float)u * M.phys_f[f].texw_p); tv = (int)((float)v * M.phys_f[f].texh_p); }
    else { tu = (int)((double)u * M.phys_d[f].texw_p); tv = (int)((double)v * M.phys_d[f].texh_p); }
    tu = min(max(tu, 0), In.tex_w - 1);
    tv = min(max(tv, 0), In.tex_h - 1);
    return In.tex_off + tu + tv * In.tex_w;
}

// RecordDirectionVector (Particle.cpp:1006-1023): Sum of v*direction and a count per cell,
// constant flow and every moment window holding t
// Particle logger (LogHit, Particle.cpp:1088-1102): an event on the logged facet takes the next
// record (u, v, theta and phi of the direction to the facet basis, oriRatio, expected decay
// moment, time, speed) while records are left
__device__ __noinline__ void log_hit(const DevModel& M, const DevTally& T, int f, double u, double v, double dx,
                                     double dy, double dz, double w, double decay_at, double time, double vel) {
    if (f != M.log_facet) return;
    const unsigned long long k = atomicAdd(T.plog_n, 1ull);
    if (k >= M.log_cap) return;
    const FacetPhysD& Ph = M.phys_d[f];
    const double* N = M.isect_d[f].v;
    const double cu = dx * Ph.nU[0] + dy * Ph.nU[1] + dz * Ph.nU[2];
    const double cv = dx * Ph.nV[0] + dy * Ph.nV[1] + dz * Ph.nV[2];
    const double cn = fmin(1.0, fmax(-1.0, dx * N[0] + dy * N[1] + dz * N[2]));
    double* r = T.plog + k * MFG_LOG_N;
    r[0] = u; r[1] = v; r[2] = acos(cn); r[3] = atan2(cv, cu);
    r[4] = w; r[5] = decay_at; r[6] = time; r[7] = vel;
}

// Force measurement (IncreaseFacetCounter, Particle.cpp:1208-1212): the momentum sgn*v*d of the
// particle onto facet f (sgn = -1 for a particle leaving it), its componentwise squares and its
// torque about the reference point, weighted by w (oriRatio), in moment 0 and every moment
// window holding `time`; FP64 atomics
__device__ __noinline__ void force_add(const DevModel& M, const DevTally& T, int f, double time, double w, double sgn,
                                       double vel, double dx, double dy, double dz, double ox, double oy, double oz) {
    const double px = sgn * vel * dx, py = sgn * vel * dy, pz = sgn * vel * dz;
    const double rx = ox - M.torque_ref[0], ry = oy - M.torque_ref[1], rz = oz - M.torque_ref[2];
    const double q[9] = {w * px, w * py, w * pz, w * px * px, w * py * py, w * pz * pz,
                         w * (ry * pz - rz * py), w * (rz * px - rx * pz), w * (rx * py - ry * px)};
    auto add = [&](int m) {
        double* b = T.force + ((size_t)m * M.nf + f) * 9;
#pragma unroll
        for (int j = 0; j < 9; ++j) atomicAdd(b + j, q[j]);
    };
    add(0);
    if (M.nm) for_moments(M, time, add);
}

__device__ __noinline__ void direction_add(const DevModel& M, const DevTally& T, int f, double u, double v, double time,
                                           double vx, double vy, double vz) {
    const FacetInfo& In = M.info[f];
    const int off = M.info2[f].dir_off;
    if (off < 0) return;
    int tu = (int)(u * M.phys_d[f].texw_p), tv = (int)(v * M.phys_d[f].texh_p);
    tu = min(max(tu, 0), In.tex_w - 1);
    tv = min(max(tv, 0), In.tex_h - 1);
    const size_t c = (size_t)off + tu + (size_t)tv * In.tex_w;
    auto add = [&](int m) {
        const size_t k = (size_t)m * M.direction_cells + c;
        atomicAdd(T.direction + 3 * k, vx);
        atomicAdd(T.direction + 3 * k + 1, vy);
        atomicAdd(T.direction + 3 * k + 2, vz);
        atomicAdd(T.dir_count + k, 1ull);
    };
    add(0);
    for_moments(M, time, add);
}

// Time-moment tallies of one event (moments >= 1): facet counter, texture cell, profile.  Inlined:
// as a called function its twenty arguments went through local memory (+8 % hits/s on the
// 100-moment tube, +1.5 % on the beam chamber, +1 % on the tube).
__device__ __forceinline__ void tally_moments(const DevModel& M, const DevTally& T, const BlockTally& B, int f, double time,
                                           unsigned long long des, unsigned long long hits, unsigned long long abs_,
                                           unsigned long long s1ov, unsigned long long svort, unsigned long long s1v,
                                           int cell, unsigned long long cell_count, unsigned long long cell_s1ov,
                                           unsigned long long cell_svort, bool count_hit,
                                           unsigned long long vf, unsigned long long of, double cosn, double vel,
                                           double u, double v, unsigned long long q1, unsigned long long q2) {
    const bool prof = (M.info[f].flags & FF_PROFILE) != 0;
    for_moments(M, time, [&](int m) {
        facet_add(M, T, B, f, m, hits, des, abs_, s1ov, svort, s1v);
        if (cell >= 0) cell_add(T.texture + ((size_t)m * M.texture_cells + cell) * TT_N, cell_count, cell_s1ov, cell_svort);
        if (prof) profile_add(M, T, f, m, count_hit, vf, of, cosn, vel, u, v, q1, q2);
    });
}

// RecordHistograms (Particle.cpp:926-975): bounces, flight distance and flight time of an
// absorbed particle, in moment 0 and every moment window holding the absorption time
__device__ __forceinline__ void hist_add(const HistDev& h, double* block, uint64_t refl, double dist, double flight,
                                         double w) {
    if (h.off < 0) return;
    double* b = block + h.off;
    if (h.nb) {
        uint64_t k = refl / h.bounce_bin;
        if (k > (uint64_t)(h.nb - 1)) k = (uint64_t)(h.nb - 1);
        atomicAdd(b + k, w);
        b += h.nb;
    }
    if (h.nd) {
        unsigned long long k = (unsigned long long)(dist / h.dist_bin);
        if (k > (unsigned long long)(h.nd - 1)) k = (unsigned long long)(h.nd - 1);
        atomicAdd(b + k, w);
        b += h.nd;
    }
    if (h.nt) {
        unsigned long long k = (unsigned long long)(flight / h.time_bin);
        if (k > (unsigned long long)(h.nt - 1)) k = (unsigned long long)(h.nt - 1);
        atomicAdd(b + k, w);
    }
}
__device__ __noinline__ void record_histograms(const DevModel& M, const DevTally& T, int f, double time, uint64_t refl,
                                               double dist, double gen_time, double w) {
    const double flight = time - gen_time;
    auto add = [&](int m) {
        double* block = T.histogram + (size_t)m * M.hist_bins;
        hist_add(M.ghist, block, refl, dist, flight, w);
        if (M.fhist) hist_add(M.fhist[f], block, refl, dist, flight, w);
    };
    add(0);
    for_moments(M, time, add);
}

// TreatMovingFacet (Physics.cpp:25-39): the moving facet's local velocity (m/s; translation,
// or rotation about the axis through mv1, position in cm) is added to the particle's
template <class R>
__device__ __noinline__ void treat_moving(const DevModel& M, double ox, double oy, double oz, R& dx, R& dy, R& dz, R& vel) {
    double ax = 0.0, ay = 0.0, az = 0.0;
    if (M.motion_type == 1) {
        ax = M.mv2[0]; ay = M.mv2[1]; az = M.mv2[2];
    } else if (M.motion_type == 2) {
        const double rx = 0.01 * (ox - M.mv1[0]), ry = 0.01 * (oy - M.mv1[1]), rz = 0.01 * (oz - M.mv1[2]);
        ax = M.mv2[1] * rz - M.mv2[2] * ry;
        ay = M.mv2[2] * rx - M.mv2[0] * rz;
        az = M.mv2[0] * ry - M.mv2[1] * rx;
    }
    const double v = (double)vel;
    const double wx = (double)dx * v + ax, wy = (double)dy * v + ay, wz = (double)dz * v + az;
    const double n = sqrt(wx * wx + wy * wy + wz * wz);
    dx = (R)(wx / n); dy = (R)(wy / n); dz = (R)(wz / n);
    vel = (R)n;
}

// PerformScatter (Particle.cpp:840-886, Physics.cpp:41-63): collision with a background-gas
// molecule at impact parameter b = rho sqrt(r); the direction turns by the scattering angle
// about an orthonormal base built on the old direction; returns false when the particle fell
// below the cutoff speed
template <class Rng, class R>
__device__ __noinline__ bool perform_scatter(const DevModel& M, Rng& rng, double dist, R& dx, R& dy, R& dz, R& vel,
                                             double& scat_at) {
    const double rho = M.sc_rho, mr = M.sc_mass_ratio;
    const double b = rho * sqrt((double)rng.next());
    const double a = sqrt(rho * rho - b * b);
    const double ctg = 1.0 / (2.0 * a * b) * (rho * rho * mr + b * b - a * a);
    const double theta = atan(1.0 / ctg);
    const double phi = 2.0 * kPi * (double)rng.next();
    const double d0 = (double)dx, d1 = (double)dy, d2 = (double)dz;
    double r0 = 1.0, r1 = 0.0, r2 = 0.0;
    if (d0 != 0.0) { r0 = 0.0; r2 = 1.0; }
    else if (d1 != 0.0) { r2 = 1.0; }
    double u0 = d1 * r2 - d2 * r1, u1 = d2 * r0 - d0 * r2, u2 = d0 * r1 - d1 * r0;
    double l = sqrt(u0 * u0 + u1 * u1 + u2 * u2);
    u0 /= l; u1 /= l; u2 /= l;
    double v0 = d1 * u2 - d2 * u1, v1 = d2 * u0 - d0 * u2, v2 = d0 * u1 - d1 * u0;
    l = sqrt(v0 * v0 + v1 * v1 + v2 * v2);
    v0 /= l; v1 /= l; v2 /= l;
    const double st = sin(theta), ct = cos(theta), sp = sin(phi), cp = cos(phi);
    dx = (R)(st * cp * u0 + st * sp * v0 + ct * d0);
    dy = (R)(st * cp * u1 + st * sp * v1 + ct * d1);
    dz = (R)(st * cp * u2 + st * sp * v2 + ct * d2);
    const double q = mr * rho / b * st;
    const double v = (double)vel;
    vel = (R)sqrt(v * v / (1.0 + q * q));
    scat_at = dist - M.sc_mfp * log(1.0 - (double)rng.next());
    return !(M.scatter_cutoff && (double)vel < M.sc_cutoff_speed);
}

// RegisterTransparentPass (Particle.cpp:1232-1257): crossing a transparent facet counts a hit
// whose 1/v_ort and v_ort sums are doubled (the particle crosses, it does not turn back), on
// the facet, its texture (countTrans), profile, direction cells and angle map, in the moment
// windows holding the crossing time.  Returns v_ort.
//
// A structure link (PerformBounce, Particle.cpp:698-724) is tallied the same way at t = 0, except
// that the facet counter gets no velocity sums (`link`).
// In low-flux mode the sums carry the particle's weight `w` and the equivalent counts go to the
// low-flux arrays.
template <bool kFP32, class R>
__device__ __noinline__ double transparent_pass(const DevModel& M, const DevTally& T, const BlockTally& B, int f,
                                                R t, R u, R v, double time, R vel, R dx, R dy, R dz,
                                                bool link = false, double w = 1.0) {
    const FacetInfo& In = M.info[f];
    R cosn;
    double tp;
    if (kFP32) {
        cosn = fabsf(dx * M.phys_f[f].N[0] + dy * M.phys_f[f].N[1] + dz * M.phys_f[f].N[2]);
        tp = time + (double)((float)t * (0.01f / (float)vel));
    } else {
        cosn = (R)fabs((double)dx * M.isect_d[f].v[0] + (double)dy * M.isect_d[f].v[1] + (double)dz * M.isect_d[f].v[2]);
        tp = time + (double)t / 100.0 / (double)vel;
    }
    R ort = vel * cosn;
    unsigned long long q1 = kFP32 ? qf((float)w * (1.0f / (float)ort), (float)MFG_SCALE_INV) : qd(w * (1.0 / (double)ort), MFG_SCALE_INV);
    unsigned long long q2 = kFP32 ? qf((float)w * (float)ort, (float)MFG_SCALE_V) : qd(w * (double)ort, MFG_SCALE_V);
    unsigned long long q3 = kFP32 ? qf((float)w * (1.0f / (float)vel), (float)MFG_SCALE_INV) : qd(w * (1.0 / (double)vel), MFG_SCALE_INV);
    const unsigned long long f1 = link ? 0ull : 2 * q1, f2 = link ? 0ull : 2 * q2;
    facet_add(M, T, B, f, 0, 1, 0, 0, f1, f2, q3);
    const int cell = (In.tex_off >= 0 && (In.count & MFG_COUNT_TRANS)) ? texture_cell<kFP32>(M, f, u, v) : -1;
    if (cell >= 0) cell_add(T.texture + (size_t)cell * TT_N, 1, 2 * q1, 2 * q2);
    if (In.count & MFG_COUNT_DIR)
        direction_add(M, T, f, (double)u, (double)v, tp, w * (double)dx * (double)vel, w * (double)dy * (double)vel,
                      w * (double)dz * (double)vel);
    if (T.lf_glob)
        lf_counts(M, T, f, tp, w, 0.0, cell, w, w, (double)cosn, (double)vel, (double)u, (double)v, link ? w : 0.0, 0.0);
    if (In.flags & FF_PROFILE) profile_add(M, T, f, 0, true, 2, 2, (double)cosn, (double)vel, (double)u, (double)v, q1, q2);
    if (In.flags & FF_ANGLEMAP) anglemap_add(M, T, f, (double)dx, (double)dy, (double)dz);
    if (M.nm)
        tally_moments(M, T, B, f, tp, 0, 1, 0, f1, f2, q3, cell, 1, 2 * q1, 2 * q2, true, 2, 2, (double)cosn,
                      (double)vel, (double)u, (double)v, q1, q2);
    return (double)ort;
}

// PerformTeleport (Particle.cpp:76-183), after the hit on facet f was recorded as a pass: the
// direction keeps its angles to the facet basis, now taken on the destination's basis (the polar
// round trip written as a projection), the particle starts at the same (u,v) on the destination,
// or, when that point is outside the destination polygon, at a uniform point of it (at most 1000
// draws: the reference's try counter never stops the loop, Particle.cpp:152-161).  The source's
// facet counter adds the velocity sums of the outgoing direction against its own normal.
template <bool kFP32, class Rng, class R>
__device__ __noinline__ void teleport_to(const DevModel& M, const DevTally& T, const BlockTally& B, int f, int dest,
                                         Rng& rng, double time, R vel, double u, double v, double& ox, double& oy,
                                         double& oz, R& dx, R& dy, R& dz) {
    const FacetPhysD& Pf = M.phys_d[f];
    const FacetPhysD& Pd = M.phys_d[dest];
    const double* Nf = M.isect_d[f].v;
    const double* Nd = M.isect_d[dest].v;
    const double ddx = (double)dx, ddy = (double)dy, ddz = (double)dz;
    const double a = ddx * Pf.nU[0] + ddy * Pf.nU[1] + ddz * Pf.nU[2];
    const double b = ddx * Pf.nV[0] + ddy * Pf.nV[1] + ddz * Pf.nV[2];
    const double c = ddx * Nf[0] + ddy * Nf[1] + ddz * Nf[2];
    const double ex = a * Pd.nU[0] + b * Pd.nV[0] + c * Nd[0];
    const double ey = a * Pd.nU[1] + b * Pd.nV[1] + c * Nd[1];
    const double ez = a * Pd.nU[2] + b * Pd.nV[2] + c * Nd[2];
    if (!in_facet_d(M, dest, u, v)) {
        for (int tr = 0; tr < 1000; ++tr) {
            const double u2 = (double)rng.next(), v2 = (double)rng.next();
            if (in_facet_d(M, dest, u2, v2)) { u = u2; v = v2; break; }
        }
    }
    const FacetIsectD& Rd = M.isect_d[dest];
    const PolyD& PD = M.poly_d[dest];
    const double ua = u * PD.su * PD.su, vb = v * PD.sv * PD.sv;   // O + u*U + v*V (record keeps U/|U|^2)
    ox = Rd.v[4] + ua * Rd.v[8] + vb * Rd.v[12];
    oy = Rd.v[5] + ua * Rd.v[9] + vb * Rd.v[13];
    oz = Rd.v[6] + ua * Rd.v[10] + vb * Rd.v[14];
    dx = (R)ex; dy = (R)ey; dz = (R)ez;
    const double ort = (double)vel * fabs(ex * Nf[0] + ey * Nf[1] + ez * Nf[2]);
    const unsigned long long q1 = qd(2.0 / ort, MFG_SCALE_INV), q2 = qd(2.0 * ort, MFG_SCALE_V);
    facet_add(M, T, B, f, 0, 0, 0, 0, q1, q2, 0);
    if (M.nm) for_moments(M, time, [&](int m) { facet_add(M, T, B, f, m, 0, 0, 0, q1, q2, 0); });
}

// General relaunch (any accommodation, temperature parameter, sojourn time, reflection
// mix): UpdateVelocity, sojourn, diffuse / specular / cos^N direction, with the random
// numbers drawn in the order of PerformBounce (Particle.cpp:769-802).  Inlined: +3 to +5 %
// hits/s on a 200k-facet chamber and on a 66-facet tube against a call (the register allocation
// of the whole loop, also where this law never runs).
template <bool kFP32, class Rng, class R>
__device__ __forceinline__ void reflect_general(const DevModel& M, int fo, bool flip, Rng& rng, double& time, R& vel,
                                                R& dx, R& dy, R& dz, const double* cv, const double* cp,
                                                const float* cvf, const float* cpf) {
    const FacetInfo& In = M.info[fo];
    const FacetPhysD& Ph = M.phys_d[fo];
    const FacetIsectD& Rr = M.isect_d[fo];
    double temp = (In.flags & FF_TEMP_PARAM) ? param_at(M, M.info2[fo].temp_param, time) : M.info2[fo].temperature;
    double sqT = (In.flags & FF_TEMP_PARAM) ? sqrt(temp) : Ph.sqrtT;
    if (Ph.accommodation > 0.9999) {
        if (M.use_maxwell) {
            if (kFP32) vel = (R)((float)sqT * interp_x_f((float)rng.next(), cvf, cpf, MFG_MAXWELL_N));
            else vel = (R)(sqT * interp_x_d((double)rng.next(), cv, cp, MFG_MAXWELL_N));
        } else {
            vel = (R)(145.469 * sqT / M.gas_mass);   // the reference's formula (Particle.cpp:1152)
        }
    } else {
        double o2 = (double)vel * (double)vel, n2;
        if (M.use_maxwell) {
            double v = sqT * interp_x_d((double)rng.next(), cv, cp, MFG_MAXWELL_N);
            n2 = v * v;
        } else {
            n2 = 29369.939 * (temp / M.gas_mass);
        }
        vel = (R)sqrt(o2 + (n2 - o2) * Ph.accommodation);
    }
    if (In.flags & FF_SOJOURN) {
        double A = exp(-Ph.soj_e / (8.31 * temp));
        time += -log(1.0 - (double)rng.next()) / (A * Ph.soj_freq);
    }
    int kind = 0;   // 0 diffuse, 1 specular, 2 cos^N
    if (!(In.flags & FF_DIFFUSE_ONLY)) {
        double rt = (double)rng.next();
        kind = (rt < Ph.diffuse) ? 0 : (rt < Ph.diffuse + Ph.specular ? 1 : 2);
    }
    if (kind == 1) {
        // mirror reflection: the normal component changes sign (Particle.cpp:790-794)
        double dn = (double)dx * Rr.v[0] + (double)dy * Rr.v[1] + (double)dz * Rr.v[2];
        dx = (R)((double)dx - 2.0 * dn * Rr.v[0]);
        dy = (R)((double)dy - 2.0 * dn * Rr.v[1]);
        dz = (R)((double)dz - 2.0 * dn * Rr.v[2]);
    } else {
        R r1 = (R)rng.next(), r2 = (R)rng.next();
        R ct = (kind == 2) ? (R)pow((double)r1, 1.0 / (Ph.cos_exp + 1.0)) : (R)sqrt(r1);
        polar_dir<kFP32>(M, fo, ct, r2, flip, dx, dy, dz);
    }
}

// output event of the sensitivity variant: y adds to output j, to the score sums of every
// earlier reflection on a parameter facet, and to the particle's source.  Inlined: as a called
// function it read the reflection list through generic loads and cost 26 % of the sensitivity
// kernel's time on the 1000-parameter tube (30.7 against 24.3 ms at 256 x 2; vectorised int4
// reads of the list measured slower still).
__device__ __forceinline__ void sens_output(const SensCtl& S, const int* traj, int ntraj, int src, int j, double y) {
    atomicAdd(S.Y + j, y);
    const int n = ntraj < MFG_SENS_TRAJ ? ntraj : MFG_SENS_TRAJ;
    for (int e = 0; e < n; ++e) atomicAdd(S.A + (size_t)traj[e] * MFG_SENS_NOUT + j, y);
    if (src >= 0) atomicAdd(S.Cs + (size_t)src * MFG_SENS_NOUT + j, y);
}

// stand-in for the pass list in variants built for models without transparent facets
struct NoTranspList {
    static constexpr int n = 0;
};

// kExt: variant for models with transparent facets or histograms (pass list, flight distance,
// desorption time and reflection count per particle)
// kTop: variant that reads the top BVH levels staged in shared memory (C.n_top nodes)
template <bool kFP32, int kMinBlocks, bool kSens = false, bool kExt = false, int kBlock = 256, bool kTop = false>
__global__ void __launch_bounds__(kBlock, kMinBlocks) trace_kernel(const __grid_constant__ DevModel M, DevTally T, LaunchCtl C) {
    typedef typename Real_<kFP32>::T R;
    extern __shared__ unsigned long long smem[];
    __shared__ double s_cdf_v[MFG_MAXWELL_N], s_cdf_p[MFG_MAXWELL_N];
    __shared__ float s_cdf_vf[MFG_MAXWELL_N], s_cdf_pf[MFG_MAXWELL_N];
    __shared__ unsigned char s_guide[MFG_GUIDE_N];
    BlockTally B;
    B.sglob = smem;
    B.sfac = C.smem_facets ? smem + TG_N : nullptr;
    const int nsm = TG_N + (C.smem_facets ? M.nf * SF_N : 0);
    for (int i = threadIdx.x; i < nsm; i += blockDim.x) smem[i] = 0ull;
    // top levels of the FP32 BVH (breadth-first NodeC records [0, n_top)), after the partials
    float4* s_top = reinterpret_cast<float4*>(smem + nsm);
    const int n_top = (kFP32 && kTop) ? C.n_top : 0;
    for (int i = threadIdx.x; i < 4 * n_top; i += blockDim.x)
        s_top[i] = __ldg(reinterpret_cast<const float4*>(M.nodes_c) + i);
    // the sensitivity variants (no staged nodes) stage their packed per-facet words after the partials
    int* s_ring = reinterpret_cast<int*>(s_top + 4 * n_top);
    const int* scodes = nullptr;
    if constexpr (kSens) {
        if (C.sens.smem_code) {
            for (int i = threadIdx.x; i < M.nf; i += blockDim.x) s_ring[i] = __ldg(C.sens.code + i);
            scodes = s_ring;
        } else {
            scodes = C.sens.code;
        }
    }
    // packed sensitivity word of a facet: parameter (bits 0-19, +1), gauge (20-23, +1), pump (24)
    auto scode = [&](int f) -> int { return kSens ? scodes[f] : 0; };
    for (int i = threadIdx.x; i < MFG_MAXWELL_N; i += blockDim.x) {
        s_cdf_v[i] = M.cdf_v[i];
        s_cdf_p[i] = M.cdf_p[i];
        s_cdf_vf[i] = (float)M.cdf_v[i];
        s_cdf_pf[i] = (float)M.cdf_p[i];
    }
    for (int b = threadIdx.x; b < MFG_GUIDE_N; b += blockDim.x) {
        const float yb = (float)b / (float)MFG_GUIDE_N;
        int c = 0;
        for (int i = 0; i < MFG_MAXWELL_N; ++i) c += ((float)M.cdf_p[i] <= yb) ? 1 : 0;
        s_guide[b] = (unsigned char)c;
    }
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const unsigned lane_lt = (1u << lane) - 1u;
    unsigned long long pool_next = 0, pool_end = 0;   // warp pool of particle ids
    const unsigned long long chunk = (unsigned long long)C.chunk;   // >= 32: one request serves a warp

    const unsigned long long n_total = C.run->n_total;
    const unsigned long long max_steps = C.run->max_steps;
    const int n_inst = C.run->n_inst;
    typename std::conditional<kFP32, RngF, RngD>::type rng;
    rng.k0 = C.run->key0;
    rng.k1 = C.run->key1;
    ParticleState P;
    P.ox = P.oy = P.oz = 0;
    P.time = 0;
    P.decay_at = 1e100;
    P.bounces = 0;
    P.last = -1;
    P.structure = 0;
    R dx = 0, dy = 0, dz = 0, vel = 1;
    R pu = 0, pv = 0;         // (u,v) on the current facet (facetHitDetails)
    bool active = true;       // lane still has particles to trace
    bool need_new = true;     // lane must desorb a new particle
    bool relink = false;      // lane crossed a structure link: trace on without a new direction
    // incoming half of the last reflection, added together with the outgoing half (moment 0)
    unsigned long long pend_s1ov = 0, pend_svort = 0, pend_s1v = 0;
    int pend_cell = -1;
    bool pend = false;
    unsigned iter = 0;
    int traj[kSens ? MFG_SENS_TRAJ : 1];   // parameters of this particle's reflections (sensitivity variant)
    int ntraj = 0, src_idx = -1;
    // per-thread global counters (no contended shared atomics on the hot path)
    unsigned long long c_hits = 0, c_des = 0, c_abs = 0, c_leak = 0, c_drop = 0, c_rechk = 0;
    unsigned long long c_dist = 0, c_distf = 0;
    unsigned long long deadline;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(deadline));
    deadline += C.run->time_limit_ns;

    auto flush_pending = [&]() {
        if (!pend) return;
        facet_add(M, T, B, P.last, 0, 1, 0, 0, pend_s1ov, pend_svort, pend_s1v);
        if (pend_cell >= 0) cell_add(T.texture + (size_t)pend_cell * TT_N, 1, pend_s1ov, pend_svort);
        pend = false;
        pend_cell = -1;
    };

    while (__any_sync(0xffffffffu, active)) {
        // ---- watchdog: kernel time limit and host abort word ----
        if ((++iter & 63u) == 0u) {
            int stop = 0;
            if (lane == 0) {
                unsigned long long now;
                asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
                if (now > deadline) { stop = 1; atomicOr(T.global + TG_STATUS, KS_TIMEOUT); }
                if (C.abort_flag && *C.abort_flag) { stop = 1; atomicOr(T.global + TG_STATUS, KS_ABORTED); }
            }
            stop = __shfl_sync(0xffffffffu, stop, 0);
            if (stop) {
                if (active) {
                    flush_pending();
                    if (!need_new) ++c_drop;
                }
                break;
            }
        }
        // ---- refill lanes that need a particle from the warp pool ----
        bool want = active && need_new;
        unsigned wmask = __ballot_sync(0xffffffffu, want);
        if (wmask) {
            unsigned n = __popc(wmask);
            unsigned rank = __popc(wmask & lane_lt);
            unsigned long long avail = pool_end - pool_next;
            if (avail < n) {
                unsigned long long base = 0;
                if (lane == 0) base = atomicAdd(C.next_particle, chunk);
                base = __shfl_sync(0xffffffffu, base, 0);
                unsigned long long mine = (rank < avail) ? pool_next + rank : base + (rank - avail);
                pool_next = base + (n - avail);
                pool_end = base + chunk;
                if (want) P.bounces = mine;   // temporary holder of the id
            } else {
                if (want) P.bounces = pool_next + rank;
                pool_next += n;
            }
            if (want && P.bounces >= n_total) { active = false; want = false; }
        }
        // lanes without a particle go on to the traversal too: they take part in its warp votes

        // ---- 1. emit: desorption (want) or reflection from P.last.  The two share the speed,
        //      direction and tally code; only short prologues differ.  Random numbers are drawn in
        //      the reference's order: desorption = source, [reverse], time, speed, [decay], (u,v)..., theta,
        //      phi (Particle.cpp:418-625); reflection = speed, [sojourn], [type], theta, phi (:769-802).
        if (active && !relink) {
            const bool des = want;
            int fo, law;              // law: 0 cosine, 1 uniform, 2 cos^N, 3 general reflection
            bool flip = false;
            bool amdes = false;   // extended variants: direction from the source's recorded angle map
            int ocell = -1;       // outgassing-map cell of the source (-1: uniform over the facet)
            R lexp = 0;
            if (des) {
                int inst = 0;
                if (n_inst > 1) {
                    int a = 0, b = n_inst;   // last instance whose prefix <= id
                    while (b - a > 1) { int mid = (a + b) >> 1; if (C.inst_prefix[mid] <= P.bounces) a = mid; else b = mid; }
                    inst = a;
                }
                rng.start(C.inst_first[inst] + (P.bounces - C.inst_prefix[inst]), (uint32_t)inst);
                // source facet by cumulative outgassing (Particle.cpp:418-464)
                const int sbase = M.inst_src_base[inst], scount = M.inst_src_count[inst];
                double sr = (double)rng.next() * M.inst_src_total[inst];
                int lo = 0, hi = scount;
                while (lo < hi) { int mid = (lo + hi) >> 1; if (M.src_cdf[sbase + mid] > sr) hi = mid; else lo = mid + 1; }
                if (lo >= scount) lo = scount - 1;
                lo += sbase;
                fo = M.src_facet[lo];
                if (M.src_cell) ocell = M.src_cell[lo];
                const FacetInfo2& I2 = M.info2[fo];
                if (M.info[fo].flags & FF_TWO_SIDED) flip = (double)rng.next() > 0.5;
                int idt = M.src_id[lo];
                if (idt >= 0) P.time = desorption_time(M, idt, (double)rng.next());
                else P.time = (double)rng.next() * M.latest;
                P.structure = I2.structure;
                P.bounces = 0;
                if constexpr (kExt) {
                    P.dist = 0.0;
                    P.gen_time = P.time;
                    P.refl = 0;
                    P.ori = 1.0;
                    P.tele_from = -1;
                }
                if (kSens) {
                    ntraj = 0;
                    src_idx = C.sens.src_of_facet[fo];
                    if (src_idx >= 0) atomicAdd(C.sens.src_count + src_idx, 1ull);
                }
                law = I2.desorb_type == MFG_DES_UNIFORM ? 1 : (I2.desorb_type == MFG_DES_COSINE_N ? 2 : 0);
                if constexpr (kExt) amdes = I2.desorb_type == MFG_DES_ANGLEMAP;
                lexp = (R)I2.desorb_exp;
                if (!M.use_maxwell) law |= 4;   // fixed speed 145.469 sqrt(T/m) (Particle.cpp:483)
            } else {
                fo = P.last;
                if (M.info[fo].flags & FF_TWO_SIDED) {
                    if (kFP32) {
                        const FacetPhysF& Pf = M.phys_f[fo];
                        flip = (dx * Pf.N[0] + dy * Pf.N[1] + dz * Pf.N[2]) > 0.0f;
                    } else {
                        const FacetIsectD& Rf = M.isect_d[fo];
                        flip = ((double)dx * Rf.v[0] + (double)dy * Rf.v[1] + (double)dz * Rf.v[2]) > 0.0;
                    }
                }
                law = (M.info[fo].flags & FF_FAST_REFL) ? 0 : 3;
            }
            // speed: Maxwell at the facet temperature (desorption and full-accommodation reflection)
            if (law < 3) {
                if (kFP32) vel = (R)(M.phys_f[fo].sqrtT * interp_x_guided((float)rng.next(), s_cdf_vf, s_cdf_pf, s_guide, MFG_MAXWELL_N));
                else vel = (R)(M.phys_d[fo].sqrtT * interp_x_d((double)rng.next(), s_cdf_v, s_cdf_p, MFG_MAXWELL_N));
            } else if (law & 4) {
                vel = (R)(145.469 * sqrt(M.info2[fo].temperature / M.gas_mass));
                law &= 3;
            }
            if (des) {
                P.decay_at = M.enable_decay ? P.time - 1.44269 * M.half_life * log(1.0 - (double)rng.next()) : 1e100;
                if constexpr (kExt) {
                    // free path to the first background-gas collision (Particle.cpp:500-504)
                    P.scat_at = M.scatter ? -M.sc_mfp * log(1.0 - (double)rng.next()) : 1e100;
                }
                // start point: rejection in the (u,v) rectangle, at most 1000 tries (Particle.cpp:513-570)
                start_point<kFP32>(M, fo, ocell, rng, P.ox, P.oy, P.oz, pu, pv);
                P.last = fo;
            }
            if (law == 3) {
                reflect_general<kFP32>(M, fo, flip, rng, P.time, vel, dx, dy, dz, s_cdf_v, s_cdf_p, s_cdf_vf, s_cdf_pf);
            } else if (amdes) {
                const double r1 = (double)rng.next(), r2 = (double)rng.next();
                double ax, ay, az;
                am_direction(M, fo, r1, r2, ax, ay, az);
                dx = (R)ax; dy = (R)ay; dz = (R)az;
            } else {
                R r1 = (R)rng.next(), r2 = (R)rng.next();
                R ct = law == 1 ? r1 : (law == 2 ? (R)pow((double)r1, 1.0 / ((double)lexp + 1.0)) : (R)sqrt(r1));
                polar_dir<kFP32>(M, fo, ct, r2, flip, dx, dy, dz);
            }
            if constexpr (kExt) {
                if (M.info[fo].flags & FF_MOVING) treat_moving(M, P.ox, P.oy, P.oz, dx, dy, dz, vel);
                if (M.force)   // desorbed particle onto its source, or reflected particle leaving the facet
                    force_add(M, T, fo, P.time, P.ori, des ? 1.0 : -1.0, (double)vel, (double)dx, (double)dy, (double)dz,
                              P.ox, P.oy, P.oz);
                if (des && M.log_facet >= 0)
                    log_hit(M, T, fo, (double)pu, (double)pv, (double)dx, (double)dy, (double)dz, P.ori, P.decay_at, P.time,
                            (double)vel);
            }
            {
                // outgoing tallies; a reflection's incoming half (pending) is added with them (moment 0)
                const FacetInfo& In = M.info[fo];
                R cosn;
                if (kFP32) cosn = fabsf(dx * M.phys_f[fo].N[0] + dy * M.phys_f[fo].N[1] + dz * M.phys_f[fo].N[2]);
                else cosn = (R)fabs((double)dx * M.isect_d[fo].v[0] + (double)dy * M.isect_d[fo].v[1] + (double)dz * M.isect_d[fo].v[2]);
                R ort = vel * cosn;
                double W = 1.0;   // low-flux weight of the outgoing half
                if constexpr (kExt) {
                    if (M.low_flux) W = P.ori;
                }
                unsigned long long q1 = kFP32 ? qf((float)W * (1.0f / (float)ort), (float)MFG_SCALE_INV) : qd(W * (1.0 / (double)ort), MFG_SCALE_INV);
                unsigned long long q2 = kFP32 ? qf((float)W * (float)ort, (float)MFG_SCALE_V) : qd(W * (double)ort, MFG_SCALE_V);
                unsigned long long q3 = 0;
                int cell = pend_cell;
                if (des) {
                    ++c_des;
                    q3 = kFP32 ? qf(1.0f / (float)vel, (float)MFG_SCALE_INV) : qd(1.0 / (double)vel, MFG_SCALE_INV);
                    cell = (In.count & MFG_COUNT_DES) ? texture_cell<kFP32>(M, fo, pu, pv) : -1;
                    if constexpr (kExt) {
                        if (M.low_flux && cell >= 0)
                            lf_counts(M, T, fo, P.time, 0.0, 0.0, cell, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0);
                    }
                }
                if (kSens && !des) {
                    const int g = ((scode(fo) >> 20) & 15) - 1;
                    if (g >= 0) sens_output(C.sens, traj, ntraj, src_idx, g, (double)ort);   // outgoing half at a gauge
                }
                const unsigned long long vf = des ? 2 : 1;   // velocity factor of the 1/v_ort sum
                const unsigned long long a1 = des ? 2 * q1 : pend_s1ov + q1;
                const unsigned long long a2 = des ? q2 : pend_svort + q2;
                const unsigned long long a3 = des ? q3 : pend_s1v;
                facet_add(M, T, B, fo, 0, des ? 0 : 1, des ? 1 : 0, 0, a1, a2, a3);
                if (cell >= 0) cell_add(T.texture + (size_t)cell * TT_N, 1, a1, a2);
                if (In.flags & FF_PROFILE) profile_add_i(M, T, fo, 0, false, vf, 1, (double)cosn, (double)vel, (double)pu, (double)pv, q1, q2);
                if (M.nm)
                    tally_moments(M, T, B, fo, P.time, des ? 1 : 0, 0, 0, vf * q1, q2, q3, cell, des ? 1 : 0, vf * q1, q2, false, vf, 1,
                                  (double)cosn, (double)vel, (double)pu, (double)pv, q1, q2);
                pend = false;
                pend_cell = -1;
                pend_s1ov = pend_svort = pend_s1v = 0;
                need_new = false;
            }
        }
        relink = false;

        // ---- 2. trace the ray ----
        int root = M.roots[P.structure];
        int hf;
        double ht;
        R hu, hv;
        const double ddx = (double)dx, ddy = (double)dy, ddz = (double)dz;
        // transparent and semi-transparent facets: passes of this ray, opacity draws keyed by
        // (particle, trace step, facet) in a stream of their own
        typename std::conditional<kExt, TranspList<R>, NoTranspList>::type tl;
        OpacCtx oc;
        TranspList<R>* tlp = nullptr;
        const OpacCtx* ocp = nullptr;
        if constexpr (kExt) {
            tl.clear((R)0);
            oc.k0 = rng.k0 ^ (rng.inst * 0x9E3779B9u);
            oc.k1 = rng.k1 ^ 0xA5A5A5A5u;
            oc.p0 = rng.p0;
            oc.p1 = rng.p1;
            oc.step = (uint32_t)P.bounces;
            oc.time = P.time;
            tlp = &tl;
            ocp = &oc;
        }
        if constexpr (kFP32) {
            bool amb = false;
            HitF h;
            {
                // Lockstep traversal: every lane of the warp visits one node or one leaf list per
                // step and the warp votes after each step, so the lanes stay converged (a lane
                // whose ray has finished waits at the vote instead of drifting into other code).
                // Measured against one traversal loop per lane: +48 % hits/s on the 200k-facet
                // beam chamber, +41 % on the tube.  Idle lanes take part in the votes.
                TravF tv;
                TravStack stk;
                if (active) trav_init(tv, stk, M.roots_c[P.structure], make_ray_f(P.ox, P.oy, P.oz, (float)dx, (float)dy, (float)dz), P.last);
                else tv.ref = kTrDone;
                // Node and leaf steps run in separate rounds: a lane that reaches a leaf list waits
                // until the lanes at leaves outnumber those at nodes three to one, then the leaf
                // lanes test their facets together (+26 % on C2, +15 % on C1 against mixed rounds;
                // ratios 1, 2, 3, 4 measured, 2 to 4 within 1 %).
                while (true) {
                    const bool live = tv.ref != kTrDone;
                    const bool node = live && tv.ref >= 0;
                    const unsigned mn = __ballot_sync(0xffffffffu, node);
                    const unsigned ml = __ballot_sync(0xffffffffu, live && !node);
                    if ((mn | ml) == 0u) break;
                    const bool leaf_round = __popc(ml) > 3 * __popc(mn);
                    if (leaf_round ? (live && !node) : node) trav_step<kExt>(M, tv, stk, T.global + TG_STATUS, tlp, ocp, s_top, n_top);
                }
                if (!active) continue;
                h = tv.h;
                amb = tv.amb;
            }
            bool retrace = amb || h.f < 0;
            if constexpr (kExt) retrace = retrace || tl.over;   // more passes than the list: all rounds in FP64
            if (retrace) {
                ++c_rechk;
                if constexpr (kExt) tl.clear((R)0);
                HitD hd = trace_d<R, kExt>(M, root, P.ox, P.oy, P.oz, ddx, ddy, ddz, P.last, T.global + TG_STATUS, tlp,
                                          ocp);
                hf = hd.f; ht = hd.t; hu = (R)hd.u; hv = (R)hd.v;
            } else {
                hf = h.f;
                hu = h.u;
                hv = h.v;
                // distance to the FP64 plane of the hit facet: FP32 estimate + FP64 residual
                const FacetIsectD& Rh = M.isect_d[hf];
                double den = Rh.v[0] * ddx + Rh.v[1] * ddy + Rh.v[2] * ddz;
                double num = Rh.v[3] - (Rh.v[0] * P.ox + Rh.v[1] * P.oy + Rh.v[2] * P.oz);
                double r = num - (double)h.t * den;
                ht = (double)h.t + (double)((float)r / (float)den);
            }
        } else {
            // the FP64 traversal in lockstep as well: one node per lane and step, a warp vote after each
            TravD td;
            TravStack stk;
            if (active) travd_init(td, stk, root, P.ox, P.oy, P.oz, ddx, ddy, ddz, P.last);
            else td.node = kTrDoneD;
            while (__any_sync(0xffffffffu, td.node != kTrDoneD))
                if (td.node != kTrDoneD) travd_step<R, kExt>(M, td, stk, T.global + TG_STATUS, tlp, ocp);
            if (!active) continue;
            hf = td.h.f; ht = td.h.t; hu = (R)td.h.u; hv = (R)td.h.v;
        }
        if (hf < 0) {   // leak (Particle.cpp:387-392)
            ++c_leak;
            need_new = true;
            continue;
        }
        // ---- 3. volume events, move (Particle.cpp:257-313) ----
        double travel = ht;
        int event = 0;
        if (!M.constant_flow) {
            double dl = (double)vel * 100.0 * (M.latest - P.time);
            if (dl < travel) { travel = dl; event = 1; }
        }
        if (M.enable_decay) {
            double dd = (double)vel * 100.0 * (P.decay_at - P.time);
            if (dd < travel) { travel = dd; event = 2; }
        }
        if constexpr (kExt) {
            if (M.scatter) {   // background-gas collision (Particle.cpp:281-287)
                const double ds = P.scat_at - P.dist;
                if (ds < travel) { travel = ds; event = 3; }
            }
            while (true) {
                for (int k = 0; k < tl.n; ++k) {
                    if (!((double)tl.t[k] < travel)) continue;
                    double ort_t = transparent_pass<kFP32>(M, T, B, tl.f[k], tl.t[k], tl.u[k], tl.v[k], P.time, vel, dx, dy, dz);
                    if (kSens) {
                        const int g = ((scode(tl.f[k]) >> 20) & 15) - 1;
                        if (g >= 0) sens_output(C.sens, traj, ntraj, src_idx, g, 2.0 * ort_t);
                    }
                }
                if (!tl.over) break;
                // the ray crosses more transparent facets than the list holds: trace it again (FP64,
                // the same hard hit) for the passes beyond the farthest one taken
                const R cut = tl.farthest();
                if (!((double)cut < travel)) break;
                tl.clear(cut);
                trace_d<R, kExt>(M, root, P.ox, P.oy, P.oz, ddx, ddy, ddz, P.last, T.global + TG_STATUS, tlp, ocp);
            }
        }
        P.ox = P.ox + travel * ddx;
        P.oy = P.oy + travel * ddy;
        P.oz = P.oz + travel * ddz;
        if (kFP32) P.time += (double)((float)travel * (0.01f / (float)vel));   // cm -> m
        else P.time += travel / 100.0 / (double)vel;
        unsigned long long qdist = kFP32 ? qf((float)travel, (float)MFG_SCALE_DIST) : qd(travel, MFG_SCALE_DIST);
        c_dist += qdist;
        if constexpr (kExt) {
            if (event == 3) {   // PerformScatter: counted as a hit, then a new flight from here
                c_distf += qdist;
                P.dist += travel;
                ++c_hits;
                if (M.low_flux)
                    lf_counts(M, T, 0, P.time, 0.0, 0.0, -1, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, P.ori, 0.0);
                ++P.refl;
                if (!perform_scatter(M, rng, P.dist, dx, dy, dz, vel, P.scat_at)) { need_new = true; continue; }
                P.last = -1;
                relink = true;
                need_new = false;
                if (++P.bounces > max_steps) {
                    ++c_drop;
                    relink = false;
                    need_new = true;
                }
                continue;
            }
        }
        if (event != 0) { need_new = true; continue; }
        c_distf += qdist;
        if constexpr (kExt) P.dist += travel;
        // ---- 4. stick or reflect at facet hf (Particle.cpp:323-357) ----
        const FacetInfo& In = M.info[hf];
        if constexpr (!kExt) {
            // plain variants: stick or reflect (Particle.cpp:323-357), one tally path per hit
            bool absorb;
            R cosn;
            if (kFP32) {
                const float s = (In.flags & FF_STICK_PARAM) ? (float)param_at(M, M.info2[hf].stick_param, P.time) : M.phys_f[hf].sticking;
                absorb = (s == 1.0f) || (s > 0.0f && (float)rng.next() < s);
                cosn = fabsf(dx * M.phys_f[hf].N[0] + dy * M.phys_f[hf].N[1] + dz * M.phys_f[hf].N[2]);
            } else {
                const FacetIsectD& Rh = M.isect_d[hf];
                const double s = (In.flags & FF_STICK_PARAM) ? param_at(M, M.info2[hf].stick_param, P.time) : M.phys_d[hf].sticking;
                absorb = (s == 1.0) || (s > 0.0 && (double)rng.next() < s);
                cosn = (R)fabs(ddx * Rh.v[0] + ddy * Rh.v[1] + ddz * Rh.v[2]);
            }
            const R ort = vel * cosn;
            const unsigned long long q1 = kFP32 ? qf(1.0f / (float)ort, (float)MFG_SCALE_INV) : qd(1.0 / (double)ort, MFG_SCALE_INV);
            const unsigned long long q2 = kFP32 ? qf((float)ort, (float)MFG_SCALE_V) : qd((double)ort, MFG_SCALE_V);
            const unsigned long long q3 = kFP32 ? qf(1.0f / (float)vel, (float)MFG_SCALE_INV) : qd(1.0 / (double)vel, MFG_SCALE_INV);
            pu = hu;
            pv = hv;
            ++c_hits;
            if (!absorb && (In.flags & FF_LINK)) {
                // structure link (PerformBounce, Particle.cpp:698-724)
                transparent_pass<kFP32>(M, T, B, hf, (R)0, hu, hv, P.time, vel, dx, dy, dz, true);
                P.structure = M.info2[hf].link;
                relink = true;
                need_new = false;
                if (++P.bounces > max_steps) {
                    ++c_drop;
                    relink = false;
                    need_new = true;
                }
                continue;
            }
            const int cell = (In.tex_off >= 0 && (In.count & (absorb ? MFG_COUNT_ABS : MFG_COUNT_REFL))) ? texture_cell<kFP32>(M, hf, hu, hv) : -1;
            if (In.flags & FF_ANGLEMAP) anglemap_add(M, T, hf, ddx, ddy, ddz);
            if (In.count & MFG_COUNT_DIR)
                direction_add(M, T, hf, (double)hu, (double)hv, P.time, ddx * (double)vel, ddy * (double)vel, ddz * (double)vel);
            if (kSens) {
                const int code = scode(hf);
                const int g = ((code >> 20) & 15) - 1;
                if (g >= 0) sens_output(C.sens, traj, ntraj, src_idx, g, (double)ort);   // incoming half / absorption
                const int k = (code & 0xFFFFF) - 1;
                if (absorb) {
                    if ((code >> 24) & 1) {
                        sens_output(C.sens, traj, ntraj, src_idx, MFG_SENS_NOUT - 1, 1.0);
                        if (k >= 0) atomicAdd(C.sens.B + (size_t)k * MFG_SENS_NOUT + MFG_SENS_NOUT - 1, 1.0);
                    }
                } else if (k >= 0) {
                    if (ntraj < MFG_SENS_TRAJ) traj[ntraj++] = k;
                    else if (ntraj == MFG_SENS_TRAJ) { atomicAdd(C.sens.overflow, 1ull); ++ntraj; }
                }
            }
            if (absorb) {   // RecordAbsorb (Particle.cpp:888-924)
                ++c_abs;
                facet_add(M, T, B, hf, 0, 1, 0, 1, 2 * q1, q2, q3);
                if (cell >= 0) cell_add(T.texture + (size_t)cell * TT_N, 1, 2 * q1, q2);
                if (In.flags & FF_PROFILE) profile_add_i(M, T, hf, 0, true, 2, 1, (double)cosn, (double)vel, (double)hu, (double)hv, q1, q2);
                if (M.nm)
                    tally_moments(M, T, B, hf, P.time, 0, 1, 1, 2 * q1, q2, q3, cell, 1, 2 * q1, q2, true, 2, 1,
                                  (double)cosn, (double)vel, (double)hu, (double)hv, q1, q2);
                need_new = true;
            } else {        // incoming half of PerformBounce (Particle.cpp:735-767)
                if (In.flags & FF_PROFILE) profile_add_i(M, T, hf, 0, true, 1, 1, (double)cosn, (double)vel, (double)hu, (double)hv, q1, q2);
                if (M.nm)
                    tally_moments(M, T, B, hf, P.time, 0, 1, 0, q1, q2, q3, cell, 1, q1, q2, true, 1, 1,
                                  (double)cosn, (double)vel, (double)hu, (double)hv, q1, q2);
                P.last = hf;
                pend = true;
                pend_s1ov = q1;
                pend_svort = q2;
                pend_s1v = q3;
                pend_cell = cell;
                need_new = false;
                if (++P.bounces > max_steps) {   // step cap: count the hit, drop the particle
                    flush_pending();
                    ++c_drop;
                    need_new = true;
                }
            }
            continue;
        }
        if constexpr (kExt) {
            if (In.flags & FF_TELEPORT) {   // teleport instead of stick or reflect (Particle.cpp:326-329)
                const int tp = M.info2[hf].teleport;
                const int dest = tp == -1 ? P.tele_from : tp - 1;
                if (dest >= 0 && dest < M.nf) {
                    // recorded like a transparent pass with the incoming direction, one hit and no sums
                    transparent_pass<kFP32>(M, T, B, hf, (R)0, hu, hv, P.time, vel, dx, dy, dz, true);
                    if (M.log_facet >= 0)
                        log_hit(M, T, hf, (double)hu, (double)hv, ddx, ddy, ddz, P.ori, P.decay_at, P.time, (double)vel);
                    teleport_to<kFP32>(M, T, B, hf, dest, rng, P.time, vel, (double)hu, (double)hv, P.ox, P.oy, P.oz, dx,
                                       dy, dz);
                    P.structure = M.info2[dest].structure;
                    P.tele_from = dest;
                    P.last = dest;
                } else {
                    P.last = hf;    // no destination: the particle passes on through the facet
                }
                relink = true;
                need_new = false;
                if (++P.bounces > max_steps) {   // step cap
                    ++c_drop;
                    relink = false;
                    need_new = true;
                }
                continue;
            }
        }
        // sticking; the regular mode draws stick or reflect (Particle.cpp:323-336), low-flux mode
        // splits the particle into an absorbed part wa and a reflected part wr (:338-356)
        bool do_abs, do_refl;
        double wa = 1.0, wr = 1.0;
        R cosn;
        {
            const double s = (In.flags & FF_STICK_PARAM) ? param_at(M, M.info2[hf].stick_param, P.time)
                                                         : (kFP32 ? (double)M.phys_f[hf].sticking : M.phys_d[hf].sticking);
            bool lf = false;
            if constexpr (kExt) lf = M.low_flux != 0;
            if (lf) {
                if constexpr (kExt) {
                    do_abs = s > 0.0;
                    wa = P.ori * s;
                    P.ori = do_abs ? P.ori * (1.0 - s) : P.ori * (1.0 - s);
                    wr = P.ori;
                    do_refl = P.ori > M.low_flux_cutoff;
                }
            } else if (kFP32) {
                const float sf = (float)s;
                do_abs = (sf == 1.0f) || (sf > 0.0f && (float)rng.next() < sf);
                do_refl = !do_abs;
            } else {
                do_abs = (s == 1.0) || (s > 0.0 && (double)rng.next() < s);
                do_refl = !do_abs;
            }
            if (kFP32) cosn = fabsf(dx * M.phys_f[hf].N[0] + dy * M.phys_f[hf].N[1] + dz * M.phys_f[hf].N[2]);
            else cosn = (R)fabs(ddx * M.isect_d[hf].v[0] + ddy * M.isect_d[hf].v[1] + ddz * M.isect_d[hf].v[2]);
        }
        const R ort = vel * cosn;
        // fixed-point sums of one part of weight w: 1/v_ort, v_ort, 1/v
        auto quant = [&](double w, unsigned long long& q1, unsigned long long& q2, unsigned long long& q3) {
            if (kFP32) {
                q1 = qf((float)w * (1.0f / (float)ort), (float)MFG_SCALE_INV);
                q2 = qf((float)w * (float)ort, (float)MFG_SCALE_V);
                q3 = qf((float)w * (1.0f / (float)vel), (float)MFG_SCALE_INV);
            } else {
                q1 = qd(w * (1.0 / (double)ort), MFG_SCALE_INV);
                q2 = qd(w * (double)ort, MFG_SCALE_V);
                q3 = qd(w * (1.0 / (double)vel), MFG_SCALE_INV);
            }
        };
        pu = hu;
        pv = hv;
        c_hits += (do_abs ? 1 : 0) + (do_refl ? 1 : 0);
        if (kSens) {
            const int g = ((scode(hf) >> 20) & 15) - 1;
            if (g >= 0) sens_output(C.sens, traj, ntraj, src_idx, g, (double)ort);   // incoming half / absorption
        }
        if (do_abs) {   // RecordAbsorb (Particle.cpp:888-924)
            unsigned long long q1, q2, q3;
            quant(wa, q1, q2, q3);
            if constexpr (kExt) {
                if (M.force) force_add(M, T, hf, P.time, wa, 1.0, (double)vel, ddx, ddy, ddz, P.ox, P.oy, P.oz);
                if (M.log_facet >= 0) log_hit(M, T, hf, (double)hu, (double)hv, ddx, ddy, ddz, wa, P.decay_at, P.time, (double)vel);
            }
            ++c_abs;
            const int cell = (In.tex_off >= 0 && (In.count & MFG_COUNT_ABS)) ? texture_cell<kFP32>(M, hf, hu, hv) : -1;
            if (In.flags & FF_ANGLEMAP) anglemap_add(M, T, hf, ddx, ddy, ddz);
            if (In.count & MFG_COUNT_DIR)
                direction_add(M, T, hf, (double)hu, (double)hv, P.time, wa * ddx * (double)vel, wa * ddy * (double)vel,
                              wa * ddz * (double)vel);
            if (kSens) {
                const int code = scode(hf);
                const int k = (code & 0xFFFFF) - 1;
                if ((code >> 24) & 1) {
                    sens_output(C.sens, traj, ntraj, src_idx, MFG_SENS_NOUT - 1, 1.0);
                    if (k >= 0) atomicAdd(C.sens.B + (size_t)k * MFG_SENS_NOUT + MFG_SENS_NOUT - 1, 1.0);
                }
            }
            if constexpr (kExt) {
                if (M.hist_bins) record_histograms(M, T, hf, P.time, P.refl, P.dist, P.gen_time, wa);
                if (M.low_flux)
                    lf_counts(M, T, hf, P.time, wa, wa, cell, wa, wa, (double)cosn, (double)vel, (double)hu, (double)hv, wa, wa);
            }
            facet_add(M, T, B, hf, 0, 1, 0, 1, 2 * q1, q2, q3);
            if (cell >= 0) cell_add(T.texture + (size_t)cell * TT_N, 1, 2 * q1, q2);
            if (In.flags & FF_PROFILE) profile_add_i(M, T, hf, 0, true, 2, 1, (double)cosn, (double)vel, (double)hu, (double)hv, q1, q2);
            if (M.nm)
                tally_moments(M, T, B, hf, P.time, 0, 1, 1, 2 * q1, q2, q3, cell, 1, 2 * q1, q2, true, 2, 1,
                              (double)cosn, (double)vel, (double)hu, (double)hv, q1, q2);
        }
        if (!do_refl) {
            need_new = true;
            continue;
        }
        if (In.flags & FF_LINK) {
            // structure link: counted as a pass, the particle goes on into the linked structure
            // with its direction, speed and last-hit facet (PerformBounce, Particle.cpp:698-724)
            transparent_pass<kFP32>(M, T, B, hf, (R)0, hu, hv, P.time, vel, dx, dy, dz, true, wr);
            P.structure = M.info2[hf].link;
            if (In.flags & FF_MOVING) treat_moving(M, P.ox, P.oy, P.oz, dx, dy, dz, vel);
            if constexpr (kExt) {
                if (M.log_facet >= 0)
                    log_hit(M, T, hf, (double)hu, (double)hv, (double)dx, (double)dy, (double)dz, wr, P.decay_at, P.time,
                            (double)vel);
            }
            relink = true;
            need_new = false;
            if (++P.bounces > max_steps) {   // step cap
                ++c_drop;
                relink = false;
                need_new = true;
            }
            continue;
        }
        {   // incoming half of PerformBounce (Particle.cpp:735-767)
            unsigned long long q1, q2, q3;
            quant(wr, q1, q2, q3);
            if constexpr (kExt) {
                if (M.force) force_add(M, T, hf, P.time, wr, 1.0, (double)vel, ddx, ddy, ddz, P.ox, P.oy, P.oz);
                if (M.log_facet >= 0) log_hit(M, T, hf, (double)hu, (double)hv, ddx, ddy, ddz, wr, P.decay_at, P.time, (double)vel);
            }
            const int cell = (In.tex_off >= 0 && (In.count & MFG_COUNT_REFL)) ? texture_cell<kFP32>(M, hf, hu, hv) : -1;
            if (In.flags & FF_ANGLEMAP) anglemap_add(M, T, hf, ddx, ddy, ddz);
            if (In.count & MFG_COUNT_DIR)
                direction_add(M, T, hf, (double)hu, (double)hv, P.time, wr * ddx * (double)vel, wr * ddy * (double)vel,
                              wr * ddz * (double)vel);
            if (kSens) {
                const int k = (scode(hf) & 0xFFFFF) - 1;
                if (k >= 0) {
                    if (ntraj < MFG_SENS_TRAJ) traj[ntraj++] = k;
                    else if (ntraj == MFG_SENS_TRAJ) { atomicAdd(C.sens.overflow, 1ull); ++ntraj; }
                }
            }
            if constexpr (kExt) {
                if (M.low_flux)
                    lf_counts(M, T, hf, P.time, wr, 0.0, cell, wr, wr, (double)cosn, (double)vel, (double)hu, (double)hv, wr, 0.0);
            }
            if (In.flags & FF_PROFILE) profile_add_i(M, T, hf, 0, true, 1, 1, (double)cosn, (double)vel, (double)hu, (double)hv, q1, q2);
            if (M.nm)
                tally_moments(M, T, B, hf, P.time, 0, 1, 0, q1, q2, q3, cell, 1, q1, q2, true, 1, 1,
                              (double)cosn, (double)vel, (double)hu, (double)hv, q1, q2);
            P.last = hf;
            if constexpr (kExt) ++P.refl;
            pend = true;
            pend_s1ov = q1;
            pend_svort = q2;
            pend_s1v = q3;
            pend_cell = cell;
            need_new = false;
            if (++P.bounces > max_steps) {   // step cap: count the hit, drop the particle
                flush_pending();
                ++c_drop;
                need_new = true;
            }
        }
    }
    // ---- flush the per-thread counters, then the block partials ----
    if (c_hits) atomicAdd(B.sglob + TG_HITS, c_hits);
    if (c_des) atomicAdd(B.sglob + TG_DES, c_des);
    if (c_abs) atomicAdd(B.sglob + TG_ABS, c_abs);
    if (c_leak) atomicAdd(B.sglob + TG_LEAK, c_leak);
    if (c_drop) atomicAdd(B.sglob + TG_DROPPED, c_drop);
    if (c_rechk) atomicAdd(B.sglob + TG_RECHECK, c_rechk);
    sadd(B.sglob + TG_DIST_LO, c_dist, T.global + TG_DIST_LO);
    sadd(B.sglob + TG_DISTF_LO, c_distf, T.global + TG_DISTF_LO);
    __syncthreads();
    if (threadIdx.x < TG_N) {
        int i = threadIdx.x;
        unsigned long long v = B.sglob[i];
        if (i == TG_DIST_LO || i == TG_DISTF_LO) add128(T.global + i, v);
        else if (i != TG_DIST_HI && i != TG_DISTF_HI && i != TG_STATUS && v) atomicAdd(T.global + i, v);
    }
    if (B.sfac) {
        for (int i = threadIdx.x; i < M.nf * SF_N; i += blockDim.x) {
            unsigned long long v = B.sfac[i];
            if (!v) continue;
            int f = i / SF_N, k = i % SF_N;
            unsigned long long* g = T.facet + (size_t)f * TF_N;
            if (k == SF_HITS) atomicAdd(g + TF_HITS, v);
            else if (k == SF_DES) atomicAdd(g + TF_DES, v);
            else if (k == SF_ABS) atomicAdd(g + TF_ABS, v);
            else if (k == SF_S1OV) add128(g + TF_S1OV, v);
            else if (k == SF_SVORT) add128(g + TF_SVORT, v);
            else add128(g + TF_S1V, v);
        }
    }
}

// ------------------------------------------------------------ replay ----
// One ray per thread.  FP32R: the warp traverses its lanes' rays in lockstep (every lane takes
// part in the votes, also those past the end), then an ambiguous or missing hit goes to the FP64
// traversal.  256 threads, at least 4 blocks per SM (64 registers): the traversal alone runs
// without spills at that budget.
constexpr int kReplayBlock = 256;
__global__ void __launch_bounds__(kReplayBlock, 4) replay_kernel(const __grid_constant__ DevModel M, int precision,
                              long long n, const double* origin, const double* dir, const int* last, int* hit_f,
                              double* hit_t, unsigned long long* rechecks, unsigned long long* status) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = i < n;
    const int root = M.roots[0];
    const OpacCtx oc = replay_opacity();
    const OpacCtx* ocp = M.has_transparent ? &oc : nullptr;
    if (precision == 0) {
        if (!active) return;
        const double ox = origin[3 * i], oy = origin[3 * i + 1], oz = origin[3 * i + 2];
        const double dx = dir[3 * i], dy = dir[3 * i + 1], dz = dir[3 * i + 2];
        HitD h = trace_d<double>(M, root, ox, oy, oz, dx, dy, dz, last[i], status, nullptr, ocp);
        hit_f[i] = h.f;
        hit_t[i] = h.f >= 0 ? h.t : -1.0;
        return;
    }
    double ox = 0, oy = 0, oz = 0, dx = 1, dy = 0, dz = 0;
    int li = -1;
    if (active) {
        ox = origin[3 * i]; oy = origin[3 * i + 1]; oz = origin[3 * i + 2];
        dx = dir[3 * i]; dy = dir[3 * i + 1]; dz = dir[3 * i + 2];
        li = last[i];
    }
    bool amb = false;
    const HitF h = trace_f_lockstep(M, active, M.roots_c[0], make_ray_f(ox, oy, oz, (float)dx, (float)dy, (float)dz), li,
                                    amb, status, ocp);
    if (!active) return;
    if (amb || h.f < 0) {
        atomicAdd(rechecks, 1ull);
        HitD hd = trace_d<double>(M, root, ox, oy, oz, dx, dy, dz, li, status, nullptr, ocp);
        hit_f[i] = hd.f;
        hit_t[i] = hd.f >= 0 ? hd.t : -1.0;
    } else {
        const FacetIsectD& Rh = M.isect_d[h.f];
        double den = Rh.v[0] * dx + Rh.v[1] * dy + Rh.v[2] * dz;
        double num = Rh.v[3] - (Rh.v[0] * ox + Rh.v[1] * oy + Rh.v[2] * oz);
        double r = num - (double)h.t * den;
        hit_f[i] = h.f;
        hit_t[i] = (double)h.t + (double)((float)r / (float)den);
    }
}

}  // namespace mfgk
