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

namespace mfgk {

constexpr int kStack = 64;
constexpr double kPi = 3.14159265358979323846;

// ------------------------------------------------------------------ Philox --
__device__ __forceinline__ void philox4x32_10(uint32_t& c0, uint32_t& c1, uint32_t& c2, uint32_t& c3,
                                              uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}
__device__ __forceinline__ double u01d(uint32_t a, uint32_t b) {
    uint64_t m = ((((uint64_t)a) << 32) | b) >> 12;
    return __longlong_as_double((long long)(0x3FF0000000000000ull | m)) - 1.0;
}
// uniform float in (0,1): (k + 1/2) * 2^-23; never 0, so cos(theta) = sqrt(u) never
// gives a direction lying in the facet plane
__device__ __forceinline__ float u01f(uint32_t a) {
    return (__uint_as_float(0x3F800000u | (a >> 9)) - 1.0f) + 5.9604645e-8f;
}

// double stream: two uniforms per Philox block (the CPU oracle's order)
struct RngD {
    uint32_t p0, p1, ctr, k0, k1;
    bool have;
    double cache;
    __device__ void start(uint64_t pid) { p0 = (uint32_t)pid; p1 = (uint32_t)(pid >> 32); ctr = 0; have = false; }
    __device__ double next() {
        if (have) { have = false; return cache; }
        uint32_t c0 = p0, c1 = p1, c2 = ctr++, c3 = 0u;
        philox4x32_10(c0, c1, c2, c3, k0, k1);
        cache = u01d(c2, c3);
        have = true;
        return u01d(c0, c1);
    }
};
// float stream: four uniforms per Philox block
struct RngF {
    uint32_t p0, p1, ctr, k0, k1;
    uint32_t w[4];
    int n;
    __device__ void start(uint64_t pid) { p0 = (uint32_t)pid; p1 = (uint32_t)(pid >> 32); ctr = 0; n = 0; }
    __device__ float next() {
        if (n == 0) {
            uint32_t c0 = p0, c1 = p1, c2 = ctr++, c3 = 0u;
            philox4x32_10(c0, c1, c2, c3, k0, k1);
            w[0] = c0; w[1] = c1; w[2] = c2; w[3] = c3;
            n = 4;
        }
        return u01f(w[--n]);
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
    int lo = 0, hi = M.nm;   // first start > t
    while (lo < hi) { int mid = (lo + hi) >> 1; if (M.mstart[mid] <= t) lo = mid + 1; else hi = mid; }
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
__device__ __forceinline__ float interp_x_f(float y, const float* xs, const float* ys, int n) {
    int lo = 0, hi = n;
    while (lo < hi) { int mid = (lo + hi) >> 1; if (ys[mid] <= y) lo = mid + 1; else hi = mid; }
    int i = lo - 1;
    if (i < 0) i = 0;
    if (i > n - 2) i = n - 2;
    float w = (y - ys[i]) / (ys[i + 1] - ys[i]);
    return xs[i] + (xs[i + 1] - xs[i]) * w;
}
// InterpolateY (no extrapolation) for time-dependent parameters
__device__ double param_at(const DevModel& M, int p, double t) {
    int s = M.par_start[p], e = M.par_start[p + 1], n = e - s;
    const double* xs = M.par_t + s;
    const double* ys = M.par_v + s;
    if (n == 1) return ys[0];
    int lo = 0, hi = n;
    while (lo < hi) { int mid = (lo + hi) >> 1; if (xs[mid] <= t) lo = mid + 1; else hi = mid; }
    int i = lo - 1;
    if (i < 0) return ys[0];
    if (i >= n - 1) return ys[n - 1];
    bool lx = M.par_logx[p], ly = M.par_logy[p];
    double w = lx ? (log10(t) - log10(xs[i])) / (log10(xs[i + 1]) - log10(xs[i])) : (t - xs[i]) / (xs[i + 1] - xs[i]);
    if (ly) return exp10(log10(ys[i]) + (log10(ys[i + 1]) - log10(ys[i])) * w);
    return ys[i] + (ys[i + 1] - ys[i]) * w;
}

// -------------------------------------------------- point in polygon ----
__device__ __forceinline__ bool crossing_d(const double2* v2, int vs, int nv, double u, double v) {
    bool in = false;
    double2 pj = v2[vs + nv - 1];
    for (int i = 0; i < nv; ++i) {
        double2 pi = v2[vs + i];
        if ((pi.y > v) != (pj.y > v)) {
            double cr = (pj.x - pi.x) * (v - pi.y) - (u - pi.x) * (pj.y - pi.y);
            if ((cr > 0) == (pj.y > pi.y)) in = !in;
        }
        pj = pi;
    }
    return in;
}
__device__ __forceinline__ bool in_facet_d(const DevModel& M, int f, double u, double v) {
    const PolyD P = M.poly_d[f];
    double du = (u - P.cu) * P.su, dv = (v - P.cv) * P.sv;
    double r2 = du * du + dv * dv;
    if (r2 < P.rin2) return true;
    if (r2 > P.rout2) return false;
    return crossing_d(M.v2_d, P.vstart, P.nv, u, v);
}

// --------------------------------------------------------- FP64 trace ---
struct HitD {
    int f;
    double t, u, v;
};

// closest hard hit of the ray (skipping facet `last`); BVH of structure `root`
__device__ __noinline__ HitD trace_d(const DevModel& M, int root, double ox, double oy, double oz,
                                     double dx, double dy, double dz, int last, unsigned long long* status) {
    HitD h;
    h.f = -1;
    h.t = 1.0e99;
    h.u = h.v = 0;
    double ix = 1.0 / dx, iy = 1.0 / dy, iz = 1.0 / dz;
    int stack[kStack];
    int sp = 0;
    int node = root;
    while (true) {
        const NodeD nd = M.nodes_d[node];
        double tx0 = (nd.lo[0] - ox) * ix, tx1 = (nd.hi[0] - ox) * ix;
        double ty0 = (nd.lo[1] - oy) * iy, ty1 = (nd.hi[1] - oy) * iy;
        double tz0 = (nd.lo[2] - oz) * iz, tz1 = (nd.hi[2] - oz) * iz;
        double tmin = fmax(fmax(fmin(tx0, tx1), fmin(ty0, ty1)), fmax(fmin(tz0, tz1), 0.0));
        double tmax = fmin(fmin(fmax(tx0, tx1), fmax(ty0, ty1)), fmin(fmax(tz0, tz1), h.t));
        bool hit = tmin <= tmax;
        if (hit && nd.b >= 0) {
            int near = nd.a, far = nd.a + 1;
            double dax = nd.b == 0 ? dx : (nd.b == 1 ? dy : dz);
            if (dax < 0) { near = nd.a + 1; far = nd.a; }
            if (sp < kStack) stack[sp++] = far;
            else atomicOr(status, KS_STACK);
            node = near;
            continue;
        }
        if (hit) {
            int cnt = -1 - nd.b;
            for (int k = 0; k < cnt; ++k) {
                int f = M.prims[nd.a + k];
                if (f == last) continue;
                const FacetIsectD& R = M.isect_d[f];
                double Nx = R.v[0], Ny = R.v[1], Nz = R.v[2], D = R.v[3];
                double den = Nx * dx + Ny * dy + Nz * dz;
                bool two = (M.info[f].flags & FF_TWO_SIDED) != 0;
                if (!two && den >= 0.0) continue;
                if (den == 0.0) continue;
                double t = (D - (Nx * ox + Ny * oy + Nz * oz)) / den;
                if (!(t > 0.0) || t > h.t) continue;
                double px = ox + t * dx - R.v[4], py = oy + t * dy - R.v[5], pz = oz + t * dz - R.v[6];
                double u = px * R.v[8] + py * R.v[9] + pz * R.v[10];
                if (u < 0.0 || u > 1.0) continue;
                double v = px * R.v[12] + py * R.v[13] + pz * R.v[14];
                if (v < 0.0 || v > 1.0) continue;
                if (!in_facet_d(M, f, u, v)) continue;
                if (t < h.t || f < h.f) { h.f = f; h.t = t; h.u = u; h.v = v; }
            }
        }
        if (sp == 0) break;
        node = stack[--sp];
    }
    return h;
}

// --------------------------------------------------------- FP32 trace ---
// FP32 traversal with per-candidate error bounds.  Returns the hit and sets
// `ambiguous` when a candidate could be classified differently in exact
// arithmetic (near an edge, near the origin, or too close to the best hit).
struct HitF {
    int f;
    float t, u, v;
};

__device__ __forceinline__ bool edge_inside_f(const DevModel& M, const PolyF& P, float u, float v, float em,
                                              bool& amb) {
    // crossing test, plus ambiguity when the point is within em (cm) of an edge line
    bool in = false;
    float pu = u * P.su, pv = v * P.sv;
    float2 pj = M.v2_f[P.vstart + P.nv - 1];
    float pju = pj.x * P.su, pjv = pj.y * P.sv;
    for (int i = 0; i < P.nv; ++i) {
        float2 pi = M.v2_f[P.vstart + i];
        float piu = pi.x * P.su, piv = pi.y * P.sv;
        float eu = pju - piu, ev = pjv - piv;
        float cr = eu * (pv - piv) - (pu - piu) * ev;
        // |cr| / |e| is the distance to the edge line; a point beyond the segment's
        // ends is at least as far from the segment, so the test stays conservative.
        float l2 = eu * eu + ev * ev;
        if (cr * cr <= em * em * l2) {
            // within em of this edge's line: ambiguous if also within em of the segment span
            float tt = ((pu - piu) * eu + (pv - piv) * ev);
            if (tt >= -em * sqrtf(l2) && tt <= l2 + em * sqrtf(l2)) amb = true;
        }
        if ((piv > pv) != (pjv > pv)) {
            if ((cr > 0) == (pjv > piv)) in = !in;
        }
        pju = piu; pjv = piv;
    }
    return in;
}

// Ray for the FP32 traversal: origin split into hi + lo floats so that O - o is
// formed to ~1e-7 of its own size, whatever the absolute coordinates.
struct RayF {
    float ohx, ohy, ohz, olx, oly, olz;
    float dx, dy, dz;
};
__device__ __forceinline__ RayF make_ray_f(double ox, double oy, double oz, float dx, float dy, float dz) {
    RayF r;
    r.ohx = (float)ox; r.ohy = (float)oy; r.ohz = (float)oz;
    r.olx = (float)(ox - (double)r.ohx); r.oly = (float)(oy - (double)r.ohy); r.olz = (float)(oz - (double)r.ohz);
    r.dx = dx; r.dy = dy; r.dz = dz;
    return r;
}

// FacetIsectF layout: [N0 N1 N2 Olo0 | Ohi0 Ohi1 Ohi2 Olo1 | Us0 Us1 Us2 Olo2 | Vs0 Vs1 Vs2 -]
__device__ __noinline__ HitF trace_f(const DevModel& M, int root, const RayF& ray, int last, bool& ambiguous,
                                     unsigned long long* status) {
    HitF h;
    h.f = -1;
    h.t = 3.0e38f;
    h.u = h.v = 0;
    float htol = 0.0f;    // error bound of h.t
    const float dx = ray.dx, dy = ray.dy, dz = ray.dz;
    const float ox = ray.ohx, oy = ray.ohy, oz = ray.ohz;
    float ix = 1.0f / dx, iy = 1.0f / dy, iz = 1.0f / dz;
    int stack[kStack];
    int sp = 0;
    int node = root;
    while (true) {
        const NodeF nd = M.nodes_f[node];
        float tx0 = (nd.lo[0] - ox) * ix, tx1 = (nd.hi[0] - ox) * ix;
        float ty0 = (nd.lo[1] - oy) * iy, ty1 = (nd.hi[1] - oy) * iy;
        float tz0 = (nd.lo[2] - oz) * iz, tz1 = (nd.hi[2] - oz) * iz;
        float tmin = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), 0.0f));
        float tmax = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), h.t + 2.0f * htol));
        bool hit = tmin <= tmax * 1.0000005f;
        if (hit && nd.b >= 0) {
            int near = nd.a, far = nd.a + 1;
            float dax = nd.b == 0 ? dx : (nd.b == 1 ? dy : dz);
            if (dax < 0) { near = nd.a + 1; far = nd.a; }
            if (sp < kStack) stack[sp++] = far;
            else atomicOr(status, KS_STACK);
            node = near;
            continue;
        }
        if (hit) {
            int cnt = -1 - nd.b;
            for (int k = 0; k < cnt; ++k) {
                int f = M.prims[nd.a + k];
                if (f == last) continue;
                const FacetIsectF& R = M.isect_f[f];
                float Nx = R.v[0], Ny = R.v[1], Nz = R.v[2];
                float den = Nx * dx + Ny * dy + Nz * dz;
                bool two = (M.info[f].flags & FF_TWO_SIDED) != 0;
                float aden = fabsf(den);
                // back-face culling is exact when N.d is well above its rounding error
                if (!two && den > 1e-6f) continue;
                if (aden < 1e-30f) continue;
                // w = O - o to ~1e-7 |w| (Sterbenz for nearby facets)
                float wx = (R.v[4] - ray.ohx) + (R.v[3] - ray.olx);
                float wy = (R.v[5] - ray.ohy) + (R.v[7] - ray.oly);
                float wz = (R.v[6] - ray.ohz) + (R.v[11] - ray.olz);
                float wabs = fabsf(wx) + fabsf(wy) + fabsf(wz);
                float num = Nx * wx + Ny * wy + Nz * wz;
                float t = num / den;
                float at = fabsf(t);
                float tol = (5e-7f * wabs + 4e-7f * at) / aden + 3e-7f * at;   // error bound of t
                if (t + tol <= 0.0f) continue;                       // certainly behind
                if (t - tol > h.t + htol) continue;                  // certainly beyond the best
                float px = t * dx - wx, py = t * dy - wy, pz = t * dz - wz;   // hit point - O
                float u = px * R.v[8] + py * R.v[9] + pz * R.v[10];
                float v = px * R.v[12] + py * R.v[13] + pz * R.v[14];
                const PolyF P = M.poly_f[f];
                float em = tol + 3e-7f * (wabs + at) + 2e-7f * fmaxf(P.su, P.sv);   // position error bound, cm
                float eu = em / P.su, ev = em / P.sv;
                if (u < -eu || u > 1.0f + eu || v < -ev || v > 1.0f + ev) continue;   // certainly outside
                bool amb = (t - tol <= 0.0f) || (!two && den >= 0.0f);
                amb = amb || u < eu || u > 1.0f - eu || v < ev || v > 1.0f - ev;
                bool inside;
                float du = (u - P.cu) * P.su, dv = (v - P.cv) * P.sv;
                float r = sqrtf(du * du + dv * dv);
                if (P.rin2 > 1e29f) {
                    inside = true;                                   // rectangle: [0,1]^2 decided above
                } else if (r * r < P.rin2 && r + em < sqrtf(P.rin2)) {
                    inside = true;
                    amb = (t - tol <= 0.0f) || (!two && den >= 0.0f);
                } else if (r - em > sqrtf(P.rout2)) {
                    continue;
                } else {
                    bool eamb = false;
                    inside = edge_inside_f(M, P, u, v, em, eamb);
                    amb = amb || eamb;
                }
                if (amb) {
                    // could be a hit closer than the best one: let FP64 decide the ray
                    if (t - tol <= h.t + htol) ambiguous = true;
                    continue;
                }
                if (!inside) continue;
                // certain hit; ambiguous ordering when it is within error bounds of the best
                if (h.f >= 0 && fabsf(t - h.t) <= tol + htol) ambiguous = true;
                if (t < h.t) { h.f = f; h.t = t; h.u = u; h.v = v; htol = tol; }
            }
        }
        if (sp == 0) break;
        node = stack[--sp];
    }
    return h;
}

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
    double u, v;              // (u,v) of the current facet (facetHitDetails)
    uint64_t bounces;
    int last, structure;
};

// ProfileFacet (Particle.cpp:1026-1085); profiles are tallied in global memory
__device__ __forceinline__ void profile_add(const DevModel& M, const DevTally& T, int f, int m, bool count_hit,
                                            unsigned long long vfac, unsigned long long ofac, double cosn, double vel,
                                            double u, double v, unsigned long long q1, unsigned long long q2) {
    const FacetInfo& In = M.info[f];
    int pt = In.profile_type;
    int pos = -1;
    bool full = false;
    if (count_hit && pt == MFG_PROFILE_ANGULAR) {
        double th = acos(fmin(cosn, 1.0));
        pos = (int)(th / (kPi / 2) * (double)MFG_PROFILE_SIZE);
        pos = min(max(pos, 0), MFG_PROFILE_SIZE - 1);
    } else if (pt == MFG_PROFILE_U || pt == MFG_PROFILE_V) {
        double x = (pt == MFG_PROFILE_U ? u : v) * (double)MFG_PROFILE_SIZE;
        if (!(x >= 0.0) || x >= (double)MFG_PROFILE_SIZE) return;
        pos = (int)x;
        full = true;
    } else if (count_hit && pt >= MFG_PROFILE_VELOCITY && pt <= MFG_PROFILE_TAN_VELOCITY) {
        double dd = (pt == MFG_PROFILE_VELOCITY) ? 1.0 : (pt == MFG_PROFILE_ORT_VELOCITY ? cosn : sqrt(fmax(0.0, 1.0 - cosn * cosn)));
        double x = dd * vel / M.info2[f].max_speed * (double)MFG_PROFILE_SIZE;
        if (!(x >= 0.0) || x >= (double)MFG_PROFILE_SIZE) return;
        pos = (int)x;
    } else {
        return;
    }
    unsigned long long* g = T.profile + (((size_t)m * M.profile_facets + In.prof_idx) * MFG_PROFILE_SIZE + pos) * TT_N;
    if (count_hit) atomicAdd(g + TT_COUNT, 1ull);
    if (full) {
        add128(g + TT_S1OV, vfac * q1);
        add128(g + TT_SVORT, ofac * q2);
    }
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

template <bool kFP32>
__global__ void __launch_bounds__(256) trace_kernel(const __grid_constant__ DevModel M, DevTally T, LaunchCtl C) {
    typedef typename Real_<kFP32>::T R;
    extern __shared__ unsigned long long smem[];
    __shared__ double s_cdf_v[MFG_MAXWELL_N], s_cdf_p[MFG_MAXWELL_N];
    __shared__ float s_cdf_vf[MFG_MAXWELL_N], s_cdf_pf[MFG_MAXWELL_N];
    BlockTally B;
    B.sglob = smem;
    B.sfac = C.smem_facets ? smem + TG_N : nullptr;
    const int nsm = TG_N + (C.smem_facets ? M.nf * SF_N : 0);
    for (int i = threadIdx.x; i < nsm; i += blockDim.x) smem[i] = 0ull;
    for (int i = threadIdx.x; i < MFG_MAXWELL_N; i += blockDim.x) {
        s_cdf_v[i] = M.cdf_v[i];
        s_cdf_p[i] = M.cdf_p[i];
        s_cdf_vf[i] = (float)M.cdf_v[i];
        s_cdf_pf[i] = (float)M.cdf_p[i];
    }
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const unsigned lane_lt = (1u << lane) - 1u;
    unsigned long long pool_next = 0, pool_end = 0;   // warp pool of particle ids
    const unsigned long long chunk = 64;

    typename std::conditional<kFP32, RngF, RngD>::type rng;
    rng.k0 = C.key0;
    rng.k1 = C.key1;
    ParticleState P;
    P.ox = P.oy = P.oz = 0;
    P.time = 0;
    P.decay_at = 1e100;
    P.u = P.v = 0;
    P.bounces = 0;
    P.last = -1;
    P.structure = 0;
    R dx = 0, dy = 0, dz = 0, vel = 1;
    bool active = true;       // lane still has particles to trace
    bool need_new = true;     // lane must desorb a new particle
    // incoming half of the last reflection, added together with the outgoing half (moment 0)
    unsigned long long pend_s1ov = 0, pend_svort = 0, pend_s1v = 0;
    int pend_cell = -1;
    bool pend = false;
    unsigned iter = 0;
    // per-thread global counters (no contended shared atomics on the hot path)
    unsigned long long c_hits = 0, c_des = 0, c_abs = 0, c_leak = 0, c_drop = 0, c_rechk = 0;
    unsigned long long c_dist = 0, c_distf = 0;
    unsigned long long deadline;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(deadline));
    deadline += C.time_limit_ns;

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
            if (want && P.bounces >= C.n_particles) { active = false; want = false; }
        }
        if (!active) continue;

        // ---- 1. emit a direction: desorption or reflection from facet fo ----
        int fo;
        if (want) {
            // StartFromSource (Particle.cpp:407-685)
            rng.start(C.first_particle + P.bounces);
            double sr = (double)rng.next() * M.src_total;
            int lo = 0, hi = M.n_src;
            while (lo < hi) { int mid = (lo + hi) >> 1; if (M.src_cdf[mid] > sr) hi = mid; else lo = mid + 1; }
            if (lo >= M.n_src) lo = M.n_src - 1;
            fo = M.src_facet[lo];
            const FacetInfo& In = M.info[fo];
            const FacetInfo2& I2 = M.info2[fo];
            bool flip = (In.flags & FF_TWO_SIDED) ? ((double)rng.next() > 0.5) : false;
            int idt = M.src_id[lo];
            if (idt >= 0) {
                int s = M.id_start[idt], e = M.id_start[idt + 1];
                double r = (double)rng.next() * M.id_cum[e - 1];
                P.time = interp_x_d(r, M.id_t + s, M.id_cum + s, e - s);
            } else {
                P.time = (double)rng.next() * M.latest;
            }
            P.structure = I2.structure;
            P.bounces = 0;
            if (M.use_maxwell) {
                if (kFP32) vel = (R)(M.phys_f[fo].sqrtT * interp_x_f((float)rng.next(), s_cdf_vf, s_cdf_pf, MFG_MAXWELL_N));
                else vel = (R)(M.phys_d[fo].sqrtT * interp_x_d((double)rng.next(), s_cdf_v, s_cdf_p, MFG_MAXWELL_N));
            } else {
                vel = (R)(145.469 * sqrt(I2.temperature / M.gas_mass));
            }
            P.decay_at = M.enable_decay ? P.time - 1.44269 * M.half_life * log(1.0 - (double)rng.next()) : 1e100;
            // start point: rejection in the (u,v) rectangle, at most 1000 tries (Particle.cpp:513-570)
            const FacetIsectD& Rr = M.isect_d[fo];
            const PolyD& PP = M.poly_d[fo];
            bool found = false;
            double su = 0.5, sv = 0.5;
            for (int tr = 0; tr < 1000 && !found; ++tr) {
                double u = (double)rng.next(), v = (double)rng.next();
                if (in_facet_d(M, fo, u, v)) { su = u; sv = v; found = true; }
            }
            if (found) {
                double a = su * PP.su * PP.su, b = sv * PP.sv * PP.sv;   // O + u*U + v*V (record keeps U/|U|^2)
                P.ox = Rr.v[4] + a * Rr.v[8] + b * Rr.v[12];
                P.oy = Rr.v[5] + a * Rr.v[9] + b * Rr.v[13];
                P.oz = Rr.v[6] + a * Rr.v[10] + b * Rr.v[14];
            } else {
                P.ox = M.center[3 * fo];
                P.oy = M.center[3 * fo + 1];
                P.oz = M.center[3 * fo + 2];
            }
            P.u = su;
            P.v = sv;
            P.last = fo;
            R r1 = (R)rng.next(), r2 = (R)rng.next();
            R ct;
            if (I2.desorb_type == MFG_DES_UNIFORM) ct = r1;
            else if (I2.desorb_type == MFG_DES_COSINE_N) ct = (R)pow((double)r1, 1.0 / (I2.desorb_exp + 1.0));
            else ct = (R)sqrt(r1);
            polar_dir<kFP32>(M, fo, ct, r2, flip, dx, dy, dz);
            // desorption tallies (Particle.cpp:646-680)
            double cosn = kFP32 ? (double)fabsf(dx * M.phys_f[fo].N[0] + dy * M.phys_f[fo].N[1] + dz * M.phys_f[fo].N[2])
                                : fabs((double)dx * Rr.v[0] + (double)dy * Rr.v[1] + (double)dz * Rr.v[2]);
            R ort = vel * (R)cosn;
            unsigned long long q1 = kFP32 ? qf(1.0f / (float)ort, (float)MFG_SCALE_INV) : qd(1.0 / (double)ort, MFG_SCALE_INV);
            unsigned long long q2 = kFP32 ? qf((float)ort, (float)MFG_SCALE_V) : qd((double)ort, MFG_SCALE_V);
            unsigned long long q3 = kFP32 ? qf(1.0f / (float)vel, (float)MFG_SCALE_INV) : qd(1.0 / (double)vel, MFG_SCALE_INV);
            ++c_des;
            int cell = -1;
            if ((In.count & MFG_COUNT_DES) && In.tex_off >= 0) {
                int tu = (int)(su * M.phys_d[fo].texw_p), tv = (int)(sv * M.phys_d[fo].texh_p);
                tu = min(max(tu, 0), In.tex_w - 1);
                tv = min(max(tv, 0), In.tex_h - 1);
                cell = In.tex_off + tu + tv * In.tex_w;
            }
            facet_add(M, T, B, fo, 0, 0, 1, 0, 2 * q1, q2, q3);
            if (cell >= 0) cell_add(T.texture + (size_t)cell * TT_N, 1, 2 * q1, q2);
            if (In.flags & FF_PROFILE) profile_add(M, T, fo, 0, false, 2, 1, cosn, (double)vel, su, sv, q1, q2);
            for_moments(M, P.time, [&](int m) {
                facet_add(M, T, B, fo, m, 0, 1, 0, 2 * q1, q2, q3);
                if (cell >= 0) cell_add(T.texture + ((size_t)m * M.texture_cells + cell) * TT_N, 1, 2 * q1, q2);
                if (In.flags & FF_PROFILE) profile_add(M, T, fo, m, false, 2, 1, cosn, (double)vel, su, sv, q1, q2);
            });
            need_new = false;
        } else {
            // relaunch half of PerformBounce (Particle.cpp:769-836)
            fo = P.last;
            const FacetInfo& In = M.info[fo];
            const FacetIsectD& Rr = M.isect_d[fo];
            const FacetPhysD& Ph = M.phys_d[fo];
            bool flip = false;
            if (In.flags & FF_TWO_SIDED)
                flip = kFP32 ? (dx * M.phys_f[fo].N[0] + dy * M.phys_f[fo].N[1] + dz * M.phys_f[fo].N[2]) > 0.0f
                             : ((double)dx * Rr.v[0] + (double)dy * Rr.v[1] + (double)dz * Rr.v[2]) > 0.0;
            double temp = (In.flags & FF_TEMP_PARAM) ? param_at(M, M.info2[fo].temp_param, P.time) : M.info2[fo].temperature;
            double sqT = (In.flags & FF_TEMP_PARAM) ? sqrt(temp) : Ph.sqrtT;
            if ((kFP32 ? (double)M.phys_f[fo].accommodation : Ph.accommodation) > 0.9999) {   // UpdateVelocity (Particle.cpp:1138-1163)
                if (M.use_maxwell) {
                    if (kFP32) vel = (R)((float)sqT * interp_x_f((float)rng.next(), s_cdf_vf, s_cdf_pf, MFG_MAXWELL_N));
                    else vel = (R)(sqT * interp_x_d((double)rng.next(), s_cdf_v, s_cdf_p, MFG_MAXWELL_N));
                } else {
                    vel = (R)(145.469 * sqT / M.gas_mass);
                }
            } else {
                double o2 = (double)vel * (double)vel, n2;
                if (M.use_maxwell) {
                    double v = sqT * interp_x_d((double)rng.next(), s_cdf_v, s_cdf_p, MFG_MAXWELL_N);
                    n2 = v * v;
                } else {
                    n2 = 29369.939 * (temp / M.gas_mass);
                }
                vel = (R)sqrt(o2 + (n2 - o2) * Ph.accommodation);
            }
            if (In.flags & FF_SOJOURN) {
                double A = exp(-Ph.soj_e / (8.31 * temp));
                P.time += -log(1.0 - (double)rng.next()) / (A * Ph.soj_freq);
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
            double cosn = kFP32 ? (double)fabsf(dx * M.phys_f[fo].N[0] + dy * M.phys_f[fo].N[1] + dz * M.phys_f[fo].N[2])
                                : fabs((double)dx * Rr.v[0] + (double)dy * Rr.v[1] + (double)dz * Rr.v[2]);
            R ort = vel * (R)cosn;
            unsigned long long q1 = kFP32 ? qf(1.0f / (float)ort, (float)MFG_SCALE_INV) : qd(1.0 / (double)ort, MFG_SCALE_INV);
            unsigned long long q2 = kFP32 ? qf((float)ort, (float)MFG_SCALE_V) : qd((double)ort, MFG_SCALE_V);
            // moment 0: incoming and outgoing halves together
            pend_s1ov += q1;
            pend_svort += q2;
            flush_pending();
            int cell = -1;
            if ((In.count & MFG_COUNT_REFL) && In.tex_off >= 0) {
                int tu = (int)(P.u * Ph.texw_p), tv = (int)(P.v * Ph.texh_p);
                tu = min(max(tu, 0), In.tex_w - 1);
                tv = min(max(tv, 0), In.tex_h - 1);
                cell = In.tex_off + tu + tv * In.tex_w;
            }
            if (In.flags & FF_PROFILE) profile_add(M, T, fo, 0, false, 1, 1, cosn, (double)vel, P.u, P.v, q1, q2);
            for_moments(M, P.time, [&](int m) {
                facet_add(M, T, B, fo, m, 0, 0, 0, q1, q2, 0);
                if (cell >= 0) cell_add(T.texture + ((size_t)m * M.texture_cells + cell) * TT_N, 0, q1, q2);
                if (In.flags & FF_PROFILE) profile_add(M, T, fo, m, false, 1, 1, cosn, (double)vel, P.u, P.v, q1, q2);
            });
        }

        // ---- 2. trace the ray ----
        int root = M.roots[P.structure];
        int hf;
        double ht, hu, hv;
        if (kFP32) {
            bool amb = false;
            HitF h = trace_f(M, root, make_ray_f(P.ox, P.oy, P.oz, (float)dx, (float)dy, (float)dz), P.last, amb,
                             T.global + TG_STATUS);
            if (amb || h.f < 0) {
                ++c_rechk;
                HitD hd = trace_d(M, root, P.ox, P.oy, P.oz, (double)dx, (double)dy, (double)dz, P.last, T.global + TG_STATUS);
                hf = hd.f; ht = hd.t; hu = hd.u; hv = hd.v;
            } else {
                hf = h.f;
                hu = h.u;
                hv = h.v;
                // distance to the FP64 plane of the hit facet: FP32 estimate + FP64 residual
                const FacetIsectD& Rh = M.isect_d[hf];
                double ddx = (double)dx, ddy = (double)dy, ddz = (double)dz;
                double den = Rh.v[0] * ddx + Rh.v[1] * ddy + Rh.v[2] * ddz;
                double num = Rh.v[3] - (Rh.v[0] * P.ox + Rh.v[1] * P.oy + Rh.v[2] * P.oz);
                double r = num - (double)h.t * den;
                ht = (double)h.t + (double)((float)r / (float)den);
            }
        } else {
            HitD h = trace_d(M, root, P.ox, P.oy, P.oz, (double)dx, (double)dy, (double)dz, P.last, T.global + TG_STATUS);
            hf = h.f; ht = h.t; hu = h.u; hv = h.v;
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
        P.ox = P.ox + travel * (double)dx;
        P.oy = P.oy + travel * (double)dy;
        P.oz = P.oz + travel * (double)dz;
        if (kFP32) P.time += (double)((float)travel * (0.01f / (float)vel));   // cm -> m
        else P.time += travel / 100.0 / (double)vel;
        unsigned long long qdist = kFP32 ? qf((float)travel, (float)MFG_SCALE_DIST) : qd(travel, MFG_SCALE_DIST);
        c_dist += qdist;
        if (event != 0) { need_new = true; continue; }
        c_distf += qdist;
        // ---- 4. stick or reflect at facet hf (Particle.cpp:323-357) ----
        const FacetInfo& In = M.info[hf];
        const FacetIsectD& Rh = M.isect_d[hf];
        bool absorb;
        double cosn;
        if (kFP32) {
            float s = (In.flags & FF_STICK_PARAM) ? (float)param_at(M, M.info2[hf].stick_param, P.time) : M.phys_f[hf].sticking;
            absorb = (s == 1.0f) || (s > 0.0f && (float)rng.next() < s);
            cosn = (double)fabsf(dx * M.phys_f[hf].N[0] + dy * M.phys_f[hf].N[1] + dz * M.phys_f[hf].N[2]);
        } else {
            double s = (In.flags & FF_STICK_PARAM) ? param_at(M, M.info2[hf].stick_param, P.time) : M.phys_d[hf].sticking;
            absorb = (s == 1.0) || (s > 0.0 && (double)rng.next() < s);
            cosn = fabs((double)dx * Rh.v[0] + (double)dy * Rh.v[1] + (double)dz * Rh.v[2]);
        }
        R ort = vel * (R)cosn;
        unsigned long long q1 = kFP32 ? qf(1.0f / (float)ort, (float)MFG_SCALE_INV) : qd(1.0 / (double)ort, MFG_SCALE_INV);
        unsigned long long q2 = kFP32 ? qf((float)ort, (float)MFG_SCALE_V) : qd((double)ort, MFG_SCALE_V);
        unsigned long long q3 = kFP32 ? qf(1.0f / (float)vel, (float)MFG_SCALE_INV) : qd(1.0 / (double)vel, MFG_SCALE_INV);
        P.u = hu;
        P.v = hv;
        int cell = -1;
        if (In.tex_off >= 0 && (In.count & (absorb ? MFG_COUNT_ABS : MFG_COUNT_REFL))) {
            int tu = (int)(hu * M.phys_d[hf].texw_p), tv = (int)(hv * M.phys_d[hf].texh_p);
            tu = min(max(tu, 0), In.tex_w - 1);
            tv = min(max(tv, 0), In.tex_h - 1);
            cell = In.tex_off + tu + tv * In.tex_w;
        }
        ++c_hits;
        if (In.flags & FF_ANGLEMAP) anglemap_add(M, T, hf, (double)dx, (double)dy, (double)dz);
        if (absorb) {   // RecordAbsorb (Particle.cpp:888-924)
            ++c_abs;
            facet_add(M, T, B, hf, 0, 1, 0, 1, 2 * q1, q2, q3);
            if (cell >= 0) cell_add(T.texture + (size_t)cell * TT_N, 1, 2 * q1, q2);
            if (In.flags & FF_PROFILE) profile_add(M, T, hf, 0, true, 2, 1, cosn, (double)vel, hu, hv, q1, q2);
            for_moments(M, P.time, [&](int m) {
                facet_add(M, T, B, hf, m, 1, 0, 1, 2 * q1, q2, q3);
                if (cell >= 0) cell_add(T.texture + ((size_t)m * M.texture_cells + cell) * TT_N, 1, 2 * q1, q2);
                if (In.flags & FF_PROFILE) profile_add(M, T, hf, m, true, 2, 1, cosn, (double)vel, hu, hv, q1, q2);
            });
            need_new = true;
        } else {        // incoming half of PerformBounce (Particle.cpp:735-767)
            if (In.flags & FF_PROFILE) profile_add(M, T, hf, 0, true, 1, 1, cosn, (double)vel, hu, hv, q1, q2);
            for_moments(M, P.time, [&](int m) {
                facet_add(M, T, B, hf, m, 1, 0, 0, q1, q2, q3);
                if (cell >= 0) cell_add(T.texture + ((size_t)m * M.texture_cells + cell) * TT_N, 1, q1, q2);
                if (In.flags & FF_PROFILE) profile_add(M, T, hf, m, true, 1, 1, cosn, (double)vel, hu, hv, q1, q2);
            });
            P.last = hf;
            pend = true;
            pend_s1ov = q1;
            pend_svort = q2;
            pend_s1v = q3;
            pend_cell = cell;
            need_new = false;
            if (++P.bounces > C.max_steps) {   // step cap: count the hit, drop the particle
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
__global__ void replay_kernel(const __grid_constant__ DevModel M, int precision, long long n, const double* origin,
                              const double* dir, const int* last, int* hit_f, double* hit_t,
                              unsigned long long* rechecks, unsigned long long* status) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double ox = origin[3 * i], oy = origin[3 * i + 1], oz = origin[3 * i + 2];
    double dx = dir[3 * i], dy = dir[3 * i + 1], dz = dir[3 * i + 2];
    int root = M.roots[0];
    if (precision == 0) {
        HitD h = trace_d(M, root, ox, oy, oz, dx, dy, dz, last[i], status);
        hit_f[i] = h.f;
        hit_t[i] = h.f >= 0 ? h.t : -1.0;
    } else {
        bool amb = false;
        HitF h = trace_f(M, root, make_ray_f(ox, oy, oz, (float)dx, (float)dy, (float)dz), last[i], amb, status);
        if (amb || h.f < 0) {
            atomicAdd(rechecks, 1ull);
            HitD hd = trace_d(M, root, ox, oy, oz, dx, dy, dz, last[i], status);
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
}

}  // namespace mfgk
