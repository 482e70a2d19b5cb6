// traversal.cuh — ray/BVH traversal for the tracer: FP64 (trace_d) and FP32 with
// error bounds (trace_f), point-in-polygon tests.  Host-compilable with the shims in
// the CPU harness of the tests; device code otherwise.
#pragma once
#include <stdint.h>

#include "device_model.h"
#include "philox.cuh"

#ifndef MFG_AMB_HOOK
#define MFG_AMB_HOOK(reason)
#endif

namespace mfgk {

constexpr int kStack = 64;
// Traversal stack of one thread, in local memory.  Keeping its top 8 or 16 entries in shared
// memory (one bank per lane) measured 2x slower on the beam chamber and 1.5x on the tube (1024 x 2
// launch shape): the rings' shared memory comes out of the L1 that holds the BVH nodes.
struct TravStack {
    int sp;
    int loc[kStack];
    __device__ __forceinline__ void push(int v) { loc[sp++] = v; }
    __device__ __forceinline__ int pop() { return loc[--sp]; }
};


// One 32-byte read-only load (two float4) per thread: half the L1 requests of two 16-byte loads
// for the scattered BVH node fetches (+3 % hits/s on the beam chamber, +2 % on the tube, +8 % for
// the traversal alone), with the hint to keep the nodes in L1 and L2 ahead of the spilled
// registers and stacks (+0.5 %).  MFG_NO_V8 builds the two 16-byte loads instead.
__device__ __forceinline__ void ldg_v8(const void* p, float4& a, float4& b) {
#if defined(__CUDA_ARCH__) && !defined(MFG_NO_V8)
    asm("ld.global.nc.L1::evict_last.L2::evict_last.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w) : "l"(p));
#else
    a = __ldg(reinterpret_cast<const float4*>(p));
    b = __ldg(reinterpret_cast<const float4*>(p) + 1);
#endif
}

// InterpolateY (no extrapolation) for time-dependent parameters
__device__ __noinline__ double param_at(const DevModel& M, int p, double t) {
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


// ---------------------------------------------------------- opacity ----
#define MFG_MAX_TRANSP 32
// Transparent passes found during one trace (candidates of RegisterTransparentPass): the nearest
// MFG_MAX_TRANSP of those beyond distance `tlo`.  When a ray crosses more, `over` is set and the
// tracer traces the same ray again for the passes beyond the farthest one kept (the hard hit is
// the same every time), so no pass is lost whatever the number of transparent facets.
template <class T>
struct TranspList {
    int n, over;
    T tlo;
    int f[MFG_MAX_TRANSP];
    T t[MFG_MAX_TRANSP], u[MFG_MAX_TRANSP], v[MFG_MAX_TRANSP];
    __device__ __forceinline__ void clear(T from) { n = 0; over = 0; tlo = from; }
    // distance of the farthest pass kept
    __device__ __forceinline__ T farthest() const {
        T m = tlo;
        for (int k = 0; k < n; ++k) m = t[k] > m ? t[k] : m;
        return m;
    }
};
// A partial-opacity decision is an order-independent draw per (particle, trace step, facet)
// from a Philox stream keyed apart from the particle's own stream.
struct OpacCtx {
    uint32_t k0, k1, p0, p1, step;
    double time;
};
__device__ __forceinline__ bool is_hard(const DevModel& M, int f, int cls, const OpacCtx* oc) {
    if (cls == 0) return true;
    if (cls == 1 || !oc) return false;
    const FacetInfo2& I2 = M.info2[f];
    double op = I2.opac_param >= 0 ? param_at(M, I2.opac_param, oc->time) : I2.opacity;
    if (op >= 1.0) return true;
    if (op <= 0.0) return false;
    uint32_t c0 = oc->p0, c1 = oc->p1, c2 = oc->step, c3 = (uint32_t)f + 1u;
    philox4x32_10(c0, c1, c2, c3, oc->k0, oc->k1);
    return u01d(c0, c1) < op;
}
// opacity draws of a ray replayed on its own: particle 0, step 0, time 0, seed 0
__device__ __forceinline__ OpacCtx replay_opacity() {
    OpacCtx oc;
    oc.k0 = 0u;
    oc.k1 = 0xA5A5A5A5u;
    oc.p0 = oc.p1 = oc.step = 0u;
    oc.time = 0.0;
    return oc;
}
template <class T>
__device__ __forceinline__ void add_transp(TranspList<T>* tl, int f, double t, double u, double v,
                                           unsigned long long* status) {
    (void)status;
    if (!tl) return;
    const T tt = (T)t;
    if (!(tt > tl->tlo)) return;   // taken in an earlier round
    int k = tl->n;
    if (k == MFG_MAX_TRANSP) {     // full: replace the farthest if this one is nearer
        tl->over = 1;
        k = 0;
        for (int j = 1; j < MFG_MAX_TRANSP; ++j) k = tl->t[j] > tl->t[k] ? j : k;
        if (!(tt < tl->t[k])) return;
    } else {
        ++tl->n;
    }
    tl->f[k] = f; tl->t[k] = tt; tl->u[k] = (T)u; tl->v[k] = (T)v;
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

// Resumable FP64 traversal of one ray (the FP64 kernel and the FP32 path's recheck): the next
// NodeD to visit (or kTrDoneD) and the closest hard hit so far; the stack is kept apart.
constexpr int kTrDoneD = -1;
struct TravD {
    double ox, oy, oz, dx, dy, dz, ix, iy, iz;
    int node, last;
    HitD h;
};

__device__ __forceinline__ void travd_init(TravD& s, TravStack& stk, int root, double ox, double oy, double oz,
                                           double dx, double dy, double dz, int last) {
    s.ox = ox; s.oy = oy; s.oz = oz;
    s.dx = dx; s.dy = dy; s.dz = dz;
    s.ix = 1.0 / dx; s.iy = 1.0 / dy; s.iz = 1.0 / dz;
    s.node = root;
    s.last = last;
    s.h.f = -1;
    s.h.t = 1.0e99;
    s.h.u = s.h.v = 0;
    stk.sp = 0;
}

// one step: visit node `s.node` (its box; a leaf's facets), then set the next node.  Transparent
// candidates (opacity 0, or a partial-opacity draw above the opacity) go to `tl`.
template <class LT = double, bool kTr = true>
__device__ __forceinline__ void travd_step(const DevModel& M, TravD& s, TravStack& stk, unsigned long long* status,
                                           TranspList<LT>* tl = nullptr, const OpacCtx* oc = nullptr) {
    const double ox = s.ox, oy = s.oy, oz = s.oz, dx = s.dx, dy = s.dy, dz = s.dz;
    const double ix = s.ix, iy = s.iy, iz = s.iz;
    const int last = s.last;
    HitD& h = s.h;
    const NodeD nd = M.nodes_d[s.node];
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
        if (stk.sp < kStack) stk.push(far);
        else atomicOr(status, KS_STACK);
        s.node = near;
        return;
    }
    if (hit) {
        int cnt = -1 - nd.b;
        for (int k = 0; k < cnt; ++k) {
            int f = M.prims[nd.a + k];
            if (f == last) continue;
            const FacetIsectD& R = M.isect_d[f];
            double Nx = R.v[0], Ny = R.v[1], Nz = R.v[2], D = R.v[3];
            double den = Nx * dx + Ny * dy + Nz * dz;
            const long long fl = __double_as_longlong(R.v[7]);   // bit 0 two-sided, bits 1-2 opacity class
            const bool two = (fl & 1) != 0;
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
            if constexpr (kTr) {
                const int cls = (int)((fl >> 1) & 3);
                if (cls != 0 && !is_hard(M, f, cls, oc)) { add_transp(tl, f, t, u, v, status); continue; }
            }
            if (t < h.t || f < h.f) { h.f = f; h.t = t; h.u = u; h.v = v; }
        }
    }
    s.node = stk.sp == 0 ? kTrDoneD : stk.pop();
}

// closest hard hit of the ray (skipping facet `last`); BVH of structure `root`
template <class LT = double, bool kTr = true>
__device__ __noinline__ HitD trace_d(const DevModel& M, int root, double ox, double oy, double oz,
                                     double dx, double dy, double dz, int last, unsigned long long* status,
                                     TranspList<LT>* tl = nullptr, const OpacCtx* oc = nullptr) {
    TravD s;
    TravStack stk;
    travd_init(s, stk, root, ox, oy, oz, dx, dy, dz, last);
    while (s.node != kTrDoneD) travd_step<LT, kTr>(M, s, stk, status, tl, oc);
    return s.h;
}

// --------------------------------------------------------- FP32 trace ---
// hit of the FP32 traversal
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

// FacetIsectF layout: [N0 N1 N2 Olo0 | Ohi0 Ohi1 Ohi2 Olo1 | Us0 Us1 Us2 Olo2 | Vs0 Vs1 Vs2 flags]

// Resumable FP32 traversal of one ray: the ref to visit next (a NodeC index >= 0, a leaf list
// -1-first < 0, or kTrDone) and the best hit so far with its error bound; the stack is kept
// apart, so that the scalar state can stay in registers.  A warp can step its lanes' traversals
// together and stop them at any step.
constexpr int kTrDone = -0x7fffffff - 1;
struct TravF {
    RayF ray;
    float ix, iy, iz;
    int ref, last;
    HitF h;
    float htol;    // error bound of h.t
    bool amb;      // a candidate could be classified differently in exact arithmetic
};

template <class Stk>
__device__ __forceinline__ void trav_init(TravF& s, Stk& stk, int root, const RayF& ray, int last) {
    s.ray = ray;
    s.ix = 1.0f / ray.dx;
    s.iy = 1.0f / ray.dy;
    s.iz = 1.0f / ray.dz;
    s.ref = root;   // the structure's root NodeC
    s.last = last;
    s.h.f = -1;
    s.h.t = 3.0e38f;
    s.h.u = s.h.v = 0;
    s.htol = 0.0f;
    s.amb = false;
    stk.sp = 0;
}

// one step: visit the node or the leaf list `s.ref`, then set the next ref.  The first n_top
// NodeC records (the top levels of structure 0, breadth-first) may be staged in shared memory at
// `top`; the others are read from global memory.
template <bool kTr = true, class Stk = TravStack>
__device__ __forceinline__ void trav_step(const DevModel& M, TravF& s, Stk& stk, unsigned long long* status,
                                          TranspList<float>* tl = nullptr, const OpacCtx* oc = nullptr,
                                          const float4* top = nullptr, int n_top = 0) {
    const RayF& ray = s.ray;
    const float dx = ray.dx, dy = ray.dy, dz = ray.dz;
    const float ox = ray.ohx, oy = ray.ohy, oz = ray.ohz;
    const float ix = s.ix, iy = s.iy, iz = s.iz;
    const int last = s.last;
    HitF& h = s.h;
    float& htol = s.htol;
    int ref = s.ref;
    bool ambiguous = false;
    if (ref >= 0) {
        // both children's boxes in one 64-byte node
        float4 q0, q1, q2, q3;
        if (ref < n_top) {
            const float4* tp = top + 4 * ref;
            q0 = tp[0]; q1 = tp[1]; q2 = tp[2]; q3 = tp[3];
        } else {
            const float4* np = reinterpret_cast<const float4*>(M.nodes_c + ref);
            ldg_v8(np, q0, q1);   // NodeC records are 64-byte aligned
            ldg_v8(np + 2, q2, q3);
        }
        const float tcap = h.t + 2.0f * htol;
        float a0 = (q0.x - ox) * ix, a1 = (q0.w - ox) * ix;
        float b0 = (q0.y - oy) * iy, b1 = (q1.x - oy) * iy;
        float c0 = (q0.z - oz) * iz, c1 = (q1.y - oz) * iz;
        const float tmin0 = fmaxf(fmaxf(fminf(a0, a1), fminf(b0, b1)), fmaxf(fminf(c0, c1), 0.0f));
        const float tmax0 = fminf(fminf(fmaxf(a0, a1), fmaxf(b0, b1)), fminf(fmaxf(c0, c1), tcap));
        a0 = (q1.z - ox) * ix; a1 = (q2.y - ox) * ix;
        b0 = (q1.w - oy) * iy; b1 = (q2.z - oy) * iy;
        c0 = (q2.x - oz) * iz; c1 = (q2.w - oz) * iz;
        const float tmin1 = fmaxf(fmaxf(fminf(a0, a1), fminf(b0, b1)), fmaxf(fminf(c0, c1), 0.0f));
        const float tmax1 = fminf(fminf(fmaxf(a0, a1), fmaxf(b0, b1)), fminf(fmaxf(c0, c1), tcap));
        const bool hit0 = tmin0 <= tmax0 * 1.0000005f, hit1 = tmin1 <= tmax1 * 1.0000005f;
        const int r0 = __float_as_int(q3.x), r1 = __float_as_int(q3.y);
        if (hit0 && hit1) {
            // nearer box first
            const bool first0 = tmin0 <= tmin1;
            if (stk.sp < kStack) stk.push(first0 ? r1 : r0);
            else atomicOr(status, KS_STACK);
            ref = first0 ? r0 : r1;
        } else if (hit0 || hit1) {
            ref = hit0 ? r0 : r1;
        } else {
            ref = stk.sp == 0 ? kTrDone : stk.pop();
        }
        s.ref = ref;
        return;
    }
    for (int k = -1 - ref;; ++k) {
        const int f = M.prims_c[k];
        if (f < 0) break;
        if (f == last) continue;
        const FacetIsectF& R = M.isect_f[f];
        float Nx = R.v[0], Ny = R.v[1], Nz = R.v[2];
        float den = Nx * dx + Ny * dy + Nz * dz;
        const int fl = (int)R.v[15];                     // bit 0 two-sided, bits 1-2 opacity class
        const bool two = (fl & 1) != 0;
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
        // reason codes: 1 near the origin, 2 nearly parallel back face, 3 near a rectangle
        // edge, 4 near a polygon edge, 5 two hits within error bounds.  A candidate that is
        // certainly outside its polygon is dropped whatever its distance (coplanar facets
        // of a baffle have t = 0 exactly for a ray leaving a neighbour).
        bool inside, eamb = false;
        if (P.rin2 > 1e29f) {
            inside = true;                                   // rectangle: [0,1]^2 decided above
            eamb = u < eu || u > 1.0f - eu || v < ev || v > 1.0f - ev;
        } else if (P.nv == 3) {
            // triangle: signed distances to the three edge lines; a point within the position
            // error (plus the rounding of the edge function) of a line is ambiguous
            const float4* te = reinterpret_cast<const float4*>(M.tri_f + f);
            bool out = false;
            inside = true;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float4 e = __ldg(te + k);
                const float au = e.x * u, bv = e.y * v;
                const float dist = au + bv + e.z;
                const float tl = em + 4e-7f * (fabsf(au) + fabsf(bv) + fabsf(e.z));
                if (dist < -tl) out = true;
                else if (dist <= tl) eamb = true;
                inside = inside && dist > tl;
            }
            if (out) continue;                               // certainly outside
        } else {
            float du = (u - P.cu) * P.su, dv = (v - P.cv) * P.sv;
            float r = sqrtf(du * du + dv * dv);
            if (r * r < P.rin2 && r + em < sqrtf(P.rin2)) inside = true;
            else if (r - em > sqrtf(P.rout2)) continue;
            else inside = edge_inside_f(M, P, u, v, em, eamb);
        }
        if (!inside && !eamb) continue;                      // certainly outside
        int why = (t - tol <= 0.0f) ? 1 : ((!two && den >= 0.0f) ? 2 : (eamb ? (P.rin2 > 1e29f ? 3 : 4) : 0));
        if (why) {
            // could be a hit closer than the best one: let FP64 decide the ray
            if (t - tol <= h.t + htol) { ambiguous = true; MFG_AMB_HOOK(why); }
            continue;
        }
        if (!inside) continue;
        if constexpr (kTr) {
            const int cls = (fl >> 1) & 3;
            if (cls != 0 && !is_hard(M, f, cls, oc)) { add_transp(tl, f, t, u, v, status); continue; }
        }
        // certain hit; ambiguous ordering when it is within error bounds of the best
        if (h.f >= 0 && fabsf(t - h.t) <= tol + htol) { ambiguous = true; MFG_AMB_HOOK(5); }
        if (t < h.t) { h.f = f; h.t = t; h.u = u; h.v = v; htol = tol; }
    }
    s.amb = s.amb || ambiguous;
    s.ref = stk.sp == 0 ? kTrDone : stk.pop();
}

// Lockstep FP32 traversal of one ray per lane, for kernels whose lanes trace independent rays
// (replay): every lane of the warp calls it, lanes without a ray with `active` false.  The warp
// visits one node or one leaf list per lane and step and votes after each step; node and leaf
// steps run in separate rounds, a leaf round once the lanes at leaves outnumber those at nodes
// three to one (the tracer's own traversal loop does the same).  Device code only (warp votes).
#ifdef __CUDACC__
template <bool kTr = true>
__device__ __forceinline__ HitF trace_f_lockstep(const DevModel& M, bool active, int root, const RayF& ray, int last,
                                                 bool& ambiguous, unsigned long long* status,
                                                 const OpacCtx* oc = nullptr) {
    TravF s;
    TravStack stk;
    if (active) trav_init(s, stk, root, ray, last);
    else s.ref = kTrDone;
    while (true) {
        const bool live = s.ref != kTrDone;
        const bool node = live && s.ref >= 0;
        const unsigned mn = __ballot_sync(0xffffffffu, node);
        const unsigned ml = __ballot_sync(0xffffffffu, live && !node);
        if ((mn | ml) == 0u) break;
        const bool leaf_round = __popc(ml) > 3 * __popc(mn);
        if (leaf_round ? (live && !node) : node) trav_step<kTr>(M, s, stk, status, nullptr, oc);
    }
    ambiguous = active && s.amb;
    return s.h;
}
#endif

// FP32 traversal with per-candidate error bounds.  Returns the hit and sets
// `ambiguous` when a candidate could be classified differently in exact
// arithmetic (near an edge, near the origin, or too close to the best hit).
template <bool kTr = true>
__device__ __noinline__ HitF trace_f(const DevModel& M, int root, const RayF& ray, int last, bool& ambiguous,
                                     unsigned long long* status, TranspList<float>* tl = nullptr,
                                     const OpacCtx* oc = nullptr) {
    TravF s;
    TravStack stk;
    trav_init(s, stk, root, ray, last);
    while (s.ref != kTrDone) trav_step<kTr>(M, s, stk, status, tl, oc);
    if (s.amb) ambiguous = true;
    return s.h;
}


}  // namespace mfgk
