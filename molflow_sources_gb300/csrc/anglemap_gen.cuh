// anglemap_gen.cuh — desorption direction drawn from a recorded incident-angle map
// (AnglemapGeneration.cpp:14-257 of the reference).
//
// The tables (AmDev, built on the host from the map) hold, per theta line, the line's count and
// its midpoint CDF value, and per phi bin the midpoint CDF and the normalised pdf of its line.
// Between two midpoints the pdf is taken as linear, so the CDF is inverted on a parabola; in the
// half bins at either end of a part the CDF is inverted linearly.  The phi distribution is the
// count-weighted blend of the two theta lines around the drawn theta.
#pragma once

#include "device_model.h"

namespace mfgk {

struct AmView {
    const AmDev& a;
    const double* p;
    __device__ __forceinline__ double tcdf(bool upper, int i) const { return p[(upper ? a.tcdf_hi : a.tcdf_lo) + i]; }
    __device__ __forceinline__ double sum(bool upper, int i) const { return p[(upper ? a.sum_hi : a.sum_lo) + i]; }
    __device__ __forceinline__ const double* pcdf(bool upper) const { return p + (upper ? a.pcdf_hi : a.pcdf_lo); }
    __device__ __forceinline__ const double* ppdf(bool upper) const { return p + (upper ? a.ppdf_hi : a.ppdf_lo); }
};

__device__ __forceinline__ double am_weigh(double x, double y, double w) { return x + w * (y - x); }

// last index with v[i] <= key (-1 below the first); optionally on the blend of two lines
__device__ __forceinline__ int am_lower_index(double key, const double* v, int n) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (v[mid] <= key) lo = mid + 1; else hi = mid;
    }
    return lo - 1;
}
__device__ __forceinline__ int am_lower_index2(double key, double w, const double* a, const double* b, int n) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (am_weigh(a[mid], b[mid], w) <= key) lo = mid + 1; else hi = mid;
    }
    return lo - 1;
}

__device__ __forceinline__ double am_theta_of(const AmDev& a, double ti) {
    if ((unsigned long long)ti < (unsigned long long)a.lo) return a.limit * ti / (double)a.lo;
    return a.limit + (kPi / 2.0 - a.limit) * (ti - (double)a.lo) / (double)a.hi;
}
__device__ __forceinline__ double am_phi_of(const AmDev& a, double pi) {
    const double w = (double)a.w;
    const double c = pi < w ? pi : pi - w;
    return -kPi + 2.0 * kPi * c / w;
}

// phi pdf at fractional theta index ti, phi bin pli (taken around the circle)
__device__ double am_phi_pdf(const AmView& v, double ti, int pli) {
    const int w = v.a.w, lo = v.a.lo, hi = v.a.hi;
    const int k = ((pli % w) + w) % w;
    if (ti < 0.5) return lo > 0 ? v.ppdf(false)[k] : v.ppdf(true)[k];
    if (ti > (double)(lo + hi) - 0.5)
        return hi > 0 ? v.ppdf(true)[(size_t)w * (hi - 1) + k] : v.ppdf(false)[(size_t)w * (lo - 1) + k];
    const unsigned long long tl = (unsigned long long)(ti - 0.5);
    const double ov = ti - 0.5 - (double)tl;
    const double v0 = tl < (unsigned long long)lo ? v.ppdf(false)[tl * w + k] : v.ppdf(true)[(tl - lo) * w + k];
    const unsigned long long tn = tl + 1;
    const double v1 = tn < (unsigned long long)lo ? v.ppdf(false)[tn * w + k] : v.ppdf(true)[(tn - lo) * w + k];
    return am_weigh(v0, v1, ov);
}

// phi CDF at fractional theta index ti, phi bin pli (pli == w: one turn plus the first midpoint)
__device__ double am_phi_cdf(const AmView& v, double ti, int pli) {
    const int w = v.a.w, lo = v.a.lo, hi = v.a.hi;
    const bool upper = !(ti < (double)lo);
    const double* c = v.pcdf(upper);
    const int base = upper ? lo : 0, n = upper ? hi : lo;
    unsigned long long l0, l1;
    double ov = 0.0;
    if (ti < (double)base + 0.5) {
        l0 = l1 = 0;
    } else if (ti > (double)(base + n) - 0.5) {
        l0 = l1 = (unsigned long long)(n - 1);
    } else {
        const unsigned long long tl = (unsigned long long)(ti - 0.5);
        ov = ti - 0.5 - (double)tl;
        l0 = tl - base;
        l1 = l0 + 1;
    }
    const double v0 = pli < w ? c[l0 * w + pli] : 1.0 + c[l0 * w];
    const double v1 = pli < w ? c[l1 * w + pli] : 1.0 + c[l1 * w];
    return l0 == l1 ? v0 : am_weigh(v0, v1, ov);
}

// GenerateThetaFromAngleMap: theta of uniform r; also the lower line index and the fraction
// of a bin above its midpoint, which select the phi distribution
__device__ double am_gen_theta(const AmView& v, double r, int& out_i, double& out_ov) {
    const AmDev& a = v.a;
    const bool upper = !(r < a.lower_ratio);
    const int base = upper ? a.lo : 0, n = upper ? a.hi : a.lo;
    const double* tc = v.p + (upper ? a.tcdf_hi : a.tcdf_lo);
    const int i = base + am_lower_index(r, tc, n);
    double ov, th;
    if (i == base - 1) {
        if (!upper) { ov = 0.5 * r / tc[0]; th = am_theta_of(a, ov); }
        else { ov = 0.5 * (r - a.lower_ratio) / (tc[0] - a.lower_ratio); th = am_theta_of(a, (double)a.lo + ov); }
    } else if (i == base + n - 1) {
        const double top = upper ? 1.0 : a.lower_ratio;
        ov = 0.5 * (r - tc[i - base]) / (top - tc[i - base]);
        th = am_theta_of(a, (double)i + 0.5 + ov);
    } else {
        const int j = i - base;
        const double s0 = v.sum(upper, j), s1 = v.sum(upper, j + 1);
        if (s0 == s1) {
            ov = (r - tc[j]) / (tc[j + 1] - tc[j]);
        } else {
            const double step = am_theta_of(a, (double)i + 1.5) - am_theta_of(a, (double)i + 0.5);
            const double b = s0 / a.total / step;
            const double q = 0.5 * (s1 - s0) / a.total / (step * step);
            const double dy = r - tc[j];
            ov = ((-b + sqrt(b * b + 4.0 * q * dy)) / (2.0 * q)) / step;
        }
        th = am_theta_of(a, (double)i + 0.5 + ov);
    }
    out_i = i;
    out_ov = ov;
    return th;
}

// GeneratePhiFromAngleMap: phi in [-pi, pi) of uniform r, given the theta line index i and the
// fraction tov returned by am_gen_theta
__device__ double am_gen_phi(const AmView& v, int i, double tov, double r) {
    const AmDev& a = v.a;
    const int w = a.w, lo = a.lo, hi = a.hi;
    if (w == 1) return -kPi + 2.0 * kPi * r;
    int pi;
    double weigh;
    if (i < lo) {
        const double* c = v.pcdf(false);
        if (i == -1) {
            r += c[0];
            pi = am_lower_index(r, c, w);
            weigh = tov;
        } else if (i == lo - 1) {
            r += c[(size_t)i * w];
            pi = am_lower_index(r, c + (size_t)i * w, w);
            weigh = tov;
        } else {
            const double s0 = v.sum(false, i), s1 = v.sum(false, i + 1);
            const double div = s0 * (1.0 - tov) + s1 * tov;
            weigh = div > 0.0 ? tov * s1 / div : tov;
            r += am_weigh(c[(size_t)i * w], c[(size_t)(i + 1) * w], weigh);
            pi = am_lower_index2(r, weigh, c + (size_t)i * w, c + (size_t)(i + 1) * w, w);
        }
    } else {
        const double* c = v.pcdf(true);
        const int j = i - lo;
        if (i == lo + hi - 1) {
            r += c[(size_t)j * w];
            pi = am_lower_index(r, c + (size_t)j * w, w);
            weigh = tov;
        } else {
            const double s0 = v.sum(true, j), s1 = v.sum(true, j + 1);
            const double div = s0 * (1.0 - tov) + s1 * tov;
            weigh = div > 0.0 ? tov * s1 / div : tov;
            r += am_weigh(c[(size_t)j * w], c[(size_t)(j + 1) * w], weigh);
            pi = am_lower_index2(r, weigh, c + (size_t)j * w, c + (size_t)(j + 1) * w, w);
        }
    }
    const double ti = (double)i + 0.5 + weigh;
    if (pi == -1) return am_phi_of(a, 0.5 * r / am_phi_cdf(v, ti, 0));
    const double p0 = am_phi_pdf(v, ti, pi), p1 = am_phi_pdf(v, ti, pi + 1);
    const double c0 = am_phi_cdf(v, ti, pi);
    double pov;
    if (p0 == p1) {
        pov = (r - c0) / (am_phi_cdf(v, ti, pi + 1) - c0);
    } else {
        const double step = 2.0 * kPi / (double)w;
        const double b = p0 / step, q = 0.5 * (p1 - p0) / (step * step), dy = r - c0;
        const double D = b * b + 4.0 * q * dy;
        if (D < 0.0) pov = (r - c0) / (am_phi_cdf(v, ti, (pi + 1) % w) - c0);   // the reference wraps here
        else pov = ((-b + sqrt(D)) / (2.0 * q)) / step;
    }
    return am_phi_of(a, (double)pi + 0.5 + pov);
}

// desorption direction of source facet f by its angle map (Particle.cpp:598-622): the map holds
// incident angles, the particle leaves at pi - theta
__device__ __noinline__ void am_direction(const DevModel& M, int f, double r1, double r2, double& dx, double& dy,
                                          double& dz) {
    const AmView v{M.am_dev[M.am_of_facet[f]], M.am_pool};
    int i;
    double tov;
    const double th = kPi - am_gen_theta(v, r1, i, tov);
    const double ph = am_gen_phi(v, i, tov, r2);
    const double st = sin(th), ct = cos(th), sp = sin(ph), cp = cos(ph);
    const FacetPhysD& Ph = M.phys_d[f];
    const FacetIsectD& Rf = M.isect_d[f];
    dx = st * cp * Ph.nU[0] + st * sp * Ph.nV[0] + ct * Rf.v[0];
    dy = st * cp * Ph.nU[1] + st * sp * Ph.nV[1] + ct * Rf.v[1];
    dz = st * cp * Ph.nU[2] + st * sp * Ph.nV[2] + ct * Rf.v[2];
}

}  // namespace mfgk
