/*
 * oracle.c — CPU FP64 restatement of MolFlow+'s test-particle Monte Carlo tracer.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  Written from the reference's
 * algorithm; each function names the reference lines it follows.  Compiled with
 * -ffp-contract=off so x86 and Arm builds give identical numbers.
 */
#include "oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PI_D 3.14159265358979323846
#define KB_MOLFLOW 1.38E-23
#define MAXWELL_CDF_N 100
#define MAX_TRANSP 256

/* ------------------------------------------------------------------ RNG -- */

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11). */
void orc_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static inline double u01_from(uint32_t a, uint32_t b) {
    /* uniform double in [0,1): 52 random mantissa bits of (a:b) in [1,2), minus 1 (exact) */
    uint64_t m = (((uint64_t)a << 32) | b) >> 12;
    uint64_t bits = 0x3FF0000000000000ull | m;
    double x;
    memcpy(&x, &bits, sizeof x);
    return x - 1.0;
}

/* MT19937 (Matsumoto & Nishimura 1998) */
typedef struct { uint32_t mt[624]; int mti; } mt19937;
static void mt_seed(mt19937* g, uint32_t s) {
    g->mt[0] = s;
    for (int i = 1; i < 624; ++i)
        g->mt[i] = 1812433253u * (g->mt[i - 1] ^ (g->mt[i - 1] >> 30)) + (uint32_t)i;
    g->mti = 624;
}
static uint32_t mt_next(mt19937* g) {
    uint32_t y;
    if (g->mti >= 624) {
        for (int k = 0; k < 624; ++k) {
            y = (g->mt[k] & 0x80000000u) | (g->mt[(k + 1) % 624] & 0x7fffffffu);
            g->mt[k] = g->mt[(k + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
        }
        g->mti = 0;
    }
    y = g->mt[g->mti++];
    y ^= (y >> 11);
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= (y >> 18);
    return y;
}

typedef struct {
    int mode;
    uint32_t key[2];
    uint64_t pid;
    uint32_t inst;
    uint32_t ctr;
    int have;
    double cache;
    mt19937 mt;
} rng_t;

static void rng_start_particle(rng_t* r, uint64_t pid) {
    r->pid = pid; r->ctr = 0; r->have = 0;
}
static double rnd(rng_t* r) {
    if (r->mode == ORC_RNG_MT) {
        uint32_t a = mt_next(&r->mt), b = mt_next(&r->mt);
        return u01_from(a, b);
    }
    if (r->have) { r->have = 0; return r->cache; }
    uint32_t c[4] = {(uint32_t)r->pid, (uint32_t)(r->pid >> 32), r->ctr++, r->inst}, o[4];
    orc_philox4x32(c, r->key, o);
    r->cache = u01_from(o[2], o[3]);
    r->have = 1;
    return u01_from(o[0], o[1]);
}
/* order-independent draw for the opacity decision of facet f at trace step s */
static double rnd_opacity(rng_t* r, uint64_t step, int f) {
    if (r->mode == ORC_RNG_MT) return rnd(r);
    uint32_t c[4] = {(uint32_t)r->pid, (uint32_t)(r->pid >> 32), (uint32_t)step, (uint32_t)f + 1u}, o[4];
    uint32_t k[2] = {r->key[0] ^ (r->inst * 0x9E3779B9u), r->key[1] ^ 0xA5A5A5A5u};   /* separate stream */
    orc_philox4x32(c, k, o);
    return u01_from(o[0], o[1]);
}

/* -------------------------------------------------------------- vectors -- */
static inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static inline void cross3(const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}
static inline double norm3(const double* a) { return sqrt(dot3(a, a)); }

/* ------------------------------------------------------- interpolation -- */
/* index of the last table entry <= key, -1 if key is below the first (MathTools lower_index contract,
 * described at Particle.cpp:435-437) */
static int lower_index(double key, const double* tab, int n) {
    int lo = 0, hi = n;  /* first index with tab[i] > key */
    while (lo < hi) { int mid = (lo + hi) >> 1; if (tab[mid] <= key) lo = mid + 1; else hi = mid; }
    return lo - 1;
}
static double weigh(double a, double b, double w) { return a + (b - a) * w; }
/* InterpolateY(x, table, logX, logY, allowExtrapolate): y at x (SimulationMC.cpp:20) */
static double interp_y(double x, const double* xs, const double* ys, int n, int logx, int logy, int extrap) {
    if (n == 1) return ys[0];
    int i = lower_index(x, xs, n);
    if (i == -1) { if (!extrap) return ys[0]; i = 0; }
    else if (i == n - 1) { if (!extrap) return ys[n - 1]; i = n - 2; }
    double x0 = xs[i], x1 = xs[i + 1], y0 = ys[i], y1 = ys[i + 1];
    double w = logx ? (log10(x) - log10(x0)) / (log10(x1) - log10(x0)) : (x - x0) / (x1 - x0);
    if (logy) return pow(10.0, weigh(log10(y0), log10(y1), w));
    return weigh(y0, y1, w);
}
/* InterpolateX(y, table, ...): x where the table reaches y (Physics.cpp:7) */
static double interp_x(double y, const double* xs, const double* ys, int n, int logx, int logy, int extrap) {
    if (n == 1) return xs[0];
    int i = lower_index(y, ys, n);
    if (i == -1) { if (!extrap) return xs[0]; i = 0; }
    else if (i == n - 1) { if (!extrap) return xs[n - 1]; i = n - 2; }
    double y0 = ys[i], y1 = ys[i + 1];
    double w = logy ? (log10(y) - log10(y0)) / (log10(y1) - log10(y0)) : (y - y0) / (y1 - y0);
    if (logx) return pow(10.0, weigh(log10(xs[i]), log10(xs[i + 1]), w));
    return weigh(xs[i], xs[i + 1], w);
}

/* Generate_CDF(1 K, gasMass): flux-weighted Maxwell CDF on 100 points (CDFGeneration.cpp:54-83) */
void orc_maxwell_cdf(double gas_mass, double* speed, double* cumul) {
    const double kb = 1.38E-23, R = 8.3144621;
    double T = 1.0;
    double a = sqrt(kb * T / (gas_mass * 1.67E-27));
    double vprob = sqrt(2.0 * R * T / (gas_mass / 1000.0));
    double bin = 4.0 * vprob / (double)MAXWELL_CDF_N;
    for (int i = 0; i < MAXWELL_CDF_N; ++i) {
        double x = (double)i * bin;
        double y = (x * x) / (2.0 * a * a);
        speed[i] = x;
        cumul[i] = 1.0 - exp(-y) * (y + 1.0);
    }
}

/* -------------------------------------------------------------- model -- */
typedef struct {
    double O[3], U[3], V[3], N[3], nU[3], nV[3];
    double center[3];
    double bbmin[3], bbmax[3];
    double area;
    double invU2, invV2;   /* 1/|U|^2, 1/|V|^2 */
    double planeD;         /* N.O */
    int vstart, nv;        /* into model->v2 (u,v pairs) */
    /* parameters */
    double sticking, opacity, outgassing, temperature, sqrtT, accommodation;
    int desorb_type; double desorb_exp;
    double diffuse, specular, cos_exp;
    int two_sided, structure, link, teleport, moving;
    double texw_p, texh_p; int texw, texh; uint32_t count;
    int profile_type; double max_speed;
    int am_record, am_phi, am_lo, am_hi; double am_limit;
    int p_stick, p_opac, p_outg, p_temp;
    int sojourn; double soj_freq, soj_e;
    /* layout */
    long tex_off, dir_off, ang_off; int prof_idx;
    /* desorption */
    int id_idx;            /* integrated desorption table index, -1 none */
    struct oamap* amd;     /* angle-map desorption tables, NULL unless DES_ANGLEMAP */
    int og_w, og_h;        /* outgassing-map grid (0: none) and its extent in cells over U, V */
    double og_wp, og_hp;
} ofacet;

typedef struct { double bmin[3], bmax[3]; int left, right, first, count; } onode;

typedef struct { int n; double* t; double* v; int logx, logy; } oparam;
typedef struct { int n; double* t; double* cum; } oid;

/* one histogram set (HistogramParams): bin sizes and bin counts, offset in a moment block */
typedef struct {
    uint32_t record;
    uint64_t bounce_bin; double dist_bin, time_bin;
    long nb, nd, nt;       /* bins; 0 when not recorded */
    long off;              /* -1 when nothing is recorded */
} ohist;

static void hist_init(ohist* h, const mfg_histogram_params* p) {
    memset(h, 0, sizeof *h);
    h->off = -1;
    if (!p || !p->record) return;
    h->record = p->record;
    h->bounce_bin = p->bounce_binsize ? p->bounce_binsize : 1;
    h->dist_bin = p->distance_binsize;
    h->time_bin = p->time_binsize;
    /* bin counts restated from the sizes the reference stores with its histograms */
    if (p->record & MFG_HIST_BOUNCE) h->nb = (long)(p->bounce_max / h->bounce_bin) + 2;
    if (p->record & MFG_HIST_DISTANCE) h->nd = (long)(size_t)(p->distance_max / p->distance_binsize) + 1;
    if (p->record & MFG_HIST_TIME) h->nt = (long)(size_t)(p->time_max / p->time_binsize) + 1;
}

/* ------------------------------------------------- angle-map desorption --
 * Tables built from a recorded incident-angle map (MolflowSimFacet::InitializeAngleMap,
 * MolflowSimFacet.cpp:90-215) and the theta / phi generation of AnglemapGeneration.cpp:14-257.
 * The map has `lo` theta lines below thetaLimit and `hi` above, `w` phi bins per line.  CDFs are
 * sampled at bin midpoints; between midpoints the pdf is interpolated linearly, so the CDF is
 * inverted on a parabola. */
typedef struct oamap {
    int w, lo, hi; double limit;
    double *tcdf_lo, *tcdf_hi;     /* theta CDF at each line's midpoint */
    double *sum_lo, *sum_hi;       /* counts per theta line */
    double *pcdf_lo, *pcdf_hi;     /* phi CDF at each bin midpoint, per line */
    double *ppdf_lo, *ppdf_hi;     /* phi pdf per line, normalised to the line */
    double lower_ratio, total;
} oamap;

static void oamap_free(oamap* a) {
    if (!a) return;
    free(a->tcdf_lo); free(a->tcdf_hi); free(a->sum_lo); free(a->sum_hi);
    free(a->pcdf_lo); free(a->pcdf_hi); free(a->ppdf_lo); free(a->ppdf_hi);
    free(a);
}

/* returns NULL (all-zero map) or the tables */
static oamap* oamap_build(const uint64_t* pdf, int w, int lo, int hi, double limit) {
    oamap* a = (oamap*)calloc(1, sizeof(oamap));
    a->w = w; a->lo = lo; a->hi = hi; a->limit = limit;
    a->tcdf_lo = (double*)calloc(lo + 1, sizeof(double)); a->tcdf_hi = (double*)calloc(hi + 1, sizeof(double));
    a->sum_lo = (double*)calloc(lo + 1, sizeof(double)); a->sum_hi = (double*)calloc(hi + 1, sizeof(double));
    a->pcdf_lo = (double*)calloc((size_t)w * lo + 1, sizeof(double)); a->pcdf_hi = (double*)calloc((size_t)w * hi + 1, sizeof(double));
    a->ppdf_lo = (double*)calloc((size_t)w * lo + 1, sizeof(double)); a->ppdf_hi = (double*)calloc((size_t)w * hi + 1, sizeof(double));
    double slo = 0, sall;
    for (int t = 0; t < lo; ++t) { for (int k = 0; k < w; ++k) a->sum_lo[t] += (double)pdf[(size_t)t * w + k]; slo += a->sum_lo[t]; }
    sall = slo;
    for (int t = 0; t < hi; ++t) { for (int k = 0; k < w; ++k) a->sum_hi[t] += (double)pdf[(size_t)(lo + t) * w + k]; sall += a->sum_hi[t]; }
    if (sall == 0) { oamap_free(a); return NULL; }
    a->total = sall;
    a->lower_ratio = slo / sall;
    const double tn = 1.0 / sall;
    for (int part = 0; part < 2; ++part) {
        const int n = part ? hi : lo, base = part ? lo : 0;
        double* tcdf = part ? a->tcdf_hi : a->tcdf_lo;
        double* sum = part ? a->sum_hi : a->sum_lo;
        double* pcdf = part ? a->pcdf_hi : a->pcdf_lo;
        double* ppdf = part ? a->ppdf_hi : a->ppdf_lo;
        for (int t = 0; t < n; ++t) {
            if (t == 0) tcdf[0] = (part ? a->lower_ratio : 0.0) + 0.5 * sum[0] * tn;
            else tcdf[t] = tcdf[t - 1] + (sum[t - 1] + sum[t]) * 0.5 * tn;
            const double pn = 1.0 / sum[t];
            const uint64_t* line = pdf + (size_t)(base + t) * w;
            for (int k = 0; k < w; ++k) {
                const size_t i = (size_t)t * w + k;
                if (sum[t] == 0) {   /* empty line: uniform phi */
                    pcdf[i] = (0.5 + k) / (double)w;
                    ppdf[i] = 1.0 / (double)w;
                } else {
                    pcdf[i] = (k == 0) ? 0.5 * (double)line[0] * pn : pcdf[i - 1] + (double)(line[k - 1] + line[k]) * 0.5 * pn;
                    ppdf[i] = (double)line[k] * pn;
                }
            }
        }
    }
    return a;
}

static inline double am_weigh(double a, double b, double w) { return a + w * (b - a); }
/* last index with v[i] <= key, -1 below the first */
static int am_lower_index(double key, const double* v, int n) {
    int lo = 0, hi = n;
    while (lo < hi) { int mid = (lo + hi) >> 1; if (v[mid] <= key) lo = mid + 1; else hi = mid; }
    return lo - 1;
}
/* the same on the line interpolated between a and b with weight w */
static int am_weighed_lower_index(double key, double w, const double* a, const double* b, int n) {
    int lo = 0, hi = n;
    while (lo < hi) { int mid = (lo + hi) >> 1; if (am_weigh(a[mid], b[mid], w) <= key) lo = mid + 1; else hi = mid; }
    return lo - 1;
}
static inline int am_circ(int i, int n) { return ((i % n) + n) % n; }
static double am_theta(const oamap* a, double ti) {
    if ((size_t)ti < (size_t)a->lo) return a->limit * ti / (double)a->lo;
    return a->limit + (PI_D / 2.0 - a->limit) * (ti - (double)a->lo) / (double)a->hi;
}
static double am_phi(const oamap* a, double pi) {
    const double w = (double)a->w;
    const double c = (pi < w) ? pi : pi - w;
    return -PI_D + 2.0 * PI_D * c / w;
}
static double am_phi_pdf(const oamap* a, double ti, int pli) {
    const int w = a->w, lo = a->lo, hi = a->hi;
    const int k = am_circ(pli, w);
    if (ti < 0.5) return lo > 0 ? a->ppdf_lo[k] : a->ppdf_hi[k];
    if (ti > (double)(lo + hi) - 0.5) return hi > 0 ? a->ppdf_hi[(size_t)w * (hi - 1) + k] : a->ppdf_lo[(size_t)w * (lo - 1) + k];
    const size_t tl = (size_t)(ti - 0.5);
    const double ov = ti - 0.5 - (double)tl;
    const double v0 = tl < (size_t)lo ? a->ppdf_lo[tl * w + k] : a->ppdf_hi[(tl - lo) * w + k];
    const size_t tn = tl + 1;
    const double v1 = tn < (size_t)lo ? a->ppdf_lo[tn * w + k] : a->ppdf_hi[(tn - lo) * w + k];
    return am_weigh(v0, v1, ov);
}
static double am_phi_cdf(const oamap* a, double ti, int pli) {
    const int w = a->w, lo = a->lo, hi = a->hi;
    const double* c = (ti < (double)lo) ? a->pcdf_lo : a->pcdf_hi;
    const int base = (ti < (double)lo) ? 0 : lo, n = (ti < (double)lo) ? lo : hi;
    size_t line0, line1;
    double ov = 0.0;
    if (ti < (double)base + 0.5) { line0 = line1 = 0; }
    else if (ti > (double)(base + n) - 0.5) { line0 = line1 = (size_t)(n - 1); }
    else {
        const size_t tl = (size_t)(ti - 0.5);
        ov = ti - 0.5 - (double)tl;
        line0 = tl - base; line1 = line0 + 1;
    }
    const double v0 = pli < w ? c[line0 * w + pli] : 1.0 + c[line0 * w];
    const double v1 = pli < w ? c[line1 * w + pli] : 1.0 + c[line1 * w];
    return line0 == line1 ? v0 : am_weigh(v0, v1, ov);
}
/* GenerateThetaFromAngleMap (AnglemapGeneration.cpp:14-109) */
static double am_gen_theta(const oamap* a, double r, int* out_i, double* out_ov) {
    const int lo = a->lo, hi = a->hi;
    int i; double ov, th;
    const int upper = !(r < a->lower_ratio);
    const double* tc = upper ? a->tcdf_hi : a->tcdf_lo;
    const double* sm = upper ? a->sum_hi : a->sum_lo;
    const int base = upper ? lo : 0, n = upper ? hi : lo;
    i = base + am_lower_index(r, tc, n);
    if (i == base - 1) {   /* below the first midpoint of the part */
        if (!upper) { ov = 0.5 * r / tc[0]; th = am_theta(a, ov); }
        else { ov = 0.5 * (r - a->lower_ratio) / (tc[0] - a->lower_ratio); th = am_theta(a, (double)lo + ov); }
    } else if (i == base + n - 1) {   /* above the last midpoint of the part */
        const double top = upper ? 1.0 : a->lower_ratio;
        ov = 0.5 * (r - tc[i - base]) / (top - tc[i - base]);
        th = am_theta(a, (double)i + 0.5 + ov);
    } else {
        const int j = i - base;
        if (sm[j] == sm[j + 1]) {
            ov = (r - tc[j]) / (tc[j + 1] - tc[j]);
        } else {
            const double step = am_theta(a, (double)i + 1.5) - am_theta(a, (double)i + 0.5);
            const double c = tc[j];
            const double b = sm[j] / a->total / step;
            const double aa = 0.5 * (sm[j + 1] - sm[j]) / a->total / (step * step);
            const double dy = r - c;
            const double dx = (-b + sqrt(b * b + 4 * aa * dy)) / (2 * aa);
            ov = dx / step;
        }
        th = am_theta(a, (double)i + 0.5 + ov);
    }
    *out_i = i; *out_ov = ov;
    return th;
}
/* GeneratePhiFromAngleMap (AnglemapGeneration.cpp:120-248) */
static double am_gen_phi(const oamap* a, int i, double tov, double r) {
    const int w = a->w, lo = a->lo, hi = a->hi;
    if (w == 1) return -PI_D + 2.0 * PI_D * r;
    int pi; double weigh;
    if (i < lo) {
        if (i == -1) {
            r += a->pcdf_lo[0];
            pi = am_lower_index(r, a->pcdf_lo, w);
            weigh = tov;
        } else if (i == lo - 1) {
            r += a->pcdf_lo[(size_t)i * w];
            pi = am_lower_index(r, a->pcdf_lo + (size_t)i * w, w);
            weigh = tov;
        } else {
            const double div = a->sum_lo[i] * (1.0 - tov) + a->sum_lo[i + 1] * tov;
            weigh = div > 0.0 ? tov * a->sum_lo[i + 1] / div : tov;
            r += am_weigh(a->pcdf_lo[(size_t)i * w], a->pcdf_lo[(size_t)(i + 1) * w], weigh);
            pi = am_weighed_lower_index(r, weigh, a->pcdf_lo + (size_t)i * w, a->pcdf_lo + (size_t)(i + 1) * w, w);
        }
    } else {
        const int j = i - lo;
        if (i == lo + hi - 1) {
            r += a->pcdf_hi[(size_t)j * w];
            pi = am_lower_index(r, a->pcdf_hi + (size_t)j * w, w);
            weigh = tov;
        } else {
            const double div = a->sum_hi[j] * (1.0 - tov) + a->sum_hi[j + 1] * tov;
            weigh = div > 0.0 ? tov * a->sum_hi[j + 1] / div : tov;
            r += am_weigh(a->pcdf_hi[(size_t)j * w], a->pcdf_hi[(size_t)(j + 1) * w], weigh);
            pi = am_weighed_lower_index(r, weigh, a->pcdf_hi + (size_t)j * w, a->pcdf_hi + (size_t)(j + 1) * w, w);
        }
    }
    const double ti = (double)i + 0.5 + weigh;
    double pov;
    if (pi == -1) {
        pov = 0.5 * r / am_phi_cdf(a, ti, 0);
        return am_phi(a, pov);
    }
    const double p0 = am_phi_pdf(a, ti, pi), p1 = am_phi_pdf(a, ti, pi + 1);
    const double c0 = am_phi_cdf(a, ti, pi);
    if (p0 == p1) {
        pov = (r - c0) / (am_phi_cdf(a, ti, pi + 1) - c0);
    } else {
        const double step = 2.0 * PI_D / (double)w;
        const double b = p0 / step, aa = 0.5 * (p1 - p0) / (step * step), dy = r - c0;
        const double D = b * b + 4 * aa * dy;
        if (D < 0) pov = (r - c0) / (am_phi_cdf(a, ti, am_circ(pi + 1, w)) - c0);
        else pov = ((-b + sqrt(D)) / (2 * aa)) / step;
    }
    return am_phi(a, (double)pi + 0.5 + pov);
}

struct orc_model {
    int nf, nstruct;
    ofacet* f;
    double* v2;            /* vertices2, 2 doubles per vertex */
    double* texinc;        /* per texture cell increment (1/area) */
    /* per-structure BVH over facet ids */
    int* nnodes; onode** nodes; int** prims;
    /* moments */
    int nm; double* mstart; double* mend; double maxwin;
    double latest;
    int constant_flow, use_maxwell, low_flux, decay;
    double low_flux_cutoff, half_life, gas_mass;
    double cdf_v[MAXWELL_CDF_N], cdf_p[MAXWELL_CDF_N];
    int nparams; oparam* params;
    int nid; oid* ids;
    double* src_prefix; int* src_facet; int* src_cell; int nsrc; double src_total;
    int motion_type; double mv1[3], mv2[3];                 /* moving facets */
    int scatter, scatter_cutoff;                            /* background-gas scattering */
    int force; double torque_ref[3];                        /* force measurement */
    int log_facet; int64_t log_cap;                         /* particle logger */
    double sc_mass_ratio, sc_mfp, sc_rho, sc_cutoff_speed;
    ohist ghist;           /* global histograms; offset 0 of each moment block */
    ohist* fhist;          /* per facet, NULL when no facet records */
    mfg_state_layout L;
};

static void set_err(char* err, size_t n, const char* msg) {
    if (err && n) { strncpy(err, msg, n - 1); err[n - 1] = 0; }
}

/* Facet basis (O,U,V,N,nU,nV) and normalised polygon vertices, restating the
 * src_shared geometry initialisation contract used by the tracer:
 * N from the first non-degenerate pair of consecutive edges (right-hand rule),
 * nU along the first edge, nV = N x nU, (u,v) of every vertex rescaled to the
 * polygon's bounding rectangle, N and nV flipped when the signed area is negative.
 * Texture dims in the fixtures confirm U runs along indices[0]->indices[1]. */
static int facet_basis(ofacet* F, const double* vert, const int32_t* idx, double* v2) {
    int n = F->nv;
    const double* p0 = vert + 3 * idx[0];
    double N[3] = {0, 0, 0};
    int ok = 0;
    for (int k = 0; k + 2 < n + 0 && !ok; ++k) {
        const double* a = vert + 3 * idx[k];
        const double* b = vert + 3 * idx[k + 1];
        const double* c = vert + 3 * idx[k + 2];
        double e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
        double e2[3] = {c[0] - b[0], c[1] - b[1], c[2] - b[2]};
        cross3(e1, e2, N);
        if (norm3(N) >= 1e-11) ok = 1;
    }
    if (!ok) return -1;
    double nn = norm3(N);
    for (int i = 0; i < 3; ++i) N[i] /= nn;
    const double* p1 = vert + 3 * idx[1];
    double U[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
    double ul = norm3(U);
    if (ul <= 0) return -1;
    for (int i = 0; i < 3; ++i) U[i] /= ul;
    double V[3];
    cross3(N, U, V);
    double umin = 0, umax = 0, vmin = 0, vmax = 0;
    for (int j = 0; j < n; ++j) {
        const double* p = vert + 3 * idx[j];
        double d[3] = {p[0] - p0[0], p[1] - p0[1], p[2] - p0[2]};
        double u = (j == 0) ? 0.0 : dot3(U, d);
        double v = (j == 0) ? 0.0 : dot3(V, d);
        v2[2 * j] = u; v2[2 * j + 1] = v;
        if (u < umin) umin = u; if (u > umax) umax = u;
        if (v < vmin) vmin = v; if (v > vmax) vmax = v;
    }
    double area2 = 0;
    for (int j = 0; j < n; ++j) {
        int jn = (j + 1) % n;
        area2 += v2[2 * j] * v2[2 * jn + 1] - v2[2 * jn] * v2[2 * j + 1];
    }
    if (area2 < 0) {
        for (int i = 0; i < 3; ++i) { N[i] = -N[i]; V[i] = -V[i]; }
        vmin = 0; vmax = 0;
        for (int j = 0; j < n; ++j) {
            v2[2 * j + 1] = -v2[2 * j + 1];
            if (v2[2 * j + 1] < vmin) vmin = v2[2 * j + 1];
            if (v2[2 * j + 1] > vmax) vmax = v2[2 * j + 1];
        }
    }
    F->area = fabs(0.5 * area2);
    double uD = umax - umin, vD = vmax - vmin;
    if (uD <= 0 || vD <= 0) return -1;
    for (int i = 0; i < 3; ++i) {
        F->N[i] = N[i]; F->nU[i] = U[i]; F->nV[i] = V[i];
        F->O[i] = p0[i] + umin * U[i] + vmin * V[i];
        F->U[i] = U[i] * uD; F->V[i] = V[i] * vD;
    }
    for (int j = 0; j < n; ++j) {
        v2[2 * j] = (v2[2 * j] - umin) / uD;
        v2[2 * j + 1] = (v2[2 * j + 1] - vmin) / vD;
    }
    F->invU2 = 1.0 / dot3(F->U, F->U);
    F->invV2 = 1.0 / dot3(F->V, F->V);
    F->planeD = dot3(F->N, F->O);
    for (int i = 0; i < 3; ++i) { F->bbmin[i] = 1e300; F->bbmax[i] = -1e300; }
    for (int j = 0; j < n; ++j) {
        const double* p = vert + 3 * idx[j];
        for (int i = 0; i < 3; ++i) {
            if (p[i] < F->bbmin[i]) F->bbmin[i] = p[i];
            if (p[i] > F->bbmax[i]) F->bbmax[i] = p[i];
        }
    }
    for (int i = 0; i < 3; ++i) F->center[i] = 0.5 * (F->bbmin[i] + F->bbmax[i]);
    return 0;
}

/* Crossing-number point-in-polygon in (u,v) space (IsInFacet contract, Particle.cpp:148,540). */
static int in_polygon(const double* v2, int n, double u, double v) {
    int inside = 0;
    for (int i = 0, j = n - 1; i < n; j = i++) {
        double ui = v2[2 * i], vi = v2[2 * i + 1], uj = v2[2 * j], vj = v2[2 * j + 1];
        if ((vi > v) != (vj > v)) {
            double cr = (uj - ui) * (v - vi) - (u - ui) * (vj - vi);
            if ((cr > 0) == (vj > vi)) inside = !inside;
        }
    }
    return inside;
}

/* area of polygon (u,v in cm) clipped to an axis-aligned rectangle, Sutherland-Hodgman */
static double clip_area(const double* poly, int n, double x0, double y0, double x1, double y1) {
    double bufA[2 * 4096], bufB[2 * 4096];
    if (n > 1000) return -1;
    int m = n;
    memcpy(bufA, poly, sizeof(double) * 2 * n);
    double* in = bufA; double* out = bufB;
    for (int edge = 0; edge < 4; ++edge) {
        int k = 0;
        for (int i = 0; i < m; ++i) {
            double* P = in + 2 * i; double* Q = in + 2 * ((i + 1) % m);
            double dp, dq;
            switch (edge) {
                case 0: dp = P[0] - x0; dq = Q[0] - x0; break;
                case 1: dp = x1 - P[0]; dq = x1 - Q[0]; break;
                case 2: dp = P[1] - y0; dq = Q[1] - y0; break;
                default: dp = y1 - P[1]; dq = y1 - Q[1]; break;
            }
            if (dp >= 0) { out[2 * k] = P[0]; out[2 * k + 1] = P[1]; ++k; }
            if ((dp >= 0) != (dq >= 0)) {
                double t = dp / (dp - dq);
                out[2 * k] = P[0] + t * (Q[0] - P[0]);
                out[2 * k + 1] = P[1] + t * (Q[1] - P[1]);
                ++k;
            }
        }
        m = k;
        double* tmp = in; in = out; out = tmp;
        if (m == 0) return 0.0;
    }
    double a = 0;
    for (int i = 0; i < m; ++i) {
        int j = (i + 1) % m;
        a += in[2 * i] * in[2 * j + 1] - in[2 * j] * in[2 * i + 1];
    }
    return fabs(0.5 * a);
}

/* ---------------------------------------------------------------- BVH -- */
typedef struct { int* ids; double* cen; const ofacet* f; onode* nodes; int nn, cap; int* prims; int np; } bvh_build;

static int bvh_rec(bvh_build* B, int* ids, int n) {
    if (B->nn >= B->cap) { B->cap *= 2; B->nodes = (onode*)realloc(B->nodes, sizeof(onode) * B->cap); }
    int me = B->nn++;
    onode nd;
    for (int i = 0; i < 3; ++i) { nd.bmin[i] = 1e300; nd.bmax[i] = -1e300; }
    for (int k = 0; k < n; ++k) {
        const ofacet* F = &B->f[ids[k]];
        for (int i = 0; i < 3; ++i) {
            if (F->bbmin[i] < nd.bmin[i]) nd.bmin[i] = F->bbmin[i];
            if (F->bbmax[i] > nd.bmax[i]) nd.bmax[i] = F->bbmax[i];
        }
    }
    nd.left = nd.right = -1;
    if (n <= 2) {   /* 2 facets per leaf (MolflowSimulation.cpp:79) */
        nd.first = B->np; nd.count = n;
        for (int k = 0; k < n; ++k) B->prims[B->np++] = ids[k];
        B->nodes[me] = nd;
        return me;
    }
    /* binned SAH on centroids, 16 bins per axis */
    double cmin[3] = {1e300, 1e300, 1e300}, cmax[3] = {-1e300, -1e300, -1e300};
    for (int k = 0; k < n; ++k)
        for (int i = 0; i < 3; ++i) {
            double c = B->f[ids[k]].center[i];
            if (c < cmin[i]) cmin[i] = c; if (c > cmax[i]) cmax[i] = c;
        }
    enum { NB = 16 };
    double best = 1e300; int bax = -1; double bsplit = 0;
    for (int ax = 0; ax < 3; ++ax) {
        double ext = cmax[ax] - cmin[ax];
        if (ext <= 0) continue;
        int cnt[NB] = {0}; double bmn[NB][3], bmx[NB][3];
        for (int b = 0; b < NB; ++b) for (int i = 0; i < 3; ++i) { bmn[b][i] = 1e300; bmx[b][i] = -1e300; }
        for (int k = 0; k < n; ++k) {
            const ofacet* F = &B->f[ids[k]];
            int b = (int)((F->center[ax] - cmin[ax]) / ext * NB); if (b >= NB) b = NB - 1; if (b < 0) b = 0;
            cnt[b]++;
            for (int i = 0; i < 3; ++i) {
                if (F->bbmin[i] < bmn[b][i]) bmn[b][i] = F->bbmin[i];
                if (F->bbmax[i] > bmx[b][i]) bmx[b][i] = F->bbmax[i];
            }
        }
        for (int s = 1; s < NB; ++s) {
            double lmn[3] = {1e300, 1e300, 1e300}, lmx[3] = {-1e300, -1e300, -1e300};
            double rmn[3] = {1e300, 1e300, 1e300}, rmx[3] = {-1e300, -1e300, -1e300};
            int lc = 0, rc = 0;
            for (int b = 0; b < s; ++b) { lc += cnt[b]; for (int i = 0; i < 3; ++i) { if (bmn[b][i] < lmn[i]) lmn[i] = bmn[b][i]; if (bmx[b][i] > lmx[i]) lmx[i] = bmx[b][i]; } }
            for (int b = s; b < NB; ++b) { rc += cnt[b]; for (int i = 0; i < 3; ++i) { if (bmn[b][i] < rmn[i]) rmn[i] = bmn[b][i]; if (bmx[b][i] > rmx[i]) rmx[i] = bmx[b][i]; } }
            if (!lc || !rc) continue;
            double dl[3] = {lmx[0] - lmn[0], lmx[1] - lmn[1], lmx[2] - lmn[2]};
            double dr[3] = {rmx[0] - rmn[0], rmx[1] - rmn[1], rmx[2] - rmn[2]};
            double sal = dl[0] * dl[1] + dl[1] * dl[2] + dl[2] * dl[0];
            double sar = dr[0] * dr[1] + dr[1] * dr[2] + dr[2] * dr[0];
            double cost = sal * lc + sar * rc;
            if (cost < best) { best = cost; bax = ax; bsplit = cmin[ax] + ext * (double)s / NB; }
        }
    }
    int mid;
    if (bax < 0) {
        mid = n / 2;   /* all centroids equal: split the list */
    } else {
        int i = 0, j = n - 1;
        while (i <= j) {
            if (B->f[ids[i]].center[bax] < bsplit) ++i;
            else { int t = ids[i]; ids[i] = ids[j]; ids[j] = t; --j; }
        }
        mid = i;
        if (mid == 0 || mid == n) mid = n / 2;
    }
    nd.first = -1; nd.count = 0;
    B->nodes[me] = nd;
    int l = bvh_rec(B, ids, mid);
    int r = bvh_rec(B, ids + mid, n - mid);
    B->nodes[me].left = l; B->nodes[me].right = r;
    return me;
}

static void build_structure_bvh(orc_model* M, int s) {
    int* ids = (int*)malloc(sizeof(int) * (M->nf + 1));
    int n = 0;
    for (int i = 0; i < M->nf; ++i)
        if (M->f[i].structure == -1 || M->f[i].structure == s) ids[n++] = i;
    bvh_build B;
    B.f = M->f; B.cap = 2 * n + 2; B.nodes = (onode*)malloc(sizeof(onode) * B.cap); B.nn = 0;
    B.prims = (int*)malloc(sizeof(int) * (n + 1)); B.np = 0;
    if (n > 0) bvh_rec(&B, ids, n);
    M->nodes[s] = B.nodes; M->nnodes[s] = B.nn; M->prims[s] = B.prims;
    free(ids);
}

/* ---------------------------------------------------- Generate_ID -------- */
/* Integrated desorption for a time-dependent outgassing parameter (IDGeneration.cpp:45-207). */
static void generate_id(const oparam* P, double latest, oid* out) {
    int cap = 16 + 12 * (P->n + 2);
    double* ot = (double*)malloc(sizeof(double) * (P->n + 3));
    double* ov = (double*)malloc(sizeof(double) * (P->n + 3));
    int no = 0;
    out->t = (double*)malloc(sizeof(double) * cap);
    out->cum = (double*)malloc(sizeof(double) * cap);
    int n = 0;
    int ia;
    for (ia = 0; ia < P->n && P->t[ia] < latest; ++ia) {}
    int last_before = 0;
    if (ia >= P->n) { ia = P->n - 1; last_before = 1; }
    out->t[n] = 0.0; out->cum[n] = 0.0; ++n;
    if (P->t[0] > 0.0) { ot[no] = 0.0; ov[no] = P->v[0]; ++no; }
    if (last_before) {
        for (int i = 0; i < P->n; ++i) { ot[no] = P->t[i]; ov[no] = P->v[i]; ++no; }
        ot[no] = latest; ov[no] = ov[no - 1]; ++no;
    } else {
        for (int i = 0; i < ia; ++i) { ot[no] = P->t[i]; ov[no] = P->v[i]; ++no; }
        if (!(fabs(ot[no - 1] - latest) < 1e-10)) {
            ot[no] = latest;
            ov[no] = interp_y(latest, P->t, P->v, P->n, P->logx, P->logy, 1);
            ++no;
        }
    }
    for (int i = 1; i < no; ++i) {
        if (fabs(ov[i] - ov[i - 1]) < 1e-10) {
            out->t[n] = ot[i];
            out->cum[n] = out->cum[n - 1] + (ot[i] - ot[i - 1]) * ov[i] * 0.1;  /* MBARLS_TO_PAM3S */
            ++n;
        } else {
            const int steps = 10;
            double t0 = ot[i - 1], t1 = ot[i], dt = t1 - t0, delta = 1.0 / steps;
            double lt0 = 0, lt1 = 0, ldt = 0, sub_dt = 0, sub_ldt = 0;
            if (P->logx) {
                lt0 = (t0 == 0) ? -99 : log10(t0); lt1 = log10(t1); ldt = lt1 - lt0; sub_ldt = ldt * delta;
            } else sub_dt = dt * delta;
            double pv = ov[i - 1], pt = t0;
            double frac = delta;
            while (frac < 1.0001) {
                double et = P->logx ? pow(10.0, lt0 + frac * ldt) : t0 + frac * dt;
                double ev = interp_y(et, ot, ov, no, P->logx, P->logy, 1);
                double g;
                if (!P->logx && !P->logy) g = sub_dt * 0.5 * (pv + ev);
                else if (P->logx && !P->logy) g = (ev - pv) * (pt - et) / log(et / pt) - pt * pv + et * ev;
                else if (!P->logx && P->logy) {
                    double le = (ev > 0) ? log10(ev) : -99, lp = (pt > 0) ? log10(pv) : -99;
                    g = sub_dt * (ev - pv) * log10(exp(1.0)) / (le - lp);
                } else {
                    double le = (ev > 0) ? log10(ev) : -99, lp = (pt > 0) ? log10(pv) : -99;
                    double m = (le - lp) / sub_ldt;
                    if (m != -1.0) g = pv / pow(pt, m) / (m + 1.0) * (pow(et, m + 1.0) - pow(pt, m + 1.0));
                    else g = pt * pv * sub_ldt;
                }
                if (n >= cap) { cap *= 2; out->t = (double*)realloc(out->t, sizeof(double) * cap); out->cum = (double*)realloc(out->cum, sizeof(double) * cap); }
                out->t[n] = et; out->cum[n] = out->cum[n - 1] + g * 0.1; ++n;
                pv = ev; pt = et;
                frac += delta;
            }
        }
    }
    out->n = n;
    free(ot); free(ov);
}

/* ------------------------------------------------------- model create -- */
#define OPT(ptr, i, def) ((ptr) ? (ptr)[i] : (def))

int orc_model_create(const mfg_model_desc* d, orc_model** out, char* err, size_t errlen) {
    *out = NULL;
    if (!d || d->abi_version != MFG_ABI_VERSION) { set_err(err, errlen, "bad descriptor version"); return MFG_ERR_INVALID_MODEL; }
    if (d->n_facets <= 0 || d->n_vertices <= 0 || !d->vertices || !d->facet_vertex_start || !d->facet_vertex_index) {
        set_err(err, errlen, "empty geometry"); return MFG_ERR_INVALID_MODEL;
    }
    orc_model* M = (orc_model*)calloc(1, sizeof(orc_model));
    M->nf = d->n_facets;
    M->nstruct = d->n_structures > 0 ? d->n_structures : 1;
    M->f = (ofacet*)calloc(M->nf, sizeof(ofacet));
    int nvt = d->facet_vertex_start[M->nf];
    M->v2 = (double*)malloc(sizeof(double) * 2 * (nvt + 1));
    M->constant_flow = d->constant_flow; M->use_maxwell = d->use_maxwell;
    M->low_flux = d->low_flux_mode; M->low_flux_cutoff = d->low_flux_cutoff;
    M->motion_type = d->motion_type;
    for (int k = 0; k < 3; ++k) { M->mv1[k] = d->motion_vector1[k]; M->mv2[k] = d->motion_vector2[k]; }
    M->scatter = d->scatter_enabled; M->scatter_cutoff = d->scatter_cutoff_enabled;
    M->force = d->enable_force_measurement != 0;
    M->log_facet = (d->log_facet >= 0 && d->log_facet < d->n_facets && d->log_limit > 0) ? d->log_facet : -1;
    M->log_cap = M->log_facet >= 0 ? d->log_limit : 0;
    for (int k = 0; k < 3; ++k) M->torque_ref[k] = d->torque_ref_point[k];
    M->sc_mass_ratio = d->scatter_mass_ratio; M->sc_mfp = d->scatter_mean_free_path_cm;
    M->sc_rho = d->scatter_rho; M->sc_cutoff_speed = d->scatter_cutoff_speed;
    M->decay = d->enable_decay; M->half_life = d->half_life; M->gas_mass = d->gas_mass;
    char msg[256];
    size_t am_cursor = 0;   /* position in desc->desorb_anglemap */
    for (int i = 0; i < M->nf; ++i) {
        ofacet* F = &M->f[i];
        F->vstart = d->facet_vertex_start[i];
        F->nv = d->facet_vertex_start[i + 1] - F->vstart;
        if (F->nv < 3) { snprintf(msg, sizeof msg, "facet %d has fewer than 3 vertices", i + 1); set_err(err, errlen, msg); orc_model_destroy(M); return MFG_ERR_INVALID_MODEL; }
        for (int k = 0; k < F->nv; ++k) {
            int vi = d->facet_vertex_index[F->vstart + k];
            if (vi < 0 || vi >= d->n_vertices) { set_err(err, errlen, "vertex index out of range"); orc_model_destroy(M); return MFG_ERR_INVALID_MODEL; }
        }
        if (facet_basis(F, d->vertices, d->facet_vertex_index + F->vstart, M->v2 + 2 * F->vstart) != 0) {
            snprintf(msg, sizeof msg, "facet %d is degenerate", i + 1); set_err(err, errlen, msg); orc_model_destroy(M); return MFG_ERR_INVALID_MODEL;
        }
        F->sticking = OPT(d->sticking, i, 0.0);
        F->opacity = OPT(d->opacity, i, 1.0);
        if (F->opacity < 0) F->opacity = 0; if (F->opacity > 1) F->opacity = 1;   /* clamp (MolflowSimGeom.cpp:148-150) */
        F->outgassing = OPT(d->outgassing, i, 0.0);
        F->temperature = OPT(d->temperature, i, 293.15);
        F->sqrtT = sqrt(F->temperature);
        F->accommodation = OPT(d->accommodation, i, 1.0);
        F->desorb_type = OPT(d->desorb_type, i, MFG_DES_NONE);
        F->desorb_exp = OPT(d->desorb_exponent, i, 0.0);
        F->diffuse = OPT(d->refl_diffuse, i, 1.0);
        F->specular = OPT(d->refl_specular, i, 0.0);
        F->cos_exp = OPT(d->refl_cos_exponent, i, 0.0);
        F->two_sided = OPT(d->is_2sided, i, 0);
        F->structure = OPT(d->structure, i, 0);
        F->link = OPT(d->link_dest, i, 0);
        F->teleport = OPT(d->teleport_dest, i, 0);
        F->texw_p = OPT(d->tex_width, i, 0.0);
        F->texh_p = OPT(d->tex_height, i, 0.0);
        F->count = OPT(d->count_flags, i, 0u);
        F->profile_type = OPT(d->profile_type, i, MFG_PROFILE_NONE);
        F->max_speed = OPT(d->max_speed, i, 0.0);
        F->am_record = OPT(d->anglemap_record, i, 0);
        F->am_phi = OPT(d->anglemap_phi_width, i, 0);
        F->am_limit = OPT(d->anglemap_theta_limit, i, 1.570796326);
        F->am_lo = OPT(d->anglemap_theta_lower_res, i, 0);
        F->am_hi = OPT(d->anglemap_theta_higher_res, i, 0);
        F->p_stick = OPT(d->sticking_param, i, -1);
        F->p_opac = OPT(d->opacity_param, i, -1);
        F->p_outg = OPT(d->outgassing_param, i, -1);
        F->p_temp = OPT(d->temperature_param, i, -1);
        F->sojourn = OPT(d->enable_sojourn, i, 0);
        F->soj_freq = OPT(d->sojourn_freq, i, 0.0);
        F->soj_e = OPT(d->sojourn_e, i, 0.0);
        if (F->link < 0 || F->link > M->nstruct) {
            set_err(err, errlen, "structure link destination out of range");
            orc_model_destroy(M);
            return MFG_ERR_INVALID_MODEL;
        }
        F->moving = OPT(d->is_moving, i, 0);
        if (F->desorb_type == MFG_DES_ANGLEMAP) {
            const int w = F->am_phi, lo = F->am_lo, hi = F->am_hi;
            const uint64_t* map = d->desorb_anglemap ? d->desorb_anglemap + am_cursor : NULL;
            if (w > 0 && lo >= 0 && hi >= 0 && lo + hi > 0) am_cursor += (size_t)w * (lo + hi);
            if (map && w > 0 && lo >= 0 && hi >= 0 && lo + hi > 0) F->amd = oamap_build(map, w, lo, hi, F->am_limit);
            if (!F->amd) {
                snprintf(msg, sizeof msg, "facet %d desorbs by angle map but has no recorded angle map", i + 1);
                set_err(err, errlen, msg); orc_model_destroy(M); return MFG_ERR_INVALID_MODEL;
            }
        }
        if (F->teleport < -1) {
            snprintf(msg, sizeof msg, "facet %d: teleport destination out of range", i + 1);
            set_err(err, errlen, msg); orc_model_destroy(M); return MFG_ERR_INVALID_MODEL;
        }
        if (F->structure < -1 || F->structure >= M->nstruct) { set_err(err, errlen, "structure index out of range"); orc_model_destroy(M); return MFG_ERR_INVALID_MODEL; }
        int textured = (F->texw_p * F->texh_p) > 0;   /* isTextured (LoaderXML.cpp:1111) */
        if (textured) {
            F->texw = (int)ceil(F->texw_p - 1e-9); F->texh = (int)ceil(F->texh_p - 1e-9);
            if (F->texw < 1) F->texw = 1; if (F->texh < 1) F->texh = 1;
        } else { F->texw = F->texh = 0; F->count = 0; }
    }
    /* time-dependent parameters */
    M->nparams = d->n_params;
    if (M->nparams > 0) {
        M->params = (oparam*)calloc(M->nparams, sizeof(oparam));
        for (int p = 0; p < M->nparams; ++p) {
            int s = d->param_start[p], e = d->param_start[p + 1];
            M->params[p].n = e - s;
            M->params[p].t = (double*)malloc(sizeof(double) * (e - s + 1));
            M->params[p].v = (double*)malloc(sizeof(double) * (e - s + 1));
            memcpy(M->params[p].t, d->param_t + s, sizeof(double) * (e - s));
            memcpy(M->params[p].v, d->param_v + s, sizeof(double) * (e - s));
            M->params[p].logx = OPT(d->param_log_x, p, 0);
            M->params[p].logy = OPT(d->param_log_y, p, 0);
            if (M->params[p].n < 1) { set_err(err, errlen, "empty parameter"); orc_model_destroy(M); return MFG_ERR_INVALID_MODEL; }
        }
    }
    for (int i = 0; i < M->nf; ++i) {
        ofacet* F = &M->f[i];
        if (F->p_stick >= M->nparams || F->p_opac >= M->nparams || F->p_outg >= M->nparams || F->p_temp >= M->nparams) {
            set_err(err, errlen, "facet refers to a missing time-dependent parameter"); orc_model_destroy(M); return MFG_ERR_INVALID_MODEL;
        }
    }
    /* moments and latest moment (PrepareToRun, MolflowSimGeom.cpp:202-206; CalcIntervalCache :255-261) */
    M->nm = d->n_moments;
    if (M->nm > 0) {
        M->mstart = (double*)malloc(sizeof(double) * M->nm);
        M->mend = (double*)malloc(sizeof(double) * M->nm);
        M->maxwin = 0;
        for (int k = 0; k < M->nm; ++k) {
            M->mstart[k] = d->moment_time[k] - 0.5 * d->moment_window[k];
            M->mend[k] = d->moment_time[k] + 0.5 * d->moment_window[k];
            if (d->moment_window[k] > M->maxwin) M->maxwin = d->moment_window[k];
            if (k > 0 && d->moment_time[k] < d->moment_time[k - 1]) { set_err(err, errlen, "moments must be sorted"); orc_model_destroy(M); return MFG_ERR_INVALID_MODEL; }
        }
        M->latest = d->moment_time[M->nm - 1] + 0.5 * d->moment_window[M->nm - 1];
    } else {
        M->latest = d->time_window * 0.5;
    }
    orc_maxwell_cdf(M->gas_mass, M->cdf_v, M->cdf_p);
    /* integrated desorption per outgassing parameter */
    M->ids = (oid*)calloc(M->nparams + 1, sizeof(oid));
    M->nid = 0;
    int* pid2id = (int*)malloc(sizeof(int) * (M->nparams + 1));
    for (int p = 0; p < M->nparams; ++p) pid2id[p] = -1;
    for (int i = 0; i < M->nf; ++i) {
        ofacet* F = &M->f[i];
        F->id_idx = -1;
        if (F->p_outg >= 0) {
            if (pid2id[F->p_outg] < 0) { generate_id(&M->params[F->p_outg], M->latest, &M->ids[M->nid]); pid2id[F->p_outg] = M->nid++; }
            F->id_idx = pid2id[F->p_outg];
        }
    }
    free(pid2id);
    /* source table: StartFromSource facet weights (Particle.cpp:421-464).  A facet with an
     * outgassing map desorbs by its cells (Particle.cpp:425-446; MolflowSimGeom.cpp:303-310):
     * here one entry per cell of non-zero rate, searched like the facets. */
    size_t nmapcells = 0;
    for (int i = 0; i < M->nf; ++i) {
        ofacet* F = &M->f[i];
        F->og_w = OPT(d->outgassing_map_width, i, 0);
        F->og_h = OPT(d->outgassing_map_height, i, 0);
        if (F->og_w > 0 && F->og_h > 0) {
            if (!d->outgassing_map) { set_err(err, errlen, "outgassing map missing"); orc_model_destroy(M); return MFG_ERR_INVALID_MODEL; }
            F->og_wp = sqrt(dot3(F->U, F->U)) * OPT(d->outgassing_map_ratio_u, i, 0.0);
            F->og_hp = sqrt(dot3(F->V, F->V)) * OPT(d->outgassing_map_ratio_v, i, 0.0);
            if (!(F->og_wp > F->og_w - 1.0 && F->og_hp > F->og_h - 1.0)) {
                set_err(err, errlen, "outgassing map has more cells than its ratio puts on the facet"); orc_model_destroy(M); return MFG_ERR_INVALID_MODEL;
            }
            nmapcells += (size_t)F->og_w * F->og_h;
        } else F->og_w = F->og_h = 0;
    }
    M->src_prefix = (double*)malloc(sizeof(double) * (M->nf + nmapcells + 1));
    M->src_facet = (int*)malloc(sizeof(int) * (M->nf + nmapcells + 1));
    M->src_cell = (int*)malloc(sizeof(int) * (M->nf + nmapcells + 1));
    M->nsrc = 0;
    double sum = 0;
    size_t cursor = 0;
    for (int i = 0; i < M->nf; ++i) {
        ofacet* F = &M->f[i];
        const int ncell = F->og_w * F->og_h;
        const double* cells = ncell ? d->outgassing_map + cursor : NULL;
        cursor += (size_t)ncell;
        if (F->desorb_type == MFG_DES_NONE) continue;
        if (ncell) {
            double tot = 0;
            for (int c = 0; c < ncell; ++c) {
                if (!(cells[c] >= 0)) { set_err(err, errlen, "negative outgassing-map cell"); orc_model_destroy(M); return MFG_ERR_INVALID_MODEL; }
                tot += cells[c];
            }
            if (!(tot > 0)) continue;
            if (F->structure == -1) { set_err(err, errlen, "a facet in all structures cannot desorb"); orc_model_destroy(M); return MFG_ERR_INVALID_MODEL; }
            for (int c = 0; c < ncell; ++c) {
                if (!(cells[c] > 0)) continue;
                sum += M->latest * cells[c] / (KB_MOLFLOW * F->temperature);
                M->src_prefix[M->nsrc] = sum; M->src_facet[M->nsrc] = i; M->src_cell[M->nsrc] = c; M->nsrc++;
            }
            continue;
        }
        double w = (F->id_idx >= 0 ? M->ids[F->id_idx].cum[M->ids[F->id_idx].n - 1] : M->latest * F->outgassing)
                   / (KB_MOLFLOW * F->temperature);
        if (!(w > 0)) continue;
        if (F->structure == -1) { set_err(err, errlen, "a facet in all structures cannot desorb"); orc_model_destroy(M); return MFG_ERR_INVALID_MODEL; }
        sum += w;
        M->src_prefix[M->nsrc] = sum; M->src_facet[M->nsrc] = i; M->src_cell[M->nsrc] = -1; M->nsrc++;
    }
    M->src_total = sum;
    for (int i = 0; i < M->nf; ++i) {   /* a teleport into a facet of all structures has no structure to go on in */
        const int t = M->f[i].teleport;
        if (t > 0 && t <= M->nf && M->f[t - 1].structure == -1) {
            set_err(err, errlen, "teleport destination is in all structures"); orc_model_destroy(M); return MFG_ERR_INVALID_MODEL;
        }
    }
    /* layout + texture increments (Initializer.cpp:433-456) */
    mfg_state_layout* L = &M->L;
    memset(L, 0, sizeof *L);
    L->n_facets = M->nf; L->n_moments = M->nm;
    for (int i = 0; i < M->nf; ++i) {
        ofacet* F = &M->f[i];
        F->tex_off = -1; F->dir_off = -1; F->ang_off = -1; F->prof_idx = -1;
        if (F->texw > 0) { F->tex_off = L->texture_cells; L->texture_cells += (long)F->texw * F->texh; }
        if ((F->count & MFG_COUNT_DIR) && F->texw > 0) { F->dir_off = L->direction_cells; L->direction_cells += (long)F->texw * F->texh; }
        if (F->profile_type != MFG_PROFILE_NONE) F->prof_idx = (int)L->profile_facets++;
        if (F->am_record && F->am_phi > 0 && F->am_lo >= 0 && F->am_hi >= 0 && F->am_lo + F->am_hi > 0) { F->ang_off = L->anglemap_cells; L->anglemap_cells += (long)F->am_phi * (F->am_lo + F->am_hi); }
    }
    int64_t B = 1 + M->nm;
    L->n_global = MFG_G_N;
    L->n_facet_counts = B * M->nf * MFG_FC_N;
    L->n_facet_sums = B * M->nf * MFG_FS_N;
    L->n_texture = B * L->texture_cells * 3;
    L->n_profile = B * L->profile_facets * MFG_PROFILE_SIZE * 3;
    L->n_direction = B * L->direction_cells * 4;
    L->n_anglemap = L->anglemap_cells;
    hist_init(&M->ghist, &d->global_histogram);
    long hb = 0;
    if (M->ghist.record) { M->ghist.off = 0; hb = M->ghist.nb + M->ghist.nd + M->ghist.nt; }
    if (d->facet_histogram) {
        M->fhist = (ohist*)calloc(M->nf, sizeof(ohist));
        for (int i = 0; i < M->nf; ++i) {
            hist_init(&M->fhist[i], &d->facet_histogram[i]);
            if (M->fhist[i].record) { M->fhist[i].off = hb; hb += M->fhist[i].nb + M->fhist[i].nd + M->fhist[i].nt; }
        }
    }
    L->histogram_bins = hb;
    L->n_histogram = B * hb;
    L->n_force = M->force ? B * (int64_t)M->nf * 9 : 0;
    M->texinc = (double*)calloc(L->texture_cells + 1, sizeof(double));
    for (int i = 0; i < M->nf; ++i) {
        ofacet* F = &M->f[i];
        if (F->texw <= 0) continue;
        double lu = norm3(F->U), lv = norm3(F->V);
        double rw = lu / F->texw_p, rh = lv / F->texh_p;
        double sides = F->two_sided ? 2.0 : 1.0;
        double* poly = (double*)malloc(sizeof(double) * 2 * F->nv);
        for (int k = 0; k < F->nv; ++k) { poly[2 * k] = M->v2[2 * (F->vstart + k)] * lu; poly[2 * k + 1] = M->v2[2 * (F->vstart + k) + 1] * lv; }
        for (int y = 0; y < F->texh; ++y)
            for (int x = 0; x < F->texw; ++x) {
                double a = clip_area(poly, F->nv, x * rw, y * rh, (x + 1) * rw, (y + 1) * rh);
                if (a < 0) a = rw * rh;
                M->texinc[F->tex_off + (long)y * F->texw + x] = (a > 1e-12 * rw * rh) ? 1.0 / (a * sides) : 0.0;
            }
        free(poly);
    }
    M->nnodes = (int*)calloc(M->nstruct, sizeof(int));
    M->nodes = (onode**)calloc(M->nstruct, sizeof(onode*));
    M->prims = (int**)calloc(M->nstruct, sizeof(int*));
    for (int s = 0; s < M->nstruct; ++s) build_structure_bvh(M, s);
    *out = M;
    return MFG_OK;
}

void orc_model_destroy(orc_model* M) {
    if (!M) return;
    free(M->v2); free(M->texinc);
    if (M->nodes) for (int s = 0; s < M->nstruct; ++s) { free(M->nodes[s]); free(M->prims[s]); }
    free(M->nodes); free(M->prims); free(M->nnodes);
    free(M->mstart); free(M->mend);
    for (int p = 0; p < M->nparams; ++p) { free(M->params[p].t); free(M->params[p].v); }
    free(M->params);
    if (M->ids) for (int k = 0; k < M->nid; ++k) { free(M->ids[k].t); free(M->ids[k].cum); }
    free(M->ids);
    free(M->src_prefix); free(M->src_facet); free(M->src_cell);
    free(M->fhist);
    if (M->f) for (int i = 0; i < M->nf; ++i) oamap_free(M->f[i].amd);
    free(M->f);
    free(M);
}

int orc_layout(const orc_model* M, mfg_state_layout* out) { *out = M->L; return MFG_OK; }

int orc_facet_geometry(const orc_model* M, double* o18, double* area) {
    for (int i = 0; i < M->nf; ++i) {
        const ofacet* F = &M->f[i];
        double* o = o18 + 18 * i;
        for (int k = 0; k < 3; ++k) { o[k] = F->O[k]; o[3 + k] = F->U[k]; o[6 + k] = F->V[k]; o[9 + k] = F->N[k]; o[12 + k] = F->nU[k]; o[15 + k] = F->nV[k]; }
        if (area) area[i] = F->area;
    }
    return MFG_OK;
}

/* ---------------------------------------------------------- intersect -- */
typedef struct { int facet; double t, u, v; } ohit;
typedef struct {
    int hard; double t, u, v;
    int ntr; ohit* tr;   /* transparent passes: every one the ray crosses (a per-thread buffer that grows) */
    uint64_t nodes, prims;
} oisect;
static _Thread_local ohit* g_tr_buf = NULL;
static _Thread_local int g_tr_cap = 0;
static void add_pass(oisect* H, int fi, double t, double u, double v) {
    if (H->ntr == g_tr_cap) {
        int cap = g_tr_cap ? 2 * g_tr_cap : MAX_TRANSP;
        ohit* nb = (ohit*)realloc(g_tr_buf, (size_t)cap * sizeof(ohit));
        if (!nb) return;   /* out of memory: the pass is dropped */
        g_tr_buf = nb;
        g_tr_cap = cap;
    }
    H->tr = g_tr_buf;
    H->tr[H->ntr].facet = fi; H->tr[H->ntr].t = t; H->tr[H->ntr].u = u; H->tr[H->ntr].v = v; H->ntr++;
}

static double param_at(const orc_model* M, int p, double t) {
    const oparam* P = &M->params[p];
    return interp_y(t, P->t, P->v, P->n, P->logx, P->logy, 0);
}

/* Ray/facet test: plane hit in front of the ray, (u,v) inside the bounding rectangle,
 * inside the polygon; back faces of one-sided facets are invisible. */
static int facet_hit(const orc_model* M, const ofacet* F, const double* o, const double* d, double* t, double* u, double* v) {
    double den = dot3(F->N, d);
    if (!F->two_sided && den >= 0.0) return 0;
    if (den == 0.0) return 0;
    double tt = (F->planeD - dot3(F->N, o)) / den;
    if (!(tt > 0.0)) return 0;
    double p[3] = {o[0] + tt * d[0] - F->O[0], o[1] + tt * d[1] - F->O[1], o[2] + tt * d[2] - F->O[2]};
    double uu = dot3(p, F->U) * F->invU2;
    if (uu < 0.0 || uu > 1.0) return 0;
    double vv = dot3(p, F->V) * F->invV2;
    if (vv < 0.0 || vv > 1.0) return 0;
    if (!in_polygon(M->v2 + 2 * F->vstart, F->nv, uu, vv)) return 0;
    *t = tt; *u = uu; *v = vv;
    return 1;
}

static inline int box_hit(const onode* n, const double* o, const double* inv, double tmax) {
    double t0 = 0.0, t1 = tmax;
    for (int a = 0; a < 3; ++a) {
        double ta = (n->bmin[a] - o[a]) * inv[a];
        double tb = (n->bmax[a] - o[a]) * inv[a];
        if (ta > tb) { double x = ta; ta = tb; tb = x; }
        if (ta != ta) ta = -1e300;   /* 0*inf */
        if (tb != tb) tb = 1e300;
        if (ta > t0) t0 = ta;
        if (tb < t1) t1 = tb;
        if (t0 > t1) return 0;
    }
    return 1;
}

static void intersect(const orc_model* M, int s, const double* o, const double* d, int last, double time,
                      rng_t* r, uint64_t step, oisect* H) {
    H->hard = -1; H->t = 1e99; H->ntr = 0; H->tr = g_tr_buf;
    if (M->nnodes[s] == 0) return;
    double inv[3] = {1.0 / d[0], 1.0 / d[1], 1.0 / d[2]};
    const onode* nodes = M->nodes[s];
    const int* prims = M->prims[s];
    int stack[128], sp = 0;
    stack[sp++] = 0;
    while (sp) {
        const onode* n = &nodes[stack[--sp]];
        H->nodes++;
        if (!box_hit(n, o, inv, H->t)) continue;
        if (n->left < 0) {
            for (int k = 0; k < n->count; ++k) {
                int fi = prims[n->first + k];
                if (fi == last) continue;
                const ofacet* F = &M->f[fi];
                H->prims++;
                double t, u, v;
                if (!facet_hit(M, F, o, d, &t, &u, &v)) continue;
                double op = (F->p_opac >= 0) ? param_at(M, F->p_opac, time) : F->opacity;
                int hard = (op >= 1.0) ? 1 : (op <= 0.0 ? 0 : (rnd_opacity(r, step, fi) < op));
                if (hard) {
                    if (t < H->t || (t == H->t && fi < H->hard)) { H->t = t; H->hard = fi; H->u = u; H->v = v; }
                } else {
                    add_pass(H, fi, t, u, v);
                }
            }
        } else {
            /* visit the child on the ray's near side first */
            const onode* L = &nodes[n->left];
            const onode* R = &nodes[n->right];
            int ax = 0; double best = -1;
            for (int a = 0; a < 3; ++a) {
                double sep = fabs((L->bmin[a] + L->bmax[a]) - (R->bmin[a] + R->bmax[a]));
                if (sep > best) { best = sep; ax = a; }
            }
            int l_first = ((L->bmin[ax] + L->bmax[ax]) < (R->bmin[ax] + R->bmax[ax])) == (d[ax] > 0);
            if (sp + 2 > 128) continue;
            if (l_first) { stack[sp++] = n->right; stack[sp++] = n->left; }
            else { stack[sp++] = n->left; stack[sp++] = n->right; }
        }
    }
}

/* ------------------------------------------------------------- tracer -- */
typedef struct {
    double* global;
    uint64_t* fc;
    double* fs;
    double* tex;
    double* prof;
    double* dir;
    uint64_t* ang;
    double* hist;
    double* force;   /* [(1+M) * nf * 9] with force measurement */
    double* plog;    /* particle log records (MFG_LOG_N doubles each) */
    int64_t plog_n;
} otally;

/* Score-function bookkeeping of one thread (orc_run_sens): the parameters of the current
 * particle's reflections on parameter facets, and the sums that give d(output)/d(sticking):
 * A[k][j] = Sum over (output event j, earlier reflection on parameter k) of the event's value,
 * B[k][j] = Sum over absorptions on parameter k counted to output j, Y[j] = Sum of values. */
#define ORC_SENS_NOUT 9
#define ORC_SENS_TRAJ 1024
typedef struct osens {
    const int32_t* pof;     /* [nf] parameter index or -1 */
    const int32_t* gof;     /* [nf] gauge index 0..7 or -1 */
    const uint8_t* pump;    /* [nf] 1: an absorption counts to the pumped flux */
    double* A;              /* [np * 9] */
    double* B;              /* [np * 9] */
    double Y[ORC_SENS_NOUT];
    int32_t traj[ORC_SENS_TRAJ];
    int ntraj;
    uint64_t overflow;
} osens;

typedef struct {
    double o[3], d[3];
    double time, velocity, ori, dist, gen_time, decay_at, scatter_at;
    int last, structure;
    int tele_from;  /* teleportedFrom: destination of the last teleport, -1 none */
    uint64_t bounces;
    double u, v;   /* facetHitDetails of the current facet */
    osens* S;      /* score-function bookkeeping, or NULL */
} opart;

/* output event j of value y: the value, and its score pairs with every earlier reflection on a
 * parameter facet (decisions after the event do not change it) */
static void sens_out(osens* S, int j, double y) {
    S->Y[j] += y;
    const int n = S->ntraj < ORC_SENS_TRAJ ? S->ntraj : ORC_SENS_TRAJ;
    for (int e = 0; e < n; ++e) S->A[(size_t)S->traj[e] * ORC_SENS_NOUT + j] += y;
}
static void sens_reflect(osens* S, int fi) {
    const int k = S->pof[fi];
    if (k < 0) return;
    if (S->ntraj < ORC_SENS_TRAJ) S->traj[S->ntraj++] = k;
    else if (S->ntraj == ORC_SENS_TRAJ) { S->overflow++; S->ntraj++; }
}

/* moment blocks of time t: all moments whose [start,end) window contains t
 * (LookupMomentIndex, Particle.cpp:1364-1379, which returns the single window
 * when windows are disjoint) */
static int moments_of(const orc_model* M, double t, int* out, int maxn) {
    if (M->nm == 0) return 0;
    int hi = lower_index(t, M->mstart, M->nm);   /* last start <= t */
    int n = 0;
    for (int k = hi; k >= 0 && M->mstart[k] > t - M->maxwin - 1e-300; --k) {
        if (M->mstart[k] <= t && t < M->mend[k]) { if (n < maxn) out[n++] = k + 1; }
    }
    return n;
}

static void polar_to_cart(const ofacet* F, double theta, double phi, int reverse, double* out) {
    double st = sin(theta), ct = cos(theta), sp = sin(phi), cp = cos(phi);
    double u = st * cp, v = st * sp, n = ct;
    if (reverse) n = -n;
    for (int k = 0; k < 3; ++k) out[k] = u * F->nU[k] + v * F->nV[k] + n * F->N[k];
}
static void cart_to_polar(const ofacet* F, const double* d, double* theta, double* phi) {
    double u = dot3(d, F->nU), v = dot3(d, F->nV), n = dot3(d, F->N);
    if (n > 1) n = 1; if (n < -1) n = -1;
    *theta = acos(n);
    *phi = atan2(v, u);
}

static void add_moment_block(const orc_model* M, otally* T, int m, int fi, double hit, double des, double absn,
                             double s1v, double svort, const opart* P) {
    uint64_t* fc = T->fc + ((size_t)m * M->nf + fi) * MFG_FC_N;
    double* fs = T->fs + ((size_t)m * M->nf + fi) * MFG_FS_N;
    double he = hit * P->ori;
    fc[MFG_FC_NBMCHIT] += (uint64_t)hit;
    fc[MFG_FC_NBDESORBED] += (uint64_t)des;
    fc[MFG_FC_NBABSORBED] += (uint64_t)absn;
    fs[MFG_FS_NBHITEQUIV] += he;
    fs[MFG_FS_NBABSEQUIV] += absn * P->ori;
    fs[MFG_FS_SUM_1_PER_ORT_VEL] += P->ori * s1v;
    fs[MFG_FS_SUM_V_ORT] += P->ori * svort;
    fs[MFG_FS_SUM_1_PER_VELOCITY] += (he + des) / P->velocity;
}
/* IncreaseFacetCounter (Particle.cpp:1194-1230) */
static void facet_counter(const orc_model* M, otally* T, const int* ms, int nms, int fi, double hit, double des,
                          double absn, double s1v, double svort, const opart* P) {
    add_moment_block(M, T, 0, fi, hit, des, absn, s1v, svort, P);
    for (int k = 0; k < nms; ++k) add_moment_block(M, T, ms[k], fi, hit, des, absn, s1v, svort, P);
}
/* LogHit (Particle.cpp:1088-1102): an event on the logged facet adds a record (u, v, theta and phi
 * of the direction to the facet basis, oriRatio, expected decay moment, time, speed) while the
 * thread's log has room */
static void log_hit(const orc_model* M, otally* T, int fi, const opart* P) {
    if (fi != M->log_facet || T->plog_n >= M->log_cap) return;
    const ofacet* F = &M->f[fi];
    double th, ph;
    cart_to_polar(F, P->d, &th, &ph);
    double* r = T->plog + (size_t)T->plog_n * MFG_LOG_N;
    r[0] = P->u; r[1] = P->v; r[2] = th; r[3] = ph;
    r[4] = P->ori; r[5] = P->decay_at; r[6] = P->time; r[7] = P->velocity;
    T->plog_n++;
}
/* force measurement (IncreaseFacetCounter, Particle.cpp:1208-1212): momentum s*v*d of the particle
 * onto facet fi (s = -1 for a particle leaving it), its squares and its torque about the
 * reference point, weighted by oriRatio, in moment 0 and the moments of the event */
static void force_add(const orc_model* M, otally* T, const int* ms, int nms, int fi, const opart* P, double s) {
    if (!M->force) return;
    const double w = P->ori;
    double p[3], r[3];
    for (int a = 0; a < 3; ++a) { p[a] = s * P->velocity * P->d[a]; r[a] = P->o[a] - M->torque_ref[a]; }
    const double q[9] = {w * p[0], w * p[1], w * p[2], w * p[0] * p[0], w * p[1] * p[1], w * p[2] * p[2],
                         w * (r[1] * p[2] - r[2] * p[1]), w * (r[2] * p[0] - r[0] * p[2]), w * (r[0] * p[1] - r[1] * p[0])};
    for (int k = -1; k < nms; ++k) {
        double* b = T->force + ((size_t)((k < 0) ? 0 : ms[k]) * M->nf + fi) * 9;
        for (int j = 0; j < 9; ++j) b[j] += q[j];
    }
}
/* RecordHitOnTexture (Particle.cpp:978-1004) */
static void texture_hit(const orc_model* M, otally* T, const int* ms, int nms, const ofacet* F, const opart* P,
                        int count_hit, double vel_factor, double ort_factor) {
    long tu = (long)(P->u * F->texw_p), tv = (long)(P->v * F->texh_p);
    if (tu >= F->texw) tu = F->texw - 1; if (tv >= F->texh) tv = F->texh - 1;
    if (tu < 0) tu = 0; if (tv < 0) tv = 0;
    long add = tu + tv * F->texw;
    double ort = (M->use_maxwell ? 1.0 : 1.1781) * P->velocity * fabs(dot3(P->d, F->N));
    double inc = M->texinc[F->tex_off + add];
    for (int k = -1; k < nms; ++k) {
        int m = (k < 0) ? 0 : ms[k];
        double* c = T->tex + ((size_t)m * M->L.texture_cells + F->tex_off + add) * 3;
        if (count_hit) c[0] += P->ori;
        c[1] += P->ori * ort_factor * ort * inc;
        c[2] += P->ori * vel_factor / ort;
    }
}
/* RecordDirectionVector (Particle.cpp:1006-1023) */
static void direction_hit(const orc_model* M, otally* T, const int* ms, int nms, const ofacet* F, const opart* P) {
    long tu = (long)(P->u * F->texw_p), tv = (long)(P->v * F->texh_p);
    if (tu >= F->texw) tu = F->texw - 1; if (tv >= F->texh) tv = F->texh - 1;
    long add = tu + tv * F->texw;
    for (int k = -1; k < nms; ++k) {
        int m = (k < 0) ? 0 : ms[k];
        double* c = T->dir + ((size_t)m * M->L.direction_cells + F->dir_off + add) * 4;
        for (int a = 0; a < 3; ++a) c[a] += P->ori * P->d[a] * P->velocity;
        c[3] += 1.0;
    }
}
/* ProfileFacet (Particle.cpp:1026-1085) */
static void profile_hit(const orc_model* M, otally* T, const int* ms, int nms, const ofacet* F, const opart* P,
                        int count_hit, double vel_factor, double ort_factor) {
    if (F->prof_idx < 0) return;
    int pt = F->profile_type;
    long pos = -1;
    int slices = 0;   /* 1: count only; 2: full slice */
    double dotn = dot3(F->N, P->d);
    if (count_hit && pt == MFG_PROFILE_ANGULAR) {
        double theta = acos(fabs(dotn));
        pos = (long)(theta / (PI_D / 2) * (double)MFG_PROFILE_SIZE);
        if (pos < 0) pos = 0; if (pos > MFG_PROFILE_SIZE - 1) pos = MFG_PROFILE_SIZE - 1;
        slices = 1;
    } else if (pt == MFG_PROFILE_U || pt == MFG_PROFILE_V) {
        double x = (pt == MFG_PROFILE_U) ? P->u : P->v;
        pos = (long)(x * (double)MFG_PROFILE_SIZE);
        if (pos < 0 || pos >= MFG_PROFILE_SIZE) return;
        slices = 2;
    } else if (count_hit && (pt == MFG_PROFILE_VELOCITY || pt == MFG_PROFILE_ORT_VELOCITY || pt == MFG_PROFILE_TAN_VELOCITY)) {
        double dd;
        if (pt == MFG_PROFILE_VELOCITY) dd = 1.0;
        else if (pt == MFG_PROFILE_ORT_VELOCITY) dd = fabs(dotn);
        else dd = sqrt(1 - dotn * dotn);
        double x = dd * P->velocity / F->max_speed * (double)MFG_PROFILE_SIZE;
        if (!(x >= 0) || x >= MFG_PROFILE_SIZE) return;
        pos = (long)x;
        slices = 1;
    } else return;
    double ort = P->velocity * fabs(dotn);
    for (int k = -1; k < nms; ++k) {
        int m = (k < 0) ? 0 : ms[k];
        double* c = T->prof + (((size_t)m * M->L.profile_facets + F->prof_idx) * MFG_PROFILE_SIZE + pos) * 3;
        if (slices == 1) { c[0] += P->ori; continue; }
        if (count_hit) c[0] += P->ori;
        c[2] += P->ori * vel_factor / ort;
        c[1] += P->ori * ort_factor * (M->use_maxwell ? 1.0 : 1.1781) * ort;
    }
}
/* RecordAngleMap (Particle.cpp:1104-1136) */
static void anglemap_hit(const orc_model* M, otally* T, const ofacet* F, const opart* P) {
    if (F->ang_off < 0) return;
    double th, ph;
    cart_to_polar(F, P->d, &th, &ph);
    if (th > PI_D / 2.0) th = fabs(PI_D - th);
    long ti;
    if (th < F->am_limit) {
        if (F->am_lo <= 0) return;
        ti = (long)(th / F->am_limit * (double)F->am_lo);
    } else {
        if (F->am_hi <= 0) return;
        ti = F->am_lo + (long)((th - F->am_limit) / (PI_D / 2.0 - F->am_limit) * (double)F->am_hi);
    }
    long pi = (long)((ph + 3.1415926) / (2.0 * PI_D) * (double)F->am_phi);
    if (ti >= F->am_lo + F->am_hi) ti = F->am_lo + F->am_hi - 1;
    if (pi >= F->am_phi) pi = F->am_phi - 1; if (pi < 0) pi = 0;
    T->ang[F->ang_off + ti * F->am_phi + pi] += 1;
}

static double maxwell_speed(const orc_model* M, double sqrtT, double r) {
    return sqrtT * interp_x(r, M->cdf_v, M->cdf_p, MAXWELL_CDF_N, 0, 0, 1);
}
static double temperature_at(const orc_model* M, const ofacet* F, double t) {
    return (F->p_temp >= 0) ? param_at(M, F->p_temp, t) : F->temperature;
}

/* StartFromSource (Particle.cpp:407-685) for facets without outgassing maps. */
/* TreatMovingFacet (Physics.cpp:25-39): the moving facet's local velocity (m/s) is added to the
 * particle's; position in cm, rotation axis base in cm, angular velocity in rad/s */
static void treat_moving(const orc_model* M, opart* P) {
    double add[3] = {0, 0, 0};
    if (M->motion_type == 1) {
        for (int k = 0; k < 3; ++k) add[k] = M->mv2[k];
    } else if (M->motion_type == 2) {
        double dv[3] = {0.01 * (P->o[0] - M->mv1[0]), 0.01 * (P->o[1] - M->mv1[1]), 0.01 * (P->o[2] - M->mv1[2])};
        cross3(M->mv2, dv, add);
    }
    double w[3];
    for (int k = 0; k < 3; ++k) w[k] = P->d[k] * P->velocity + add[k];
    double n = sqrt(dot3(w, w));
    for (int k = 0; k < 3; ++k) P->d[k] = w[k] / n;
    P->velocity = n;
}

static int start_from_source(const orc_model* M, otally* T, rng_t* r, opart* P) {
    double sr = rnd(r) * M->src_total;
    int lo = 0, hi = M->nsrc;   /* first k with prefix[k] > sr */
    while (lo < hi) { int mid = (lo + hi) >> 1; if (M->src_prefix[mid] > sr) hi = mid; else lo = mid + 1; }
    if (lo >= M->nsrc) return 0;
    int fi = M->src_facet[lo];
    const int cell = M->src_cell[lo];
    const ofacet* F = &M->f[fi];
    int reverse = F->two_sided ? (rnd(r) > 0.5) : 0;
    P->last = fi;
    if (F->id_idx >= 0) {
        const oid* I = &M->ids[F->id_idx];
        P->time = interp_x(rnd(r) * I->cum[I->n - 1], I->t, I->cum, I->n, 0, 0, 1);
    } else P->time = rnd(r) * M->latest;
    P->gen_time = P->time;
    if (M->use_maxwell) P->velocity = maxwell_speed(M, F->sqrtT, rnd(r));
    else P->velocity = 145.469 * sqrt(F->temperature / M->gas_mass);
    P->ori = 1.0;
    if (M->decay) {
        double tau = 1.44269 * M->half_life;
        P->decay_at = P->time - tau * log(1.0 - rnd(r));
    } else P->decay_at = 1e100;
    /* free path to the first background-gas collision (Particle.cpp:500-504) */
    P->scatter_at = M->scatter ? -M->sc_mfp * log(1.0 - rnd(r)) : 1e100;
    P->tele_from = -1;
    P->bounces = 0; P->dist = 0;
    int found = 0;
    /* outgassing-map cell (Particle.cpp:513-535): u, v uniform in the cell, the last column and
     * row of the grid only as far as the facet reaches */
    const int cw = cell >= 0 ? cell % F->og_w : 0, ch = cell >= 0 ? cell / F->og_w : 0;
    for (int tries = 0; tries < 1000 && !found; ++tries) {
        double u, v;
        if (cell >= 0) {
            u = (cw < F->og_w - 1) ? (cw + rnd(r)) / F->og_wp : (cw + rnd(r) * (F->og_wp - (F->og_w - 1.0))) / F->og_wp;
            v = (ch < F->og_h - 1) ? (ch + rnd(r)) / F->og_hp : (ch + rnd(r) * (F->og_hp - (F->og_h - 1.0))) / F->og_hp;
        } else {
            u = rnd(r); v = rnd(r);
        }
        if (in_polygon(M->v2 + 2 * F->vstart, F->nv, u, v)) {
            for (int k = 0; k < 3; ++k) P->o[k] = F->O[k] + u * F->U[k] + v * F->V[k];
            P->u = u; P->v = v; found = 1;
        }
    }
    if (!found) {
        if (cell >= 0) {   /* the cell's centre */
            P->u = (cw + 0.5) / F->og_wp; P->v = (ch + 0.5) / F->og_hp;
            for (int k = 0; k < 3; ++k) P->o[k] = F->O[k] + P->u * F->U[k] + P->v * F->V[k];
        } else { P->u = 0.5; P->v = 0.5; for (int k = 0; k < 3; ++k) P->o[k] = F->center[k]; }
    }
    double th, ph;
    switch (F->desorb_type) {
        case MFG_DES_UNIFORM: th = acos(rnd(r)); ph = rnd(r) * 2.0 * PI_D; break;
        case MFG_DES_COSINE_N: th = acos(pow(rnd(r), 1.0 / (F->desorb_exp + 1.0))); ph = rnd(r) * 2.0 * PI_D; break;
        case MFG_DES_ANGLEMAP: {   /* the map holds incident angles: leave at pi - theta (Particle.cpp:598-622) */
            int ti; double tov;
            const double r1 = rnd(r);
            th = am_gen_theta(F->amd, r1, &ti, &tov);
            ph = am_gen_phi(F->amd, ti, tov, rnd(r));
            th = PI_D - th;
            reverse = 0;
            break;
        }
        default: th = acos(sqrt(rnd(r))); ph = rnd(r) * 2.0 * PI_D; break;
    }
    polar_to_cart(F, th, ph, reverse, P->d);
    P->structure = F->structure;
    if (F->moving) treat_moving(M, P);
    T->global[MFG_G_NBDESORBED] += 1.0;
    double ort = P->velocity * fabs(dot3(P->d, F->N));
    int ms[256]; int nms = moments_of(M, P->time, ms, 256);
    facet_counter(M, T, ms, nms, fi, 0, 1, 0, 2.0 / ort, (M->use_maxwell ? 1.0 : 1.1781) * ort, P);
    force_add(M, T, ms, nms, fi, P, 1.0);
    log_hit(M, T, fi, P);
    profile_hit(M, T, ms, nms, F, P, 0, 2.0, 1.0);
    if (F->count & MFG_COUNT_DES) texture_hit(M, T, ms, nms, F, P, 1, 2.0, 1.0);
    return 1;
}

/* RegisterTransparentPass (Particle.cpp:1232-1257) */
static void transparent_pass(const orc_model* M, otally* T, int fi, const ohit* h, opart* P) {
    const ofacet* F = &M->f[fi];
    double df = fabs(dot3(P->d, F->N));
    int ms[256]; int nms = moments_of(M, P->time + h->t / 100.0 / P->velocity, ms, 256);
    double su = P->u, sv = P->v;
    P->u = h->u; P->v = h->v;
    facet_counter(M, T, ms, nms, fi, 1, 0, 0, 2.0 / (P->velocity * df),
                  2.0 * (M->use_maxwell ? 1.0 : 1.1781) * P->velocity * df, P);
    if (P->S && P->S->gof[fi] >= 0) sens_out(P->S, P->S->gof[fi], 2.0 * P->velocity * df);
    if (F->count & MFG_COUNT_TRANS) texture_hit(M, T, ms, nms, F, P, 1, 2.0, 2.0);
    if ((F->count & MFG_COUNT_DIR) && F->dir_off >= 0) direction_hit(M, T, ms, nms, F, P);
    profile_hit(M, T, ms, nms, F, P, 1, 2.0, 2.0);
    if (F->ang_off >= 0) anglemap_hit(M, T, F, P);
    P->u = su; P->v = sv;
}

/* RecordHistograms (Particle.cpp:926-975): bounces, flight distance and flight time of the
 * absorbed particle, in moment 0 and the moments of the absorption time */
static void hist_add(const ohist* h, double* block, const opart* P) {
    if (h->off < 0) return;
    double* b = block + h->off;
    if (h->nb) {
        uint64_t k = P->bounces / h->bounce_bin;
        if (k > (uint64_t)(h->nb - 1)) k = (uint64_t)(h->nb - 1);
        b[k] += P->ori;
        b += h->nb;
    }
    if (h->nd) {
        size_t k = (size_t)(P->dist / h->dist_bin);
        if (k > (size_t)(h->nd - 1)) k = (size_t)(h->nd - 1);
        b[k] += P->ori;
        b += h->nd;
    }
    if (h->nt) {
        size_t k = (size_t)((P->time - P->gen_time) / h->time_bin);
        if (k > (size_t)(h->nt - 1)) k = (size_t)(h->nt - 1);
        b[k] += P->ori;
    }
}
static void record_histograms(const orc_model* M, otally* T, const int* ms, int nms, int fi, const opart* P) {
    const long hb = M->L.histogram_bins;
    if (!hb) return;
    for (int k = -1; k < nms; ++k) {
        double* block = T->hist + (size_t)((k < 0) ? 0 : ms[k]) * hb;
        hist_add(&M->ghist, block, P);
        if (M->fhist) hist_add(&M->fhist[fi], block, P);
    }
}

/* RecordAbsorb (Particle.cpp:888-924) */
static void record_absorb(const orc_model* M, otally* T, int fi, opart* P) {
    const ofacet* F = &M->f[fi];
    T->global[MFG_G_NBMCHIT] += 1; T->global[MFG_G_NBHITEQUIV] += P->ori; T->global[MFG_G_NBABSEQUIV] += P->ori;
    int ms[256]; int nms = moments_of(M, P->time, ms, 256);
    double ort = P->velocity * fabs(dot3(P->d, F->N));
    facet_counter(M, T, ms, nms, fi, 1, 0, 1, 2.0 / ort, (M->use_maxwell ? 1.0 : 1.1781) * ort, P);
    if (P->S) {
        osens* S = P->S;
        if (S->gof[fi] >= 0) sens_out(S, S->gof[fi], ort);
        if (S->pump[fi]) {
            sens_out(S, ORC_SENS_NOUT - 1, 1.0);
            if (S->pof[fi] >= 0) S->B[(size_t)S->pof[fi] * ORC_SENS_NOUT + ORC_SENS_NOUT - 1] += 1.0;
        }
    }
    force_add(M, T, ms, nms, fi, P, 1.0);
    log_hit(M, T, fi, P);
    profile_hit(M, T, ms, nms, F, P, 1, 2.0, 1.0);
    if (F->ang_off >= 0) anglemap_hit(M, T, F, P);
    record_histograms(M, T, ms, nms, fi, P);
    if (F->count & MFG_COUNT_ABS) texture_hit(M, T, ms, nms, F, P, 1, 2.0, 1.0);
    if ((F->count & MFG_COUNT_DIR) && F->dir_off >= 0) direction_hit(M, T, ms, nms, F, P);
}

/* UpdateVelocity (Particle.cpp:1138-1163) */
static void update_velocity(const orc_model* M, const ofacet* F, rng_t* r, opart* P) {
    double temp = temperature_at(M, F, P->time);
    double sqrtT = (F->p_temp < 0) ? F->sqrtT : sqrt(temp);
    if (F->accommodation > 0.9999) {
        if (M->use_maxwell) P->velocity = maxwell_speed(M, sqrtT, rnd(r));
        else P->velocity = 145.469 * sqrtT / M->gas_mass;   /* reference quirk kept (Particle.cpp:1152) */
    } else {
        double old2 = P->velocity * P->velocity, new2;
        if (M->use_maxwell) { double v = maxwell_speed(M, sqrtT, rnd(r)); new2 = v * v; }
        else new2 = 29369.939 * (temp / M->gas_mass);
        P->velocity = sqrt(old2 + (new2 - old2) * F->accommodation);
    }
}

/* PerformTeleport (Particle.cpp:76-183): the hit on facet fi is recorded like a transparent pass
 * (texture, direction, profile, angle map with the incoming direction); the particle leaves the
 * destination facet at the same (u,v) with the same angles to the destination's basis (the
 * reference's polar round trip, written as the projection onto the destination basis), in the
 * destination's structure.  The facet counter takes one hit and the velocity sums of the
 * outgoing direction against the source normal; the global hit count is not increased.  A
 * destination -1 means the facet the particle last teleported to; without one (or with an
 * invalid one) the particle passes on through fi.  When (u,v) is outside the destination
 * polygon, new points are drawn until one is inside: the reference draws without limit (its try
 * counter sits outside the loop); here at most 1000 draws, then the mapped point is kept. */
static void perform_teleport(const orc_model* M, otally* T, int fi, rng_t* r, opart* P) {
    const ofacet* F = &M->f[fi];
    const int dest = F->teleport == -1 ? P->tele_from : F->teleport - 1;
    if (dest < 0 || dest >= M->nf) { P->last = fi; return; }
    const ofacet* D = &M->f[dest];
    P->structure = D->structure;
    P->tele_from = dest;
    int ms[256]; int nms = moments_of(M, P->time, ms, 256);
    if (F->count & MFG_COUNT_TRANS) texture_hit(M, T, ms, nms, F, P, 1, 2.0, 2.0);
    if ((F->count & MFG_COUNT_DIR) && F->dir_off >= 0) direction_hit(M, T, ms, nms, F, P);
    profile_hit(M, T, ms, nms, F, P, 1, 2.0, 2.0);
    if (F->ang_off >= 0) anglemap_hit(M, T, F, P);
    log_hit(M, T, fi, P);
    const double a = dot3(P->d, F->nU), b = dot3(P->d, F->nV), c = dot3(P->d, F->N);
    for (int k = 0; k < 3; ++k) P->d[k] = a * D->nU[k] + b * D->nV[k] + c * D->N[k];
    double u = P->u, v = P->v;
    if (!in_polygon(M->v2 + 2 * D->vstart, D->nv, u, v)) {
        for (int tries = 0; tries < 1000; ++tries) {
            const double u2 = rnd(r), v2 = rnd(r);
            if (in_polygon(M->v2 + 2 * D->vstart, D->nv, u2, v2)) { u = u2; v = v2; break; }
        }
    }
    for (int k = 0; k < 3; ++k) P->o[k] = D->O[k] + u * D->U[k] + v * D->V[k];
    P->last = dest;
    const double ort = P->velocity * fabs(dot3(P->d, F->N));
    facet_counter(M, T, ms, nms, fi, 1, 0, 0, 2.0 / ort, 2.0 * (M->use_maxwell ? 1.0 : 1.1781) * ort, P);
}

/* PerformBounce (Particle.cpp:691-838), no moving facets */
static void perform_bounce(const orc_model* M, otally* T, int fi, rng_t* r, opart* P) {
    const ofacet* F = &M->f[fi];
    T->global[MFG_G_NBMCHIT] += 1; T->global[MFG_G_NBHITEQUIV] += P->ori;
    if (F->link) {
        /* structure link (Particle.cpp:698-724): counted like a transparent pass without
         * velocity sums on the facet counter; the particle continues in structure link-1 with
         * its direction, speed and last-hit facet unchanged */
        int ms[256]; int nms = moments_of(M, P->time, ms, 256);
        facet_counter(M, T, ms, nms, fi, 1, 0, 0, 0.0, 0.0, P);
        profile_hit(M, T, ms, nms, F, P, 1, 2.0, 2.0);
        if (F->ang_off >= 0) anglemap_hit(M, T, F, P);
        if (F->count & MFG_COUNT_TRANS) texture_hit(M, T, ms, nms, F, P, 1, 2.0, 2.0);
        if ((F->count & MFG_COUNT_DIR) && F->dir_off >= 0) direction_hit(M, T, ms, nms, F, P);
        P->structure = F->link - 1;
        if (F->moving) treat_moving(M, P);
        log_hit(M, T, fi, P);
        return;
    }
    int revert = F->two_sided ? (dot3(P->d, F->N) > 0.0) : 0;
    double ort = P->velocity * fabs(dot3(P->d, F->N));
    double vf = M->use_maxwell ? 1.0 : 1.1781;
    int ms[256]; int nms = moments_of(M, P->time, ms, 256);
    facet_counter(M, T, ms, nms, fi, 1, 0, 0, 1.0 / ort, vf * ort, P);
    if (P->S) {
        if (P->S->gof[fi] >= 0) sens_out(P->S, P->S->gof[fi], ort);
        sens_reflect(P->S, fi);
    }
    force_add(M, T, ms, nms, fi, P, 1.0);
    log_hit(M, T, fi, P);
    P->bounces++;
    if (F->count & MFG_COUNT_REFL) texture_hit(M, T, ms, nms, F, P, 1, 1.0, 1.0);
    if ((F->count & MFG_COUNT_DIR) && F->dir_off >= 0) direction_hit(M, T, ms, nms, F, P);
    profile_hit(M, T, ms, nms, F, P, 1, 1.0, 1.0);
    if (F->ang_off >= 0) anglemap_hit(M, T, F, P);
    update_velocity(M, F, r, P);
    if (F->sojourn) {
        double A = exp(-F->soj_e / (8.31 * temperature_at(M, F, P->time)));
        P->time += -log(1.0 - rnd(r)) / (A * F->soj_freq);
        nms = moments_of(M, P->time, ms, 256);
    }
    if (F->diffuse > 0.999999) {
        double th = acos(sqrt(rnd(r))); double ph = rnd(r) * 2.0 * PI_D;
        polar_to_cart(F, th, ph, revert, P->d);
    } else {
        double rt = rnd(r);
        if (rt < F->diffuse) {
            double th = acos(sqrt(rnd(r))); double ph = rnd(r) * 2.0 * PI_D;
            polar_to_cart(F, th, ph, revert, P->d);
        } else if (rt < F->diffuse + F->specular) {
            double th, ph; cart_to_polar(F, P->d, &th, &ph);
            polar_to_cart(F, PI_D - th, ph, 0, P->d);
        } else {
            double th = acos(pow(rnd(r), 1.0 / (F->cos_exp + 1.0))); double ph = rnd(r) * 2.0 * PI_D;
            polar_to_cart(F, th, ph, revert, P->d);
        }
    }
    if (F->moving) treat_moving(M, P);
    ort = P->velocity * fabs(dot3(P->d, F->N));
    facet_counter(M, T, ms, nms, fi, 0, 0, 0, 1.0 / ort, vf * ort, P);
    if (P->S && P->S->gof[fi] >= 0) sens_out(P->S, P->S->gof[fi], ort);
    force_add(M, T, ms, nms, fi, P, -1.0);
    if (F->count & MFG_COUNT_REFL) texture_hit(M, T, ms, nms, F, P, 0, 1.0, 1.0);
    profile_hit(M, T, ms, nms, F, P, 0, 1.0, 1.0);
    P->last = fi;
}

typedef struct { otally T; orc_stats st; osens* S; } othread;

static void tally_alloc(const orc_model* M, otally* T) {
    const mfg_state_layout* L = &M->L;
    T->global = (double*)calloc(L->n_global, sizeof(double));
    T->fc = (uint64_t*)calloc(L->n_facet_counts + 1, sizeof(uint64_t));
    T->fs = (double*)calloc(L->n_facet_sums + 1, sizeof(double));
    T->tex = (double*)calloc(L->n_texture + 1, sizeof(double));
    T->prof = (double*)calloc(L->n_profile + 1, sizeof(double));
    T->dir = (double*)calloc(L->n_direction + 1, sizeof(double));
    T->ang = (uint64_t*)calloc(L->n_anglemap + 1, sizeof(uint64_t));
    T->hist = (double*)calloc(L->n_histogram + 1, sizeof(double));
    T->force = (double*)calloc(L->n_force + 1, sizeof(double));
    T->plog = (double*)calloc((size_t)M->log_cap * MFG_LOG_N + 1, sizeof(double));
    T->plog_n = 0;
}
static void tally_free(otally* T) {
    free(T->global); free(T->fc); free(T->fs); free(T->tex); free(T->prof); free(T->dir); free(T->ang); free(T->hist);
    free(T->force); free(T->plog);
}

/* trace one particle to absorption/leak: the body of SimulationMCStep (Particle.cpp:221-393) */
/* PerformScatter (Particle.cpp:840-886, Physics.cpp:41-63): collision with a background-gas
 * molecule; returns 0 when the particle fell below the cutoff speed */
static int perform_scatter(const orc_model* M, otally* T, rng_t* r, opart* P) {
    T->global[MFG_G_NBMCHIT] += 1; T->global[MFG_G_NBHITEQUIV] += P->ori;
    P->bounces++;
    const double rho = M->sc_rho, mr = M->sc_mass_ratio;
    const double b = rho * sqrt(rnd(r));
    const double a = sqrt(rho * rho - b * b);
    const double ctg = 1.0 / (2.0 * a * b) * (rho * rho * mr + b * b - a * a);
    const double theta = atan(1.0 / ctg);
    const double phi = 2.0 * PI_D * rnd(r);
    double rv[3] = {1.0, 0.0, 0.0};
    if (P->d[0] != 0.0) { rv[0] = 0.0; rv[2] = 1.0; }
    else if (P->d[1] != 0.0) { rv[2] = 1.0; }
    double un[3], vn[3];
    cross3(P->d, rv, un);
    double l = sqrt(dot3(un, un));
    for (int k = 0; k < 3; ++k) un[k] /= l;
    cross3(P->d, un, vn);
    l = sqrt(dot3(vn, vn));
    for (int k = 0; k < 3; ++k) vn[k] /= l;
    const double st = sin(theta), ct = cos(theta), sp = sin(phi), cp = cos(phi);
    double nd[3];
    for (int k = 0; k < 3; ++k) nd[k] = st * cp * un[k] + st * sp * vn[k] + ct * P->d[k];
    for (int k = 0; k < 3; ++k) P->d[k] = nd[k];
    const double q = mr * rho / b * st;
    P->velocity = sqrt(P->velocity * P->velocity / (1.0 + q * q));
    P->scatter_at = P->dist - M->sc_mfp * log(1.0 - rnd(r));
    return !(M->scatter_cutoff && P->velocity < M->sc_cutoff_speed);
}

static int trace_particle(const orc_model* M, otally* T, rng_t* r, uint64_t max_steps, orc_stats* st,
                          int64_t* nrec, int64_t maxrec, double* ro, double* rd, int32_t* rl, int32_t* rh, double* rt,
                          osens* S) {
    opart P;
    P.S = NULL;
    if (!start_from_source(M, T, r, &P)) return -1;
    P.S = S;
    if (S) S->ntraj = 0;
    st->desorbed++;
    oisect H;
    for (uint64_t step = 0;; ++step) {
        if (step >= max_steps) { st->dropped++; return 0; }
        H.nodes = 0; H.prims = 0;
        intersect(M, P.structure, P.o, P.d, P.last, P.time, r, step, &H);
        st->rays++; st->node_visits += H.nodes; st->prim_tests += H.prims;
        if (nrec && *nrec < maxrec) {
            int64_t k = (*nrec)++;
            for (int a = 0; a < 3; ++a) { ro[3 * k + a] = P.o[a]; rd[3 * k + a] = P.d[a]; }
            rl[k] = P.last; rh[k] = H.hard; rt[k] = H.t;
        }
        if (H.hard < 0) {
            T->global[MFG_G_NBLEAK] += 1; st->leaks++;
            return 0;
        }
        int fi = H.hard;
        const ofacet* F = &M->f[fi];
        double travel = H.t;
        int event = 0;   /* 0 facet hit, 1 overtime, 2 decay */
        if (!M->constant_flow) {
            double dl = P.velocity * 100.0 * (M->latest - P.time);
            if (dl < travel) { travel = dl; event = 1; }
        }
        if (M->decay) {
            double dd = P.velocity * 100.0 * (P.decay_at - P.time);
            if (dd < travel) { travel = dd; event = 2; }
        }
        if (M->scatter) {   /* background-gas collision (Particle.cpp:281-287) */
            double ds = P.scatter_at - P.dist;
            if (ds < travel) { travel = ds; event = 3; }
        }
        for (int k = 0; k < H.ntr; ++k)
            if (H.tr[k].t < travel) transparent_pass(M, T, H.tr[k].facet, &H.tr[k], &P);
        for (int a = 0; a < 3; ++a) P.o[a] = P.o[a] + travel * P.d[a];
        P.time += travel / 100.0 / P.velocity;
        if (event == 3) {
            T->global[MFG_G_DIST_TOTAL] += travel; T->global[MFG_G_DIST_FULLHITS] += travel; P.dist += travel;
            st->hits++;
            if (!perform_scatter(M, T, r, &P)) return 0;
            P.last = -1;   /* any facet may be hit after a volume collision */
            continue;
        }
        if (event != 0) {
            T->global[MFG_G_DIST_TOTAL] += travel;
            return 0;
        }
        T->global[MFG_G_DIST_TOTAL] += travel; T->global[MFG_G_DIST_FULLHITS] += travel; P.dist += travel;
        P.u = H.u; P.v = H.v;
        if (F->teleport) { perform_teleport(M, T, fi, r, &P); continue; }   /* Particle.cpp:326-329 */
        double s = (F->p_stick >= 0) ? param_at(M, F->p_stick, P.time) : F->sticking;
        if (!M->low_flux) {
            if (s == 1.0 || (s > 0.0 && rnd(r) < s)) { record_absorb(M, T, fi, &P); st->hits++; return 0; }
            perform_bounce(M, T, fi, r, &P); st->hits++;
        } else {
            st->hits++;
            if (s > 0.0) {
                double before = P.ori;
                P.ori *= s;
                record_absorb(M, T, fi, &P);
                P.ori = before * (1.0 - s);
            } else P.ori *= (1.0 - s);
            if (P.ori > M->low_flux_cutoff) perform_bounce(M, T, fi, r, &P);
            else return 0;
        }
    }
}

static double now_s(void) {
    struct timespec ts; clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

int orc_run(orc_model* M, uint64_t n_des, const orc_run_opts* o, mfg_state_view* view, orc_stats* st) {
    return orc_run_logged(M, n_des, o, view, st, NULL, 0, NULL);
}

/* sensitivity set-up of a run: facet maps, parameter count and the caller's sums (NULL: none) */
typedef struct {
    const int32_t* pof; const int32_t* gof; const uint8_t* pump;
    int np;
    double* A; double* B; double* Y; uint64_t* overflow;
} osens_run;

static int run_impl(orc_model* M, uint64_t n_des, const orc_run_opts* o, mfg_state_view* view, orc_stats* st,
                    double* log, int64_t log_capacity, int64_t* log_n, const osens_run* sr);

int orc_run_logged(orc_model* M, uint64_t n_des, const orc_run_opts* o, mfg_state_view* view, orc_stats* st,
                   double* log, int64_t log_capacity, int64_t* log_n) {
    return run_impl(M, n_des, o, view, st, log, log_capacity, log_n, NULL);
}

int orc_run_sens(orc_model* M, uint64_t n_des, const orc_run_opts* o, mfg_state_view* view, orc_stats* st,
                 const int32_t* param_of_facet, const int32_t* gauge_of_facet, const uint8_t* pump_of_facet,
                 int32_t n_params, double* A, double* B, double* Y, uint64_t* overflow) {
    osens_run sr = {param_of_facet, gauge_of_facet, pump_of_facet, n_params, A, B, Y, overflow};
    return run_impl(M, n_des, o, view, st, NULL, 0, NULL, &sr);
}

static int run_impl(orc_model* M, uint64_t n_des, const orc_run_opts* o, mfg_state_view* view, orc_stats* st,
                    double* log, int64_t log_capacity, int64_t* log_n, const osens_run* sr) {
    if (log_n) *log_n = 0;
    if (M->nsrc == 0) return MFG_ERR_NO_SOURCE;
    int nt = o->n_threads;
#ifdef _OPENMP
    if (nt <= 0) nt = omp_get_max_threads();
#else
    nt = 1;
#endif
    uint64_t max_steps = o->max_steps ? o->max_steps : ((uint64_t)1 << 40);
    othread* th = (othread*)calloc(nt, sizeof(othread));
    double t0 = now_s();
    int err = 0;
#pragma omp parallel num_threads(nt)
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        othread* me = &th[tid];
        tally_alloc(M, &me->T);
        if (sr) {
            me->S = (osens*)calloc(1, sizeof(osens));
            me->S->pof = sr->pof; me->S->gof = sr->gof; me->S->pump = sr->pump;
            me->S->A = (double*)calloc((size_t)sr->np * ORC_SENS_NOUT + 1, sizeof(double));
            me->S->B = (double*)calloc((size_t)sr->np * ORC_SENS_NOUT + 1, sizeof(double));
        }
        rng_t r; memset(&r, 0, sizeof r);
        r.mode = o->rng_mode;
        r.key[0] = (uint32_t)o->seed; r.key[1] = (uint32_t)(o->seed >> 32);
        r.inst = o->instance;
        if (r.mode == ORC_RNG_MT) mt_seed(&r.mt, 42424242u + (uint32_t)tid);
#pragma omp for schedule(dynamic, 256)
        for (long long i = 0; i < (long long)n_des; ++i) {
            rng_start_particle(&r, o->first_particle + (uint64_t)i);
            if (trace_particle(M, &me->T, &r, max_steps, &me->st, NULL, 0, NULL, NULL, NULL, NULL, NULL, me->S) < 0) err = 1;
        }
    }
    double t1 = now_s();
    /* reduce into the view (GlobalSimuState::operator+=, MolflowSimGeom.cpp:452-458) */
    const mfg_state_layout* L = &M->L;
    memset(st, 0, sizeof *st);
    for (int t = 0; t < nt; ++t) {
        otally* T = &th[t].T;
        if (view->global) for (int64_t k = 0; k < L->n_global; ++k) view->global[k] += T->global[k];
        if (view->facet_counts) for (int64_t k = 0; k < L->n_facet_counts; ++k) view->facet_counts[k] += T->fc[k];
        if (view->facet_sums) for (int64_t k = 0; k < L->n_facet_sums; ++k) view->facet_sums[k] += T->fs[k];
        if (view->texture) for (int64_t k = 0; k < L->n_texture; ++k) view->texture[k] += T->tex[k];
        if (view->profile) for (int64_t k = 0; k < L->n_profile; ++k) view->profile[k] += T->prof[k];
        if (view->direction) for (int64_t k = 0; k < L->n_direction; ++k) view->direction[k] += T->dir[k];
        if (view->anglemap) for (int64_t k = 0; k < L->n_anglemap; ++k) view->anglemap[k] += T->ang[k];
        if (view->histogram) for (int64_t k = 0; k < L->n_histogram; ++k) view->histogram[k] += T->hist[k];
        if (view->force) for (int64_t k = 0; k < L->n_force; ++k) view->force[k] += T->force[k];
        if (log && log_n) {   /* the threads' logs one after the other, up to the capacity */
            int64_t take = T->plog_n;
            if (take > log_capacity - *log_n) take = log_capacity - *log_n;
            if (take > 0) memcpy(log + (size_t)(*log_n) * MFG_LOG_N, T->plog, (size_t)take * MFG_LOG_N * sizeof(double));
            if (take > 0) *log_n += take;
        }
        st->desorbed += th[t].st.desorbed; st->hits += th[t].st.hits; st->leaks += th[t].st.leaks;
        st->dropped += th[t].st.dropped; st->rays += th[t].st.rays;
        st->node_visits += th[t].st.node_visits; st->prim_tests += th[t].st.prim_tests;
        tally_free(T);
        if (th[t].S) {   /* per-thread score sums, added in thread order */
            osens* S = th[t].S;
            for (size_t k = 0; k < (size_t)sr->np * ORC_SENS_NOUT; ++k) { sr->A[k] += S->A[k]; sr->B[k] += S->B[k]; }
            for (int j = 0; j < ORC_SENS_NOUT; ++j) sr->Y[j] += S->Y[j];
            if (sr->overflow) *sr->overflow += S->overflow;
            free(S->A); free(S->B); free(S);
        }
    }
    st->seconds = t1 - t0;
    st->threads = nt;
    free(th);
    return err ? MFG_ERR_NO_SOURCE : MFG_OK;
}

int orc_replay(orc_model* M, int64_t n, const double* origin, const double* dir, const int32_t* last,
               int32_t* hit_facet, double* hit_t, orc_stats* st) {
    uint64_t nodes = 0, prims = 0;
#pragma omp parallel for reduction(+:nodes, prims) schedule(static)
    for (long long i = 0; i < (long long)n; ++i) {
        oisect H; H.nodes = 0; H.prims = 0;
        rng_t r; memset(&r, 0, sizeof r);
        intersect(M, 0, origin + 3 * i, dir + 3 * i, last[i], 0.0, &r, 0, &H);
        hit_facet[i] = H.hard; hit_t[i] = (H.hard >= 0) ? H.t : -1.0;
        nodes += H.nodes; prims += H.prims;
    }
    if (st) { memset(st, 0, sizeof *st); st->rays = n; st->node_visits = nodes; st->prim_tests = prims; }
    return MFG_OK;
}

int64_t orc_record_rays(orc_model* M, uint64_t n_des, uint64_t seed, int64_t max_rays,
                        double* origin, double* dir, int32_t* last, int32_t* hit_facet, double* hit_t) {
    otally T; tally_alloc(M, &T);
    orc_stats st; memset(&st, 0, sizeof st);
    rng_t r; memset(&r, 0, sizeof r);
    r.key[0] = (uint32_t)seed; r.key[1] = (uint32_t)(seed >> 32);
    int64_t nrec = 0;
    for (uint64_t i = 0; i < n_des && nrec < max_rays; ++i) {
        rng_start_particle(&r, i);
        trace_particle(M, &T, &r, (uint64_t)1 << 40, &st, &nrec, max_rays, origin, dir, last, hit_facet, hit_t, NULL);
    }
    tally_free(&T);
    return nrec;
}

/* Angle-map desorption check: draw n (theta, phi) pairs from a recorded map with uniforms
 * r[2k], r[2k+1] as the tracer would, and re-bin the incident angles into the map's bins. */
int orc_anglemap_resample(const uint64_t* pdf, int w, int lo, int hi, double limit, int64_t n, const double* r,
                          uint64_t* out) {
    oamap* a = oamap_build(pdf, w, lo, hi, limit);
    if (!a) return MFG_ERR_INVALID_MODEL;
    for (int64_t k = 0; k < n; ++k) {
        int ti; double tov;
        const double th = am_gen_theta(a, r[2 * k], &ti, &tov);
        const double ph = am_gen_phi(a, ti, tov, r[2 * k + 1]);
        long t;
        if (th < limit) t = (long)(th / limit * (double)lo);
        else t = lo + (long)((th - limit) / (PI_D / 2.0 - limit) * (double)hi);
        long p = (long)((ph + 3.1415926) / (2.0 * PI_D) * (double)w);
        if (t >= lo + hi) t = lo + hi - 1; if (t < 0) t = 0;
        if (p >= w) p = w - 1; if (p < 0) p = 0;
        out[t * w + p] += 1;
    }
    oamap_free(a);
    return MFG_OK;
}
