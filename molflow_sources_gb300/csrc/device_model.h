// device_model.h — data layout of a model in GPU memory, shared by host and kernels.
//
// One model = facets (planar polygons), a BVH per structure and the tables the
// tracer samples from.  Records are AoS and 16-byte aligned so a thread fetches
// one facet with a few vector loads; the FP32 copies are half the size for the
// FP32 traversal.
#pragma once
#include <stdint.h>

#define MFG_MAXWELL_N 100

// BVH nodes are stored breadth-first, so the two children of an internal node
// are adjacent.  Internal node: a = index of the left child (right = a+1),
// b = split axis (0..2).  Leaf: a = first index into the prim list, b = -1 - count.
// FP64 bounds (64 B):
struct __align__(16) NodeD {
    double lo[3];
    double hi[3];
    int32_t a, b;
    int32_t pad0, pad1;
};
// FP32 traversal node holding its two children's boxes, rounded outward and padded by a
// scene-relative margin (64 B, four 16-byte loads), so one fetch decides which children to visit
// and a missed child costs no fetch.  Child reference: >= 0 another NodeC, < 0 a leaf whose
// facets are prims_c[-1 - ref ...] up to a -1 sentinel.  Every structure starts at a root NodeC
// whose child 0 is the whole tree and child 1 an empty leaf far away.
struct __align__(16) NodeC {
    float lo0[3], hi0[3];
    float lo1[3], hi1[3];
    int32_t c0, c1;
    int32_t pad0, pad1;
};

// Facet intersection record FP64 (128 B):
//  [0..2] N, [3] D = N.O, [4..6] O, [7] flags as integer bits (bit 0 two-sided, bits 1-2 opacity
//  class: 0 opaque, 1 transparent, 2 partial or time-dependent), [8..10] U/|U|^2, [11] pad,
//  [12..14] V/|V|^2, [15] pad
struct __align__(16) FacetIsectD { double v[16]; };
// FP32 copy (64 B): [0..2] N, [3] Olo.x, [4..6] Ohi, [7] Olo.y, [8..10] U/|U|^2, [11] Olo.z,
// [12..14] V/|V|^2, [15] the same flags as a float — O as a hi+lo float pair for the origin-relative test
struct __align__(16) FacetIsectF { float v[16]; };

// Polygon record: circle shortcut + vertex range (64 B / 32 B).
//  cu, cv: centre in normalised (u,v); su = |U|, sv = |V|; rin2/rout2: squared radii (cm^2)
//  of a disk certainly inside / a disk containing the polygon; vstart, nv.
struct __align__(16) PolyD { double cu, cv, su, sv, rin2, rout2; int32_t vstart, nv; };
struct __align__(16) PolyF { float cu, cv, su, sv, rin2, rout2; int32_t vstart, nv; };
// Triangle edges for the FP32 test: edge i as a function of (u,v) giving the signed distance (cm)
// of the point from the edge line, positive inside: e_i = a u + b v + c in e[i] = (a, b, c, 0).
// All zero for a degenerate triangle (every point then goes to the FP64 test).
struct __align__(16) TriF { float e[3][4]; };

// Facet flags
#define FF_TWO_SIDED   1u
#define FF_TEXTURED    2u
#define FF_STICK_PARAM 4u
#define FF_TEMP_PARAM  8u
#define FF_SOJOURN     16u
#define FF_ANGLEMAP    32u
#define FF_PROFILE     64u
#define FF_DIFFUSE_ONLY 128u
#define FF_FAST_REFL   256u   // diffuse, full accommodation, Maxwell speeds, no sojourn, constant temperature
#define FF_LINK        512u   // structure link: the particle passes into structure FacetInfo2::link
#define FF_MOVING      1024u  // moving facet: its velocity is added to particles leaving it
#define FF_TELEPORT    2048u  // teleport source: the particle leaves FacetInfo2::teleport instead

// Per-facet physics record (FP64, 128 B).
struct __align__(16) FacetPhysD {
    double nU[3], nV[3];
    double sticking, sqrtT, accommodation, diffuse, specular, cos_exp;
    double texw_p, texh_p;
    double soj_freq, soj_e;
};
struct __align__(16) FacetPhysF {
    float nU[3], nV[3];
    float N[3];
    float sticking, sqrtT, accommodation, diffuse, specular, cos_exp;
    float texw_p, texh_p;
    float pad;
};
// Per-facet integer info (32 B).
struct __align__(16) FacetInfo {
    uint32_t flags, count;      // FF_*, MFG_COUNT_*
    int32_t tex_off, tex_w;     // texture cell offset in one moment block, width in cells
    int32_t tex_h, prof_idx;
    int32_t ang_off, profile_type;
};
struct __align__(16) FacetInfo2 {
    int32_t structure, desorb_type, stick_param, temp_param;
    int32_t am_phi, am_lo, am_hi, dir_off;   // dir_off: direction-cell offset, -1 when not recorded
    double am_limit, max_speed, desorb_exp, temperature;
    double opacity;
    int32_t opac_param, link;   // link: destination structure of a link facet, -1 none
    int32_t teleport;           // teleportDest: 0 none, -1 the facet last teleported to, k facet k-1
    int32_t pad_t;
};

// Device-resident tallies.  Fixed-point scales: velocities (m/s) * 2^20,
// inverse velocities (s/m) * 2^32, distances (cm) * 2^20.
#define MFG_SCALE_V    1048576.0              /* 2^20 */
#define MFG_SCALE_INV  4294967296.0           /* 2^32 */
#define MFG_SCALE_DIST 1048576.0              /* 2^20 */
#define MFG_Q_MAX      1125899906842624.0     /* 2^50: per-sample clamp */
#define MFG_SMEM_FLUSH (1ull << 60)           /* shared partial sums move to global above this */

// global (u64 pairs = 128-bit fixed point where noted)
#define TG_HITS 0
#define TG_DES 1
#define TG_ABS 2
#define TG_LEAK 3
#define TG_DIST_LO 4   // 128-bit: distTraveled_total
#define TG_DIST_HI 5
#define TG_DISTF_LO 6  // 128-bit: distTraveledTotal_fullHitsOnly
#define TG_DISTF_HI 7
#define TG_DROPPED 8
#define TG_RECHECK 9
#define TG_STATUS 10
#define TG_N 16
// per facet per moment block (u64): counts then 128-bit sums
#define TF_HITS 0
#define TF_DES 1
#define TF_ABS 2
#define TF_S1OV 3   // lo, hi
#define TF_SVORT 5  // lo, hi
#define TF_S1V 7    // lo, hi
#define TF_N 9
// per texture cell / profile bin per moment block (u64)
#define TT_COUNT 0
#define TT_S1OV 1   // lo, hi
#define TT_SVORT 3  // lo, hi
#define TT_N 5
// shared-memory partial layouts (u64)
#define SF_HITS 0
#define SF_DES 1
#define SF_ABS 2
#define SF_S1OV 3
#define SF_SVORT 4
#define SF_S1V 5
#define SF_N 6
#define ST_N 3

// kernel status bits (TG_STATUS)
#define KS_TIMEOUT 1ull
#define KS_ABORTED 2ull
#define KS_NO_SOURCE 4ull
#define KS_STACK 8ull

// Angle-map desorption tables of one source facet (built from its recorded incident-angle map,
// MolflowSimFacet.cpp:90-215): `lo` theta lines below the limit, `hi` above, `w` phi bins; the
// offsets index DevModel::am_pool
struct AmDev {
    int32_t w, lo, hi, pad;
    double limit, lower_ratio, total;
    int32_t tcdf_lo, tcdf_hi, sum_lo, sum_hi;      // theta CDF at line midpoints, line sums
    int32_t pcdf_lo, pcdf_hi, ppdf_lo, ppdf_hi;    // phi CDFs at bin midpoints, phi pdfs
};

// Outgassing map of a source facet (MolflowSimFacet::InitializeOutgassingMap): cells along U and
// V, and the grid's extent in cells over the facet (ratio x |U|, ratio x |V|; the last row and
// column may be partial)
struct OgDev {
    int32_t w, h;
    double wp, hp;
};

// one histogram set (RecordHistograms, Particle.cpp:926-975): bin sizes, bin counts (0 = not
// recorded) and offset of the set in a moment block (-1 = none)
struct HistDev {
    uint32_t record;
    int32_t off;
    uint64_t bounce_bin;
    double dist_bin, time_bin;
    int32_t nb, nd, nt, pad;
};

struct DevModel {
    int32_t nf, nstruct;
    int32_t n_src, nm;
    const NodeD* nodes_d;
    const NodeC* nodes_c;          // FP32 two-child nodes (trace_f)
    const int32_t* prims_c;        // leaf facet lists of nodes_c, each ended by -1
    const int32_t* roots_c;        // root NodeC per structure
    const int32_t* roots;        // root node per structure
    const int32_t* prims;        // facet ids in leaf order
    const FacetIsectD* isect_d;
    const FacetIsectF* isect_f;
    const PolyD* poly_d;
    const PolyF* poly_f;
    const TriF* tri_f;             // [nf] edges of triangular facets (unused for other polygons)
    const double2* v2_d;
    const float2* v2_f;
    const FacetPhysD* phys_d;
    const FacetPhysF* phys_f;
    const FacetInfo* info;
    const FacetInfo2* info2;
    const double* center;        // 3 per facet (start point fallback)
    const double* src_cdf;       // prefix sums of source weights
    const int32_t* src_facet;
    const int32_t* src_id;       // integrated-desorption table index per source (-1 none)
    const int32_t* src_cell;     // outgassing-map cell per source (-1 none), or null without maps
    const OgDev* og;             // [nf] outgassing-map grids, or null without maps
    double src_total;
    double latest;               // latestMoment
    const double* mstart;        // moment window starts (sorted)
    const double* mend;
    double maxwin;
    // guide to the moment search: mguide[b] = number of window starts <= 2^(mg_l0 + b / mg_scale),
    // a lower bound of the search's answer for times in bucket b (null: binary search)
    const int32_t* mguide;
    double mg_t0;                // 2^mg_l0, the first bucket's start
    float mg_l0, mg_scale;
    int32_t mg_n;
    // integrated desorption tables (concatenated)
    const int32_t* id_start;
    const double* id_t;
    const double* id_cum;
    // time-dependent parameters (concatenated)
    const int32_t* par_start;
    const double* par_t;
    const double* par_v;
    const uint8_t* par_logx;
    const uint8_t* par_logy;
    double cdf_v[MFG_MAXWELL_N];
    double cdf_p[MFG_MAXWELL_N];
    double gas_mass;
    double ort_factor;           // 1.0 with Maxwell speeds, 1.1781 without (Particle.cpp:673)
    double half_life;
    int32_t use_maxwell, constant_flow, enable_decay, pad0;
    int64_t texture_cells;       // per moment block
    int64_t profile_facets;
    int64_t anglemap_cells;
    int64_t direction_cells;
    int32_t has_transparent;     // some facet has opacity < 1 or an opacity parameter
    int32_t has_ext;             // traced by the extended kernel variants (transparency, histograms, low flux)
    int32_t low_flux, pad4;      // low-flux mode (otfParams.lowFluxMode) and its cutoff weight
    double low_flux_cutoff;
    // moving facets: motion type (1 translation, 2 rotation), axis base (cm), velocity or
    // angular velocity vector
    int32_t motion_type, scatter;   // scatter: background-gas collisions on
    double mv1[3], mv2[3];
    int32_t force, log_facet;       // force measurement on; particle logger facet (-1 none)
    unsigned long long log_cap;     // particle logger capacity (records)
    double torque_ref[3];           // sp.torqueRefPoint (cm)
    int32_t scatter_cutoff, pad5;
    double sc_mass_ratio, sc_mfp, sc_rho, sc_cutoff_speed;
    // histograms recorded at absorptions: global set and per-facet sets, hist_bins per moment block
    HistDev ghist;
    const HistDev* fhist;        // [nf] or null
    const int32_t* am_of_facet;  // angle-map desorption table of each facet (-1 none), or null
    const AmDev* am_dev;
    const double* am_pool;
    int64_t hist_bins;
    double scene_scale;          // max |coordinate| of the scene (for FP32 tolerances)
    // instances of a batch (one for a plain model): source-table range and total weight
    int32_t n_inst, pad1;
    const int32_t* inst_src_base;
    const int32_t* inst_src_count;
    const double* inst_src_total;
};

struct DevTally {
    double* histogram;               // (1+M) * hist_bins (FP64 atomics)
    double* force;                   // (1+M) * nf * 9: impulse, its squares, torque (FP64 atomics), or null
    double* plog;                    // particle log: log_cap records of 8 doubles, or null
    unsigned long long* plog_n;      // records claimed (may exceed log_cap; only log_cap are written)
    // low-flux mode: weighted ("equivalent") counts, FP64 atomics; null otherwise
    double* lf_glob;                 // [2] nbHitEquiv, nbAbsEquiv
    double* lf_facet;                // (1+M) * nf * 2 (nbHitEquiv, nbAbsEquiv)
    double* lf_tex;                  // (1+M) * texture_cells (countEquiv)
    double* lf_prof;                 // (1+M) * profile_facets * 100 (countEquiv)
    unsigned long long* global;      // TG_N
    unsigned long long* facet;       // (1+M) * nf * TF_N
    unsigned long long* texture;     // (1+M) * texture_cells * TT_N
    unsigned long long* profile;     // (1+M) * profile_facets * 100 * TT_N
    unsigned long long* anglemap;    // anglemap_cells
    double* direction;               // (1+M) * direction_cells * 3: Sum of velocity vectors (FP64 atomics)
    unsigned long long* dir_count;   // (1+M) * direction_cells
};

// Per-run values live in device memory so one captured CUDA graph serves every run:
// the host fills a pinned staging copy and the graph's first node copies it over.
struct RunDesc {
    unsigned long long n_total;          // particles of all instances
    unsigned long long max_steps;
    unsigned long long time_limit_ns;    // a warp stops this long after it started
    uint32_t key0, key1;                 // Philox key
    int32_t n_inst, pad;
    // followed in memory by inst_prefix[n_inst + 1] and inst_first[n_inst] (u64)
};

// Score-function sensitivity bookkeeping (sensitivity kernel variant only)
#define MFG_SENS_NOUT 9          // 8 gauge pressures + pumped flux
#define MFG_SENS_TRAJ 1024       // reflections remembered per particle
struct SensCtl {
    const int32_t* param_of_facet;   // [nf] parameter index, -1 if the facet's sticking is not a parameter
    const int32_t* gauge_of_facet;   // [nf] gauge index 0..7, -1 otherwise
    const uint8_t* pump_of_facet;    // [nf] 1 when an absorption counts to the pumped flux
    const int32_t* src_of_facet;     // [nf] source index for outgassing gradients, -1 otherwise
    // [nf] the three maps above packed into one word per facet, read once per hit: bits 0-19
    // parameter index + 1, bits 20-23 gauge index + 1 (0: none), bit 24 pump
    const int32_t* code;
    int32_t smem_code;               // 1: the packed words are staged in shared memory
    int32_t pad_code;
    double* A;                       // [P][9] sum over (output event, earlier reflection on parameter k) of y
    double* B;                       // [P][9] sum over absorptions on parameter k of y
    double* Cs;                      // [S][9] sum of y per source
    double* Y;                       // [9] sum of y
    unsigned long long* src_count;   // [S] desorptions per source
    unsigned long long* overflow;    // particles whose reflection list overflowed
};

struct LaunchCtl {
    unsigned long long* next_particle;   // work counter (particles handed out)
    const RunDesc* run;
    const unsigned long long* inst_prefix;   // particle index ranges per instance
    const unsigned long long* inst_first;    // Philox counter of each instance's first particle
    const volatile int* abort_flag;          // host-mapped
    int smem_facets;                         // 1: moment-0 facet partials in shared memory
    int n_top;                               // FP32 BVH nodes [0, n_top) staged in shared memory
    int chunk;                               // particle ids a warp takes per work-queue request (>= 32)
    SensCtl sens;                            // used by the sensitivity variant
};
