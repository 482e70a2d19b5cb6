/*
 * mfg.h — C ABI of the GB300 test-particle Monte Carlo tracer.
 *
 * This library replaces the CPU worker threads that run MolFlow+'s
 * `MFSim::ParticleTracer::SimulationMCStep` (src/Simulation/Particle.cpp:207-396)
 * and the BVH `Intersect` it calls (src/Simulation/Particle.cpp:245).  The caller
 * hands over a `MolflowSimulationModel`-equivalent flat descriptor and reads back
 * a `GlobalSimuState`-shaped result (src/Simulation/MolflowSimGeom.h:106-154).
 *
 * Conventions
 *   - Plain C: pointers, sizes, int status codes.  No exception crosses the ABI.
 *   - Every `const` pointer in a descriptor is read during the call that takes it
 *     and copied; the caller keeps ownership.
 *   - Units follow the reference: lengths in cm, time in s, speeds in m/s,
 *     outgassing in Pa*m^3/s, temperature in K, gas mass in g/mol.
 *   - One handle is used by one host thread at a time (the library serialises
 *     calls on a handle with a mutex); different handles are independent.
 */
#ifndef MFG_H
#define MFG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MFG_ABI_VERSION 6u

/* ---- status codes (replace the reference's exceptions / MCStepResult,
 *      src/Simulation/Particle.h:24-28, src/Simulation/MolflowSimGeom.cpp:219-247) ---- */
#define MFG_OK                       0
#define MFG_ERR_INVALID_MODEL        1  /* model descriptor rejected (SanityCheck, MolflowSimGeom.cpp:337-404) */
#define MFG_ERR_NO_SOURCE            2  /* no desorbing facet (MCStepResult::DesorptionError, Particle.cpp:228-231,466-469) */
#define MFG_ERR_TIMEOUT              3  /* wait or kernel time limit reached (GetHitLock timeout, MolflowSimGeom.cpp:1239-1248) */
#define MFG_ERR_ABORTED              4  /* mfg_abort() was called while running */
#define MFG_ERR_CUDA                 5  /* CUDA runtime error; text in mfg_last_error */
#define MFG_ERR_UNSUPPORTED_FEATURE  6  /* model uses a feature the library does not trace */
#define MFG_ERR_INVALID_ARGUMENT     7
#define MFG_ERR_BUSY                 8  /* a run is still in flight on this handle */
#define MFG_ERR_NO_DEVICE            9
#define MFG_ERR_LIMIT               10  /* a size exceeds a documented limit */

/* Size limits of a model (MFG_ERR_LIMIT past them): structures; texture, direction and angle-map
 * cells and histogram bins of one moment block, each at most 2^31-1 (32-bit device offsets). */
#define MFG_MAX_STRUCTURES       65536

/* desorption types, src/MolflowTypes.h:17-21 */
#define MFG_DES_NONE      0
#define MFG_DES_UNIFORM   1
#define MFG_DES_COSINE    2
#define MFG_DES_COSINE_N  3
#define MFG_DES_ANGLEMAP  4

/* profile types, src/MolflowTypes.h:29-35 */
#define MFG_PROFILE_NONE          0
#define MFG_PROFILE_U             1
#define MFG_PROFILE_V             2
#define MFG_PROFILE_ANGULAR       3
#define MFG_PROFILE_VELOCITY      4
#define MFG_PROFILE_ORT_VELOCITY  5
#define MFG_PROFILE_TAN_VELOCITY  6
#define MFG_PROFILE_SIZE        100   /* bins per profile (value stored by the reference's fixtures) */

/* texture recording flags (facet sh.countDes/countAbs/countRefl/countTrans/countDirection) */
#define MFG_COUNT_DES    1u
#define MFG_COUNT_ABS    2u
#define MFG_COUNT_REFL   4u
#define MFG_COUNT_TRANS  8u
#define MFG_COUNT_DIR   16u

/* fields of one FacetHitBuffer in a state view (fields named at Particle.cpp:1200-1207) */
#define MFG_FC_NBMCHIT    0   /* facet_counts: u64 */
#define MFG_FC_NBDESORBED 1
#define MFG_FC_NBABSORBED 2
#define MFG_FC_N          3
#define MFG_FS_NBHITEQUIV          0   /* facet_sums: double */
#define MFG_FS_NBABSEQUIV          1
#define MFG_FS_SUM_1_PER_ORT_VEL   2
#define MFG_FS_SUM_V_ORT           3
#define MFG_FS_SUM_1_PER_VELOCITY  4
#define MFG_FS_N                   5
/* global counters (GlobalHitBuffer, Particle.cpp:36-45) */
#define MFG_G_NBMCHIT      0
#define MFG_G_NBHITEQUIV   1
#define MFG_G_NBDESORBED   2
#define MFG_G_NBABSEQUIV   3
#define MFG_G_NBLEAK       4
#define MFG_G_DIST_TOTAL   5
#define MFG_G_DIST_FULLHITS 6
#define MFG_G_N            8

/* Histogram settings (HistogramParams): which of the number of bounces, the flight distance
 * (cm) and the flight time (s) since desorption an absorption is binned by.  Bin counts: bounces
 * bounce_max/bounce_binsize + 2 (integer division), distance and time (size_t)(max/binsize) + 1;
 * the last bin takes every larger value. */
#define MFG_HIST_BOUNCE   1u
#define MFG_HIST_DISTANCE 2u
#define MFG_HIST_TIME     4u
typedef struct mfg_histogram_params {
    uint32_t record;                   /* MFG_HIST_* bits */
    uint32_t pad;
    uint64_t bounce_binsize, bounce_max;
    double   distance_binsize, distance_max;
    double   time_binsize, time_max;
} mfg_histogram_params;

/*
 * Model descriptor: the fields of MolflowSimulationModel that the tracer reads
 * (src/Simulation/MolflowSimGeom.h:158-232, facet fields used in Particle.cpp).
 * Per-facet arrays have n_facets entries.  Optional arrays may be NULL and then
 * take the reference's defaults (given in brackets).
 */
typedef struct mfg_model_desc {
    uint32_t abi_version;              /* MFG_ABI_VERSION */
    int32_t  n_vertices;
    const double*  vertices;           /* [n_vertices*3] (x,y,z) cm — vertices3 */
    int32_t  n_facets;
    const int32_t* facet_vertex_start; /* [n_facets+1] offsets into facet_vertex_index */
    const int32_t* facet_vertex_index; /* polygon vertex indices (facet->indices), right-hand rule gives N */

    const double*  sticking;           /* sh.sticking                     [0] */
    const double*  opacity;            /* sh.opacity                      [1] */
    const double*  outgassing;         /* sh.outgassing Pa*m3/s           [0] */
    const double*  temperature;        /* sh.temperature K                [293.15] */
    const double*  accommodation;      /* sh.accomodationFactor           [1] */
    const int32_t* desorb_type;        /* sh.desorbType                   [DES_NONE] */
    const double*  desorb_exponent;    /* sh.desorbTypeN                  [0] */
    const double*  refl_diffuse;       /* sh.reflection.diffusePart       [1] */
    const double*  refl_specular;      /* sh.reflection.specularPart      [0] */
    const double*  refl_cos_exponent;  /* sh.reflection.cosineExponent    [0] */
    const uint8_t* is_2sided;          /* sh.is2sided                     [0] */
    const int32_t* structure;          /* sh.superIdx (-1: all structures) [0] */
    const int32_t* link_dest;          /* sh.superDest (0: none)          [0] */
    const int32_t* teleport_dest;      /* sh.teleportDest (0: none)       [0] */
    const double*  tex_width;          /* sh.texWidth_precise (0: no texture)  [0] */
    const double*  tex_height;         /* sh.texHeight_precise            [0] */
    const uint32_t* count_flags;       /* MFG_COUNT_* bits                [0] */
    const int32_t* profile_type;       /* sh.profileType                  [PROFILE_NONE] */
    const double*  max_speed;          /* sh.maxSpeed for velocity profiles [0] */
    const int32_t* anglemap_phi_width;       /* anglemapParams.phiWidth (record when >0 and record flag) [0] */
    const double*  anglemap_theta_limit;     /* anglemapParams.thetaLimit  [1.570796326] */
    const int32_t* anglemap_theta_lower_res; /* anglemapParams.thetaLowerRes [0] */
    const int32_t* anglemap_theta_higher_res;/* anglemapParams.thetaHigherRes [0] */
    const uint8_t* anglemap_record;          /* anglemapParams.record [0] */
    const int32_t* sticking_param;     /* index into params (-1: constant) [-1] */
    const int32_t* opacity_param;      /* [-1] */
    const int32_t* outgassing_param;   /* [-1] */
    const int32_t* temperature_param;  /* [-1] */
    const uint8_t* enable_sojourn;     /* sh.enableSojournTime [0] */
    const double*  sojourn_freq;       /* sh.sojournFreq [0] */
    const double*  sojourn_e;          /* sh.sojournE J/mol [0] */
    const uint8_t* is_moving;          /* sh.isMoving [0] */

    /* simulation parameters (MolflowSimulationModel::sp, otfParams) */
    double   gas_mass;                 /* sp.gasMass g/mol */
    int32_t  use_maxwell;              /* sp.useMaxwellDistribution */
    int32_t  constant_flow;            /* sp.calcConstantFlow */
    double   time_window;              /* sp.timeWindowSize s (latestMoment when no moments) */
    int32_t  enable_decay;             /* sp.enableDecay */
    double   half_life;                /* sp.halfLife s */
    int32_t  low_flux_mode;            /* otfParams.lowFluxMode */
    double   low_flux_cutoff;          /* otfParams.lowFluxCutoff */
    int32_t  n_structures;             /* sh.nbSuper (>=1, at most MFG_MAX_STRUCTURES) */

    /* time moments (tdParams.moments): centre and window, sorted by centre */
    int32_t  n_moments;
    const double* moment_time;
    const double* moment_window;

    /* time-dependent parameters (tdParams.parameters): piecewise (t, value) tables */
    int32_t  n_params;
    const int32_t* param_start;        /* [n_params+1] offsets into param_t/param_v */
    const double*  param_t;
    const double*  param_v;
    const uint8_t* param_log_x;        /* logXinterp [0] */
    const uint8_t* param_log_y;        /* logYinterp [0] */

    /* histograms recorded at each absorption (RecordHistograms, Particle.cpp:926-975) */
    mfg_histogram_params global_histogram;          /* sp.globalHistogramParams */
    const mfg_histogram_params* facet_histogram;    /* sh.facetHistogramParams [n_facets] or NULL */

    /* moving facets (sp.motionType, motionVector1/2; Physics::TreatMovingFacet, Physics.cpp:25-39):
     * 0 none, 1 translation with velocity motion_vector2 (m/s), 2 rotation about the axis
     * through motion_vector1 (cm) with angular velocity vector motion_vector2 (rad/s).  The
     * facet's velocity is added to a particle leaving a facet with is_moving set. */
    int32_t  motion_type;
    double   motion_vector1[3];
    double   motion_vector2[3];
    /* background-gas scattering (sp.scattering; PerformScatter, Particle.cpp:840-886): free
     * paths exponential with mean scatter_mean_free_path_cm, impact parameter within
     * scatter_rho, test/background mass ratio scatter_mass_ratio; with the cutoff on, a particle
     * slower than scatter_cutoff_speed (m/s) after a collision ends */
    int32_t  scatter_enabled;
    int32_t  scatter_cutoff_enabled;
    double   scatter_mass_ratio;
    double   scatter_mean_free_path_cm;
    double   scatter_rho;
    double   scatter_cutoff_speed;
    /* angle-map desorption (DES_ANGLEMAP; AnglemapGeneration.cpp): the recorded incident-angle
     * counts of every facet with desorb_type MFG_DES_ANGLEMAP, in facet order, each
     * anglemap_phi_width * (lower_res + higher_res) counts (theta-major, as recorded); NULL when
     * no facet desorbs by angle map */
    const uint64_t* desorb_anglemap;
    /* outgassing maps (useOutgassingFile; StartFromSource, Particle.cpp:425-446 and 513-535;
     * MolflowSimFacet::InitializeOutgassingMap, MolflowSimFacet.cpp:224-239).  A facet with
     * outgassing_map_width[i] > 0 (array NULL: none) desorbs from its map instead of
     * `outgassing`: outgassing_map holds, for those facets in facet order, width x height cell
     * rates (Pa m^3/s, row-major: height rows of width cells along U).  The facet's weight among
     * the sources is the sum of its cells, a cell is chosen by its rate and the start point is
     * uniform in the cell; the grid has ratio_u * |U| by ratio_v * |V| cells over the facet
     * (outgassingFileRatioU/V), so its last row and column may be partial. */
    const int32_t*  outgassing_map_width;
    const int32_t*  outgassing_map_height;
    const double*   outgassing_map_ratio_u;
    const double*   outgassing_map_ratio_v;
    const double*   outgassing_map;
    /* force measurement (sp.enableForceMeasurement, sp.torqueRefPoint; IncreaseFacetCounter,
     * Particle.cpp:1194-1230): per facet and moment, the sums of the momentum v*d carried onto the
     * facet (a leaving particle counts -v*d), of its componentwise squares, and of the torque
     * (o - ref) x v*d about torque_ref_point (cm x m/s), for desorptions, hits and absorptions;
     * passes carry none */
    int32_t  enable_force_measurement;
    double   torque_ref_point[3];
    /* BVH split weights, one per facet (RebuildAccelStructure with SplitMethod::ProbSplit,
     * MolflowSimGeom.cpp:155-169: the share of nbHitEquiv each facet took in a prior run); NULL
     * builds by the surface-area heuristic alone.  Only the tree changes, never the results. */
    const double* bvh_facet_weight;
    /* particle logger (otfParams.enableLogging, logFacetId, logLimit; LogHit, Particle.cpp:1088-1102):
     * each desorption from, hit on, absorption on, link pass through and teleport from facet
     * log_facet (0-based; -1 none) is recorded, up to log_limit records until mfg_reset (mfg_fetch_log) */
    int32_t  log_facet;
    int64_t  log_limit;
} mfg_model_desc;

/*
 * Result view: caller-owned buffers laid out like GlobalSimuState
 * (src/Simulation/MolflowSimGeom.h:56-154).  Sizes come from mfg_state_layout().
 * Moment block 0 is constant flow, blocks 1..n_moments the time moments.
 * Any pointer may be NULL (that part is skipped).
 */
typedef struct mfg_state_layout {
    int64_t n_facets;
    int64_t n_moments;             /* blocks per facet = 1 + n_moments */
    int64_t texture_cells;         /* sum over textured facets of texWidth*texHeight */
    int64_t profile_facets;        /* facets with a profile */
    int64_t direction_cells;       /* sum over facets with countDirection of texWidth*texHeight */
    int64_t anglemap_cells;        /* sum over recording facets of phiWidth*(lowerRes+higherRes) */
    /* element counts of each view array */
    int64_t n_global;              /* MFG_G_N */
    int64_t n_facet_counts;        /* (1+M)*F*MFG_FC_N */
    int64_t n_facet_sums;          /* (1+M)*F*MFG_FS_N */
    int64_t n_texture;             /* (1+M)*texture_cells*3  (countEquiv, sum_v_ort_per_area, sum_1_per_ort_velocity) */
    int64_t n_profile;             /* (1+M)*profile_facets*PROFILE_SIZE*3 (countEquiv, sum_v_ort, sum_1_per_ort_velocity) */
    int64_t n_direction;           /* (1+M)*direction_cells*4 (dir.x, dir.y, dir.z, count) */
    int64_t n_anglemap;            /* anglemap_cells */
    int64_t histogram_bins;        /* bins of one moment block: the global histograms (bounce,
                                      distance, time, those recorded), then each facet's in id order */
    int64_t n_histogram;           /* (1+M)*histogram_bins */
    int64_t n_force;               /* (1+M)*F*9 with force measurement (impulse, impulse_square,
                                      impulse_momentum, x y z each), else 0 */
} mfg_state_layout;

typedef struct mfg_state_view {
    double*   global;        /* [n_global] */
    uint64_t* facet_counts;  /* [n_facet_counts] */
    double*   facet_sums;    /* [n_facet_sums] */
    double*   texture;       /* [n_texture] */
    double*   profile;       /* [n_profile] */
    double*   direction;     /* [n_direction] */
    uint64_t* anglemap;      /* [n_anglemap] */
    double*   histogram;     /* [n_histogram] */
    double*   force;         /* [n_force] */
} mfg_state_view;

/* Run options (precision, RNG, launch shape). */
#define MFG_PREC_FP64    0   /* plain FP64 traversal, polygon tests and physics */
#define MFG_PREC_FP32R   1   /* FP32 traversal/tests + FP64 recheck and FP64 new origin */

typedef struct mfg_run_options {
    int32_t  precision;          /* MFG_PREC_* */
    uint64_t seed;               /* Philox key; replaces MersenneTwister seeding (MolflowSimulation.cpp:44-55) */
    int32_t  block_size;         /* threads per block, 0 = autotuned default */
    int32_t  blocks_per_sm;      /* 0 = occupancy maximum */
    int32_t  smem_bvh_levels;    /* FP32R: the first 2^levels FP32 BVH nodes (breadth-first: the top levels) are
                                    staged in shared memory per block, 1..12; 0 = the autotuned choice (none
                                    before mfg_autotune); -1 = none */
    double   time_limit_s;       /* kernel self-stops after this wall time (status MFG_ERR_TIMEOUT), 0 = 600 s */
    uint64_t max_steps_per_particle; /* a particle that exceeds this many bounces is dropped and counted, 0 = 2^40 */
    int32_t  use_graph;          /* 1: launch through a captured CUDA graph (captured once per launch shape) */
    int32_t  particles_per_request; /* particle ids a warp takes from the shared work queue per request,
                                    32..65536; 0 = the autotuned choice (64 before mfg_autotune) */
} mfg_run_options;

/* Run statistics of the last run (filled by mfg_run / mfg_wait). */
typedef struct mfg_run_stats {
    uint64_t desorbed;           /* particles started in this run */
    uint64_t hits;               /* nbMCHit added in this run */
    uint64_t leaks;
    uint64_t rechecks;           /* FP32R: rays re-intersected in FP64 */
    uint64_t dropped;            /* particles dropped at max_steps_per_particle */
    double   kernel_ms;          /* tracing kernel time, CUDA events on the launch stream */
    double   total_ms;           /* whole call incl. set-up and flushes */
    int32_t  status;
    int32_t  kernel_launches;    /* kernels this library launched for the run */
} mfg_run_stats;

typedef struct mfg_model mfg_model;
typedef struct mfg_sim mfg_sim;

/* ---- library ---- */
uint32_t mfg_abi_version(void);
/* Last error text of the calling thread (copied into buf, NUL terminated). Returns its length. */
size_t   mfg_last_error(char* buf, size_t buflen);

/* ---- model: replaces MolflowSimulationModel construction + PrepareToRun +
 *      BuildAccelStructure (MolflowSimGeom.cpp:124-253) ---- */
int mfg_model_create(const mfg_model_desc* desc, mfg_model** out);
void mfg_model_destroy(mfg_model* model);
int mfg_state_layout_of(const mfg_model* model, mfg_state_layout* out);
/* Merge prepared models into one batch model of n instances (C4-style batching; no reference
 * counterpart: the reference runs one model per process).  Instances keep their own geometry,
 * BVH, sources and tallies; they must share gas, speed law, flow mode and moments. */
int mfg_model_merge(const mfg_model* const* models, int32_t n, mfg_model** out);
int32_t mfg_model_instances(const mfg_model* model);
/* Layout of instance i's own GlobalSimuState (for mfg_fetch_instance). */
int mfg_instance_layout(const mfg_model* model, int32_t i, mfg_state_layout* out);
/* Derived per-facet geometry as computed by the library (O,U,V,N,nU,nV as 18 doubles per facet, area) for checks. */
int mfg_model_facet_geometry(const mfg_model* model, double* out18, double* area);
/* Outgassing totals of the model (CalcTotalOutgassing, MolflowSimGeom.cpp:290-335): molecules desorbed
 * up to the latest moment (sp.totalDesorbedMolecules), the final outgassing rate in molecules/s
 * (sp.finalOutgassingRate) and in Pa*m3/s (sp.finalOutgassingRate_Pa_m3_sec).  Any pointer may be NULL. */
int mfg_model_outgassing(const mfg_model* model, double* total_desorbed_molecules, double* final_rate,
                         double* final_rate_pa_m3_s);
/* ---- MolFlow+ files on the host (LoaderXML.cpp:31-1130): a .xml file, or the .xml inside a
 *      .zip (the form the reference saves and its test cases use), read into a model descriptor
 *      that the handle owns (valid until mfg_xml_close), plus the file's stored results. ---- */
typedef struct mfg_xml mfg_xml;
int mfg_xml_open(const char* path, mfg_xml** out);
/* The same with a parameter catalog folder (LoadParameterCatalog, MolflowSimGeom.cpp:1250-1319): its
 * .csv parameters ("[catalog] <file name>", file-name order) follow the file's own parameters, as
 * the reference inserts them; facets may refer to them by name or index.  NULL: no catalog. */
int mfg_xml_open_catalog(const char* path, const char* catalog_dir, mfg_xml** out);
const mfg_model_desc* mfg_xml_desc(const mfg_xml* file);
/* 1 when the file holds stored results (a MolflowResults element), else 0. */
int32_t mfg_xml_has_results(const mfg_xml* file);
/* Stored results (MolflowResults, LoaderXML.cpp:366-760) into a view laid out for `model`, a model
 * created from mfg_xml_desc of the same file: every array of the view is cleared, then filled. */
int mfg_xml_read_state(const mfg_xml* file, const mfg_model* model, mfg_state_view* out);
void mfg_xml_close(mfg_xml* file);
/* GlobalSimuState::Compare (MolflowSimGeom.cpp:559-1148), the test suite's acceptance rule (called
 * with 0.009 and 0.07, tests/testsuite.cpp:460): two results laid out for `model` (every array of its
 * layout present) -> counts[0..2] = global, facet and fine error counts (facet and fine -1 when the
 * states have no desorptions); a run passes when the first two are 0.  `messages` (may be NULL)
 * receives one line per difference, global and facet ones first, cut to buflen - 1 bytes. */
int mfg_compare_states(const mfg_model* model, const mfg_state_view* a, const mfg_state_view* b, double glob_threshold,
                       double loc_threshold, int64_t counts[3], char* messages, size_t buflen);
/* SaveGeometry + SaveSimulationState (WriterXML.cpp:72-903): the model `desc` (as `model` was created
 * from it) and the results in `state` (a view laid out for `model`; NULL: geometry and settings only)
 * as a MolFlow+ file; a path ending in ".zip" gets one stored .xml entry.  `param_names`: n_params
 * names of the time-dependent parameters, or NULL ("param<i>"). */
int mfg_xml_save(const char* path, const mfg_model_desc* desc, const mfg_model* model, const mfg_state_view* state,
                 const char* const* param_names);

/* BVH statistics: node count, depth, leaf count. */
int mfg_model_bvh_info(const mfg_model* model, int64_t* nodes, int64_t* depth, int64_t* leaves);

/* ---- simulation: replaces MolflowSimulation (MolflowSimulation.h:22-45) and the
 *      ParticleTracer worker threads (Particle.h:40-129) ---- */
int mfg_sim_create(const mfg_model* model, int device, mfg_sim** out);
void mfg_sim_destroy(mfg_sim* sim);
/* Zero all tallies (GlobalSimuState::Reset, MolflowSimGeom.cpp:527-548).  The particle
 * counter keeps running, as the reference's random generators do across a reset. */
int mfg_reset(mfg_sim* sim);
/* Philox counter of the next particle to desorb (0 after mfg_sim_create).  Ranks or
 * replicas that split one run use disjoint ranges. */
int mfg_set_particle_offset(mfg_sim* sim, uint64_t first_particle);
uint64_t mfg_particle_offset(const mfg_sim* sim);
/* Desorb and trace n_desorptions particles to absorption or leak; blocking.
 * Replaces SimulationMCStep(nbStep, threadNum, remainingDes) over all threads
 * (Particle.cpp:207-396) with the desorption limit as the work unit. */
int mfg_run(mfg_sim* sim, uint64_t n_desorptions, const mfg_run_options* opt, mfg_run_stats* stats);
/* Batch (several models merged with mfg_model_merge): counts[i] particles for instance i, one
 * persistent launch over a shared particle queue.  mfg_run gives every instance n particles. */
int mfg_run_batch(mfg_sim* sim, const uint64_t* counts, const mfg_run_options* opt, mfg_run_stats* stats);
int mfg_run_batch_async(mfg_sim* sim, const uint64_t* counts, const mfg_run_options* opt);
/* Asynchronous form: mfg_run_async returns at once; mfg_wait blocks up to timeout_ms. */
int mfg_run_async(mfg_sim* sim, uint64_t n_desorptions, const mfg_run_options* opt);
int mfg_poll(mfg_sim* sim);                      /* MFG_OK when done, MFG_ERR_BUSY while running */
int mfg_wait(mfg_sim* sim, int64_t timeout_ms, mfg_run_stats* stats);
int mfg_abort(mfg_sim* sim);                     /* sets the host-mapped abort word read by the kernel */
/* Copy accumulated tallies into the caller's view (overwrites). Replaces
 * UpdateMCHits / GlobalSimuState::operator+= (Particle.cpp:21-73, MolflowSimGeom.cpp:452-458). */
int mfg_fetch(mfg_sim* sim, mfg_state_view* view);

/* Particle log of the runs since the last mfg_reset (ParticleLog, MolflowSimGeom.h:242-270; merged
 * by UpdateHitsAndLog, Particle.cpp:1294-1312): up to `capacity` records of MFG_LOG_N doubles
 * (u, v, theta, phi to the facet basis, oriRatio, expected decay moment, time, speed), in no
 * particular order; *n_records receives the number copied. */
#define MFG_LOG_N 8
int mfg_fetch_log(mfg_sim* sim, double* records, int64_t capacity, int64_t* n_records);

/* Autotuner: times short trial runs (n_trial desorptions each) over block sizes and register
 * budgets for the given precision, keeps the fastest launch shape as this handle's default
 * (used when mfg_run_options.block_size and blocks_per_sm are 0) and writes it to *best.
 * Trial tallies are cleared; the particle counter keeps running.  No reference counterpart:
 * the reference has fixed CPU threads (MolflowSimulation.cpp:44-55). */
int mfg_autotune(mfg_sim* sim, uint64_t n_trial, int32_t precision, uint64_t seed, mfg_run_options* best);

/* Tallies of one instance of a batch, in that instance's own layout (overwrites). */
int mfg_fetch_instance(mfg_sim* sim, int32_t instance, mfg_state_view* view);

/* Change sticking coefficients of facets between runs (parameter sweeps, finite differences).
 * Replaces editing sh.sticking and reloading (ParameterParser.cpp:240-248). */
int mfg_update_sticking(mfg_sim* sim, int32_t n, const int32_t* facets, const double* values);

/* Score-function sensitivities, an autograd-Function-shaped pair (no reference counterpart).
 * Outputs y[9]: Sum v_ort per desorbed particle on up to 8 gauge facets (pressure up to
 * MolPerTP/area) and absorptions per desorbed particle on the pump facets (pumped flux).
 * Parameters: sticking of param_facets (each in (0,1)) and the outgassing of every source.
 * mfg_sens_forward traces n particles with the sensitivity kernel and stores the Jacobian;
 * mfg_sens_backward returns dL/dsticking[P] and dL/doutgassing[S] for a given dL/dy[9]. */
int mfg_sens_setup(mfg_sim* sim, int32_t n_params, const int32_t* param_facets, int32_t n_gauges,
                   const int32_t* gauge_facets, int32_t n_pumps, const int32_t* pump_facets);
int32_t mfg_sens_sources(const mfg_sim* sim);
int mfg_sens_forward(mfg_sim* sim, uint64_t n, const mfg_run_options* opt, double* outputs, mfg_run_stats* stats);
/* d y / d sticking [P x 9], d y / d outgassing [S x 9] (per molecule/s of source s), source facet ids [S] */
int mfg_sens_jacobian(mfg_sim* sim, double* d_sticking, double* d_outgassing, int32_t* source_facets);
int mfg_sens_backward(mfg_sim* sim, const double* dl_dy, double* dl_dsticking, double* dl_doutgassing);

/* Replay mode: intersect caller-given rays (no physics).  For ray i:
 * origin[3i..], direction[3i..], last_facet[i] (facet to skip, -1 none).
 * Out: hit_facet[i] (-1 = no hit), hit_t[i] (distance in |direction| units).
 * Replaces one `Intersect(ray)` call per ray (Particle.cpp:245). Host buffers. */
int mfg_replay(mfg_sim* sim, int32_t precision, int64_t n_rays,
               const double* origin, const double* direction, const int32_t* last_facet,
               int32_t* hit_facet, double* hit_t, uint64_t* n_rechecks);

/* Replay that allocates no device memory.  No counterpart in the reference.
 * For callers that cannot allocate on the device during a query: a process whose device memory
 * belongs to another framework's pool allocator, or a loop that must not block in cudaMalloc or
 * cudaFree (they can synchronise the device).  d_origin, d_direction, d_last, d_hit_facet and
 * d_hit_t are device pointers with the meaning of mfg_replay's host buffers.  The FP64 recheck
 * queue lives in a fixed 8 MiB array in the library, so n may not exceed 1,048,576 rays
 * (MFG_ERR_LIMIT otherwise).  The first call on a device looks up that array's device address;
 * make it before any stream capture.  The array is shared by all calls and keeps the last
 * call's contents: each call clears the counters it needs, and calls that overlap on the GPU
 * race.  Runs on the handle's stream and returns when the results are written. */
int mfg_replay_noalloc(mfg_sim* sim, int32_t precision, int64_t n, const double* d_origin, const double* d_direction,
                       const int32_t* d_last, int32_t* d_hit_facet, double* d_hit_t, uint64_t* n_rechecks);

#ifdef __cplusplus
}
#endif
#endif /* MFG_H */
