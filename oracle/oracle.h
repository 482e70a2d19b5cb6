/*
 * oracle.h — CPU FP64 restatement of MolFlow+'s test-particle tracer.
 *
 * TEST INFRASTRUCTURE.  This code is the checker for the GB300 library: only the
 * tests, the smoke check and bench.py's CPU-baseline leg may load it.  The product
 * path never calls it.
 *
 * It restates, in plain C with OpenMP (one tracer per thread, as
 * src/Simulation/MolflowSimulation.cpp:44-55), the algorithm of
 *   src/Simulation/Particle.cpp:207-1379   (SimulationMCStep and the Record* tallies)
 *   src/Simulation/Physics.cpp:6-19         (Maxwell speed, desorption time)
 *   src/Simulation/CDFGeneration.cpp:54-83  (Maxwell CDF)
 *   src/Simulation/IDGeneration.cpp:45-207  (integrated desorption)
 *   src/Simulation/MolflowSimGeom.cpp:194-335 (PrepareToRun, CalcTotalOutgassing)
 *   src/Simulation/SimulationMC.cpp:15-40   (time-dependent sticking/opacity/temperature)
 * plus the geometry primitives that live in the (absent) src_shared submodule,
 * restated from their observable contract: facet (O,U,V,N) basis, crossing-number
 * point-in-polygon, SAH BVH with 2 facets per leaf, ray/facet intersection that
 * skips the last hit facet and back faces of one-sided facets.
 *
 * Parity status: pinned statistically against the reference's stored converged
 * states (tests/TestCases/B01, B02, 01 via tests/golden); bit-level parity with
 * the reference is unpinned because its RNG and intersection code are absent.
 */
#ifndef MFG_ORACLE_H
#define MFG_ORACLE_H

#include "../include/mfg.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_model orc_model;

#define ORC_RNG_PHILOX 0   /* Philox4x32-10 stream per particle (same streams as the GPU kernels) */
#define ORC_RNG_MT     1   /* MT19937 per thread seeded 42424242+thread (MolflowSimulation.cpp:50) */

typedef struct orc_run_opts {
    uint64_t seed;
    uint64_t first_particle;   /* particle id of the first desorption (Philox counter) */
    int32_t  n_threads;        /* 0 = all cores */
    int32_t  rng_mode;         /* ORC_RNG_* */
    uint64_t max_steps;        /* bounce cap per particle, 0 = 2^40 */
    uint32_t instance;         /* batch instance id: word 3 of the Philox counter */
} orc_run_opts;

typedef struct orc_stats {
    uint64_t desorbed, hits, leaks, dropped;
    uint64_t rays;             /* Intersect calls */
    uint64_t node_visits;      /* BVH nodes whose box was tested */
    uint64_t prim_tests;       /* facet intersection tests */
    double   seconds;
    int32_t  threads;
} orc_stats;

int  orc_model_create(const mfg_model_desc* desc, orc_model** out, char* err, size_t errlen);
void orc_model_destroy(orc_model* m);
int  orc_layout(const orc_model* m, mfg_state_layout* out);
/* derived facet basis: O,U,V,N,nU,nV (18 doubles per facet) and area */
int  orc_facet_geometry(const orc_model* m, double* out18, double* area);
/* Simulate n_des particles and ADD the tallies into view (like UpdateMCHits). */
int  orc_run(orc_model* m, uint64_t n_des, const orc_run_opts* o, mfg_state_view* view, orc_stats* st);
/* orc_run that also returns the particle log (LogHit records, MFG_LOG_N doubles each) of all
 * threads, up to log_capacity records; *log_n receives the number returned. */
int  orc_run_logged(orc_model* m, uint64_t n_des, const orc_run_opts* o, mfg_state_view* view, orc_stats* st,
                    double* log, int64_t log_capacity, int64_t* log_n);
/* orc_run with score-function sensitivity sums (the GPU's mfg_sens_forward bookkeeping): per
 * facet its parameter index (-1 none), gauge index 0..7 (-1 none) and whether absorptions count
 * to the pumped flux (output 8).  Adds into A[n_params*9] (Sum over output events and earlier
 * reflections on parameter k of the event's value), B[n_params*9] (absorptions on parameter k
 * counted to the pumped flux), Y[9] (Sum of values), *overflow (particles whose reflection list
 * overflowed).  d output_j / d sticking_k = (-A[k][j]/(1-s_k) + B[k][j]/s_k) / n. */
int  orc_run_sens(orc_model* m, uint64_t n_des, const orc_run_opts* o, mfg_state_view* view, orc_stats* st,
                  const int32_t* param_of_facet, const int32_t* gauge_of_facet, const uint8_t* pump_of_facet,
                  int32_t n_params, double* A, double* B, double* Y, uint64_t* overflow);
/* Intersect given rays (replay mode). */
int  orc_replay(orc_model* m, int64_t n, const double* origin, const double* dir, const int32_t* last,
                int32_t* hit_facet, double* hit_t, orc_stats* st);
/* Record the first max_rays rays traced by a Philox run (origin, direction, last facet, hit facet, t). */
int64_t orc_record_rays(orc_model* m, uint64_t n_des, uint64_t seed, int64_t max_rays,
                        double* origin, double* dir, int32_t* last, int32_t* hit_facet, double* hit_t);
/* Philox4x32-10 block for tests: out[4] from counter[4], key[2]. */
void orc_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* Angle-map desorption check: resample n incident-angle pairs from a recorded map (uniforms
 * r[2n]) and bin them like the map (out[(lo+hi)*w] is added to). */
int orc_anglemap_resample(const uint64_t* pdf, int w, int lo, int hi, double limit, int64_t n, const double* r,
                          uint64_t* out);
/* Maxwell CDF at 1 K (100 entries of speed, cumulative probability). */
void orc_maxwell_cdf(double gas_mass, double* speed, double* cumul);

#ifdef __cplusplus
}
#endif
#endif
