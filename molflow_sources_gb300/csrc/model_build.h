// model_build.h — host-side preparation of a model for the GPU tracer.
//
// Replaces the parts of MolflowSimulationModel preparation the tracer depends on:
// facet geometry (the src_shared geometry initialisation), PrepareToRun
// (src/Simulation/MolflowSimGeom.cpp:194-253: latest moment, interval cache,
// Maxwell CDF, integrated desorption), CalcTotalOutgassing (:290-335), the
// texture-cell increments (src/Initializer.cpp:433-456) and BuildAccelStructure
// (:124-184, SAH BVH).  Produces flat arrays ready for upload.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/mfg.h"
#include "device_model.h"

namespace mfg {

struct HostFacet {
    double O[3], U[3], V[3], N[3], nU[3], nV[3];
    double center[3], bbmin[3], bbmax[3];
    double area;
    int vstart, nv;
};

struct HostModel {
    int nf = 0, nstruct = 1, nm = 0;
    std::vector<HostFacet> facets;
    std::vector<double> v2;               // normalised (u,v) per polygon vertex
    // parameters copied from the descriptor
    std::vector<double> sticking, opacity, outgassing, temperature, accommodation, desorb_exp;
    std::vector<double> diffuse, specular, cos_exp, texw_p, texh_p, max_speed, am_limit, soj_freq, soj_e;
    std::vector<int32_t> desorb_type, structure, link, teleport, profile_type, am_phi, am_lo, am_hi;
    std::vector<int32_t> p_stick, p_opac, p_outg, p_temp;
    std::vector<uint8_t> two_sided, am_record, sojourn, moving;
    std::vector<uint32_t> count;
    double gas_mass = 28, time_window = 1e-10, half_life = 1, low_flux_cutoff = 1e-7;
    int use_maxwell = 1, constant_flow = 1, enable_decay = 0, low_flux = 0;
    int motion_type = 0, scatter = 0, scatter_cutoff = 0;
    double mv1[3] = {0, 0, 0}, mv2[3] = {0, 0, 0};
    double sc_mass_ratio = 1, sc_mfp = 1e30, sc_rho = 0, sc_cutoff_speed = 0;
    int log_facet = -1;                   // particle logger facet (-1 none) and capacity
    int64_t log_cap = 0;
    int force = 0;                        // force measurement
    double torque_ref[3] = {0, 0, 0};
    // derived
    double latest = 0;
    std::vector<double> mstart, mend;
    double maxwin = 0;
    std::vector<int32_t> mguide;          // log-time guide to the moment search (empty: none)
    double mg_t0 = 0;
    float mg_l0 = 0, mg_scale = 0;
    double cdf_v[MFG_MAXWELL_N], cdf_p[MFG_MAXWELL_N];
    std::vector<int32_t> par_start;       // time-dependent parameters
    std::vector<double> par_t, par_v;
    std::vector<uint8_t> par_logx, par_logy;
    std::vector<int32_t> id_start;        // integrated desorption tables
    std::vector<double> id_t, id_cum;
    std::vector<int32_t> facet_id;        // ID table per facet (-1 none)
    std::vector<double> src_cdf;
    std::vector<int32_t> src_facet, src_id;
    std::vector<int32_t> src_cell;        // outgassing-map cell of each source (empty: no maps)
    std::vector<int32_t> og_w, og_h;      // outgassing-map grid per facet (0: none)
    std::vector<double> og_ru, og_rv;
    std::vector<OgDev> og;                // per facet (empty: no maps)
    double src_total = 0;
    // CalcTotalOutgassing (MolflowSimGeom.cpp:290-335): molecules desorbed up to latestMoment, and the
    // final outgassing rate in molecules/s and Pa*m3/s (the last value of a time-dependent rate)
    double total_desorbed_molecules = 0, final_outgassing_rate = 0, final_outgassing_rate_pa = 0;
    // layout
    mfg_state_layout layout{};
    std::vector<int64_t> tex_off, dir_off, ang_off, prof_idx;
    std::vector<int32_t> tex_w, tex_h;
    std::vector<double> tex_inc;          // 1/(cell area * sides) per texture cell
    // BVH (all structures concatenated, breadth-first per structure)
    std::vector<NodeD> nodes_d;
    std::vector<NodeC> nodes_c;           // FP32 two-child layout
    std::vector<int32_t> roots_c, prims_c;
    std::vector<int32_t> roots, prims;
    int64_t bvh_depth = 0, bvh_leaves = 0;
    // device records
    std::vector<FacetIsectD> isect_d;
    std::vector<FacetIsectF> isect_f;
    std::vector<PolyD> poly_d;
    std::vector<PolyF> poly_f;
    std::vector<TriF> tri_f;
    std::vector<double2> v2_d;
    std::vector<float2> v2_f;
    std::vector<FacetPhysD> phys_d;
    std::vector<FacetPhysF> phys_f;
    std::vector<FacetInfo> info;
    std::vector<FacetInfo2> info2;
    std::vector<double> centers;
    double scene_scale = 1;
    int has_transparent = 0;
    int has_ext = 0;                      // needs the extended kernel variants
    std::vector<int32_t> am_of_facet;     // angle-map desorption tables (empty: none)
    std::vector<AmDev> am_dev;
    std::vector<double> am_pool;
    HistDev ghist{};                      // histograms (off -1: none)
    std::vector<HistDev> fhist;           // per facet, empty when no facet records
    bool gpu_supported = true;
    std::string gpu_unsupported_reason;
    // instances (one for a plain model; several after merge_host_models)
    struct Instance {
        int facet_base = 0, nf = 0, struct_base = 0, nstruct = 1, src_base = 0, nsrc = 0;
        int64_t tex_base = 0, prof_base = 0, ang_base = 0, dir_base = 0;
        double src_total = 0;
    // CalcTotalOutgassing (MolflowSimGeom.cpp:290-335): molecules desorbed up to latestMoment, and the
    // final outgassing rate in molecules/s and Pa*m3/s (the last value of a time-dependent rate)
    double total_desorbed_molecules = 0, final_outgassing_rate = 0, final_outgassing_rate_pa = 0;
        mfg_state_layout layout{};
    };
    std::vector<Instance> instances;
};

// Merge prepared models into one multi-instance model (batch of independent geometries).
// All parts must share the global settings (gas, speed law, flow mode, moments).
int merge_host_models(const std::vector<const HostModel*>& parts, HostModel& out, std::string& err);

// Build a HostModel from a descriptor.  Returns MFG_OK or an error code with a message.
int build_host_model(const mfg_model_desc* d, HostModel& m, std::string& err, int leaf_max = 2);

}  // namespace mfg
