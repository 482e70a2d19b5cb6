// xml_model.h — a MolFlow+ XML file read into a model descriptor it owns, and its stored results.
#pragma once
#include <string>
#include <vector>

#include "../../include/mfg.h"
#include "model_build.h"
#include "xml_file.h"

namespace mfgx {

struct XmlModel {
    XDoc doc;                              // kept for the results
    std::vector<double> vertices;
    std::vector<int32_t> fv_start, fv_index;
    std::vector<double> sticking, opacity, outgassing, temperature, accommodation, desorb_exponent;
    std::vector<double> refl_diffuse, refl_specular, refl_cos_exponent, tex_width, tex_height, max_speed;
    std::vector<double> am_theta_limit, sojourn_freq, sojourn_e;
    std::vector<int32_t> desorb_type, structure, link_dest, teleport_dest, profile_type;
    std::vector<int32_t> am_phi_width, am_lower, am_higher;
    std::vector<int32_t> sticking_param, opacity_param, outgassing_param, temperature_param;
    std::vector<uint8_t> is_2sided, am_record, enable_sojourn, is_moving;
    std::vector<uint32_t> count_flags;
    std::vector<mfg_histogram_params> facet_hist;
    std::vector<double> moment_time, moment_window;
    std::vector<int32_t> param_start;
    std::vector<double> param_t, param_v;
    std::vector<uint8_t> param_log_x, param_log_y;
    std::vector<std::string> param_names;
    std::vector<uint64_t> desorb_anglemap;
    std::vector<int32_t> og_w, og_h;
    std::vector<double> og_ru, og_rv, og_cells;
    mfg_model_desc desc{};

    // Read `path` (.xml, or the .xml inside a .zip) and fill `desc`; false with `err` on failure.
    // `catalog_dir`: a parameter catalog folder whose parameters follow the file's own (or null).
    bool load(const std::string& path, std::string& err, const char* catalog_dir = nullptr);
};

// Stored results of the document (MolflowResults, LoaderXML.cpp:366-760) into a view laid out for
// the model built from the same file; MFG_ERR_INVALID_ARGUMENT when the file holds none.
int read_results(const XNode* root, const mfg::HostModel& h, mfg_state_view* view, std::string& err);

}  // namespace mfgx
