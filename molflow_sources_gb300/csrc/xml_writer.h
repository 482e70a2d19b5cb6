// xml_writer.h — a model and its results as a MolFlow+ file (.xml, or a .zip holding one .xml).
#pragma once
#include <string>
#include <vector>

#include "../../include/mfg.h"
#include "model_build.h"

namespace mfgx {

// Write `d` (the model's descriptor), laid out as `h` (the model built from it), and the results in
// `st` (a view laid out for that model; null: geometry and settings only).  `param_names`: names of
// the time-dependent parameters (missing or empty: "param<i>").  False with `err` on failure.
bool write_file(const std::string& path, const mfg_model_desc& d, const mfg::HostModel& h, const mfg_state_view* st,
                const std::vector<std::string>& param_names, std::string& err);

}  // namespace mfgx
