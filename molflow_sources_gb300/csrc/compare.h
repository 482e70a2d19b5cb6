// compare.h — GlobalSimuState::Compare (MolflowSimGeom.cpp:559-1148) on the C++ host.
#pragma once
#include <string>
#include <vector>

#include "../../include/mfg.h"
#include "model_build.h"

namespace mfgx {

struct CompareResult {
    int64_t global = 0, facet = 0, fine = 0;   // error counts (facet and fine -1 when not compared)
    std::vector<std::string> messages;         // global and facet differences first, then fine ones
};

// `l` and `r`: results laid out for the model `h` (every array that the layout has, non-null).
CompareResult compare_states(const mfg::HostModel& h, const mfg_state_view& l, const mfg_state_view& r, double glob,
                             double loc_threshold);

}  // namespace mfgx
