// Host build of the GPU angle-map desorption generator (molflow_sources_gb300/csrc/anglemap_gen.cuh)
// with the tables the library builds (model_build.cpp), for CPU tests: draws (theta, phi) pairs of
// a source facet from given uniforms.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include <vector_types.h>

#define __device__
#define __forceinline__ inline
#define __noinline__
#include "../../molflow_sources_gb300/csrc/device_model.h"
namespace mfgk {
constexpr double kPi = 3.14159265358979323846;
}
#include "../../molflow_sources_gb300/csrc/anglemap_gen.cuh"
#include "../../molflow_sources_gb300/csrc/model_build.h"

extern "C" int am_draw(const mfg_model_desc* d, int facet, int64_t n, const double* r, double* theta, double* phi) {
    mfg::HostModel h;
    std::string err;
    if (mfg::build_host_model(d, h, err) != MFG_OK) return 1;
    if (h.am_of_facet.empty() || h.am_of_facet[facet] < 0) return 2;
    const mfgk::AmView v{h.am_dev[h.am_of_facet[facet]], h.am_pool.data()};
    for (int64_t k = 0; k < n; ++k) {
        int i;
        double tov;
        theta[k] = mfgk::am_gen_theta(v, r[2 * k], i, tov);
        phi[k] = mfgk::am_gen_phi(v, i, tov, r[2 * k + 1]);
    }
    return 0;
}
