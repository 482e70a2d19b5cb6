// Drives the C++ adapter (include/mfg_simulation.hpp) the way molflowCLI drives
// MolflowSimulation: build a 32-sided L/R=10 tube descriptor, load, step, merge.
// Prints "transmission <p> hits <n>" or "no-device"; exit code 0 on success.
#include <cmath>
#include <cstdio>
#include <vector>

#include "mfg_simulation.hpp"

int main(int argc, char** argv) {
    const int step = 32;
    const double L = 10.0, R = 1.0;
    std::vector<double> v(3 * 2 * step);
    for (int i = 0; i < step; ++i) {
        double a = 2.0 * M_PI * i / step;
        v[6 * i + 0] = R * std::cos(a); v[6 * i + 1] = R * std::sin(a); v[6 * i + 2] = 0.0;
        v[6 * i + 3] = R * std::cos(a); v[6 * i + 4] = R * std::sin(a); v[6 * i + 5] = L;
    }
    std::vector<int32_t> start{0}, idx;
    for (int i = 0; i < step; ++i) idx.push_back(2 * i);
    start.push_back(int32_t(idx.size()));
    for (int k = 0; k < step; ++k) idx.push_back(2 * (step - 1 - k) + 1);
    start.push_back(int32_t(idx.size()));
    for (int i = 0; i < step; ++i) {
        int j = (i + 1) % step;
        idx.insert(idx.end(), {2 * i, 2 * i + 1, 2 * j + 1, 2 * j});
        start.push_back(int32_t(idx.size()));
    }
    const int nf = step + 2;
    std::vector<double> sticking(nf, 0.0), outgassing(nf, 0.0);
    std::vector<int32_t> des(nf, MFG_DES_NONE);
    sticking[0] = sticking[1] = 1.0;
    outgassing[0] = 1.0;
    des[0] = MFG_DES_COSINE;
    mfg_model_desc d{};
    d.abi_version = MFG_ABI_VERSION;
    d.n_vertices = 2 * step;
    d.vertices = v.data();
    d.n_facets = nf;
    d.facet_vertex_start = start.data();
    d.facet_vertex_index = idx.data();
    d.sticking = sticking.data();
    d.outgassing = outgassing.data();
    d.desorb_type = des.data();
    d.gas_mass = 28.0;
    d.use_maxwell = 1;
    d.constant_flow = 1;
    d.time_window = 1e-10;
    d.n_structures = 1;
    mfg::GpuSimulation sim(0);
    try {
        sim.LoadSimulation(d);
    } catch (const mfg::Error& e) {
        if (e.code == MFG_ERR_NO_DEVICE) { std::printf("no-device\n"); return 0; }
        std::printf("error %d %s\n", e.code, e.what());
        return 1;
    }
    mfg_run_options o{};
    o.precision = argc > 1 ? MFG_PREC_FP32R : MFG_PREC_FP64;
    o.seed = 0x4D6F6C66;
    mfg::HostState global;
    for (int t = 0; t < 4; ++t) {
        if (sim.SimulationMCStep(50000, o) != mfg::MCStepResult::Success) return 2;
        if (!sim.UpdateHitsAndLog(global, 1000)) return 3;
    }
    double p = double(global.facet_counts[1 * MFG_FC_N + MFG_FC_NBABSORBED]) / global.global[MFG_G_NBDESORBED];
    std::printf("transmission %.6f hits %.0f desorbed %.0f\n", p, global.global[MFG_G_NBMCHIT], global.global[MFG_G_NBDESORBED]);
    return 0;
}
