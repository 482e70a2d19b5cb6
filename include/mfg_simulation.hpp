// mfg_simulation.hpp — C++ host adapter over the C ABI (include/mfg.h).
//
// GpuSimulation offers the surface molflowCLI's thread controller uses on
// MolflowSimulation (src/Simulation/MolflowSimulation.h:22-45) and on each
// MFSim::ParticleTracer (src/Simulation/Particle.h:45,86): load a model, reset,
// step a number of desorptions, and add the results into a GlobalSimuState-shaped
// container under a timed lock (UpdateHitsAndLog, src/Simulation/Particle.cpp:21-73,
// 1294-1312).  Header-only; link against libmfg.so.  Errors are reported as
// return codes from the ABI and raised here as mfg::Error.
#pragma once
#include <chrono>
#include <cstdint>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "mfg.h"

namespace mfg {

class Error : public std::runtime_error {
public:
    Error(int code, const std::string& what) : std::runtime_error(what), code(code) {}
    int code;
};

inline std::string last_error() {
    char buf[1024];
    mfg_last_error(buf, sizeof buf);
    return buf;
}
inline void check(int rc) {
    if (rc != MFG_OK) throw Error(rc, last_error());
}

// MCStepResult of the reference (src/Simulation/Particle.h:24-28)
enum class MCStepResult { Success, DesorptionError, MaxReached };

// GlobalSimuState-shaped tallies in host memory (src/Simulation/MolflowSimGeom.h:56-154)
struct HostState {
    mfg_state_layout layout{};
    std::vector<double> global;
    std::vector<uint64_t> facet_counts;
    std::vector<double> facet_sums, texture, profile, direction;
    std::vector<uint64_t> anglemap;
    std::vector<double> histogram;
    std::vector<double> force;   // impulse, impulse_square, impulse_momentum per facet and moment
    std::timed_mutex mutex;   // simuStateMutex

    void resize(const mfg_state_layout& L) {
        layout = L;
        global.assign(size_t(L.n_global), 0.0);
        facet_counts.assign(size_t(L.n_facet_counts), 0);
        facet_sums.assign(size_t(L.n_facet_sums), 0.0);
        texture.assign(size_t(L.n_texture), 0.0);
        profile.assign(size_t(L.n_profile), 0.0);
        direction.assign(size_t(L.n_direction), 0.0);
        anglemap.assign(size_t(L.n_anglemap), 0);
        histogram.assign(size_t(L.n_histogram), 0.0);
        force.assign(size_t(L.n_force), 0.0);
    }
    mfg_state_view view() {
        return mfg_state_view{global.data(), facet_counts.data(), facet_sums.data(), texture.data(),
                              profile.data(), direction.data(), anglemap.data(), histogram.data(),
                              force.empty() ? nullptr : force.data()};
    }
    // GlobalSimuState::operator+= (src/Simulation/MolflowSimGeom.cpp:452-458)
    HostState& operator+=(const HostState& o) {
        for (size_t i = 0; i < global.size(); ++i) global[i] += o.global[i];
        for (size_t i = 0; i < facet_counts.size(); ++i) facet_counts[i] += o.facet_counts[i];
        for (size_t i = 0; i < facet_sums.size(); ++i) facet_sums[i] += o.facet_sums[i];
        for (size_t i = 0; i < texture.size(); ++i) texture[i] += o.texture[i];
        for (size_t i = 0; i < profile.size(); ++i) profile[i] += o.profile[i];
        for (size_t i = 0; i < direction.size(); ++i) direction[i] += o.direction[i];
        for (size_t i = 0; i < anglemap.size(); ++i) anglemap[i] += o.anglemap[i];
        for (size_t i = 0; i < histogram.size(); ++i) histogram[i] += o.histogram[i];
        for (size_t i = 0; i < force.size(); ++i) force[i] += o.force[i];
        return *this;
    }
};

// A MolFlow+ file (.xml, or the .xml inside a .zip; LoaderXML.cpp:31-1130): the model descriptor
// it holds (valid while the object lives) and its stored results.  `catalog_dir`: a parameter
// catalog folder whose parameters follow the file's own (LoadParameterCatalog), or null.
class XmlFile {
public:
    explicit XmlFile(const std::string& path, const char* catalog_dir = nullptr) {
        check(mfg_xml_open_catalog(path.c_str(), catalog_dir, &f_));
    }
    ~XmlFile() { mfg_xml_close(f_); }
    XmlFile(const XmlFile&) = delete;
    XmlFile& operator=(const XmlFile&) = delete;
    const mfg_model_desc& desc() const { return *mfg_xml_desc(f_); }
    bool has_results() const { return mfg_xml_has_results(f_) != 0; }
    mfg_xml* handle() const { return f_; }

private:
    mfg_xml* f_ = nullptr;
};

// The stored results of `file` laid out for `model` (a model created from file.desc()).
inline void ReadStoredResults(const XmlFile& file, const mfg_model* model, HostState& out) {
    mfg_state_layout L{};
    check(mfg_state_layout_of(model, &L));
    out.resize(L);
    mfg_state_view v = out.view();
    check(mfg_xml_read_state(file.handle(), model, &v));
}

class GpuSimulation {
public:
    explicit GpuSimulation(int device = 0) : device_(device) {}
    ~GpuSimulation() { release(); }
    GpuSimulation(const GpuSimulation&) = delete;
    GpuSimulation& operator=(const GpuSimulation&) = delete;

    // LoadSimulation (MolflowSimulation.cpp:92-154): prepare geometry, BVH, tables; upload.
    void LoadSimulation(const mfg_model_desc& desc) {
        release();
        check(mfg_model_create(&desc, &model_));
        check(mfg_sim_create(model_, device_, &sim_));
        check(mfg_state_layout_of(model_, &layout_));
    }
    // LoadSimulation from a MolFlow+ file; with `stored`, the file's results (when it holds
    // some) are read into it, the state a saved run resumes from.  Returns whether it held results.
    bool LoadSimulation(const XmlFile& file, HostState* stored = nullptr) {
        LoadSimulation(file.desc());
        if (!stored || !file.has_results()) return false;
        ReadStoredResults(file, model_, *stored);
        return true;
    }
    // SaveGeometry + SaveSimulationState (WriterXML.cpp:72-903): the loaded model (`desc`, as given
    // to LoadSimulation) and `state` (null: geometry and settings only) as a MolFlow+ file; a path
    // ending in ".zip" gets one .xml entry.  `param_names`: n_params names, or null.
    void SaveSimulationState(const std::string& path, const mfg_model_desc& desc, HostState* state,
                             const char* const* param_names = nullptr) const {
        mfg_state_view v{};
        if (state) v = state->view();
        check(mfg_xml_save(path.c_str(), &desc, model_, state ? &v : nullptr, param_names));
    }
    void ResetSimulation() { check(mfg_reset(sim_)); }
    const mfg_state_layout& layout() const { return layout_; }

    // SimulationMCStep: desorb and trace nbDesorptions particles (Particle.cpp:207-396).
    MCStepResult SimulationMCStep(uint64_t nbDesorptions, const mfg_run_options& opt, mfg_run_stats* stats = nullptr) {
        mfg_run_stats st{};
        int rc = mfg_run(sim_, nbDesorptions, &opt, &st);
        if (stats) *stats = st;
        if (rc == MFG_ERR_NO_SOURCE) return MCStepResult::DesorptionError;
        check(rc);
        return MCStepResult::Success;
    }

    // UpdateHitsAndLog: add the tallies into the global state under its timed lock, append the
    // particle log records (MFG_LOG_N doubles each) to `log` up to `log_limit` records, then clear.
    bool UpdateHitsAndLog(HostState& global, size_t timeout_ms, std::vector<double>* log = nullptr,
                          size_t log_limit = 0) {
        HostState local;
        local.resize(layout_);
        mfg_state_view v = local.view();
        check(mfg_fetch(sim_, &v));
        std::vector<double> recs;
        if (log && log_limit * MFG_LOG_N > log->size()) {
            const int64_t room = int64_t(log_limit - log->size() / MFG_LOG_N);
            recs.resize(size_t(room) * MFG_LOG_N);
            int64_t n = 0;
            check(mfg_fetch_log(sim_, recs.data(), room, &n));
            recs.resize(size_t(n) * MFG_LOG_N);
        }
        std::unique_lock<std::timed_mutex> lk(global.mutex, std::defer_lock);
        if (!lk.try_lock_for(std::chrono::milliseconds(timeout_ms))) return false;   // GetHitLock timeout
        if (global.global.empty()) global.resize(layout_);
        global += local;
        if (log) log->insert(log->end(), recs.begin(), recs.end());
        lk.unlock();
        check(mfg_reset(sim_));
        return true;
    }

    mfg_sim* handle() const { return sim_; }

private:
    void release() {
        if (sim_) mfg_sim_destroy(sim_);
        if (model_) mfg_model_destroy(model_);
        sim_ = nullptr;
        model_ = nullptr;
    }
    int device_;
    mfg_model* model_ = nullptr;
    mfg_sim* sim_ = nullptr;
    mfg_state_layout layout_{};
};

}  // namespace mfg
