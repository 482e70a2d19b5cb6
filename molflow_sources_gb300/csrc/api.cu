// api.cu — the extern "C" boundary declared in include/mfg.h.
//
// Owns the CUDA side: device copies of a model, tally buffers, the launch of the
// persistent tracer on a private stream, host-side waits with time limits, and
// the conversion of fixed-point tallies to the GlobalSimuState field layout.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/mfg.h"
#include "model_build.h"
#include "trace_kernels.cuh"
#include "xml_model.h"
#include "xml_writer.h"
#include "compare.h"

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}
int cuda_fail(cudaError_t e, const char* what) {
    g_err = std::string(what) + ": " + cudaGetErrorString(e);
    return MFG_ERR_CUDA;
}
#define CK(call)                                         \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

template <class T>
int upload(std::vector<void*>& owned, const std::vector<T>& v, const T** out) {
    if (v.empty()) { *out = nullptr; return MFG_OK; }
    void* p = nullptr;
    CK(cudaMalloc(&p, sizeof(T) * v.size()));
    owned.push_back(p);
    CK(cudaMemcpy(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
    *out = static_cast<const T*>(p);
    return MFG_OK;
}

inline double u128(const unsigned long long* p) {
    return double(p[1]) * 18446744073709551616.0 + double(p[0]);
}

}  // namespace

struct mfg_model {
    mfg::HostModel h;
};

struct mfg_sim {
    const mfg_model* model = nullptr;
    int device = 0;
    int sm_count = 0;
    std::vector<void*> owned;
    DevModel dm{};
    DevTally dt{};
    unsigned long long* d_counter = nullptr;
    int* h_abort = nullptr;      // host-mapped
    int* d_abort = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    size_t n_global = TG_N, n_facet = 0, n_texture = 0, n_profile = 0, n_anglemap = 0, n_dir = 0, n_hist = 0;
    size_t n_lf = 0;   // low-flux equivalent counts: 2 global + facet pairs + texture cells + profile bins
    size_t n_force = 0;   // force measurement sums
    std::vector<uint64_t> particles_started;   // per instance
    unsigned char* h_run = nullptr;            // pinned RunDesc + prefix + first (staging)
    unsigned char* d_run = nullptr;
    size_t run_bytes = 0;
    cudaGraphExec_t graph_exec = nullptr;
    long long graph_key[6] = {-1, -1, -1, -1, -1, -1};   // launch shape of the captured graph
    bool running = false;
    mfg_run_stats pending{};
    std::vector<unsigned long long> g_before;
    std::chrono::steady_clock::time_point t_start;
    std::mutex mu;
    int launches = 0;
    int tuned_block[2] = {0, 0};     // per precision, from mfg_autotune
    int tuned_bps[2] = {0, 0};
    int tuned_levels[2] = {0, 0};    // top BVH levels staged in shared memory (FP32R)
    int tuned_chunk[2] = {0, 0};     // particle ids per work-queue request
    std::vector<double> sticking;    // current sticking per facet (mfg_update_sticking)
    // sensitivity state (mfg_sens_*)
    bool sens_ready = false;
    std::vector<int32_t> sens_params, sens_src;
    SensCtl sens{};
    size_t sens_bytes = 0;
    void* sens_block = nullptr;
    std::vector<double> js, jq, jy;
    // pinned staging of the tallies for mfg_fetch (allocated at the first fetch, kept)
    unsigned long long* h_stage = nullptr;
    size_t stage_words = 0;
};

// Runs fn(begin, end) over [0, n) on up to 16 host threads (one when n is small): the conversion
// of fixed-point tallies into the caller's FP64 layout, tens of MB for a 200k-facet model.
template <class Fn>
static void parallel_range(size_t n, Fn fn) {
    const size_t grain = 1 << 16;
    unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    nt = unsigned(std::min<size_t>(nt, (n + grain - 1) / grain));
    if (nt <= 1) { fn(size_t(0), n); return; }
    std::vector<std::thread> th;
    const size_t chunk = (n + nt - 1) / nt;
    for (unsigned t = 0; t < nt; ++t) {
        const size_t b = size_t(t) * chunk, e = std::min(n, b + chunk);
        if (b < e) th.emplace_back(fn, b, e);
    }
    for (auto& x : th) x.join();
}

extern "C" {

uint32_t mfg_abi_version(void) { return MFG_ABI_VERSION; }

size_t mfg_last_error(char* buf, size_t buflen) {
    if (buf && buflen) {
        size_t n = std::min(buflen - 1, g_err.size());
        std::memcpy(buf, g_err.data(), n);
        buf[n] = 0;
    }
    return g_err.size();
}

int mfg_model_create(const mfg_model_desc* desc, mfg_model** out) {
    if (!out) return fail(MFG_ERR_INVALID_ARGUMENT, "out is null");
    *out = nullptr;
    auto* m = new mfg_model();
    std::string err;
    int rc = mfg::build_host_model(desc, m->h, err);
    if (rc != MFG_OK) {
        delete m;
        return fail(rc, err);
    }
    if (m->h.bvh_depth >= mfgk::kStack - 2) {
        delete m;
        return fail(MFG_ERR_LIMIT, "BVH deeper than the traversal stack");
    }
    *out = m;
    return MFG_OK;
}

void mfg_model_destroy(mfg_model* model) { delete model; }

int mfg_state_layout_of(const mfg_model* model, mfg_state_layout* out) {
    if (!model || !out) return fail(MFG_ERR_INVALID_ARGUMENT, "null argument");
    *out = model->h.layout;
    return MFG_OK;
}

int mfg_model_facet_geometry(const mfg_model* model, double* out18, double* area) {
    if (!model) return fail(MFG_ERR_INVALID_ARGUMENT, "null model");
    for (int i = 0; i < model->h.nf; ++i) {
        const auto& F = model->h.facets[i];
        if (out18) {
            double* o = out18 + 18 * size_t(i);
            for (int a = 0; a < 3; ++a) {
                o[a] = F.O[a]; o[3 + a] = F.U[a]; o[6 + a] = F.V[a];
                o[9 + a] = F.N[a]; o[12 + a] = F.nU[a]; o[15 + a] = F.nV[a];
            }
        }
        if (area) area[i] = F.area;
    }
    return MFG_OK;
}

int mfg_model_outgassing(const mfg_model* model, double* total_desorbed_molecules, double* final_rate,
                         double* final_rate_pa_m3_s) {
    if (!model) return fail(MFG_ERR_INVALID_ARGUMENT, "null model");
    if (total_desorbed_molecules) *total_desorbed_molecules = model->h.total_desorbed_molecules;
    if (final_rate) *final_rate = model->h.final_outgassing_rate;
    if (final_rate_pa_m3_s) *final_rate_pa_m3_s = model->h.final_outgassing_rate_pa;
    return MFG_OK;
}

// ---- MolFlow+ files on the host (LoaderXML.cpp:31-1130) ----
struct mfg_xml {
    mfgx::XmlModel m;
};

int mfg_xml_open(const char* path, mfg_xml** out) { return mfg_xml_open_catalog(path, nullptr, out); }

int mfg_xml_open_catalog(const char* path, const char* catalog_dir, mfg_xml** out) {
    if (!path || !out) return fail(MFG_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    auto* f = new mfg_xml();
    std::string err;
    if (!f->m.load(path, err, catalog_dir)) {
        delete f;
        return fail(MFG_ERR_INVALID_ARGUMENT, std::string(path) + ": " + err);
    }
    *out = f;
    return MFG_OK;
}

const mfg_model_desc* mfg_xml_desc(const mfg_xml* file) { return file ? &file->m.desc : nullptr; }

int32_t mfg_xml_has_results(const mfg_xml* file) {
    return file && file->m.doc.root() && file->m.doc.root()->child("MolflowResults") ? 1 : 0;
}

int mfg_xml_read_state(const mfg_xml* file, const mfg_model* model, mfg_state_view* out) {
    if (!file || !model || !out) return fail(MFG_ERR_INVALID_ARGUMENT, "null argument");
    if (model->h.nf != file->m.desc.n_facets)
        return fail(MFG_ERR_INVALID_ARGUMENT, "the model has " + std::to_string(model->h.nf) + " facets, the file " +
                                                  std::to_string(file->m.desc.n_facets));
    std::string err;
    const int rc = mfgx::read_results(file->m.doc.root(), model->h, out, err);
    return rc == MFG_OK ? MFG_OK : fail(rc, err);
}

void mfg_xml_close(mfg_xml* file) { delete file; }

int mfg_compare_states(const mfg_model* model, const mfg_state_view* a, const mfg_state_view* b, double glob_threshold,
                       double loc_threshold, int64_t counts[3], char* messages, size_t buflen) {
    if (!model || !a || !b || !counts) return fail(MFG_ERR_INVALID_ARGUMENT, "null argument");
    const mfg_state_layout& L = model->h.layout;
    for (const mfg_state_view* v : {a, b})
        if (!v->global || !v->facet_counts || !v->facet_sums || (L.n_texture && !v->texture) || (L.n_profile && !v->profile) ||
            (L.n_direction && !v->direction) || (L.n_histogram && !v->histogram))
            return fail(MFG_ERR_INVALID_ARGUMENT, "a compared view lacks an array of the model's layout");
    const mfgx::CompareResult r = mfgx::compare_states(model->h, *a, *b, glob_threshold, loc_threshold);
    counts[0] = r.global;
    counts[1] = r.facet;
    counts[2] = r.fine;
    if (messages && buflen) {
        std::string all;
        for (const std::string& m : r.messages) { all += m; all += '\n'; }
        const size_t n = std::min(all.size(), buflen - 1);
        std::memcpy(messages, all.data(), n);
        messages[n] = '\0';
    }
    return MFG_OK;
}

int mfg_xml_save(const char* path, const mfg_model_desc* desc, const mfg_model* model, const mfg_state_view* state,
                 const char* const* param_names) {
    if (!path || !desc || !model) return fail(MFG_ERR_INVALID_ARGUMENT, "null argument");
    if (desc->n_facets != model->h.nf)
        return fail(MFG_ERR_INVALID_ARGUMENT, "the descriptor has " + std::to_string(desc->n_facets) + " facets, the model " +
                                                  std::to_string(model->h.nf));
    std::vector<std::string> names;
    if (param_names)
        for (int p = 0; p < desc->n_params; ++p) names.push_back(param_names[p] ? param_names[p] : "");
    std::string err;
    if (!mfgx::write_file(path, *desc, model->h, state, names, err)) return fail(MFG_ERR_INVALID_ARGUMENT, err);
    return MFG_OK;
}

int mfg_model_bvh_info(const mfg_model* model, int64_t* nodes, int64_t* depth, int64_t* leaves) {
    if (!model) return fail(MFG_ERR_INVALID_ARGUMENT, "null model");
    if (nodes) *nodes = int64_t(model->h.nodes_d.size());
    if (depth) *depth = model->h.bvh_depth;
    if (leaves) *leaves = model->h.bvh_leaves;
    return MFG_OK;
}

static int sim_upload(mfg_sim* s) {
    const mfg::HostModel& h = s->model->h;
    DevModel& M = s->dm;
    std::memset(&M, 0, sizeof M);
    M.nf = h.nf;
    M.nstruct = h.nstruct;
    M.n_src = int32_t(h.src_facet.size());
    M.nm = h.nm;
    int rc;
#define UP(vec, field) if ((rc = upload(s->owned, vec, &M.field)) != MFG_OK) return rc
    UP(h.nodes_d, nodes_d);
    UP(h.nodes_c, nodes_c);
    UP(h.prims_c, prims_c);
    UP(h.roots_c, roots_c);
    UP(h.roots, roots);
    UP(h.prims, prims);
    UP(h.isect_d, isect_d);
    UP(h.isect_f, isect_f);
    UP(h.poly_d, poly_d);
    UP(h.poly_f, poly_f);
    UP(h.tri_f, tri_f);
    UP(h.v2_d, v2_d);
    UP(h.v2_f, v2_f);
    UP(h.phys_d, phys_d);
    UP(h.phys_f, phys_f);
    UP(h.info, info);
    UP(h.info2, info2);
    UP(h.centers, center);
    UP(h.src_cdf, src_cdf);
    UP(h.src_facet, src_facet);
    UP(h.src_id, src_id);
    UP(h.src_cell, src_cell);
    UP(h.og, og);
    UP(h.mstart, mstart);
    UP(h.mend, mend);
    UP(h.mguide, mguide);
    UP(h.id_start, id_start);
    UP(h.id_t, id_t);
    UP(h.id_cum, id_cum);
    UP(h.par_start, par_start);
    UP(h.par_t, par_t);
    UP(h.par_v, par_v);
    UP(h.par_logx, par_logx);
    UP(h.par_logy, par_logy);
    UP(h.fhist, fhist);
    UP(h.am_of_facet, am_of_facet);
    UP(h.am_dev, am_dev);
    UP(h.am_pool, am_pool);
#undef UP
    M.src_total = h.src_total;
    M.latest = h.latest;
    M.maxwin = h.maxwin;
    M.mg_t0 = h.mg_t0;
    M.mg_l0 = h.mg_l0;
    M.mg_scale = h.mg_scale;
    M.mg_n = int32_t(h.mguide.size());
    for (int i = 0; i < MFG_MAXWELL_N; ++i) { M.cdf_v[i] = h.cdf_v[i]; M.cdf_p[i] = h.cdf_p[i]; }
    M.gas_mass = h.gas_mass;
    M.ort_factor = h.use_maxwell ? 1.0 : 1.1781;
    M.half_life = h.half_life;
    M.use_maxwell = h.use_maxwell;
    M.constant_flow = h.constant_flow;
    M.enable_decay = h.enable_decay;
    M.texture_cells = h.layout.texture_cells;
    M.profile_facets = h.layout.profile_facets;
    M.anglemap_cells = h.layout.anglemap_cells;
    M.direction_cells = h.layout.direction_cells;
    M.scene_scale = h.scene_scale;
    M.has_transparent = h.has_transparent;
    M.has_ext = h.has_ext;
    M.low_flux = h.low_flux;
    M.pad4 = 0;
    M.low_flux_cutoff = h.low_flux_cutoff;
    M.motion_type = h.motion_type;
    M.scatter = h.scatter;
    for (int k = 0; k < 3; ++k) { M.mv1[k] = h.mv1[k]; M.mv2[k] = h.mv2[k]; }
    M.force = h.force;
    M.log_facet = h.log_facet;
    M.log_cap = (unsigned long long)h.log_cap;
    for (int k = 0; k < 3; ++k) M.torque_ref[k] = h.torque_ref[k];
    M.scatter_cutoff = h.scatter_cutoff;
    M.pad5 = 0;
    M.sc_mass_ratio = h.sc_mass_ratio;
    M.sc_mfp = h.sc_mfp;
    M.sc_rho = h.sc_rho;
    M.sc_cutoff_speed = h.sc_cutoff_speed;
    M.ghist = h.ghist;
    M.hist_bins = h.layout.histogram_bins;
    {
        std::vector<int32_t> sb, sc;
        std::vector<double> st;
        for (const auto& in : h.instances) { sb.push_back(in.src_base); sc.push_back(in.nsrc); st.push_back(in.src_total); }
        M.n_inst = int32_t(h.instances.size());
        if ((rc = upload(s->owned, sb, &M.inst_src_base)) != MFG_OK) return rc;
        if ((rc = upload(s->owned, sc, &M.inst_src_count)) != MFG_OK) return rc;
        if ((rc = upload(s->owned, st, &M.inst_src_total)) != MFG_OK) return rc;
        s->particles_started.assign(h.instances.size(), 0);
        s->run_bytes = sizeof(RunDesc) + 8 * (2 * h.instances.size() + 1);
        CK(cudaHostAlloc((void**)&s->h_run, s->run_bytes, cudaHostAllocDefault));
        void* q = nullptr;
        CK(cudaMalloc(&q, s->run_bytes));
        s->owned.push_back(q);
        s->d_run = static_cast<unsigned char*>(q);
    }
    // tallies
    const size_t B = 1 + size_t(h.nm);
    s->n_facet = B * size_t(h.nf) * TF_N;
    s->n_texture = B * size_t(h.layout.texture_cells) * TT_N;
    s->n_profile = B * size_t(h.layout.profile_facets) * MFG_PROFILE_SIZE * TT_N;
    s->n_anglemap = size_t(h.layout.anglemap_cells);
    s->n_dir = B * size_t(h.layout.direction_cells);
    s->n_hist = B * size_t(h.layout.histogram_bins);
    auto alloc = [&](unsigned long long** p, size_t n) -> int {
        *p = nullptr;
        if (!n) return MFG_OK;
        void* q = nullptr;
        CK(cudaMalloc(&q, n * sizeof(unsigned long long)));
        s->owned.push_back(q);
        *p = static_cast<unsigned long long*>(q);
        return MFG_OK;
    };
    if ((rc = alloc(&s->dt.global, TG_N))) return rc;
    if ((rc = alloc(&s->dt.facet, s->n_facet))) return rc;
    if ((rc = alloc(&s->dt.texture, s->n_texture))) return rc;
    if ((rc = alloc(&s->dt.profile, s->n_profile))) return rc;
    if ((rc = alloc(&s->dt.anglemap, s->n_anglemap))) return rc;
    if ((rc = alloc(&s->dt.dir_count, s->n_dir))) return rc;
    if ((rc = alloc(reinterpret_cast<unsigned long long**>(&s->dt.direction), 3 * s->n_dir))) return rc;
    if ((rc = alloc(reinterpret_cast<unsigned long long**>(&s->dt.histogram), s->n_hist))) return rc;
    s->n_force = size_t(h.layout.n_force);
    if ((rc = alloc(reinterpret_cast<unsigned long long**>(&s->dt.force), s->n_force))) return rc;
    if (h.log_cap > 0) {
        if ((rc = alloc(reinterpret_cast<unsigned long long**>(&s->dt.plog), size_t(h.log_cap) * MFG_LOG_N))) return rc;
        if ((rc = alloc(&s->dt.plog_n, 1))) return rc;
    }
    if (h.low_flux) {
        const size_t nfc = B * size_t(h.nf) * 2, ntx = B * size_t(h.layout.texture_cells),
                     npr = B * size_t(h.layout.profile_facets) * MFG_PROFILE_SIZE;
        s->n_lf = 2 + nfc + ntx + npr;
        double* base = nullptr;
        if ((rc = alloc(reinterpret_cast<unsigned long long**>(&base), s->n_lf))) return rc;
        s->dt.lf_glob = base;
        s->dt.lf_facet = base + 2;
        s->dt.lf_tex = base + 2 + nfc;
        s->dt.lf_prof = base + 2 + nfc + ntx;
    }
    if ((rc = alloc(&s->d_counter, 1))) return rc;
    return MFG_OK;
}

int mfg_reset(mfg_sim* s) {
    if (!s) return fail(MFG_ERR_INVALID_ARGUMENT, "null sim");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->running) return fail(MFG_ERR_BUSY, "run in flight");
    CK(cudaSetDevice(s->device));
    CK(cudaMemsetAsync(s->dt.global, 0, TG_N * 8, s->stream));
    if (s->n_facet) CK(cudaMemsetAsync(s->dt.facet, 0, s->n_facet * 8, s->stream));
    if (s->n_texture) CK(cudaMemsetAsync(s->dt.texture, 0, s->n_texture * 8, s->stream));
    if (s->n_profile) CK(cudaMemsetAsync(s->dt.profile, 0, s->n_profile * 8, s->stream));
    if (s->n_anglemap) CK(cudaMemsetAsync(s->dt.anglemap, 0, s->n_anglemap * 8, s->stream));
    if (s->n_dir) {
        CK(cudaMemsetAsync(s->dt.dir_count, 0, s->n_dir * 8, s->stream));
        CK(cudaMemsetAsync(s->dt.direction, 0, s->n_dir * 24, s->stream));
    }
    if (s->n_hist) CK(cudaMemsetAsync(s->dt.histogram, 0, s->n_hist * 8, s->stream));
    if (s->n_force) CK(cudaMemsetAsync(s->dt.force, 0, s->n_force * 8, s->stream));
    if (s->dt.plog_n) CK(cudaMemsetAsync(s->dt.plog_n, 0, 8, s->stream));
    if (s->n_lf) CK(cudaMemsetAsync(s->dt.lf_glob, 0, s->n_lf * 8, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return MFG_OK;
}

int mfg_set_particle_offset(mfg_sim* s, uint64_t first_particle) {
    if (!s) return fail(MFG_ERR_INVALID_ARGUMENT, "null sim");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->running) return fail(MFG_ERR_BUSY, "run in flight");
    for (auto& p : s->particles_started) p = first_particle;
    return MFG_OK;
}

uint64_t mfg_particle_offset(const mfg_sim* s) { return (s && !s->particles_started.empty()) ? s->particles_started[0] : 0; }

int mfg_sim_create(const mfg_model* model, int device, mfg_sim** out) {
    if (!model || !out) return fail(MFG_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) return fail(MFG_ERR_NO_DEVICE, "no CUDA device available");
    if (device < 0 || device >= ndev) return fail(MFG_ERR_NO_DEVICE, "device index out of range");
    auto* s = new mfg_sim();
    s->model = model;
    s->device = device;
    auto bail = [&](int rc) {
        mfg_sim_destroy(s);
        return rc;
    };
    if ((e = cudaSetDevice(device)) != cudaSuccess) return bail(cuda_fail(e, "cudaSetDevice"));
    cudaDeviceProp prop;
    if ((e = cudaGetDeviceProperties(&prop, device)) != cudaSuccess) return bail(cuda_fail(e, "cudaGetDeviceProperties"));
    s->sm_count = prop.multiProcessorCount;
    if ((e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking)) != cudaSuccess) return bail(cuda_fail(e, "stream"));
    if ((e = cudaEventCreate(&s->ev0)) != cudaSuccess) return bail(cuda_fail(e, "event"));
    if ((e = cudaEventCreate(&s->ev1)) != cudaSuccess) return bail(cuda_fail(e, "event"));
    if ((e = cudaHostAlloc(&s->h_abort, sizeof(int), cudaHostAllocMapped)) != cudaSuccess) return bail(cuda_fail(e, "cudaHostAlloc"));
    *s->h_abort = 0;
    if ((e = cudaHostGetDevicePointer(&s->d_abort, s->h_abort, 0)) != cudaSuccess) return bail(cuda_fail(e, "mapped pointer"));
    int rc = sim_upload(s);
    if (rc != MFG_OK) return bail(rc);
    s->sticking.resize(model->h.nf);
    for (int i = 0; i < model->h.nf; ++i) s->sticking[i] = model->h.phys_d[i].sticking;
    rc = mfg_reset(s);
    if (rc != MFG_OK) return bail(rc);
    *out = s;
    return MFG_OK;
}

void mfg_sim_destroy(mfg_sim* s) {
    if (!s) return;
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    for (void* p : s->owned) cudaFree(p);
    if (s->h_abort) cudaFreeHost(s->h_abort);
    if (s->h_run) cudaFreeHost(s->h_run);
    if (s->h_stage) cudaFreeHost(s->h_stage);
    if (s->graph_exec) cudaGraphExecDestroy(s->graph_exec);
    if (s->sens_block) cudaFree(s->sens_block);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

static int read_global(mfg_sim* s, std::vector<unsigned long long>& g) {
    g.assign(TG_N, 0);
    CK(cudaMemcpyAsync(g.data(), s->dt.global, TG_N * 8, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return MFG_OK;
}

// tracer kernel of a launch variant (see launch_run)
static const void* kernel_of(int variant) {
    switch (variant) {
        case 2: return (const void*)mfgk::trace_kernel<true, 2>;
        case 3: return (const void*)mfgk::trace_kernel<true, 3>;
        case 4: return (const void*)mfgk::trace_kernel<true, 4>;
        case 6: return (const void*)mfgk::trace_kernel<true, 6>;
        case 8: return (const void*)mfgk::trace_kernel<true, 8>;
        case 9: return (const void*)mfgk::trace_kernel<true, 4, false, false, 512>;
        case 10: return (const void*)mfgk::trace_kernel<true, 2, false, false, 1024>;
        case 18: return (const void*)mfgk::trace_kernel<true, 8, false, false, 256, true>;
        case 20: return (const void*)mfgk::trace_kernel<true, 2, false, false, 1024, true>;
        case 12: return (const void*)mfgk::trace_kernel<false, 2, true>;
        case 13: return (const void*)mfgk::trace_kernel<true, 3, true>;
        case 14: return (const void*)mfgk::trace_kernel<true, 2, true>;
        case 15: return (const void*)mfgk::trace_kernel<true, 4, true>;
        case 100: return (const void*)mfgk::trace_kernel<false, 2, false, true>;
        case 102: return (const void*)mfgk::trace_kernel<true, 2, false, true>;
        case 112: return (const void*)mfgk::trace_kernel<false, 2, true, true>;
        case 113: return (const void*)mfgk::trace_kernel<true, 3, true, true>;
        case 203: return (const void*)mfgk::trace_kernel<false, 3>;
        case 204: return (const void*)mfgk::trace_kernel<false, 4>;
        default: return (const void*)mfgk::trace_kernel<false, 2>;
    }
}

static int launch_run(mfg_sim* s, const uint64_t* counts, const mfg_run_options* opt, bool sens = false) {
    const mfg::HostModel& h = s->model->h;
    if (!h.gpu_supported) return fail(MFG_ERR_UNSUPPORTED_FEATURE, "not traced on the GPU: " + h.gpu_unsupported_reason);
    const int ni = int(h.instances.size());
    for (int i = 0; i < ni; ++i)
        if (counts[i] > 0 && h.instances[i].nsrc == 0)
            return fail(MFG_ERR_NO_SOURCE, "no desorbing facet (total outgassing is zero) in instance " + std::to_string(i));
    mfg_run_options o{};
    if (opt) o = *opt;
    if (o.precision != MFG_PREC_FP64 && o.precision != MFG_PREC_FP32R) return fail(MFG_ERR_INVALID_ARGUMENT, "unknown precision");
    CK(cudaSetDevice(s->device));
    int rc = read_global(s, s->g_before);
    if (rc) return rc;
    *s->h_abort = 0;
    // per-run descriptor into the pinned staging buffer
    RunDesc* R = reinterpret_cast<RunDesc*>(s->h_run);
    unsigned long long* prefix = reinterpret_cast<unsigned long long*>(s->h_run + sizeof(RunDesc));
    unsigned long long* first = prefix + ni + 1;
    uint64_t total = 0;
    prefix[0] = 0;
    for (int i = 0; i < ni; ++i) {
        first[i] = s->particles_started[i];
        total += counts[i];
        prefix[i + 1] = total;
    }
    R->n_total = total;
    R->max_steps = o.max_steps_per_particle ? o.max_steps_per_particle : (1ull << 40);
    double lim = o.time_limit_s > 0 ? o.time_limit_s : 600.0;
    R->time_limit_ns = (unsigned long long)(lim * 1e9);
    R->key0 = uint32_t(o.seed);
    R->key1 = uint32_t(o.seed >> 32);
    R->n_inst = ni;
    LaunchCtl C{};
    C.next_particle = s->d_counter;
    C.run = reinterpret_cast<const RunDesc*>(s->d_run);
    C.inst_prefix = reinterpret_cast<const unsigned long long*>(s->d_run + sizeof(RunDesc));
    C.inst_first = C.inst_prefix + ni + 1;
    C.abort_flag = s->d_abort;
    if (sens) {
        C.sens = s->sens;
        C.sens.smem_code = size_t(h.nf) * 4 <= 48 * 1024 ? 1 : 0;   // packed per-facet words in shared memory
    }
    // the autotuned shape, unless it is one the sensitivity variants are not compiled for (512- and
    // 1024-thread blocks): those runs keep their default shape
    if (o.block_size == 0 && o.blocks_per_sm == 0 && s->tuned_block[o.precision] &&
        !(sens && s->tuned_block[o.precision] > 256)) {
        o.block_size = s->tuned_block[o.precision];
        o.blocks_per_sm = s->tuned_bps[o.precision];
    }
    // staged BVH levels: 0 = the autotuned choice (none before mfg_autotune), -1 = none
    if (o.smem_bvh_levels == 0) o.smem_bvh_levels = s->tuned_levels[o.precision];
    int block = o.block_size > 0 ? o.block_size : 256;
    if (block % 32 || (block > 256 && block != 512 && block != 1024) || (block > 256 && (sens || h.has_ext)))
        return fail(MFG_ERR_INVALID_ARGUMENT,
                    "block_size must be a multiple of 32 up to 256, or 512 / 1024 (plain FP32R models)");
    if (block > 256 && o.precision != MFG_PREC_FP32R)
        return fail(MFG_ERR_INVALID_ARGUMENT, "512- and 1024-thread blocks are compiled for FP32R only");
    if (o.smem_bvh_levels > 12) return fail(MFG_ERR_INVALID_ARGUMENT, "smem_bvh_levels is at most 12");
    if (o.particles_per_request == 0) o.particles_per_request = s->tuned_chunk[o.precision] ? s->tuned_chunk[o.precision] : 64;
    if (o.particles_per_request < 32 || o.particles_per_request > 65536)
        return fail(MFG_ERR_INVALID_ARGUMENT, "particles_per_request must be 32..65536");
    C.chunk = o.particles_per_request;
    const int bps_req = block == 512 ? 4 : (block == 1024 ? 2 : std::max(1, int(o.blocks_per_sm)));
    // moment-0 facet partials in shared memory when they fit the block's share of the SM (228 KB)
    const size_t fac_bytes = size_t(h.nf) * SF_N * 8;
    C.smem_facets = fac_bytes <= std::min<size_t>(96 * 1024, 200 * 1024 / size_t(bps_req)) ? 1 : 0;
    C.n_top = o.precision == MFG_PREC_FP32R && o.smem_bvh_levels > 0 && !sens
                  ? int(std::min<size_t>(size_t(1) << o.smem_bvh_levels, h.nodes_c.size())) : 0;
    size_t dyn = (TG_N + (C.smem_facets ? size_t(h.nf) * SF_N : 0)) * 8 + size_t(C.n_top) * sizeof(NodeC) +
                 (sens && C.sens.smem_code ? size_t(h.nf) * 4 : 0);
    // kernel variant: FP64 compiled for at least 2, 3 or 4 resident blocks per SM (register budgets
    // 128, 80, 64), FP32R for 2, 3, 4, 6 or 8 (128, 80, 64, 40, 32); blocks_per_sm selects the
    // variant.  Models with transparent facets, histograms, low-flux mode, scattering, moving
    // facets, angle-map desorption, teleports, forces or the particle logger use the extended
    // variants.
    int variant = 0;
    const int b = int(o.blocks_per_sm);
    if (sens) {   // FP32R sensitivity kernel at the register budget of 2, 3 or 4 resident blocks
        variant = o.precision == MFG_PREC_FP32R ? (b >= 4 ? 15 : (b == 3 ? 13 : 14)) : 12;
    } else if (o.precision == MFG_PREC_FP32R) {
        variant = (b == 3 || b == 4 || b == 6 || b == 8) ? b : (b == 5 ? 4 : (b == 7 ? 6 : (b > 8 ? 8 : 2)));
        if (block == 512) variant = 9;     // 4 blocks of 512 threads, 32 registers
        if (block == 1024) variant = 10;   // 2 blocks of 1024 threads, 32 registers
        if (C.n_top > 0) {                 // staged BVH levels: compiled for 8 x 256 and 2 x 1024
            if (variant != 8 && variant != 10)
                return fail(MFG_ERR_INVALID_ARGUMENT, "smem_bvh_levels is compiled for the 256x8 and 1024x2 launch shapes");
            variant += 10;
        }
    } else {
        variant = b == 3 ? 203 : (b >= 4 ? 204 : 0);
    }
    // extended variants: FP64 100, FP32R 102; with sensitivities FP64 112, FP32R 113 (any budget)
    if (h.has_ext) {
        if (C.n_top > 0) return fail(MFG_ERR_INVALID_ARGUMENT, "smem_bvh_levels is compiled for plain models");
        variant = sens ? (o.precision == MFG_PREC_FP64 ? 112 : 113) : (o.precision == MFG_PREC_FP64 ? 100 : 102);
    }
    const void* fn = kernel_of(variant);
    CK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(dyn)));
    int per_sm = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, block, dyn));
    if (per_sm < 1) return fail(MFG_ERR_LIMIT, "kernel does not fit on an SM with this block size");
    if (o.blocks_per_sm > 0) per_sm = std::min(per_sm, std::max(int(o.blocks_per_sm), 1));
    long long grid = (long long)per_sm * s->sm_count;
    if (!o.use_graph) grid = std::max(1LL, std::min(grid, (long long)((total + block - 1) / block)));
    auto enqueue = [&]() -> cudaError_t {
        cudaError_t e = cudaMemcpyAsync(s->d_run, s->h_run, s->run_bytes, cudaMemcpyHostToDevice, s->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(s->d_counter, 0, 8, s->stream);
        if (e != cudaSuccess) return e;
        void* args[] = {(void*)&s->dm, (void*)&s->dt, (void*)&C};
        e = cudaLaunchKernel(fn, dim3(unsigned(grid)), dim3(block), args, dyn, s->stream);
        if (e != cudaSuccess) return e;
        return cudaGetLastError();
    };
    s->t_start = std::chrono::steady_clock::now();
    if (o.use_graph && !sens) {
        // one captured graph per launch shape: [run descriptor copy, counter reset, tracer]
        const long long key[6] = {variant, block, grid, C.n_top, (long long)dyn, C.chunk};
        if (!s->graph_exec || !std::equal(key, key + 6, s->graph_key)) {
            if (s->graph_exec) { cudaGraphExecDestroy(s->graph_exec); s->graph_exec = nullptr; }
            cudaGraph_t g = nullptr;
            CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
            cudaError_t e = enqueue();
            cudaError_t e2 = cudaStreamEndCapture(s->stream, &g);
            if (e != cudaSuccess) { if (g) cudaGraphDestroy(g); return cuda_fail(e, "graph capture"); }
            if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture");
            e = cudaGraphInstantiate(&s->graph_exec, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) { s->graph_exec = nullptr; return cuda_fail(e, "cudaGraphInstantiate"); }
            std::copy(key, key + 6, s->graph_key);
        }
        CK(cudaEventRecord(s->ev0, s->stream));
        CK(cudaGraphLaunch(s->graph_exec, s->stream));
    } else {
        CK(cudaEventRecord(s->ev0, s->stream));
        cudaError_t e = enqueue();
        if (e != cudaSuccess) return cuda_fail(e, "tracer launch");
    }
    CK(cudaEventRecord(s->ev1, s->stream));
    s->launches = 1;
    s->running = true;
    s->pending = mfg_run_stats{};
    s->pending.desorbed = total;
    for (int i = 0; i < ni; ++i) s->particles_started[i] += counts[i];
    return MFG_OK;
}

int mfg_run_async(mfg_sim* s, uint64_t n, const mfg_run_options* opt) {
    if (!s) return fail(MFG_ERR_INVALID_ARGUMENT, "null sim");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->running) return fail(MFG_ERR_BUSY, "run in flight");
    std::vector<uint64_t> counts(s->model->h.instances.size(), n);
    return launch_run(s, counts.data(), opt);
}

int mfg_run_batch_async(mfg_sim* s, const uint64_t* counts, const mfg_run_options* opt) {
    if (!s || !counts) return fail(MFG_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->running) return fail(MFG_ERR_BUSY, "run in flight");
    return launch_run(s, counts, opt);
}

int mfg_run_batch(mfg_sim* s, const uint64_t* counts, const mfg_run_options* opt, mfg_run_stats* stats) {
    int rc = mfg_run_batch_async(s, counts, opt);
    if (rc != MFG_OK) return rc;
    return mfg_wait(s, -1, stats);
}

int mfg_poll(mfg_sim* s) {
    if (!s) return fail(MFG_ERR_INVALID_ARGUMENT, "null sim");
    if (!s->running) return MFG_OK;
    cudaError_t e = cudaEventQuery(s->ev1);
    if (e == cudaErrorNotReady) return MFG_ERR_BUSY;
    if (e != cudaSuccess) return cuda_fail(e, "kernel");
    return MFG_OK;
}

int mfg_wait(mfg_sim* s, int64_t timeout_ms, mfg_run_stats* stats) {
    if (!s) return fail(MFG_ERR_INVALID_ARGUMENT, "null sim");
    std::lock_guard<std::mutex> lk(s->mu);
    if (!s->running) {
        if (stats) *stats = s->pending;
        return s->pending.status;
    }
    CK(cudaSetDevice(s->device));
    auto t0 = std::chrono::steady_clock::now();
    while (true) {
        cudaError_t e = cudaEventQuery(s->ev1);
        if (e == cudaSuccess) break;
        if (e != cudaErrorNotReady) { s->running = false; return cuda_fail(e, "tracer kernel"); }
        if (timeout_ms >= 0 &&
            std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0).count() > timeout_ms)
            return fail(MFG_ERR_TIMEOUT, "run still in flight after the wait limit");
        std::this_thread::sleep_for(std::chrono::microseconds(200));
    }
    s->running = false;
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
    std::vector<unsigned long long> g;
    int rc = read_global(s, g);
    if (rc) return rc;
    mfg_run_stats& st = s->pending;
    st.hits = g[TG_HITS] - s->g_before[TG_HITS];
    st.leaks = g[TG_LEAK] - s->g_before[TG_LEAK];
    st.rechecks = g[TG_RECHECK] - s->g_before[TG_RECHECK];
    st.dropped = g[TG_DROPPED] - s->g_before[TG_DROPPED];
    st.kernel_ms = ms;
    st.total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - s->t_start).count();
    st.kernel_launches = s->launches;
    unsigned long long status = g[TG_STATUS];
    st.status = MFG_OK;
    if (status & KS_STACK) st.status = MFG_ERR_LIMIT;
    if (status & KS_TIMEOUT) st.status = MFG_ERR_TIMEOUT;
    if (status & KS_ABORTED) st.status = MFG_ERR_ABORTED;
    if (status) {
        unsigned long long zero = 0;
        CK(cudaMemcpyAsync(s->dt.global + TG_STATUS, &zero, 8, cudaMemcpyHostToDevice, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        g_err = st.status == MFG_ERR_TIMEOUT ? "kernel time limit reached; particles in flight were dropped"
              : st.status == MFG_ERR_ABORTED ? "run aborted"
              : "BVH traversal stack overflow";
    }
    if (stats) *stats = st;
    return st.status;
}

int mfg_autotune(mfg_sim* s, uint64_t n_trial, int32_t precision, uint64_t seed, mfg_run_options* best) {
    if (!s || (precision != MFG_PREC_FP64 && precision != MFG_PREC_FP32R)) return fail(MFG_ERR_INVALID_ARGUMENT, "bad argument");
    const mfg::HostModel& h = s->model->h;
    // candidate launch shapes (threads per block, resident blocks per SM): FP64 at register budgets
    // of 2, 3 and 4 blocks of 256; FP32R at 2 to 8 blocks of 256, and for plain models the 32-register
    // budget as 4 blocks of 512 or 2 of 1024 threads (shared-memory stagings then serve more warps)
    std::vector<std::pair<int, int>> shapes;
    if (precision == MFG_PREC_FP64) {
        shapes = {{256, 2}, {256, 3}, {256, 4}};
    } else {
        shapes = {{256, 2}, {256, 3}, {256, 4}, {256, 6}, {256, 8}};
        if (!h.has_ext) { shapes.push_back({512, 4}); shapes.push_back({1024, 2}); }
    }
    auto trial = [&](int block, int bps, int levels, double& rate, int chunk = 64) -> int {
        mfg_run_options o{};
        o.precision = precision;
        o.seed = seed;
        o.block_size = block;
        o.blocks_per_sm = bps;
        o.smem_bvh_levels = levels;
        o.particles_per_request = chunk;
        o.time_limit_s = 60;
        mfg_run_stats st{};
        for (int rep = 0; rep < 2; ++rep) {   // the second run is timed
            int rc = mfg_run(s, n_trial, &o, &st);
            if (rc != MFG_OK) return rc;
            rate = double(st.hits) / (st.kernel_ms * 1e-3 + 1e-12);
        }
        return MFG_OK;
    };
    // stage 1: every shape without staged BVH levels
    std::vector<std::pair<double, int>> ranked;
    for (size_t k = 0; k < shapes.size(); ++k) {
        double rate = 0;
        int rc = trial(shapes[k].first, shapes[k].second, -1, rate);
        if (rc != MFG_OK) return rc;
        ranked.push_back({rate, int(k)});
    }
    std::sort(ranked.begin(), ranked.end(), [](const std::pair<double, int>& a, const std::pair<double, int>& b) { return a.first > b.first; });
    int best_shape = ranked[0].second, best_levels = -1;
    double best_rate = ranked[0].first;
    // stage 2 (FP32R, plain models): the 8 x 256 and 2 x 1024 shapes with the top 2^5, 2^7 or 2^9
    // nodes in shared memory
    if (precision == MFG_PREC_FP32R && !h.has_ext)
        for (size_t r = 0; r < ranked.size(); ++r)
            for (int levels : {5, 7, 9}) {
                const auto& sh = shapes[ranked[r].second];
                if (!(sh.first == 256 && sh.second == 8) && !(sh.first == 1024 && sh.second == 2)) continue;
                double rate = 0;
                int rc = trial(sh.first, sh.second, levels, rate);
                if (rc != MFG_OK) return rc;
                if (rate > best_rate) { best_rate = rate; best_shape = ranked[r].second; best_levels = levels; }
            }
    // stage 3: particles per work-queue request at the chosen shape (64 is the default)
    int best_chunk = 64;
    for (int chunk : {32, 256}) {
        double rate = 0;
        int rc = trial(shapes[best_shape].first, shapes[best_shape].second, best_levels, rate, chunk);
        if (rc != MFG_OK) return rc;
        if (rate > best_rate) { best_rate = rate; best_chunk = chunk; }
    }
    s->tuned_block[precision] = shapes[best_shape].first;
    s->tuned_bps[precision] = shapes[best_shape].second;
    s->tuned_levels[precision] = best_levels;
    s->tuned_chunk[precision] = best_chunk;
    if (best) {
        *best = mfg_run_options{};
        best->precision = precision;
        best->seed = seed;
        best->block_size = shapes[best_shape].first;
        best->blocks_per_sm = shapes[best_shape].second;
        best->smem_bvh_levels = best_levels;
        best->particles_per_request = best_chunk;
    }
    return mfg_reset(s);
}

int mfg_run(mfg_sim* s, uint64_t n, const mfg_run_options* opt, mfg_run_stats* stats) {
    int rc = mfg_run_async(s, n, opt);
    if (rc != MFG_OK) return rc;
    return mfg_wait(s, -1, stats);
}

int mfg_abort(mfg_sim* s) {
    if (!s) return fail(MFG_ERR_INVALID_ARGUMENT, "null sim");
    *(volatile int*)s->h_abort = 1;
    return MFG_OK;
}

// Copy tallies of facets [fb, fb+nf), texture cells [tb, tb+nt), profiles [pb, pb+np),
// angle-map cells [ab, ab+na) into a view laid out for exactly that range.
static int fetch_range(mfg_sim* s, mfg_state_view* v, int fb, int nf, int64_t tb, int64_t nt, int64_t pb, int64_t np,
                       int64_t ab, int64_t na, bool whole) {
    CK(cudaSetDevice(s->device));
    const mfg::HostModel& h = s->model->h;
    const double f = h.use_maxwell ? 1.0 : 1.1781;
    const size_t B = 1 + size_t(h.nm);
    const size_t NF = size_t(h.nf), NT = size_t(h.layout.texture_cells), NP = size_t(h.layout.profile_facets) * MFG_PROFILE_SIZE;
    const size_t words = TG_N + s->n_facet + s->n_texture + s->n_profile + s->n_anglemap;
    if (s->stage_words < words) {
        if (s->h_stage) cudaFreeHost(s->h_stage);
        s->h_stage = nullptr;
        s->stage_words = 0;
        CK(cudaMallocHost(&s->h_stage, words * 8));
        s->stage_words = words;
    }
    unsigned long long* const g = s->h_stage;
    unsigned long long* const fa = g + TG_N;
    unsigned long long* const tx = fa + s->n_facet;
    unsigned long long* const pr = tx + s->n_texture;
    unsigned long long* const am = pr + s->n_profile;
    CK(cudaMemcpyAsync(g, s->dt.global, TG_N * 8, cudaMemcpyDeviceToHost, s->stream));
    // the stage mirrors the device arrays; one instance of a batch copies only its own rows of each
    // moment block (a copy per block and array, into the same stage offsets)
    auto rows = [&](unsigned long long* dst, const unsigned long long* src, size_t total, size_t block, size_t first,
                    size_t count, size_t width) -> int {
        if (!total || !count) return MFG_OK;
        if (whole) {
            CK(cudaMemcpyAsync(dst, src, total * 8, cudaMemcpyDeviceToHost, s->stream));
            return MFG_OK;
        }
        for (size_t m = 0; m < B; ++m) {
            const size_t o = (m * block + first) * width;
            CK(cudaMemcpyAsync(dst + o, src + o, count * width * 8, cudaMemcpyDeviceToHost, s->stream));
        }
        return MFG_OK;
    };
    int rc;
    if ((rc = rows(fa, s->dt.facet, s->n_facet, NF, size_t(fb), size_t(nf), TF_N)) != MFG_OK) return rc;
    if (v->texture && (rc = rows(tx, s->dt.texture, s->n_texture, NT, size_t(tb), size_t(nt), TT_N)) != MFG_OK) return rc;
    if (v->profile && (rc = rows(pr, s->dt.profile, s->n_profile, NP, size_t(pb) * MFG_PROFILE_SIZE,
                                 size_t(np) * MFG_PROFILE_SIZE, TT_N)) != MFG_OK)
        return rc;
    if (s->n_anglemap && v->anglemap && na > 0)
        CK(cudaMemcpyAsync(am + (whole ? 0 : ab), s->dt.anglemap + (whole ? 0 : ab), (whole ? s->n_anglemap : size_t(na)) * 8,
                           cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    uint64_t sh = 0, sd = 0, sa = 0;
    for (int i = 0; i < nf; ++i) {
        const unsigned long long* t = &fa[(fb + i) * TF_N];
        sh += t[TF_HITS]; sd += t[TF_DES]; sa += t[TF_ABS];
    }
    parallel_range(B * size_t(nf), [&](size_t k0, size_t k1) {
        for (size_t k = k0; k < k1; ++k) {
            const size_t m = k / size_t(nf), i = k % size_t(nf);
            const unsigned long long* t = &fa[(m * NF + fb + i) * TF_N];
            if (v->facet_counts) {
                v->facet_counts[k * MFG_FC_N + MFG_FC_NBMCHIT] = t[TF_HITS];
                v->facet_counts[k * MFG_FC_N + MFG_FC_NBDESORBED] = t[TF_DES];
                v->facet_counts[k * MFG_FC_N + MFG_FC_NBABSORBED] = t[TF_ABS];
            }
            if (v->facet_sums) {
                double* o = v->facet_sums + k * MFG_FS_N;
                o[MFG_FS_NBHITEQUIV] = double(t[TF_HITS]);
                o[MFG_FS_NBABSEQUIV] = double(t[TF_ABS]);
                o[MFG_FS_SUM_1_PER_ORT_VEL] = u128(t + TF_S1OV) / MFG_SCALE_INV;
                o[MFG_FS_SUM_V_ORT] = u128(t + TF_SVORT) / MFG_SCALE_V * f;
                o[MFG_FS_SUM_1_PER_VELOCITY] = u128(t + TF_S1V) / MFG_SCALE_INV;
            }
        }
    });
    if (v->global) {
        std::fill(v->global, v->global + MFG_G_N, 0.0);
        if (whole) {
            v->global[MFG_G_NBMCHIT] = double(g[TG_HITS]);
            v->global[MFG_G_NBHITEQUIV] = double(g[TG_HITS]);
            v->global[MFG_G_NBDESORBED] = double(g[TG_DES]);
            v->global[MFG_G_NBABSEQUIV] = double(g[TG_ABS]);
            v->global[MFG_G_NBLEAK] = double(g[TG_LEAK]);
            v->global[MFG_G_DIST_TOTAL] = u128(&g[TG_DIST_LO]) / MFG_SCALE_DIST;
            v->global[MFG_G_DIST_FULLHITS] = u128(&g[TG_DISTF_LO]) / MFG_SCALE_DIST;
        } else {   // one instance of a batch: counters summed over its facets (leaks and distances are batch totals)
            v->global[MFG_G_NBMCHIT] = double(sh);
            v->global[MFG_G_NBHITEQUIV] = double(sh);
            v->global[MFG_G_NBDESORBED] = double(sd);
            v->global[MFG_G_NBABSEQUIV] = double(sa);
        }
    }
    if (v->texture)
        parallel_range(B * size_t(nt), [&](size_t k0, size_t k1) {
            for (size_t k = k0; k < k1; ++k) {
                const size_t m = k / size_t(nt), c = k % size_t(nt);
                const unsigned long long* t = &tx[(m * NT + tb + c) * TT_N];
                double* o = v->texture + k * 3;
                o[0] = double(t[TT_COUNT]);
                o[1] = u128(t + TT_SVORT) / MFG_SCALE_V * f * h.tex_inc[tb + c];
                o[2] = u128(t + TT_S1OV) / MFG_SCALE_INV / f;
            }
        });
    if (v->profile)
        for (size_t m = 0; m < B; ++m)
            for (int64_t c = 0; c < np * MFG_PROFILE_SIZE; ++c) {
                const unsigned long long* t = &pr[(m * NP + pb * MFG_PROFILE_SIZE + c) * TT_N];
                double* o = v->profile + (m * size_t(np) * MFG_PROFILE_SIZE + c) * 3;
                o[0] = double(t[TT_COUNT]);
                o[1] = u128(t + TT_SVORT) / MFG_SCALE_V * f;
                o[2] = u128(t + TT_S1OV) / MFG_SCALE_INV;
            }
    if (v->anglemap)
        for (int64_t c = 0; c < na; ++c) v->anglemap[c] = am[ab + c];
    if (v->histogram && s->n_hist && whole)
        CK(cudaMemcpy(v->histogram, s->dt.histogram, s->n_hist * 8, cudaMemcpyDeviceToHost));
    if (v->force && s->n_force) {   // facets [fb, fb+nf) of every moment block
        std::vector<double> fr(s->n_force);
        CK(cudaMemcpy(fr.data(), s->dt.force, s->n_force * 8, cudaMemcpyDeviceToHost));
        for (size_t m = 0; m < B; ++m)
            std::memcpy(v->force + (m * size_t(nf)) * 9, fr.data() + (m * NF + fb) * 9, size_t(nf) * 9 * 8);
    }
    if (s->n_lf && whole) {
        // low-flux mode: equivalent (weighted) hits, absorptions and texture / profile counts
        std::vector<double> lf(s->n_lf);
        CK(cudaMemcpy(lf.data(), s->dt.lf_glob, s->n_lf * 8, cudaMemcpyDeviceToHost));
        const double* lfc = lf.data() + 2;
        const double* lft = lfc + B * NF * 2;
        const double* lfp = lft + B * NT;
        if (v->global) {
            v->global[MFG_G_NBHITEQUIV] = lf[0];
            v->global[MFG_G_NBABSEQUIV] = lf[1];
        }
        if (v->facet_sums)
            for (size_t m = 0; m < B; ++m)
                for (int i = 0; i < nf; ++i) {
                    double* o = v->facet_sums + (m * size_t(nf) + i) * MFG_FS_N;
                    o[MFG_FS_NBHITEQUIV] = lfc[(m * NF + fb + i) * 2];
                    o[MFG_FS_NBABSEQUIV] = lfc[(m * NF + fb + i) * 2 + 1];
                }
        if (v->texture)
            for (size_t m = 0; m < B; ++m)
                for (int64_t c = 0; c < nt; ++c) v->texture[(m * size_t(nt) + c) * 3] = lft[m * NT + tb + c];
        if (v->profile)
            for (size_t m = 0; m < B; ++m)
                for (int64_t c = 0; c < np * MFG_PROFILE_SIZE; ++c)
                    v->profile[(m * size_t(np) * MFG_PROFILE_SIZE + c) * 3] = lfp[m * NP + pb * MFG_PROFILE_SIZE + c];
    }
    if (v->direction) {
        // direction cells of facets [fb, fb+nf): contiguous range starting at the first one's offset
        int64_t d0 = -1, nd = 0;
        for (int i = 0; i < nf; ++i)
            if (h.dir_off[fb + i] >= 0) {
                if (d0 < 0) d0 = h.dir_off[fb + i];
                nd += int64_t(h.tex_w[fb + i]) * h.tex_h[fb + i];
            }
        const size_t ND = size_t(h.layout.direction_cells);
        if (nd > 0) {
            std::vector<double> dv(3 * s->n_dir);
            std::vector<unsigned long long> dc(s->n_dir);
            CK(cudaMemcpy(dv.data(), s->dt.direction, 24 * s->n_dir, cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(dc.data(), s->dt.dir_count, 8 * s->n_dir, cudaMemcpyDeviceToHost));
            for (size_t m = 0; m < B; ++m)
                for (int64_t c = 0; c < nd; ++c) {
                    size_t k = m * ND + size_t(d0 + c);
                    double* o = v->direction + (m * size_t(nd) + c) * 4;
                    o[0] = dv[3 * k]; o[1] = dv[3 * k + 1]; o[2] = dv[3 * k + 2];
                    o[3] = double(dc[k]);
                }
        }
    }
    return MFG_OK;
}

int mfg_fetch(mfg_sim* s, mfg_state_view* v) {
    if (!s || !v) return fail(MFG_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->running) return fail(MFG_ERR_BUSY, "run in flight");
    const mfg::HostModel& h = s->model->h;
    return fetch_range(s, v, 0, h.nf, 0, h.layout.texture_cells, 0, h.layout.profile_facets, 0, h.layout.anglemap_cells, true);
}

int mfg_fetch_log(mfg_sim* s, double* records, int64_t capacity, int64_t* n_records) {
    if (!s || capacity < 0 || (capacity > 0 && !records)) return fail(MFG_ERR_INVALID_ARGUMENT, "bad argument");
    if (n_records) *n_records = 0;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->running) return fail(MFG_ERR_BUSY, "run in flight");
    if (!s->dt.plog_n) return MFG_OK;
    CK(cudaSetDevice(s->device));
    unsigned long long claimed = 0;
    CK(cudaMemcpy(&claimed, s->dt.plog_n, 8, cudaMemcpyDeviceToHost));
    const int64_t n = std::min<int64_t>({int64_t(claimed), int64_t(s->model->h.log_cap), capacity});
    if (n > 0) CK(cudaMemcpy(records, s->dt.plog, size_t(n) * MFG_LOG_N * 8, cudaMemcpyDeviceToHost));
    if (n_records) *n_records = n;
    return MFG_OK;
}

int mfg_fetch_instance(mfg_sim* s, int32_t i, mfg_state_view* v) {
    if (!s || !v) return fail(MFG_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->running) return fail(MFG_ERR_BUSY, "run in flight");
    const mfg::HostModel& h = s->model->h;
    if (i < 0 || i >= int(h.instances.size())) return fail(MFG_ERR_INVALID_ARGUMENT, "instance index out of range");
    const auto& in = h.instances[i];
    return fetch_range(s, v, in.facet_base, in.nf, in.tex_base, in.layout.texture_cells, in.prof_base,
                       in.layout.profile_facets, in.ang_base, in.layout.anglemap_cells, h.instances.size() == 1);
}

int mfg_model_merge(const mfg_model* const* models, int32_t n, mfg_model** out) {
    if (!models || n <= 0 || !out) return fail(MFG_ERR_INVALID_ARGUMENT, "bad argument");
    *out = nullptr;
    std::vector<const mfg::HostModel*> parts;
    for (int i = 0; i < n; ++i) {
        if (!models[i]) return fail(MFG_ERR_INVALID_ARGUMENT, "null model in batch");
        parts.push_back(&models[i]->h);
    }
    auto* m = new mfg_model();
    std::string err;
    int rc = mfg::merge_host_models(parts, m->h, err);
    if (rc != MFG_OK) { delete m; return fail(rc, err); }
    *out = m;
    return MFG_OK;
}

int32_t mfg_model_instances(const mfg_model* m) { return m ? int32_t(m->h.instances.size()) : 0; }

int mfg_instance_layout(const mfg_model* m, int32_t i, mfg_state_layout* out) {
    if (!m || !out || i < 0 || i >= int(m->h.instances.size())) return fail(MFG_ERR_INVALID_ARGUMENT, "bad argument");
    *out = m->h.instances[i].layout;
    return MFG_OK;
}

int mfg_update_sticking(mfg_sim* s, int32_t n, const int32_t* facets, const double* values) {
    if (!s || n < 0 || (n && (!facets || !values))) return fail(MFG_ERR_INVALID_ARGUMENT, "bad argument");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->running) return fail(MFG_ERR_BUSY, "run in flight");
    const mfg::HostModel& h = s->model->h;
    CK(cudaSetDevice(s->device));
    for (int i = 0; i < n; ++i) {
        int f = facets[i];
        if (f < 0 || f >= h.nf || !(values[i] >= 0.0 && values[i] <= 1.0)) return fail(MFG_ERR_INVALID_ARGUMENT, "bad facet or sticking value");
        s->sticking[f] = values[i];
        double d = values[i];
        float fl = float(values[i]);
        CK(cudaMemcpyAsync((char*)s->dm.phys_d + sizeof(FacetPhysD) * size_t(f) + offsetof(FacetPhysD, sticking), &d, sizeof d,
                           cudaMemcpyHostToDevice, s->stream));
        CK(cudaMemcpyAsync((char*)s->dm.phys_f + sizeof(FacetPhysF) * size_t(f) + offsetof(FacetPhysF, sticking), &fl, sizeof fl,
                           cudaMemcpyHostToDevice, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    return MFG_OK;
}

int mfg_sens_setup(mfg_sim* s, int32_t n_params, const int32_t* param_facets, int32_t n_gauges, const int32_t* gauge_facets,
                   int32_t n_pumps, const int32_t* pump_facets) {
    if (!s || n_params < 0 || n_gauges < 0 || n_gauges > MFG_SENS_NOUT - 1 || n_pumps < 0 || (n_params && !param_facets) ||
        (n_gauges && !gauge_facets) || (n_pumps && !pump_facets))
        return fail(MFG_ERR_INVALID_ARGUMENT, "bad argument (at most 8 gauges)");
    if (n_params >= (1 << 20) - 1) return fail(MFG_ERR_INVALID_ARGUMENT, "at most 2^20 - 2 parameters");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->running) return fail(MFG_ERR_BUSY, "run in flight");
    const mfg::HostModel& h = s->model->h;
    if (h.instances.size() != 1) return fail(MFG_ERR_INVALID_ARGUMENT, "sensitivities are for single models");
    // the score function needs a stick-or-reflect draw at every hit on a parameter facet: low-flux
    // mode splits particles by weight instead of drawing
    if (h.low_flux) return fail(MFG_ERR_UNSUPPORTED_FEATURE, "sensitivities need stick/reflect draws; low-flux mode has none");
    std::vector<int32_t> pof(h.nf, -1), gof(h.nf, -1), sof(h.nf, -1);
    std::vector<uint8_t> pump(h.nf, 0);
    for (int i = 0; i < n_params; ++i) {
        int f = param_facets[i];
        if (f < 0 || f >= h.nf || pof[f] >= 0) return fail(MFG_ERR_INVALID_ARGUMENT, "bad or repeated parameter facet");
        if (!(s->sticking[f] > 0.0 && s->sticking[f] < 1.0)) return fail(MFG_ERR_INVALID_ARGUMENT, "parameter sticking must be in (0,1)");
        if (h.info[f].flags & FF_STICK_PARAM)
            return fail(MFG_ERR_INVALID_ARGUMENT, "parameter facet has a time-dependent sticking");
        if (h.info[f].flags & (FF_LINK | FF_TELEPORT))
            return fail(MFG_ERR_INVALID_ARGUMENT, "parameter facet is a link or teleport (no stick/reflect draw)");
        pof[f] = i;
    }
    for (int i = 0; i < n_gauges; ++i) {
        int f = gauge_facets[i];
        if (f < 0 || f >= h.nf) return fail(MFG_ERR_INVALID_ARGUMENT, "bad gauge facet");
        gof[f] = i;
    }
    for (int i = 0; i < n_pumps; ++i) {
        int f = pump_facets[i];
        if (f < 0 || f >= h.nf) return fail(MFG_ERR_INVALID_ARGUMENT, "bad pump facet");
        pump[f] = 1;
    }
    s->js.clear();   // a Jacobian of the previous setup has other sizes
    s->jq.clear();
    s->jy.clear();
    s->sens_src.clear();
    for (size_t k = 0; k < h.src_facet.size(); ++k) { sof[h.src_facet[k]] = int32_t(k); s->sens_src.push_back(h.src_facet[k]); }
    s->sens_params.assign(param_facets, param_facets + n_params);
    const size_t P = size_t(std::max(n_params, 1)), S = std::max<size_t>(s->sens_src.size(), 1), nf = size_t(h.nf);
    std::vector<int32_t> code(h.nf, 0);   // packed: parameter + 1 (bits 0-19), gauge + 1 (20-23), pump (24)
    for (int f = 0; f < h.nf; ++f)
        code[f] = (pof[f] + 1) | ((gof[f] + 1) << 20) | (int32_t(pump[f]) << 24);
    const size_t off_pof = 0, off_gof = off_pof + 4 * nf, off_sof = off_gof + 4 * nf, off_code = off_sof + 4 * nf;
    const size_t off_pump = off_code + 4 * nf;
    const size_t off_A = (off_pump + nf + 255) / 256 * 256, off_B = off_A + 8 * P * MFG_SENS_NOUT;
    const size_t off_C = off_B + 8 * P * MFG_SENS_NOUT, off_Y = off_C + 8 * S * MFG_SENS_NOUT;
    const size_t off_cnt = off_Y + 8 * MFG_SENS_NOUT, off_ovf = off_cnt + 8 * S, total = off_ovf + 8;
    CK(cudaSetDevice(s->device));
    s->sens_ready = false;   // until the new block is filled
    if (s->sens_block) { cudaFree(s->sens_block); s->sens_block = nullptr; }
    CK(cudaMalloc(&s->sens_block, total));
    char* b = static_cast<char*>(s->sens_block);
    CK(cudaMemcpy(b + off_pof, pof.data(), 4 * nf, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(b + off_gof, gof.data(), 4 * nf, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(b + off_sof, sof.data(), 4 * nf, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(b + off_pump, pump.data(), nf, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(b + off_code, code.data(), 4 * nf, cudaMemcpyHostToDevice));
    s->sens.code = reinterpret_cast<const int32_t*>(b + off_code);
    s->sens.param_of_facet = reinterpret_cast<const int32_t*>(b + off_pof);
    s->sens.gauge_of_facet = reinterpret_cast<const int32_t*>(b + off_gof);
    s->sens.src_of_facet = reinterpret_cast<const int32_t*>(b + off_sof);
    s->sens.pump_of_facet = reinterpret_cast<const uint8_t*>(b + off_pump);
    s->sens.A = reinterpret_cast<double*>(b + off_A);
    s->sens.B = reinterpret_cast<double*>(b + off_B);
    s->sens.Cs = reinterpret_cast<double*>(b + off_C);
    s->sens.Y = reinterpret_cast<double*>(b + off_Y);
    s->sens.src_count = reinterpret_cast<unsigned long long*>(b + off_cnt);
    s->sens.overflow = reinterpret_cast<unsigned long long*>(b + off_ovf);
    s->sens_bytes = total - off_A;
    s->sens_ready = true;
    return MFG_OK;
}

int32_t mfg_sens_sources(const mfg_sim* s) { return s ? int32_t(s->sens_src.size()) : 0; }

int mfg_sens_forward(mfg_sim* s, uint64_t n, const mfg_run_options* opt, double* outputs, mfg_run_stats* stats) {
    if (!s || !outputs) return fail(MFG_ERR_INVALID_ARGUMENT, "null argument");
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (!s->sens_ready) return fail(MFG_ERR_INVALID_ARGUMENT, "call mfg_sens_setup first");
        if (s->running) return fail(MFG_ERR_BUSY, "run in flight");
        CK(cudaSetDevice(s->device));
        CK(cudaMemsetAsync(reinterpret_cast<char*>(s->sens.A), 0, s->sens_bytes, s->stream));
        uint64_t counts[1] = {n};
        int rc = launch_run(s, counts, opt, true);
        if (rc != MFG_OK) return rc;
    }
    int rc = mfg_wait(s, -1, stats);
    if (rc != MFG_OK) return rc;
    std::lock_guard<std::mutex> lk(s->mu);
    const size_t P = s->sens_params.size(), S = s->sens_src.size();
    std::vector<double> A(P * MFG_SENS_NOUT), B(P * MFG_SENS_NOUT), Cs(S * MFG_SENS_NOUT), Y(MFG_SENS_NOUT);
    std::vector<unsigned long long> cnt(S);
    unsigned long long ovf = 0;
    if (P) {
        CK(cudaMemcpy(A.data(), s->sens.A, 8 * P * MFG_SENS_NOUT, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(B.data(), s->sens.B, 8 * P * MFG_SENS_NOUT, cudaMemcpyDeviceToHost));
    }
    if (S) {
        CK(cudaMemcpy(Cs.data(), s->sens.Cs, 8 * S * MFG_SENS_NOUT, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(cnt.data(), s->sens.src_count, 8 * S, cudaMemcpyDeviceToHost));
    }
    CK(cudaMemcpy(Y.data(), s->sens.Y, 8 * MFG_SENS_NOUT, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&ovf, s->sens.overflow, 8, cudaMemcpyDeviceToHost));
    const double N = double(n);
    s->jy.assign(MFG_SENS_NOUT, 0.0);
    for (int j = 0; j < MFG_SENS_NOUT; ++j) { s->jy[j] = Y[j] / N; outputs[j] = s->jy[j]; }
    s->js.assign(P * MFG_SENS_NOUT, 0.0);
    for (size_t k = 0; k < P; ++k) {
        double st = s->sticking[s->sens_params[k]];
        for (int j = 0; j < MFG_SENS_NOUT; ++j)
            s->js[k * MFG_SENS_NOUT + j] = (-A[k * MFG_SENS_NOUT + j] / (1.0 - st) + B[k * MFG_SENS_NOUT + j] / st) / N;
    }
    s->jq.assign(S * MFG_SENS_NOUT, 0.0);
    for (size_t q = 0; q < S; ++q)
        for (int j = 0; j < MFG_SENS_NOUT; ++j)
            s->jq[q * MFG_SENS_NOUT + j] = cnt[q] ? Cs[q * MFG_SENS_NOUT + j] / double(cnt[q]) : 0.0;
    if (ovf) { g_err = "reflection list overflowed for " + std::to_string(ovf) + " particles"; return MFG_ERR_LIMIT; }
    return MFG_OK;
}

int mfg_sens_jacobian(mfg_sim* s, double* d_sticking, double* d_outgassing, int32_t* source_facets) {
    if (!s || s->jy.empty()) return fail(MFG_ERR_INVALID_ARGUMENT, "no forward pass yet");
    if (d_sticking) std::copy(s->js.begin(), s->js.end(), d_sticking);
    if (d_outgassing) std::copy(s->jq.begin(), s->jq.end(), d_outgassing);
    if (source_facets) std::copy(s->sens_src.begin(), s->sens_src.end(), source_facets);
    return MFG_OK;
}

int mfg_sens_backward(mfg_sim* s, const double* dl_dy, double* dl_dsticking, double* dl_doutgassing) {
    if (!s || !dl_dy) return fail(MFG_ERR_INVALID_ARGUMENT, "null argument");
    if (s->jy.empty()) return fail(MFG_ERR_INVALID_ARGUMENT, "no forward pass yet");
    const size_t P = s->sens_params.size(), S = s->sens_src.size();
    if (dl_dsticking)
        for (size_t k = 0; k < P; ++k) {
            double a = 0;
            for (int j = 0; j < MFG_SENS_NOUT; ++j) a += dl_dy[j] * s->js[k * MFG_SENS_NOUT + j];
            dl_dsticking[k] = a;
        }
    if (dl_doutgassing)
        for (size_t q = 0; q < S; ++q) {
            double a = 0;
            for (int j = 0; j < MFG_SENS_NOUT; ++j) a += dl_dy[j] * s->jq[q * MFG_SENS_NOUT + j];
            dl_doutgassing[q] = a;
        }
    return MFG_OK;
}

int mfg_replay(mfg_sim* s, int32_t precision, int64_t n, const double* origin, const double* direction,
               const int32_t* last_facet, int32_t* hit_facet, double* hit_t, uint64_t* n_rechecks) {
    if (!s || n < 0 || (n > 0 && (!origin || !direction || !last_facet || !hit_facet || !hit_t)))
        return fail(MFG_ERR_INVALID_ARGUMENT, "null argument");
    if (n == 0) { if (n_rechecks) *n_rechecks = 0; return MFG_OK; }
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->running) return fail(MFG_ERR_BUSY, "run in flight");
    CK(cudaSetDevice(s->device));
    double *d_o = nullptr, *d_d = nullptr, *d_t = nullptr;
    int *d_l = nullptr, *d_f = nullptr;
    unsigned long long* d_r = nullptr;
    auto cleanup = [&]() { cudaFree(d_o); cudaFree(d_d); cudaFree(d_t); cudaFree(d_l); cudaFree(d_f); cudaFree(d_r); };
    cudaError_t e = cudaSuccess;
    if ((e = cudaMalloc(&d_o, 24 * n)) || (e = cudaMalloc(&d_d, 24 * n)) || (e = cudaMalloc(&d_t, 8 * n)) ||
        (e = cudaMalloc(&d_l, 4 * n)) || (e = cudaMalloc(&d_f, 4 * n)) || (e = cudaMalloc(&d_r, 16))) {
        cleanup();
        return cuda_fail(e, "cudaMalloc (replay)");
    }
    cudaMemcpyAsync(d_o, origin, 24 * n, cudaMemcpyHostToDevice, s->stream);
    cudaMemcpyAsync(d_d, direction, 24 * n, cudaMemcpyHostToDevice, s->stream);
    cudaMemcpyAsync(d_l, last_facet, 4 * n, cudaMemcpyHostToDevice, s->stream);
    cudaMemsetAsync(d_r, 0, 16, s->stream);
    const int block = mfgk::kReplayBlock;
    long long grid = (n + block - 1) / block;
    mfgk::replay_kernel<<<unsigned(grid), block, 0, s->stream>>>(s->dm, precision, n, d_o, d_d, d_l, d_f, d_t, d_r,
                                                                d_r + 1);
    e = cudaGetLastError();
    if (e == cudaSuccess) {
        unsigned long long r[2] = {0, 0};
        cudaMemcpyAsync(hit_facet, d_f, 4 * n, cudaMemcpyDeviceToHost, s->stream);
        cudaMemcpyAsync(hit_t, d_t, 8 * n, cudaMemcpyDeviceToHost, s->stream);
        cudaMemcpyAsync(r, d_r, 16, cudaMemcpyDeviceToHost, s->stream);
        e = cudaStreamSynchronize(s->stream);
        if (n_rechecks) *n_rechecks = r[0];
        if (e == cudaSuccess && (r[1] & KS_STACK)) { cleanup(); return fail(MFG_ERR_LIMIT, "BVH traversal stack overflow"); }
    }
    cleanup();
    if (e != cudaSuccess) return cuda_fail(e, "replay kernel");
    return MFG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Replay without device allocations.
//
// For callers that cannot allocate device memory during a query: a process whose device
// memory belongs to another framework's pool allocator (a stray cudaMalloc would fall outside
// that pool's budget), or a control loop that must not block in cudaMalloc/cudaFree, which can
// synchronise the whole device.  The caller passes device-resident inputs and outputs; the
// FP64 recheck queue lives in the fixed array below.
//
// The array is shared by every call in the process and keeps the last call's contents: each
// call clears the queue counter and status word before its first kernel, and calls that
// overlap on the GPU (different streams or threads at the same time) race on it.
// ---------------------------------------------------------------------------
#define MFG_NOALLOC_MAX_RAYS (1 << 20)
// [0] rays queued for the FP64 pass, [1] status bits, [2 ..] queued ray indices  (8 MiB + 16 B)
static __device__ __align__(256) unsigned long long g_noalloc_scratch[2 + MFG_NOALLOC_MAX_RAYS];

namespace {
std::mutex g_noalloc_mu;
unsigned long long* g_noalloc_addr[256];   // device address of g_noalloc_scratch, per device

// FP32R: lockstep traversal of the warp's rays (lanes past the end take part in the votes)
__global__ void __launch_bounds__(mfgk::kReplayBlock, 4) noalloc_pass1(const __grid_constant__ DevModel M, int precision,
                              long long n, const double* origin, const double* dir, const int* last, int* hit_f,
                              double* hit_t, unsigned long long* scratch) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = i < n;
    int root = M.roots[0];
    const mfgk::OpacCtx oc = mfgk::replay_opacity();
    const mfgk::OpacCtx* ocp = M.has_transparent ? &oc : nullptr;
    if (precision == MFG_PREC_FP64) {
        if (!active) return;
        mfgk::HitD h = mfgk::trace_d<double>(M, root, origin[3 * i], origin[3 * i + 1], origin[3 * i + 2], dir[3 * i],
                                             dir[3 * i + 1], dir[3 * i + 2], last[i], scratch + 1, nullptr, ocp);
        hit_f[i] = h.f;
        hit_t[i] = h.f >= 0 ? h.t : -1.0;
        return;
    }
    double ox = 0, oy = 0, oz = 0, dx = 1, dy = 0, dz = 0;
    int li = -1;
    if (active) {
        ox = origin[3 * i]; oy = origin[3 * i + 1]; oz = origin[3 * i + 2];
        dx = dir[3 * i]; dy = dir[3 * i + 1]; dz = dir[3 * i + 2];
        li = last[i];
    }
    bool amb = false;
    mfgk::HitF h = mfgk::trace_f_lockstep(M, active, M.roots_c[0], mfgk::make_ray_f(ox, oy, oz, (float)dx, (float)dy, (float)dz),
                                          li, amb, scratch + 1, ocp);
    if (!active) return;
    if (amb || h.f < 0) {   // queue the ray for the FP64 pass
        unsigned long long k = atomicAdd(scratch, 1ull);
        scratch[2 + k] = (unsigned long long)i;
        return;
    }
    const FacetIsectD& Rh = M.isect_d[h.f];
    double den = Rh.v[0] * dx + Rh.v[1] * dy + Rh.v[2] * dz;
    double num = Rh.v[3] - (Rh.v[0] * ox + Rh.v[1] * oy + Rh.v[2] * oz);
    double r = num - (double)h.t * den;
    hit_f[i] = h.f;
    hit_t[i] = (double)h.t + (double)((float)r / (float)den);
}

__global__ void noalloc_pass2(const __grid_constant__ DevModel M, const double* origin, const double* dir,
                              const int* last, int* hit_f, double* hit_t, unsigned long long* scratch) {
    unsigned long long k = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= scratch[0]) return;
    long long i = (long long)scratch[2 + k];
    const mfgk::OpacCtx oc = mfgk::replay_opacity();
    mfgk::HitD h = mfgk::trace_d<double>(M, M.roots[0], origin[3 * i], origin[3 * i + 1], origin[3 * i + 2], dir[3 * i],
                                         dir[3 * i + 1], dir[3 * i + 2], last[i], scratch + 1, nullptr,
                                         M.has_transparent ? &oc : nullptr);
    hit_f[i] = h.f;
    hit_t[i] = h.f >= 0 ? h.t : -1.0;
}
}  // namespace

extern "C" int mfg_replay_noalloc(mfg_sim* s, int32_t precision, int64_t n, const double* d_origin,
                                  const double* d_direction, const int32_t* d_last, int32_t* d_hit_facet,
                                  double* d_hit_t, uint64_t* n_rechecks) {
    if (!s || n < 0) return fail(MFG_ERR_INVALID_ARGUMENT, "null simulation or negative ray count");
    if (precision != MFG_PREC_FP64 && precision != MFG_PREC_FP32R) return fail(MFG_ERR_INVALID_ARGUMENT, "unknown precision");
    if (n > MFG_NOALLOC_MAX_RAYS)
        return fail(MFG_ERR_LIMIT, "mfg_replay_noalloc takes at most " + std::to_string(MFG_NOALLOC_MAX_RAYS) +
                                       " rays per call (" + std::to_string(n) + " given); split the batch");
    if (n > 0 && (!d_origin || !d_direction || !d_last || !d_hit_facet || !d_hit_t))
        return fail(MFG_ERR_INVALID_ARGUMENT, "null buffer");
    if (n_rechecks) *n_rechecks = 0;
    if (n == 0) return MFG_OK;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->running) return fail(MFG_ERR_BUSY, "run in flight");
    if (s->device < 0 || s->device >= 256) return fail(MFG_ERR_NO_DEVICE, "device index out of range");
    CK(cudaSetDevice(s->device));
    unsigned long long* scratch;
    {
        // set-up, once per device, with that device current: the host-side name of the array is
        // not a device address, so ask the runtime for the device address
        std::lock_guard<std::mutex> g(g_noalloc_mu);
        if (!g_noalloc_addr[s->device]) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
            g_noalloc_addr[s->device] = static_cast<unsigned long long*>(p);
        }
        scratch = g_noalloc_addr[s->device];
    }
    CK(cudaMemsetAsync(scratch, 0, 2 * sizeof(unsigned long long), s->stream));   // queue counter and status
    const int block = mfgk::kReplayBlock;
    const unsigned grid = unsigned((n + block - 1) / block);
    noalloc_pass1<<<grid, block, 0, s->stream>>>(s->dm, precision, n, d_origin, d_direction, d_last, d_hit_facet,
                                                  d_hit_t, scratch);
    CK(cudaGetLastError());
    if (precision == MFG_PREC_FP32R) {
        noalloc_pass2<<<grid, block, 0, s->stream>>>(s->dm, d_origin, d_direction, d_last, d_hit_facet, d_hit_t, scratch);
        CK(cudaGetLastError());
    }
    unsigned long long head[2] = {0, 0};
    CK(cudaMemcpyAsync(head, scratch, sizeof head, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    if (head[1] & KS_STACK) return fail(MFG_ERR_LIMIT, "BVH traversal stack overflow");
    if (n_rechecks) *n_rechecks = head[0];
    return MFG_OK;
}
