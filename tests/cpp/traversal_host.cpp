// Host build of the GPU traversal (molflow_sources_gb300/csrc/traversal.cuh) for CPU tests:
// runs the FP32 traversal with its error bounds and the FP64 traversal on given rays and
// reports hit facets and the reasons that sent rays to the FP64 recheck.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include <vector_types.h>

#define __device__
#define __forceinline__ inline
#define __noinline__
static int64_t g_reasons[8];
#define MFG_AMB_HOOK(r) (++g_reasons[(r)])
static inline long long __double_as_longlong(double x) { long long i; std::memcpy(&i, &x, sizeof i); return i; }
static inline double __longlong_as_double(long long i) { double x; std::memcpy(&x, &i, sizeof x); return x; }
static inline float __uint_as_float(unsigned u) { float x; std::memcpy(&x, &u, sizeof x); return x; }
static inline unsigned __umulhi(unsigned a, unsigned b) { return (unsigned)(((unsigned long long)a * b) >> 32); }
static inline float4 __ldg(const float4* p) { return *p; }
static inline int __float_as_int(float x) { int i; std::memcpy(&i, &x, sizeof i); return i; }
static inline unsigned long long atomicOr(unsigned long long* p, unsigned long long v) {
    unsigned long long o = *p; *p |= v; return o;
}
#include "../../molflow_sources_gb300/csrc/traversal.cuh"
#include "../../molflow_sources_gb300/csrc/model_build.h"

extern "C" int trav_run(const mfg_model_desc* d, int64_t n, const double* o, const double* dir, const int32_t* last,
                        int32_t* hit32, int32_t* hit64, int64_t* reasons, int64_t* n_amb) {
    mfg::HostModel h;
    std::string err;
    if (mfg::build_host_model(d, h, err) != MFG_OK) return 1;
    DevModel M;
    std::memset(&M, 0, sizeof M);
    M.nf = h.nf;
    M.nodes_d = h.nodes_d.data();
    M.nodes_c = h.nodes_c.data();
    M.prims_c = h.prims_c.data();
    M.roots_c = h.roots_c.data();
    M.roots = h.roots.data();
    M.prims = h.prims.data();
    M.isect_d = h.isect_d.data();
    M.isect_f = h.isect_f.data();
    M.poly_d = h.poly_d.data();
    M.poly_f = h.poly_f.data();
    M.tri_f = h.tri_f.data();
    M.v2_d = h.v2_d.data();
    M.v2_f = h.v2_f.data();
    M.info = h.info.data();
    M.scene_scale = h.scene_scale;
    std::memset(g_reasons, 0, sizeof g_reasons);
    unsigned long long status = 0;
    int64_t amb = 0;
    for (int64_t i = 0; i < n; ++i) {
        const double* p = o + 3 * i;
        const double* q = dir + 3 * i;
        bool a = false;
        mfgk::HitF hf = mfgk::trace_f(M, h.roots_c[0], mfgk::make_ray_f(p[0], p[1], p[2], float(q[0]), float(q[1]), float(q[2])),
                                      last[i], a, &status);
        mfgk::HitD hd = mfgk::trace_d(M, h.roots[0], p[0], p[1], p[2], double(float(q[0])), double(float(q[1])),
                                      double(float(q[2])), last[i], &status);
        if (hf.f < 0 && !a) { ++g_reasons[6]; a = true; }
        amb += a;
        hit32[i] = a ? hd.f : hf.f;
        hit64[i] = hd.f;
    }
    for (int k = 0; k < 8; ++k) reasons[k] = g_reasons[k];
    *n_amb = amb;
    return status ? 2 : 0;
}
