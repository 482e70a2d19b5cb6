// philox.cuh — Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw, SC'11)
// and the uniform constructions used by the tracer.
#pragma once
#include <stdint.h>

namespace mfgk {

__device__ __forceinline__ void philox4x32_10(uint32_t& c0, uint32_t& c1, uint32_t& c2, uint32_t& c3,
                                              uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}
// uniform double in [0,1): 52 random mantissa bits of (a:b) in [1,2), minus 1 (exact)
__device__ __forceinline__ double u01d(uint32_t a, uint32_t b) {
    uint64_t m = ((((uint64_t)a) << 32) | b) >> 12;
    return __longlong_as_double((long long)(0x3FF0000000000000ull | m)) - 1.0;
}
// uniform float in (0,1): (k + 1/2) * 2^-23; never 0, so cos(theta) = sqrt(u) never
// gives a direction lying in the facet plane
__device__ __forceinline__ float u01f(uint32_t a) {
    return (__uint_as_float(0x3F800000u | (a >> 9)) - 1.0f) + 5.9604645e-8f;
}

}  // namespace mfgk
