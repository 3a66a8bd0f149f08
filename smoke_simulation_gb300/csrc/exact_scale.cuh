// Exact float arithmetic of the reference's projection step without the FP64 pipe (host and
// device).  The reference computes p_t = (-div / acc) * OVER_RELAXATION with a float quotient and
// a double constant (project/smokeSimulation.cu:38, :384): float(double(q) * omega), one
// rounding to 53 bits and one to 24.  GB300's FP64 rate is a small fraction of its FP32 and
// integer rates, and the one-pass projection kernel is bound by it (its FP64 pipe runs at ~48 %
// of peak), so:
//   omega_scale  forms the 24 x 53-bit significand product with two 32 x 32-bit integer
//                multiplies, rounds it to 53 and then to 24 bits with ties to even, and builds the
//                float; zeros directly; operands whose result could leave the normal float range
//                take the double product (checked against the double product on every non-NaN
//                float for omega = 1.9 and on strided samples for other omegas: same bits);
//   div_small    x / d for d = 1..6, correctly rounded: y = x * RN(1/d) corrected once by the
//                exact remainder fma(-y, d, x) (Markstein's correction step), on 2^-100 <= |x|
//                < 2^100 (every float x in that range gave the IEEE quotient's bits for each d);
//                zeros return x, other operands take the IEEE division.
#pragma once
#include <stdint.h>
#include <string.h>

#include <cmath>

#include "kernels.h"

namespace smk {

__host__ __device__ __forceinline__ uint32_t es_funnel_r(uint32_t lo, uint32_t hi, int s) {
#ifdef __CUDA_ARCH__
    return __funnelshift_r(lo, hi, (unsigned)s);
#else
    return (uint32_t)((((uint64_t)hi << 32) | lo) >> s);
#endif
}

__host__ __device__ __forceinline__ float es_bits(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}

__host__ __device__ __forceinline__ uint32_t es_uint(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}

// The operands outside the fast paths' range, out of line (a device call the compiler cannot
// evaluate for every lane and select).
#ifdef __CUDA_ARCH__
__device__ __noinline__ float es_scale_slow(float q, double omega) { return __double2float_rn((double)q * omega); }
__device__ __noinline__ float es_div_slow(float x, float d) { return x / d; }
#else
inline float es_scale_slow(float q, double omega) { return (float)((double)q * omega); }
inline float es_div_slow(float x, float d) { return x / d; }
#endif

// float(double(q) * omega) with omega split by omega_split (kernels_vsweep_tb.cu).
__host__ __device__ __forceinline__ float omega_scale(float q, const OmegaSplit& s, double omega) {
    const uint32_t bits = es_uint(q);
    const uint32_t E = (bits >> 23) & 0xffu;
    const uint32_t sign = (bits ^ (s.sign << 31)) & 0x80000000u;
    if ((bits << 1) == 0u) return es_bits(sign);
    if ((uint32_t)((int)E - s.emin) > (uint32_t)(s.emax - s.emin)) return es_scale_slow(q, omega);
    const uint32_t mq = (bits & 0x7fffffu) | 0x800000u;
    const uint64_t A = (uint64_t)mq * s.mo_lo;  // < 2^56
    const uint64_t B = (uint64_t)mq * s.mo_hi;  // < 2^45
    // the product P = w2:w1:w0 (96-bit words), P in [2^75, 2^77)
    const uint32_t w0 = (uint32_t)A;
    const uint64_t mid = (A >> 32) + (uint32_t)B;
    const uint32_t w1 = (uint32_t)mid;
    const uint32_t w2 = (uint32_t)(B >> 32) + (uint32_t)(mid >> 32);
    const int big = w2 >= (1u << 12) ? 1 : 0;                       // P has 76 + big bits
    uint32_t t24 = es_funnel_r(w1, w2, 20 + big);                    // P >> (52 + big): 24 bits
    uint32_t rh = es_funnel_r(w0, w1, 23 + big) & 0x1fffffffu;       // the next 29 bits
    const uint32_t fr = w0 << (9 - big);                              // the lowest 23 + big, left-aligned
    rh += (fr > 0x80000000u || (fr == 0x80000000u && (rh & 1u))) ? 1u : 0u;     // to 53 bits
    t24 += (rh > 0x10000000u || (rh == 0x10000000u && (t24 & 1u))) ? 1u : 0u;  // to 24 bits
    // value = t24 * 2^((E - 127) + eo + big - 23); adding t24 (implicit bit included) to the
    // exponent field one below carries into it correctly, also when t24 rounded up to 2^24
    return es_bits(sign + ((uint32_t)((int)E + s.eo + big - 1) << 23) + t24);
}

// x / d, d = 1..6 given as the float df, r = RN(1/d).
__host__ __device__ __forceinline__ float div_small(float x, float df, float r) {
    const float ax = fabsf(x);
    if (ax == 0.0f) return x;
    if (!(ax >= 0x1p-100f && ax < 0x1p100f)) return es_div_slow(x, df);
    const float y = x * r;
    const float e = fmaf(-y, df, x);
    return fmaf(e, r, y);
}

}  // namespace smk
