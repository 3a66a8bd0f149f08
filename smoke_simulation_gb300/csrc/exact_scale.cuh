// Exact float arithmetic of the reference's projection step without the FP64 pipe (host and
// device).  The reference computes p_t = (-div / acc) * OVER_RELAXATION with a float quotient and
// a double constant (project/smokeSimulation.cu:38, :384): float(double(q) * omega), one
// rounding to 53 bits and one to 24.  GB300's FP64 rate is a small fraction of its FP32 and
// integer rates, and the one-pass projection kernel is bound by it (its FP64 pipe runs at ~48 %
// of peak), so:
//   omega_scale  forms the 24 x 53-bit significand product with two 32 x 32-bit integer
//                multiplies, rounds it to 53 and then to 24 bits with ties to even, and builds the
//                float; zeros directly.  Operands whose result can fall below the normal range
//                (subnormal q included) take omega_scale_tiny: q normalised, the same product
//                rounded to 53 bits, then to a multiple of 2^-149 where the result is below
//                2^-126.  Operands whose result could overflow take the double product.  (Checked
//                against the double product on every non-NaN float for omega = 1.9 and on
//                strided samples for other omegas: same bits);
//   div_small    x / d for d = 1..6, correctly rounded: y = x * RN(1/d) corrected once by the
//                exact remainder fma(-y, d, x) (Markstein's correction step), on 2^-100 <= |x|
//                < 2^100 (every float x in that range gave the IEEE quotient's bits for each d);
//                below that range div_tiny applies the same step to x * 2^64 and scales back
//                where the quotient is normal, and rounds m / d to the nearest integer (ties to
//                even) for the quotients below 2^-126, x = m * 2^-149; zeros return x, other
//                operands take the IEEE division.
// In a fresh simulation the red-black passes spread values far below 2^-100 (subnormals among
// them) ahead of the first smoke: about 1 % of the faces for a few steps, so that about half the
// warps of a pass hold such a lane.  div_scale_fast keeps the common lanes free of branches and
// the tiny paths keep the rare ones off the FP64 pipe and the general division.
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

__host__ __device__ __forceinline__ int es_clz(uint32_t v) {
#ifdef __CUDA_ARCH__
    return __clz(v);
#else
    return __builtin_clz(v);
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

// The significand product of omega_scale: mq (24 bits, leading bit 23) times omega's 53-bit
// significand, P = w2:w1:w0 in [2^75, 2^77); t24 = its leading 24 bits, rh = the next 29 bits
// rounded (ties to even) on the rest, so that t24 * 2^29 + rh is P rounded to 53 bits; big = 1
// when P has 77 bits.
struct EsProduct {
    uint32_t t24, rh;
    int big;
};

__host__ __device__ __forceinline__ EsProduct es_product(uint32_t mq, uint32_t mo_hi, uint32_t mo_lo) {
    const uint64_t A = (uint64_t)mq * mo_lo;  // < 2^56
    const uint64_t B = (uint64_t)mq * mo_hi;  // < 2^45
    const uint32_t w0 = (uint32_t)A;
    const uint64_t mid = (A >> 32) + (uint32_t)B;
    const uint32_t w1 = (uint32_t)mid;
    const uint32_t w2 = (uint32_t)(B >> 32) + (uint32_t)(mid >> 32);
    EsProduct r;
    r.big = w2 >= (1u << 12) ? 1 : 0;                                  // P has 76 + big bits
    r.t24 = es_funnel_r(w1, w2, 20 + r.big);                           // P >> (52 + big): 24 bits
    r.rh = es_funnel_r(w0, w1, 23 + r.big) & 0x1fffffffu;              // the next 29 bits
    const uint32_t fr = w0 << (9 - r.big);                             // the lowest 23 + big, left-aligned
    r.rh += (fr > 0x80000000u || (fr == 0x80000000u && (r.rh & 1u))) ? 1u : 0u;  // to 53 bits
    return r;
}

// omega_scale for the operands whose result can fall below the normal float range (biased
// exponent E < emin, subnormal q included; q != 0 and omega_split gave a valid split).  The
// result's biased exponent is Eb = Eq + eo + big (Eq = E, or 1 - shift for a subnormal q whose
// significand was shifted left to bit 23); below 1 the 53-bit value V * 2^(Eb - 179),
// V = t24 * 2^29 + rh, is rounded to a multiple of 2^-149 as the conversion of the double does.
__host__ __device__ __forceinline__ float omega_scale_tiny(uint32_t bits, uint32_t mo_hi, uint32_t mo_lo, int eo,
                                                           uint32_t osign) {
    const uint32_t E = (bits >> 23) & 0xffu;
    const uint32_t sign = (bits ^ (osign << 31)) & 0x80000000u;
    const uint32_t mant = bits & 0x7fffffu;
    int Eq = (int)E;
    uint32_t mq = mant | 0x800000u;
    if (E == 0) {
        const int sh = es_clz(mant) - 8;  // mant != 0: its leading bit moves to bit 23
        mq = mant << sh;
        Eq = 1 - sh;
    }
    EsProduct p = es_product(mq, mo_hi, mo_lo);
    const int Eb = Eq + eo + p.big;
    if (Eb >= 1) {
        p.t24 += (p.rh > 0x10000000u || (p.rh == 0x10000000u && (p.t24 & 1u))) ? 1u : 0u;
        return es_bits(sign + ((uint32_t)(Eb - 1) << 23) + p.t24);
    }
    const uint64_t V = ((uint64_t)p.t24 << 29) + p.rh;  // <= 2^53
    const int sh = 30 - Eb;                              // the value in units of 2^-149 is V / 2^sh
    if (sh >= 55) return es_bits(sign);                  // below half of 2^-149 (V / 2^55 < 1/4)
    uint64_t qv = V >> sh;
    const uint64_t rem = V & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    qv += (rem > half || (rem == half && (qv & 1u))) ? 1u : 0u;
    return es_bits(sign | (uint32_t)qv);  // qv <= 2^23: a subnormal, or the smallest normal
}

// float(double(q) * omega) with omega split by omega_split (kernels_vsweep_tb.cu).
__host__ __device__ __forceinline__ float omega_scale(float q, const OmegaSplit& s, double omega) {
    const uint32_t bits = es_uint(q);
    const uint32_t E = (bits >> 23) & 0xffu;
    const uint32_t sign = (bits ^ (s.sign << 31)) & 0x80000000u;
    if ((bits << 1) == 0u) return es_bits(sign);
    if ((uint32_t)((int)E - s.emin) > (uint32_t)(s.emax - s.emin)) {
        if ((int)E < s.emin && s.emin <= s.emax) return omega_scale_tiny(bits, s.mo_hi, s.mo_lo, s.eo, s.sign);
        return es_scale_slow(q, omega);
    }
    EsProduct p = es_product((bits & 0x7fffffu) | 0x800000u, s.mo_hi, s.mo_lo);
    p.t24 += (p.rh > 0x10000000u || (p.rh == 0x10000000u && (p.t24 & 1u))) ? 1u : 0u;  // to 24 bits
    // value = t24 * 2^((E - 127) + eo + big - 23); adding t24 (implicit bit included) to the
    // exponent field one below carries into it correctly, also when t24 rounded up to 2^24
    return es_bits(sign + ((uint32_t)((int)E + s.eo + p.big - 1) << 23) + p.t24);
}

// x / d for 0 < |x| < 2^-100, d = 1..6 given as the float df, r = RN(1/d).  x * 2^64 is exact
// and inside the corrected multiply's range; the quotient ys scales back exactly when it is at
// least 2^-62 (the result is normal).  Below, |x / d| < 2^-126 and |x| < 6 * 2^-126, so
// x = m * 2^-149 with m < 2^26, and the result is RN(m / d) * 2^-149 (<= 2^-126).
__host__ __device__ __forceinline__ float div_tiny(float x, float df, float r) {
    const float xs = x * 0x1p64f;
    const float y = xs * r;
    const float e = fmaf(-y, df, xs);
    const float ys = fmaf(e, r, y);
    if (fabsf(ys) >= 0x1p-62f) return ys * 0x1p-64f;
    const uint32_t bits = es_uint(x);
    const uint32_t E = (bits >> 23) & 0xffu;
    const uint32_t mant = bits & 0x7fffffu;
    const uint32_t m = E == 0 ? mant : ((mant | 0x800000u) << (E - 1));
    const uint32_t d = (uint32_t)df;
    uint32_t qi = m / d;
    const uint32_t rem = m - qi * d;
    qi += (2u * rem > d || (2u * rem == d && (qi & 1u))) ? 1u : 0u;
    return es_bits((bits & 0x80000000u) | qi);
}

// x / d, d = 1..6 given as the float df, r = RN(1/d).
__host__ __device__ __forceinline__ float div_small(float x, float df, float r) {
    const float ax = fabsf(x);
    if (ax == 0.0f) return x;
    if (ax < 0x1p-100f) return div_tiny(x, df, r);
    if (!(ax < 0x1p100f)) return es_div_slow(x, df);
    const float y = x * r;
    const float e = fmaf(-y, df, x);
    return fmaf(e, r, y);
}

// float(double(x / d) * omega) for a cell update, without branches on the common operands:
// the corrected multiply and the integer product run for every lane, and a select gives zeros
// (signed as the quotient and product of a zero are).  `rare` is set for the operands that need
// the full functions (|x| below 2^-100 or not below 2^100, a quotient outside the integer
// product's exponent range): the caller then takes div_scale_full, so that a warp diverges only
// where one of its lanes has such an operand.
__host__ __device__ __forceinline__ float div_scale_fast(float x, float df, float r, const OmegaSplit& s,
                                                        bool& rare) {
    const float ax = fabsf(x);
    const float y = x * r;
    const float e = fmaf(-y, df, x);
    float q = fmaf(e, r, y);
    q = ax == 0.0f ? x : q;
    const uint32_t bits = es_uint(q);
    const uint32_t E = (bits >> 23) & 0xffu;
    const uint32_t sign = (bits ^ (s.sign << 31)) & 0x80000000u;
    EsProduct p = es_product((bits & 0x7fffffu) | 0x800000u, s.mo_hi, s.mo_lo);
    p.t24 += (p.rh > 0x10000000u || (p.rh == 0x10000000u && (p.t24 & 1u))) ? 1u : 0u;
    const uint32_t pt = sign + ((uint32_t)((int)E + s.eo + p.big - 1) << 23) + p.t24;
    const bool zero = ax == 0.0f;
    rare = !zero && (!(ax >= 0x1p-100f && ax < 0x1p100f) ||
                     (uint32_t)((int)E - s.emin) > (uint32_t)(s.emax - s.emin));
    return es_bits(zero ? sign : pt);
}

// The same value through the full functions (every operand), out of line on the device.  The
// split is passed as scalars: the call then needs no stack frame.
__host__ __device__ __forceinline__ float div_scale_full(float x, float df, float r, uint32_t mo_hi, uint32_t mo_lo, int eo, uint32_t osign, int emin,
                     int emax, double omega) {
    OmegaSplit s;
    s.mo_hi = mo_hi;
    s.mo_lo = mo_lo;
    s.eo = eo;
    s.sign = osign;
    s.emin = emin;
    s.emax = emax;
    return omega_scale(div_small(x, df, r), s, omega);
}

}  // namespace smk
