// FP64 <-> FP32-pair conversions by integer operations on the IEEE-754 bit patterns.
//
// On this GPU the conversions between FP32 and FP64 run on the FP64 pipe (2 lanes per SM and
// cycle), which bounds the element kernel; these versions use only integer operations.  They are
// plain C++ on fixed-width integers, so the same source compiles for the device (the element
// kernel) and for the host (the test that checks them against exact arithmetic).
//
//   split_bits(d, &hi, &lo): hi = d with its significand truncated to 24 bits, lo = d - hi (the
//     remaining 29 bits, truncated to 24, or to the FP32 subnormal grid): |d - hi - lo| <=
//     max(2^-47 |d|, 2^-149).  Values below 2^-126 in magnitude give (0, 0); beyond the FP32 range
//     (inf, 0); NaN gives (NaN, 0).
//   widen_bits(f): the FP64 value of the FP32 number f, exact (subnormals included);
//     infinities and NaNs stay infinities and NaNs.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define EF_HD __host__ __device__ __forceinline__
#else
#define EF_HD inline
#endif

namespace ef {

EF_HD int clz32(uint32_t v) {
#if defined(__CUDA_ARCH__)
    return __clz((int)v);
#else
    int n = 0;
    if (v == 0) return 32;
    while (!(v & 0x80000000u)) {
        v <<= 1;
        ++n;
    }
    return n;
#endif
}

EF_HD void split_bits(uint64_t b, uint32_t* hiBits, uint32_t* loBits) {
    const uint32_t hw = (uint32_t)(b >> 32), lw = (uint32_t)b;
    const uint32_t sgn = hw & 0x80000000u;
    const int e = (int)((hw >> 20) & 0x7FFu);
    const uint32_t m23 = ((hw & 0xFFFFFu) << 3) | (lw >> 29);  // top 23 fraction bits
    const uint32_t r29 = lw & 0x1FFFFFFFu;                       // the 29 bits below them
    if (e == 0x7FF) {  // infinity or NaN (a quiet NaN for any NaN)
        const bool nan = (m23 | r29) != 0u;
        *hiBits = sgn | 0x7F800000u | (nan ? 0x400000u : 0u);
        *loBits = 0u;
        return;
    }
    if (e < 897) {  // |d| < 2^-126 (FP32 subnormal range and zero)
        *hiBits = sgn;
        *loBits = sgn;
        return;
    }
    if (e > 1150) {  // beyond the FP32 range
        *hiBits = sgn | 0x7F800000u;
        *loBits = 0u;
        return;
    }
    *hiBits = sgn | ((uint32_t)(e - 896) << 23) | m23;
    if (r29 == 0u) {
        *loBits = sgn;
        return;
    }
    // lo = r29 2^(e - 1075), the most significant set bit of r29 at position p
    const int p = 31 - clz32(r29);
    const int ef = p + e - 948;  // its FP32 exponent field
    if (ef < 1) {  // FP32 subnormal: significand r29 2^(e - 926) (below 2^23 here), truncated
        *loBits = sgn | (e >= 926 ? (r29 << (e - 926)) : (r29 >> (926 - e)));
        return;
    }
    const uint32_t mant = (p >= 23 ? (r29 >> (p - 23)) : (r29 << (23 - p))) & 0x7FFFFFu;
    *loBits = sgn | ((uint32_t)ef << 23) | mant;
}

EF_HD uint64_t widen_bits(uint32_t u) {
    const uint32_t e = (u >> 23) & 0xFFu;
    const uint64_t sgn = (uint64_t)(u & 0x80000000u) << 32;
    if (e == 0u) {  // zero or subnormal: m 2^-149, normalised
        const uint32_t m = u & 0x7FFFFFu;
        if (m == 0u) return sgn;
        const int p = 31 - clz32(m);
        return sgn | ((uint64_t)(p + 874) << 52) | (((uint64_t)m << (52 - p)) & 0xFFFFFFFFFFFFFull);
    }
    const uint64_t ed = e == 0xFFu ? 0x7FFull : (uint64_t)(e + 896u);
    return sgn | (ed << 52) | ((uint64_t)(u & 0x7FFFFFu) << 29);
}

}  // namespace ef

#undef EF_HD
