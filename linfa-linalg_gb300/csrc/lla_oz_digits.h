// lla_oz_digits.h -- the exact-slice digits of a double, as packed BF16 pairs.
// Host and device code: the slicing kernels use these functions, and a host
// test checks them against an independent restatement (digits of
// floor(|a| 2^(56-e)) and the BF16 bits of each signed digit).
#pragma once

#include <stdint.h>
#include <string.h>

#include <cmath>

#ifndef __CUDACC__  // host-only compilers: the qualifiers vanish
#ifndef __host__
#define __host__
#endif
#ifndef __device__
#define __device__
#endif
#ifndef __forceinline__
#define __forceinline__ inline
#endif
#endif

namespace lla {

constexpr int kOzDigits = 8;  // 7-bit digits of a 56-bit magnitude

// The magnitude |a| 2^(56 - e) (|a| < 2^e) as a 56-bit integer, low bits
// truncated (below 2^-56 of the scale), split into its high 28 bits (digits
// 0..3) and low 28 bits (digits 4..7); neg: the sign of a.  Integer operations
// only.  Zero, inf and NaN give 0.
__host__ __device__ __forceinline__ void oz_magnitude(int64_t bits, int e, uint32_t &hi, uint32_t &lo, bool &neg) {
    const int eb = (int)((bits >> 52) & 0x7ff);
    uint64_t mant = (uint64_t)bits & ((1ull << 52) - 1);
    int ea;  // a = mant * 2^ea
    if (eb == 0) {
        ea = -1074;
    } else {
        mant |= 1ull << 52;
        ea = eb - 1075;
    }
    const int shift = ea + 56 - e;  // <= 3 since |a| < 2^e
    uint64_t T = 0;
    if (mant != 0 && eb != 0x7ff) {
        if (shift >= 0)
            T = mant << shift;
        else if (shift > -64)
            T = mant >> (-shift);
    }
    hi = (uint32_t)(T >> 28);
    lo = (uint32_t)(T & 0xfffffffu);
    neg = ((uint64_t)bits >> 63) != 0;
}

// FP32 bits of the signed digit (h >> s) & 127: the digit d is placed in the
// mantissa of 2^23 (exact), and sgn * (2^23 + d) + nsc with (sgn, nsc) = (1,
// -2^23) or (-1, 2^23) is +-d, +0 for d = 0 (an exact zero sum rounds to +0).
// A digit has at most 7 significant bits, so the upper 16 bits are its BF16.
__host__ __device__ __forceinline__ uint32_t oz_digit_f32_bits(uint32_t h, int s, float sgn, float nsc) {
    const uint32_t m = 0x4b000000u | ((h >> s) & 127u);
    float mf, f;
    memcpy(&mf, &m, 4);
#ifdef __CUDA_ARCH__
    f = __fmaf_rn(sgn, mf, nsc);
#else
    f = std::fma(sgn, mf, nsc);
#endif
    uint32_t w;
    memcpy(&w, &f, 4);
    return w;
}

// Two BF16 (the upper halves of two FP32 bit patterns) packed, a in the low half.
__host__ __device__ __forceinline__ uint32_t oz_pack_bf16(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
    return __byte_perm(a, b, 0x7632);
#else
    return (a >> 16) | (b & 0xffff0000u);
#endif
}

// Digits p = 0..7 of four consecutive elements (bits b[0..3], common scale
// exponent e) as BF16: out[p] holds elements 0..3 of plane p, element 0 in the
// lowest 16 bits.
__host__ __device__ __forceinline__ void oz_digits_packed4(const int64_t (&b)[4], int e, uint32_t (&out)[kOzDigits][2]) {
    uint32_t hi[4], lo[4];
    float sgn[4], nsc[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        bool neg;
        oz_magnitude(b[u], e, hi[u], lo[u], neg);
        sgn[u] = neg ? -1.f : 1.f;
        nsc[u] = neg ? 8388608.f : -8388608.f;
    }
#pragma unroll
    for (int p = 0; p < kOzDigits; ++p) {
        const int s = p < 4 ? 7 * (3 - p) : 7 * (7 - p);
        uint32_t f[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) f[u] = oz_digit_f32_bits(p < 4 ? hi[u] : lo[u], s, sgn[u], nsc[u]);
        out[p][0] = oz_pack_bf16(f[0], f[1]);
        out[p][1] = oz_pack_bf16(f[2], f[3]);
    }
}

}  // namespace lla
