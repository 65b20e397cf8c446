// lla_f32_bits.h -- double -> float conversions on bit patterns (integer
// operations only), for kernels where FP64 arithmetic is the scarce resource.
// Host and device code: a host test checks sym_to_f32 against the compiler's
// own conversion.
#pragma once

#include <stdint.h>
#include <string.h>

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

__host__ __device__ __forceinline__ float f32_from_bits(uint32_t w) {
    float f;
    memcpy(&f, &w, 4);
    return f;
}
__host__ __device__ __forceinline__ double f64_from_bits(int64_t b) {
    double d;
    memcpy(&d, &b, 8);
    return d;
}

#ifdef __CUDACC__
#define LLA_OUT_OF_LINE __noinline__
#else
#define LLA_OUT_OF_LINE __attribute__((noinline))
#endif
// The hardware conversion, out of line: a predicated copy in the common path
// would still take FP64 issue slots for every element.
static LLA_OUT_OF_LINE __host__ __device__ float f32_hw_convert(int64_t b) { return (float)f64_from_bits(b); }

// fp32(x) rounded to nearest even, from the bits b of a double whose FP32
// exponent is normal (the mantissa's low 29 bits decide the rounding; a carry
// into the exponent field is the correctly rounded result, infinity
// included); any other value (zero, FP32 subnormal or overflow, inf, NaN)
// through the hardware conversion.
__host__ __device__ __forceinline__ float sym_to_f32(int64_t b) {
    const int fe = (int)((b >> 52) & 0x7ff) - (1023 - 127);
    if (fe < 1 || fe > 254) return f32_hw_convert(b);
    const uint64_t mant = (uint64_t)b & 0xfffffffffffffull;
    const uint32_t m = (uint32_t)(mant >> 29), rem = (uint32_t)(mant & 0x1fffffffull);
    uint32_t w = ((uint32_t)fe << 23) | m;
    w += (rem > 0x10000000u || (rem == 0x10000000u && (m & 1u))) ? 1u : 0u;
    return f32_from_bits(w | ((uint32_t)((uint64_t)b >> 32) & 0x80000000u));
}

// |a| as FP32, truncated, from the bits v of a non-negative double that is
// zero or lies in [2^-100, 2^100] (sym_f32_range): for partial sums only.
__host__ __device__ __forceinline__ bool sym_f32_range(uint64_t v) {
    const int e = (int)(v >> 52) - 1023;
    return v == 0ull || (e >= -100 && e <= 100);
}
__host__ __device__ __forceinline__ float sym_abs_f32(uint64_t v) {
    if (v == 0ull) return 0.f;
    const uint32_t fe = (uint32_t)(v >> 52) - (1023u - 127u);
    return f32_from_bits((fe << 23) | (uint32_t)((v >> 29) & 0x7fffffull));
}

}  // namespace lla
