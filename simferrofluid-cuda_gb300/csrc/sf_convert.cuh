// Conversions between IEEE 754 binary64 and binary32 in 32-bit integer arithmetic, with the results the standard
// defines for convertFormat: double -> float rounds to nearest, ties to even; float -> double is exact.
//
// On this GPU the hardware conversion instructions between the two formats issue on the FP64 pipe (2 lanes per
// clock per SM), so in kernels that are already FP64-bound a conversion costs as much as a double-precision
// add.  These versions run on the integer pipe for the values the solver stores (zero, and normal numbers whose
// float result is normal); anything else (subnormal results, overflow, infinities, NaN) takes the hardware
// conversion, so every input gets the standard's result.  The same functions compile for the host, where
// tests compare them with the compiler's own casts bit for bit.
#pragma once
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define SF_CONV_FN __host__ __device__ __forceinline__
#else
#define SF_CONV_FN inline
#endif

namespace sf {

SF_CONV_FN void f64_words(double v, uint32_t &hi, uint32_t &lo) {
#if defined(__CUDA_ARCH__)
    hi = (uint32_t)__double2hiint(v);
    lo = (uint32_t)__double2loint(v);
#else
    uint64_t b;
    std::memcpy(&b, &v, 8);
    hi = (uint32_t)(b >> 32);
    lo = (uint32_t)b;
#endif
}

SF_CONV_FN double f64_from_words(uint32_t hi, uint32_t lo) {
#if defined(__CUDA_ARCH__)
    return __hiloint2double((int)hi, (int)lo);
#else
    const uint64_t b = ((uint64_t)hi << 32) | lo;
    double v;
    std::memcpy(&v, &b, 8);
    return v;
#endif
}

SF_CONV_FN float f32_from_bits(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float v;
    std::memcpy(&v, &u, 4);
    return v;
#endif
}

SF_CONV_FN uint32_t f32_bits(float v) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(v);
#else
    uint32_t u;
    std::memcpy(&u, &v, 4);
    return u;
#endif
}

// double -> float, round to nearest, ties to even.
SF_CONV_FN float f64_to_f32(double v) {
    uint32_t hi, lo;
    f64_words(v, hi, lo);
    const uint32_t sign = hi & 0x80000000u;
    if (((hi << 1) | lo) == 0u) return f32_from_bits(sign);  // +-0
    // binary64 exponent field e (bias 1023) -> binary32 field e - 896 (bias 127); the integer path covers
    // results in the normal range, fields 1 .. 254
    const int fe = (int)((hi >> 20) & 0x7ffu) - 896;
    if ((unsigned)(fe - 1) >= 254u) return (float)v;
    // 52-bit significand: the top 23 bits are kept, the low 29 decide the rounding
    const uint32_t mant = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const uint32_t rest = lo & 0x1fffffffu;
    uint32_t out = ((uint32_t)fe << 23) | mant;
    // more than half an ulp, or exactly half with an odd last bit: round up (a carry out of the significand
    // moves into the exponent field, which is the correctly rounded result, up to infinity)
    out += (rest > 0x10000000u || (rest == 0x10000000u && (mant & 1u))) ? 1u : 0u;
    return f32_from_bits(sign | out);
}

// float -> double, exact.
SF_CONV_FN double f32_to_f64(float v) {
    const uint32_t u = f32_bits(v);
    const uint32_t sign = u & 0x80000000u;
    if ((u << 1) == 0u) return f64_from_words(sign, 0u);  // +-0
    const uint32_t e = (u >> 23) & 0xffu;
    if (e == 0u || e == 0xffu) return (double)v;  // subnormal, infinity, NaN
    const uint32_t m = u & 0x7fffffu;
    return f64_from_words(sign | ((e + 896u) << 20) | (m >> 3), m << 29);
}

}  // namespace sf
