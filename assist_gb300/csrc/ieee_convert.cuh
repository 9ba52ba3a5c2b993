/*
 * ieee_convert.cuh -- float <-> double conversions on the integer pipes.
 *
 * On GB300 a conversion between float and double is an instruction of the
 * FP64 pipe and occupies it as long as an FP64 multiply-add, while the
 * block-cooperative kernel's float-pair terms convert every particle
 * position and partial sum.  These functions do the same conversions with
 * integer operations on the two 32-bit halves of the double, as IEEE 754
 * defines them: float -> double exactly, double -> float rounded to nearest
 * with ties to even.  Inputs whose result is not a normal number (zeros,
 * subnormals, infinities, NaN, overflow of the float range) take the
 * hardware conversion, so every input converts exactly as the hardware does.
 * Host-compilable for the tests (plain C++ without CUDA).
 */
#ifndef ASSIST_GB300_IEEE_CONVERT_CUH
#define ASSIST_GB300_IEEE_CONVERT_CUH

#include <cstring>

#ifdef __CUDACC__
#define AG_HD __host__ __device__ __forceinline__
#else
#define AG_HD inline
#endif

AG_HD unsigned ag_hi_word(double x) {
#ifdef __CUDA_ARCH__
    return (unsigned)__double2hiint(x);
#else
    unsigned long long u;
    std::memcpy(&u, &x, 8);
    return (unsigned)(u >> 32);
#endif
}
AG_HD unsigned ag_lo_word(double x) {
#ifdef __CUDA_ARCH__
    return (unsigned)__double2loint(x);
#else
    unsigned long long u;
    std::memcpy(&u, &x, 8);
    return (unsigned)u;
#endif
}
AG_HD double ag_from_words(unsigned hi, unsigned lo) {
#ifdef __CUDA_ARCH__
    return __hiloint2double((int)hi, (int)lo);
#else
    const unsigned long long u = ((unsigned long long)hi << 32) | lo;
    double x;
    std::memcpy(&x, &u, 8);
    return x;
#endif
}
AG_HD unsigned ag_float_bits(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    unsigned u;
    std::memcpy(&u, &f, 4);
    return u;
#endif
}
AG_HD float ag_float_of_bits(unsigned u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    std::memcpy(&f, &u, 4);
    return f;
#endif
}

/* float -> double: sign, exponent rebiased by 1023 - 127 = 896, the 23
 * mantissa bits at the top of the double's 52. */
AG_HD double ag_f2d_int(float f) {
    const unsigned u = ag_float_bits(f);
    const unsigned e = (u >> 23) & 0xffu;
    if (e == 0u || e == 0xffu) return (double)f;
    return ag_from_words((u & 0x80000000u) | ((e + 896u) << 20) | ((u & 0x7fffffu) >> 3), u << 29);
}

/* double -> float, round to nearest even: the top 23 of the 52 mantissa
 * bits, plus one where the 29 dropped bits exceed half a unit (or equal it
 * and the kept mantissa is odd); a carry out of the mantissa increments the
 * exponent, to infinity past the largest float, as IEEE rounding does. */
AG_HD float ag_d2f_int(double x) {
    const unsigned hi = ag_hi_word(x), lo = ag_lo_word(x);
    const int e = (int)((hi >> 20) & 0x7ffu) - 896;
    if (e <= 0 || e >= 255) return (float)x;
    const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const unsigned rem = lo & 0x1fffffffu;
    unsigned r = ((unsigned)e << 23) | m;
    if (rem > 0x10000000u || (rem == 0x10000000u && (m & 1u))) r += 1u;
    return ag_float_of_bits((hi & 0x80000000u) | r);
}

#endif
