// Exact FP32 <-> FP64 steps from the bit patterns, and the cell key of a
// double position in float-float arithmetic.
//
// GB300 issues FP64 arithmetic and every conversion to or from FP64 to a
// pipe about 60 times slower than FP32 (2 lanes per clock per SM).  The
// FP32 form keeps FP64 where it is required (positions, energies) and does
// everything else with FP32 and integer instructions; these helpers are the
// integer-only pieces.  The header compiles as C (gcc) and as CUDA, so the
// CPU test in tests/ checks the same code that the kernels run.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define FPS_HD __host__ __device__ __forceinline__
#else
#define FPS_HD static inline
#endif

FPS_HD uint64_t fps_d2u(double x) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u;
    memcpy(&u, &x, 8);
    return u;
#endif
}

FPS_HD double fps_u2d(uint64_t u) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)u);
#else
    double x;
    memcpy(&x, &u, 8);
    return x;
#endif
}

FPS_HD uint32_t fps_f2u(float x) {
#ifdef __CUDA_ARCH__
    return (uint32_t)__float_as_uint(x);
#else
    uint32_t u;
    memcpy(&u, &x, 4);
    return u;
#endif
}

FPS_HD float fps_u2f(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float x;
    memcpy(&x, &u, 4);
    return x;
#endif
}

FPS_HD int fps_clz32(uint32_t v) {
#ifdef __CUDA_ARCH__
    return __clz((int)v);
#else
    return v ? __builtin_clz(v) : 32;
#endif
}

// Uncontracted float products and sums (device code is built with FMA
// contraction on; these steps must round separately).
FPS_HD float fps_mul(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}

FPS_HD float fps_add(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}

// (double)f for every float: zeros and normal numbers by moving the fields
// (exponent rebias 127 -> 1023, fraction shifted up by 29 bits); subnormal,
// infinite and NaN inputs by the conversion instruction.
FPS_HD double fps_f2d(float f) {
    const uint32_t u = fps_f2u(f);
    const uint32_t e = (u >> 23) & 0xffu;
    const uint64_t sign = (uint64_t)(u & 0x80000000u) << 32;
    if (e == 0u) {
        if ((u & 0x7fffffu) == 0u) return fps_u2d(sign);
        return (double)f;
    }
    if (e == 255u) return (double)f;
    return fps_u2d(sign | ((uint64_t)(e + 896u) << 52) | ((uint64_t)(u & 0x7fffffu) << 29));
}

// Cell index and cell-local coordinate along one axis.  With
// y = RN64(1/h) = ih + il (il = RN32(y - ih)), x is split exactly into
// hi (its leading 24 significand bits) and lo (the remaining 29, rounded
// down to 24), and q = x*y is formed as p + t with p = RN32(hi*ih),
// t = hi*il + lo*ih + (hi*ih - p) (the last term exact by FMA).  For
// |p| < 2^20, |p + t - x/h| < 2^-43 |x/h|, and the float fraction
// fr = (p - floor(p)) + t is within 2e-7 of the fraction of RN64(x/h).  So
// when fr lies more than 1e-4 from 0 and 1, floor(p) is the floor of the
// correctly rounded quotient and fr its cell-local coordinate: returns 1.
// Otherwise (and for zero, tiny, huge or non-finite x) returns 0 and the
// caller decides with the exact FP64 quotient.
FPS_HD int fps_cell(double x, float ih, float il, float* fl, float* u) {
    const uint64_t b = fps_d2u(x);
    const int e = (int)((b >> 52) & 0x7ffu);
    if (e < 949 || e > 1150) return 0;
    const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
    const uint64_t mant = b & 0xfffffffffffffULL;
    const float hi = fps_u2f(sign | ((uint32_t)(e - 896) << 23) | (uint32_t)(mant >> 29));
    const uint32_t L = (uint32_t)(mant & 0x1fffffffu);
    float lo = 0.0f;
    if (L) {
        const int tb = 31 - fps_clz32(L);                    // leading bit, <= 28
        const uint32_t m24 = tb >= 23 ? (L >> (tb - 23)) : (L << (23 - tb));
        lo = fps_u2f(sign | ((uint32_t)(tb + e - 1075 + 127) << 23) | (m24 & 0x7fffffu));
    }
    const float p = fps_mul(hi, ih);
    if (!(fabsf(p) < 1048576.0f)) return 0;
    const float pe = fmaf(hi, ih, -p);
    const float t = fmaf(hi, il, fmaf(lo, ih, pe));
    const float f = floorf(p);
    const float fr = fps_add(fps_add(p, -f), t);
    if (!(fr > 1.0e-4f && fr < 1.0f - 1.0e-4f)) return 0;
    *fl = f;
    *u = fr;
    return 1;
}

// The largest float m0 with (m > m0) == (m > threshold) for every float m:
// the threshold rounded down to float.
FPS_HD float fps_float_threshold(double threshold) {
    float r = (float)threshold;
    if ((double)r > threshold) r = nextafterf(r, -INFINITY);
    return r;
}
