// fpconv.cuh -- FP32 <-> FP64 conversions on the integer pipe.
//
// On GB300 the FP64 pipe (about 2 operations per clock per SM) also executes
// the F2F conversions between float and double.  Kernels that move FP32
// increments into an FP64 state, or FP64 state into FP32 mirrors, are then
// bound by that pipe rather than by HBM.  These functions do the IEEE-754
// conversions with integer operations instead:
//
//   f2d_exact(f): float -> double, exact (every float is a double).
//   d2f_rn(d):    double -> float, round to nearest, ties to even (the
//                 rounding of a C cast and of cvt.rn.f32.f64).
//
// Both take a fast path for normal results and zeros and fall back to the
// hardware conversion for the rest (subnormal results, overflow, Inf, NaN),
// so the results are those of the plain casts bit for bit.  The fallbacks
// are calls of non-inlined functions: the compiler may not execute them
// speculatively on the fast path (it would, for an inline conversion, and
// the FP64 pipe would be as busy as before).
//
// Binary layouts (IEEE 754-2008): float = 1 sign, 8 exponent (bias 127),
// 23 fraction bits; double = 1 sign, 11 exponent (bias 1023), 52 fraction
// bits.  Exponents differ by 1023 - 127 = 896.
#pragma once
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define FPC_HD __host__ __device__ __forceinline__
#else
#define FPC_HD static inline
#endif

FPC_HD uint32_t fpc_f2u(float f)
{
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}
FPC_HD float fpc_u2f(uint32_t u)
{
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}
FPC_HD uint64_t fpc_d2u(double d)
{
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(d);
#else
    uint64_t u;
    memcpy(&u, &d, 8);
    return u;
#endif
}
FPC_HD double fpc_u2d(uint64_t u)
{
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)u);
#else
    double d;
    memcpy(&d, &u, 8);
    return d;
#endif
}

#ifdef __CUDACC__
static __device__ __noinline__ double fpc_f2d_slow(float f) { return (double)f; }
static __device__ __noinline__ float fpc_d2f_slow(double d) { return (float)d; }
#endif
#ifdef __CUDA_ARCH__
#define FPC_F2D_SLOW(f) fpc_f2d_slow(f)
#define FPC_D2F_SLOW(d) fpc_d2f_slow(d)
#else
#define FPC_F2D_SLOW(f) ((double)(f))
#define FPC_D2F_SLOW(d) ((float)(d))
#endif

// float -> double (exact)
FPC_HD double f2d_exact(float f)
{
    const uint32_t u = fpc_f2u(f);
    const uint32_t e = (u >> 23) & 0xffu;
    if (e == 0u || e == 0xffu) {
        if ((u & 0x7fffffffu) == 0u) return fpc_u2d((uint64_t)(u & 0x80000000u) << 32);   // +-0
        return FPC_F2D_SLOW(f);                                                           // subnormal, Inf, NaN
    }
    const uint32_t hi = (u & 0x80000000u) | ((e + 896u) << 20) | ((u & 0x7fffffu) >> 3);
    const uint32_t lo = (u & 7u) << 29;
    return fpc_u2d(((uint64_t)hi << 32) | lo);
}

// double -> float, round to nearest even
FPC_HD float d2f_rn(double d)
{
    const uint64_t u = fpc_d2u(d);
    const uint32_t hi = (uint32_t)(u >> 32), lo = (uint32_t)u;
    const uint32_t sign = hi & 0x80000000u;
    const int ef = (int)((hi >> 20) & 0x7ffu) - 896;   // the float's biased exponent
    if (ef < 1 || ef > 254) {
        if ((hi & 0x7fffffffu) == 0u && lo == 0u) return fpc_u2f(sign);                  // +-0
        return FPC_D2F_SLOW(d);                  // subnormal or zero result, overflow, Inf, NaN
    }
    // the top 23 of the 52 fraction bits, and the 29 bits below them
    const uint32_t man = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const uint32_t rem = lo & 0x1fffffffu;
    const uint32_t half = 0x10000000u;
    const uint32_t up = (rem > half || (rem == half && (man & 1u))) ? 1u : 0u;
    // a carry out of the fraction moves into the exponent (and to Inf at the top)
    return fpc_u2f(sign | ((((uint32_t)ef << 23) | man) + up));
}

// double -> float by truncation of the fraction, integer operations only:
// relative error < 2^-23 in the normal range; results below it become +-0,
// above it +-Inf, NaN stays NaN (for estimates, not for state)
FPC_HD float d2f_est(double d)
{
    const uint64_t u = fpc_d2u(d);
    const uint32_t hi = (uint32_t)(u >> 32);
    const uint32_t sign = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7ffu);
    const int ef = e - 896;
    if (ef < 1) return fpc_u2f(sign);
    if (ef > 254) {
        const int nan = e == 0x7ff && ((hi & 0xfffffu) | (uint32_t)u) != 0u;
        return fpc_u2f(sign | (nan ? 0x7fc00000u : 0x7f800000u));
    }
    return fpc_u2f(sign | ((uint32_t)ef << 23) | ((hi & 0xfffffu) << 3) | ((uint32_t)u >> 29));
}
