// Exact FP64 helpers of the FP64 step kernels: each returns the very double
// the plain IEEE operation would, with fewer instructions on the FP64 pipe
// (1/64 of the FP32 rate on GB300).  Only CUDA's IEEE intrinsics are used, so
// the results do not depend on the translation unit's -fmad setting.
#pragma once

#include <cuda_runtime.h>

namespace lat {

// x * p for an exact power of two p = 2^e.  When x and the result are normal
// numbers the product only moves the exponent field, which integer
// instructions do off the FP64 pipe (1/64 of the FP32 rate on GB300); zeros,
// subnormals, Inf/NaN and results outside the normal range take the FP64
// multiply.  Both give the same double.
__device__ __forceinline__ double mul_pow2(double x, double p)
{
    const long long bx = __double_as_longlong(x);
    const int ex = (int)(bx >> 52) & 0x7ff;
    const int e = ((int)(__double_as_longlong(p) >> 52) & 0x7ff) - 1023;
    const int ey = ex + e;
    if (ex == 0 || ex == 0x7ff || ey <= 0 || ey >= 0x7ff) return x * p;
    return __longlong_as_double(bx + ((long long)e << 52));
}

// a / b for a divisor b whose reciprocal y = RN(1/b) was computed on the host:
// q = a*y, then two residual corrections q += (a - b*q)*y with exact FMA
// residuals.  The first makes q a faithful quotient; from a faithful q and
// |y - 1/b| < 2^-53 |1/b|, the second returns the correctly rounded a / b
// (Markstein's theorem; P. Markstein, IBM J. Res. Dev. 34(1), 1990, and the
// Handbook of Floating-Point Arithmetic, ch. 4).  So the double is the IEEE
// quotient, at five FP64 instructions instead of a full division's reciprocal
// refinement.  A zero a returns a*y (the IEEE quotient +-0); otherwise |a|
// or |b| outside [2^-400, 2^401) (subnormals, Inf/NaN, and wherever quotient
// or residual could leave the normal range) take the IEEE division.
__device__ __forceinline__ bool is_zero(double a) { return (__double_as_longlong(a) << 1) == 0; }

__device__ __forceinline__ double cdiv(double a, double b, double y)
{
    constexpr unsigned lo = 1023 - 400, span = 800;  // biased exponents lo .. lo + span
    const unsigned ea = ((unsigned)__double2hiint(a) >> 20) & 0x7ffu;
    const unsigned eb = ((unsigned)__double2hiint(b) >> 20) & 0x7ffu;
    if (eb - lo > span) return a / b;
    if (is_zero(a)) return __dmul_rn(a, y);
    if (ea - lo > span) return a / b;
    double q = __dmul_rn(a, y);
    q = __fma_rn(__fma_rn(-q, b, a), y, q);
    return __fma_rn(__fma_rn(-q, b, a), y, q);
}

}  // namespace lat
