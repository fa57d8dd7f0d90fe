// Double-precision sine and cosine for the FP64 step kernels.
//
// GB300 issues FP64 at 1/64 of the FP32 rate, and the FP64 step spends most
// of its FP64 instructions in sin/cos of link phases and plaquette angles.
// These functions use a table-driven reduction (P. T. P. Tang, "Table-lookup
// algorithms for elementary functions and their error analysis", ARITH-10,
// 1991):
//
//   x = k*pi/256 + r,  |r| <= pi/512,  j = k mod 512,
//   sin x = sin(a) cos(r) + cos(a) sin(r),  cos x = cos(a) cos(r) - sin(a) sin(r),
//
// with a = j*pi/256 read from a 512-entry table of correctly rounded doubles
// (dtrig_table.inc, written by gen_dtrig_table.py), r from a three-part
// Cody-Waite reduction (Cody & Waite 1980),
// and sin r = r + r^3 (s3 + s5 r^2), cos r - 1 = r^2 (c2 + c4 r^2) with the
// linear factors interpolated at Chebyshev nodes in r^2: their errors are
// below 1.4e-18 relative and 1e-17 absolute for |r| <= pi/512.  The zeros of
// sin and cos are table points, so the two products never cancel fully;
// where the result is about half the table value, the table entry's own
// rounding (half an ulp) doubles in relative terms.  Against 40-digit values
// the error was at most 2.45 ulps (mean 0.4) over 3.7 million samples of
// |x| < 6e4, against glibc at most 3 ulps; CUDA documents 2 ulps for its
// double sin.
//
// FP64 cost: 13 instructions for sin and 15 for sincos, all DFMA/DMUL/DADD.
// The index, the range checks and the table load are integer and memory
// instructions, which leave the FP64 pipe (1/64 of the FP32 rate on GB300)
// to the arithmetic; CUDA's sin spends conversions and compares there too.
//
// Every operation is an explicit IEEE intrinsic, so the results do not
// depend on the translation unit's -fmad setting: the strict and fast FP64
// kernels and the one-pass kernel get the very same doubles.
//
// |x| >= 2^16 (beyond the split's exact range for k) and NaN/Inf go to CUDA's
// sin/cos; |x| < 2^-27 returns sin x = x, cos x = 1.
#pragma once

#include <cuda_runtime.h>

namespace lat {

#include "dtrig_table.inc"

namespace dtrig {

constexpr double kShift = 6755399441055744.0;  // 1.5 * 2^52: adding it rounds to an integer
constexpr int kHiLarge = 0x40f00000;  // high word of 2^16
constexpr int kHiTiny = 0x3e400000;   // high word of 2^-27

// r and the table entry of x (|x| < 2^16)
__device__ __forceinline__ double reduce(double x, double2& a)
{
    const double t = __fma_rn(x, kDtrigInvStep, kShift);
    const double k = __dadd_rn(t, -kShift);
    const int j = __double2loint(t) & (kDtrigEntries - 1);
    double r = __fma_rn(-k, kDtrigStepA, x);
    r = __fma_rn(-k, kDtrigStepB, r);
    r = __fma_rn(-k, kDtrigStepC, r);
    a = __ldg(&kDtrigTable[j]);
    return r;
}

// sin r and cos r - 1
__device__ __forceinline__ void kernels(double r, double& sr, double& cm)
{
    const double r2 = __dmul_rn(r, r);
    sr = __fma_rn(__dmul_rn(r, r2), __fma_rn(r2, kDtrigS5, kDtrigS3), r);
    cm = __dmul_rn(r2, __fma_rn(r2, kDtrigC4, kDtrigC2));
}

}  // namespace dtrig

__device__ __forceinline__ double dsin(double x)
{
    const int hi = __double2hiint(x) & 0x7fffffff;
    if (hi >= dtrig::kHiLarge) return ::sin(x);
    double2 a;
    const double r = dtrig::reduce(x, a);
    double sr, cm;
    dtrig::kernels(r, sr, cm);
    const double s = __fma_rn(a.y, sr, __fma_rn(a.x, cm, a.x));
    return hi < dtrig::kHiTiny ? x : s;
}

__device__ __forceinline__ void dsincos(double x, double* sp, double* cp)
{
    const int hi = __double2hiint(x) & 0x7fffffff;
    if (hi >= dtrig::kHiLarge) {
        ::sincos(x, sp, cp);
        return;
    }
    double2 a;
    const double r = dtrig::reduce(x, a);
    double sr, cm;
    dtrig::kernels(r, sr, cm);
    const double s = __fma_rn(a.y, sr, __fma_rn(a.x, cm, a.x));
    const double c = __fma_rn(-a.x, sr, __fma_rn(a.y, cm, a.y));
    *sp = hi < dtrig::kHiTiny ? x : s;
    *cp = hi < dtrig::kHiTiny ? 1.0 : c;
}

}  // namespace lat
