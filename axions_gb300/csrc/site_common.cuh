// Device helpers shared by the site kernels.
#pragma once

#include "dtrig.cuh"
#include "fp64_exact.cuh"
#include "lattice_internal.cuh"

namespace lat {

// Transcendentals by precision.  The FP64 path uses the table-driven sine and
// cosine of dtrig.cuh (about two ulps, 15-17 FP64 instructions); the FP32 path
// the reduced hardware approximations below.
template <class T>
struct Trig;
template <>
struct Trig<double> {
    static __device__ __forceinline__ double sin(double x) { return dsin(x); }
    static __device__ __forceinline__ double cos(double x)
    {
        double s, c;
        dsincos(x, &s, &c);
        return c;
    }
    static __device__ __forceinline__ void sincos(double x, double* s, double* c) { dsincos(x, s, c); }
};
// FP32: the argument is reduced to [-pi, pi] by Cody-Waite with 2*pi split in
// two parts (Cody & Waite 1980; 6.28125 has 8 significant bits, so k*6.28125 is
// exact for |k| < 2^16, i.e. |x| < 4e5), then the hardware approximations
// __sinf/__cosf are used (documented absolute error 2^-21.41 on [-pi, pi]).
// That error is below the rounding an FP32 phase or plaquette angle already
// carries (|theta| up to ~10 gives ~1e-6), and it costs a few instructions
// instead of a full-range software sine.
template <>
struct Trig<float> {
    static __device__ __forceinline__ float reduce(float x)
    {
        const float k = rintf(x * 0.159154943091895336f);  // x / (2 pi)
        const float r = fmaf(-k, 6.28125f, x);
        return fmaf(-k, 1.93530717958647692e-3f, r);      // 2 pi - 6.28125
    }
    static __device__ __forceinline__ float sin(float x) { return __sinf(reduce(x)); }
    static __device__ __forceinline__ float cos(float x) { return __cosf(reduce(x)); }
    static __device__ __forceinline__ void sincos(float x, float* s, float* c) { __sincosf(reduce(x), s, c); }
};

// a / b.  FP64: the IEEE quotient (the reference's rounding) by cdiv from the
// host reciprocal inv_b = RN(1/b), five FP64 instructions; FP32 multiplies by
// the reciprocal.
template <class T>
__device__ __forceinline__ T qdiv(T a, T b, T inv_b)
{
    if constexpr (sizeof(T) == 8) return cdiv(a, b, inv_b);
    else return a * inv_b;
}

// Leapfrog update X^{n+1} from X^n, X^{n-1} and the acceleration.
// FP64 keeps the reference's expression 2*X - Xp + dt^2*a
// (mpi_evolution.cpp:432).  FP32 uses X + (X - Xp) + dt^2*a: the difference
// of two consecutive levels is exact in floating point (they are within a
// factor two of each other), so only the velocity term is rounded.
template <class T>
__device__ __forceinline__ T leapfrog(T xn, T xp, T dt2, T acc)
{
    if constexpr (sizeof(T) == 8) return 2 * xn - xp + dt2 * acc;
    else return xn + (xn - xp) + dt2 * acc;
}

// Periodic / fixed neighbour offsets of one site.
struct Nbr {
    int s, xp, xm, yp, ym, zp, zm;  // xp = offset to i+1 etc.
};

__device__ __forceinline__ Nbr make_nbr(const Geom& g, int i, int j, int k)
{
    Nbr n;
    n.s = (i * g.ny + j) * g.nz + k;
    n.xp = (i + 1 == g.nx) ? -(g.nx - 1) * g.syz : g.syz;
    n.xm = (i == 0) ? (g.nx - 1) * g.syz : -g.syz;
    n.yp = (j + 1 == g.ny) ? -(g.ny - 1) * g.nz : g.nz;
    n.ym = (j == 0) ? (g.ny - 1) * g.nz : -g.nz;
    n.zp = (k + 1 == g.nz) ? -(g.nz - 1) : 1;
    n.zm = (k == 0) ? (g.nz - 1) : -1;
    return n;
}

// Sum two doubles over the block (BLOCK threads) and write them to
// partials[2*b], partials[2*b+1].  Fixed tree: deterministic for a fixed grid.
__device__ __forceinline__ void block_sum2_store(double a, double b, double* partials)
{
    __shared__ double red[2][BLOCK / 32];
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    if ((tid & 31) == 0) {
        red[0][tid >> 5] = a;
        red[1][tid >> 5] = b;
    }
    __syncthreads();
    if (tid == 0) {
        double sa = 0, sb = 0;
        for (int w = 0; w < BLOCK / 32; ++w) {
            sa += red[0][w];
            sb += red[1][w];
        }
        const int blk = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
        partials[2 * blk] = sa;
        partials[2 * blk + 1] = sb;
    }
}

}  // namespace lat
