// Neumann and absorbing boundaries of the Abelian-Higgs lattice
// (evolution.cpp:194-265, 446-691, 1375-1402; ic_w_evolution.cpp has the same).
//
// Neumann: before a step the outer layer of the current level is set from the
// next layer in -- the links copied, phi transported along the link -- in the
// reference's order: y faces (x interior), then x faces (all y), then z faces
// (over x planes i < nz).  Each pass is one kernel; within a pass every thread
// writes boundary sites and reads only sites no thread of the pass writes.
//
// Absorbing (x and y): the outer layer evolves with one-sided first-order
// updates.  Their second time derivatives read the past level of the next
// layer in, which the interior step overwrites, so they are computed into a
// compact buffer (perimeter x evolved z) before the interior step and applied
// after it.
//
// FP64 follows the reference's expressions operation by operation (-fmad=false);
// FP32 evaluates the same expressions in float, and its update is written
// X + (X - X') + dt^2 a like the FP32 interior step.
#include <cuda_runtime.h>

#include "lattice_internal.cuh"

namespace lat {
namespace {

struct BGeom {
    int nx, ny, nz, syz;
    int loz, hiz;  // evolved z range
    int P;         // perimeter sites of an xy plane: 2(nx + ny) - 4
};

__device__ __forceinline__ int at(const BGeom& g, int i, int j, int k) { return (i * g.ny + j) * g.nz + k; }

template <class T>
struct Lv {  // one level: phi_re, phi_im, theta_x, theta_y, theta_z
    T* v[5];
};

// ---------------------------------------------------------------------------
// Neumann
// ---------------------------------------------------------------------------
// boundary b0 from interior i0 (low face), boundary b1 from interior i1 (high
// face), along axis mu (evolution.cpp:202-208)
template <class T>
__device__ __forceinline__ void neumann_pair(const Lv<T>& L, int mu, int b0, int i0, int b1, int i1)
{
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        L.v[2 + m][b0] = L.v[2 + m][i0];
        L.v[2 + m][b1] = L.v[2 + m][i1];
    }
    const T t0 = L.v[2 + mu][b0], t1 = L.v[2 + mu][i1];
    const T c0 = cos(t0), s0 = sin(t0), c1 = cos(t1), s1 = sin(t1);
    const T p0 = L.v[0][i0], q0 = L.v[1][i0], p1 = L.v[0][i1], q1 = L.v[1][i1];
    // comp 0 (c = +1, partner comp 1); comp 1 (c = -1, partner comp 0)
    L.v[0][b0] = c0 * p0 + (T)1 * s0 * q0;
    L.v[0][b1] = c1 * p1 - (T)1 * s1 * q1;
    L.v[1][b0] = c0 * q0 + (T)-1 * s0 * p0;
    L.v[1][b1] = c1 * q1 - (T)-1 * s1 * p1;
}

template <class T>
__global__ void neumann_y_kernel(const BGeom g, const Lv<T> L)
{
    const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int k = g.loz + (int)blockIdx.y;
    if (i >= g.nx - 1 || k >= g.hiz) return;
    neumann_pair(L, 1, at(g, i, 0, k), at(g, i, 1, k), at(g, i, g.ny - 1, k), at(g, i, g.ny - 2, k));
}

template <class T>
__global__ void neumann_x_kernel(const BGeom g, const Lv<T> L)
{
    const int j = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int k = g.loz + (int)blockIdx.y;
    if (j >= g.ny || k >= g.hiz) return;
    neumann_pair(L, 0, at(g, 0, j, k), at(g, 1, j, k), at(g, g.nx - 1, j, k), at(g, g.nx - 2, j, k));
}

template <class T>
__global__ void neumann_z_kernel(const BGeom g, const Lv<T> L, int ni)
{
    const int j = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int i = (int)blockIdx.y;
    if (j >= g.ny || i >= ni) return;
    neumann_pair(L, 2, at(g, i, j, 0), at(g, i, j, 1), at(g, i, j, g.nz - 1), at(g, i, j, g.nz - 2));
}

// Moore (mooreEvol.cpp:114-160): phi_a transported along q_a * theta;
// components phi1 (0, 1), phi2 (2, 3), theta (4, 5, 6)
template <class T>
struct Lv7 {
    T* v[7];
};

template <class T>
__device__ __forceinline__ void neumann_pair_moore(const Lv7<T>& L, T q1, T q2, int mu, int b0, int i0, int b1, int i1)
{
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        L.v[4 + m][b0] = L.v[4 + m][i0];
        L.v[4 + m][b1] = L.v[4 + m][i1];
    }
    const T t0 = L.v[4 + mu][b0], t1 = L.v[4 + mu][i1];
#pragma unroll
    for (int a = 0; a < 2; ++a) {
        const T q = a == 0 ? q1 : q2;
        const T c0 = cos(q * t0), s0 = sin(q * t0), c1 = cos(q * t1), s1 = sin(q * t1);
        const T p0 = L.v[2 * a][i0], r0 = L.v[2 * a + 1][i0], p1 = L.v[2 * a][i1], r1 = L.v[2 * a + 1][i1];
        L.v[2 * a][b0] = c0 * p0 + (T)1 * s0 * r0;
        L.v[2 * a][b1] = c1 * p1 - (T)1 * s1 * r1;
        L.v[2 * a + 1][b0] = c0 * r0 + (T)-1 * s0 * p0;
        L.v[2 * a + 1][b1] = c1 * r1 - (T)-1 * s1 * p1;
    }
}

template <class T>
__global__ void neumann_y_moore_kernel(const BGeom g, const Lv7<T> L, T q1, T q2)
{
    const int i = 1 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int k = g.loz + (int)blockIdx.y;
    if (i >= g.nx - 1 || k >= g.hiz) return;
    neumann_pair_moore(L, q1, q2, 1, at(g, i, 0, k), at(g, i, 1, k), at(g, i, g.ny - 1, k), at(g, i, g.ny - 2, k));
}

template <class T>
__global__ void neumann_x_moore_kernel(const BGeom g, const Lv7<T> L, T q1, T q2)
{
    const int j = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int k = g.loz + (int)blockIdx.y;
    if (j >= g.ny || k >= g.hiz) return;
    neumann_pair_moore(L, q1, q2, 0, at(g, 0, j, k), at(g, 1, j, k), at(g, g.nx - 1, j, k), at(g, g.nx - 2, j, k));
}

// ---------------------------------------------------------------------------
// absorbing x/y layer (evolution.cpp:446-691)
// ---------------------------------------------------------------------------
// covariant second difference of phi component `comp` along mu at s
template <class T>
__device__ __forceinline__ T cov2(const Lv<T>& A, int comp, int mu, int s, int sp, int sm, T d)
{
    const int oc = comp ^ 1;
    const T cc = comp == 0 ? (T)1 : (T)-1;
    return (cos(A.v[2 + mu][s]) * A.v[comp][sp] + cc * sin(A.v[2 + mu][s]) * A.v[oc][sp] - (T)2 * A.v[comp][s] +
            cos(A.v[2 + mu][sm]) * A.v[comp][sm] - cc * sin(A.v[2 + mu][sm]) * A.v[oc][sm]) /
           (d * d);
}

// one-sided time-space difference at the low face: s0 on the face, s1 = s0 + mu
template <class T>
__device__ __forceinline__ T near_ts(const Lv<T>& A, const Lv<T>& B, int comp, int mu, int s0, int s1, T dt, T d)
{
    const int oc = comp ^ 1;
    const T cc = comp == 0 ? (T)1 : (T)-1;
    return (cos(A.v[2 + mu][s0]) * A.v[comp][s1] + cc * sin(A.v[2 + mu][s0]) * A.v[oc][s1] - A.v[comp][s0] -
            cos(B.v[2 + mu][s0]) * B.v[comp][s1] - cc * sin(B.v[2 + mu][s0]) * B.v[oc][s1] + B.v[comp][s0]) /
           (dt * d);
}

// at the high face: s0 on the face, s1 = s0 - mu; the past cos reads the link
// at sc (s1, except the (nx-1, ny-1) corner's x term, evolution.cpp:656)
template <class T>
__device__ __forceinline__ T far_ts(const Lv<T>& A, const Lv<T>& B, int comp, int mu, int s0, int s1, int sc, T dt,
                                    T d)
{
    const int oc = comp ^ 1;
    const T cc = comp == 0 ? (T)1 : (T)-1;
    return (A.v[comp][s0] - cos(A.v[2 + mu][s1]) * A.v[comp][s1] + cc * sin(A.v[2 + mu][s1]) * A.v[oc][s1] -
            B.v[comp][s0] + cos(B.v[2 + mu][sc]) * B.v[comp][s1] - cc * sin(B.v[2 + mu][s1]) * B.v[oc][s1]) /
           (dt * d);
}

template <class T>
__device__ __forceinline__ T th2(const Lv<T>& A, int m, int sp, int s, int sm, T d)
{
    return (A.v[2 + m][sp] - (T)2 * A.v[2 + m][s] + A.v[2 + m][sm]) / (d * d);
}

template <class T>
__device__ __forceinline__ T th_near(const Lv<T>& A, const Lv<T>& B, int m, int s0, int s1, T dt, T d)
{
    return (A.v[2 + m][s1] - A.v[2 + m][s0] - B.v[2 + m][s1] + B.v[2 + m][s0]) / (dt * d);
}

template <class T>
__device__ __forceinline__ T th_far(const Lv<T>& A, const Lv<T>& B, int m, int s0, int s1, T dt, T d)
{
    return (A.v[2 + m][s0] - A.v[2 + m][s1] - B.v[2 + m][s0] + B.v[2 + m][s1]) / (dt * d);
}

// perimeter position p -> (i, j): x = 0 column, x = nx-1 column, then the
// y = 0 and y = ny-1 rows without their corners
__device__ __forceinline__ void perimeter(const BGeom& g, int p, int& i, int& j)
{
    if (p < g.ny) {
        i = 0;
        j = p;
    } else if (p < 2 * g.ny) {
        i = g.nx - 1;
        j = p - g.ny;
    } else if (p < 2 * g.ny + g.nx - 2) {
        i = p - 2 * g.ny + 1;
        j = 0;
    } else {
        i = p - (2 * g.ny + g.nx - 2) + 1;
        j = g.ny - 1;
    }
}

struct BSpacing {
    double dx, dy, dz, dt;
};

template <class T>
__global__ void absorb_tt_kernel(const BGeom g, const Lv<T> A, const Lv<T> B, T* __restrict__ tt, const BSpacing sp)
{
    const int p = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int k = g.loz + (int)blockIdx.y;
    if (p >= g.P || k >= g.hiz) return;
    const T dx = (T)sp.dx, dy = (T)sp.dy, dz = (T)sp.dz, dt = (T)sp.dt;
    const int kp = (k + 1) % g.nz, km = (k - 1 + g.nz) % g.nz;
    int i, j;
    perimeter(g, p, i, j);
    const int s = at(g, i, j, k), szp = at(g, i, j, kp), szm = at(g, i, j, km);
    const int nx1 = g.nx - 1, ny1 = g.ny - 1;
    T r[5];
    const bool xface = i == 0 || i == nx1, yface = j == 0 || j == ny1;
    if (xface && !yface) {  // evolution.cpp:447-509
        const int syp = at(g, i, j + 1, k), sym = at(g, i, j - 1, k);
        const int s1 = at(g, i == 0 ? 1 : nx1 - 1, j, k);
        for (int c = 0; c < 2; ++c) {
            const T yy = cov2(A, c, 1, s, syp, sym, dy), zz = cov2(A, c, 2, s, szp, szm, dz);
            const T tx = i == 0 ? near_ts(A, B, c, 0, s, s1, dt, dx) : far_ts(A, B, c, 0, s, s1, s1, dt, dx);
            r[c] = (i == 0 ? tx : -tx) + (T)0.5 * (yy + zz);
        }
        for (int m = 0; m < 3; ++m) {
            const T yy = th2(A, m, syp, s, sym, dy), zz = th2(A, m, szp, s, szm, dz);
            const T tx = i == 0 ? th_near(A, B, m, s, s1, dt, dx) : th_far(A, B, m, s, s1, dt, dx);
            r[2 + m] = (i == 0 ? tx : -tx) + (T)0.5 * (yy + zz);
        }
    } else if (yface && !xface) {  // :511-573
        const int sxp = at(g, i + 1, j, k), sxm = at(g, i - 1, j, k);
        const int s1 = at(g, i, j == 0 ? 1 : ny1 - 1, k);
        for (int c = 0; c < 2; ++c) {
            const T xx = cov2(A, c, 0, s, sxp, sxm, dx), zz = cov2(A, c, 2, s, szp, szm, dz);
            const T ty = j == 0 ? near_ts(A, B, c, 1, s, s1, dt, dy) : far_ts(A, B, c, 1, s, s1, s1, dt, dy);
            r[c] = (j == 0 ? ty : -ty) + (T)0.5 * (xx + zz);
        }
        for (int m = 0; m < 3; ++m) {
            const T xx = th2(A, m, sxp, s, sxm, dx), zz = th2(A, m, szp, s, szm, dz);
            const T ty = j == 0 ? th_near(A, B, m, s, s1, dt, dy) : th_far(A, B, m, s, s1, dt, dy);
            r[2 + m] = (j == 0 ? ty : -ty) + (T)0.5 * (xx + zz);
        }
    } else {  // corners, :575-689
        const bool hx = i == nx1, hy = j == ny1;
        const int sx1 = at(g, hx ? nx1 - 1 : 1, j, k), sy1 = at(g, i, hy ? ny1 - 1 : 1, k);
        for (int c = 0; c < 2; ++c) {
            const T zz = cov2(A, c, 2, s, szp, szm, dz);
            const T tx = hx ? far_ts(A, B, c, 0, s, sx1, hy ? s : sx1, dt, dx) : near_ts(A, B, c, 0, s, sx1, dt, dx);
            const T ty = hy ? far_ts(A, B, c, 1, s, sy1, sy1, dt, dy) : near_ts(A, B, c, 1, s, sy1, dt, dy);
            if (!hx && !hy) r[c] = (zz + (T)2 * (tx + ty)) / (T)3;
            else if (!hx) r[c] = (zz + (T)2 * (tx - ty)) / (T)3;
            else if (!hy) r[c] = (zz - (T)2 * (tx - ty)) / (T)3;
            else r[c] = (zz - (T)2 * (tx + ty)) / (T)3;
        }
        for (int m = 0; m < 3; ++m) {
            const T zz = th2(A, m, szp, s, szm, dz);
            const T tx = hx ? th_far(A, B, m, s, sx1, dt, dx) : th_near(A, B, m, s, sx1, dt, dx);
            const T ty = hy ? th_far(A, B, m, s, sy1, dt, dy) : th_near(A, B, m, s, sy1, dt, dy);
            if (!hx && !hy) r[2 + m] = (zz + (T)2 * (tx + ty)) / (T)3;
            else if (!hx) r[2 + m] = (zz + (T)2 * (tx - ty)) / (T)3;
            else if (!hy) r[2 + m] = (zz - (T)2 * (tx - ty)) / (T)3;
            else r[2 + m] = (zz - (T)2 * (tx + ty)) / (T)3;
        }
    }
    const size_t slot = (size_t)(k - g.loz) * g.P + p, stride = (size_t)(g.hiz - g.loz) * g.P;
#pragma unroll
    for (int c = 0; c < 5; ++c) tt[c * stride + slot] = r[c];
}

// the outer x/y layer's update (evolution.cpp:1375-1402)
template <class T>
__global__ void absorb_update_kernel(const BGeom g, const Lv<T> A, const Lv<T> B, const T* __restrict__ tt, const double dt2)
{
    const int p = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    const int k = g.loz + (int)blockIdx.y;
    if (p >= g.P || k >= g.hiz) return;
    int i, j;
    perimeter(g, p, i, j);
    const int s = at(g, i, j, k);
    const size_t slot = (size_t)(k - g.loz) * g.P + p, stride = (size_t)(g.hiz - g.loz) * g.P;
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        const T a = tt[c * stride + slot];
        if constexpr (sizeof(T) == 8) B.v[c][s] = (T)2 * A.v[c][s] - B.v[c][s] + (T)dt2 * a;
        else B.v[c][s] = A.v[c][s] + (A.v[c][s] - B.v[c][s]) + (T)dt2 * a;
    }
}

}  // namespace

namespace {

BGeom bgeom(const Geom& g)
{
    BGeom b;
    b.nx = g.nx;
    b.ny = g.ny;
    b.nz = g.nz;
    b.syz = g.syz;
    b.loz = g.loz;
    b.hiz = g.hiz;
    b.P = 2 * (g.nx + g.ny) - 4;
    return b;
}

template <class T>
Lv<T> level(void* const* slots)
{
    Lv<T> L;
    for (int c = 0; c < 5; ++c) L.v[c] = (T*)slots[c];
    return L;
}

constexpr int BT = 128;

template <class T>
cudaError_t neumann_moore_t(const Geom& g, int kxy, double q1, double q2, void* const* now, cudaStream_t st,
                            int* launches)
{
    const BGeom b = bgeom(g);
    Lv7<T> L;
    for (int c = 0; c < 7; ++c) L.v[c] = (T*)now[c];
    const unsigned zs = (unsigned)(g.hiz - g.loz);
    if (kxy == LAT_BC_NEUMANN && zs > 0) {
        neumann_y_moore_kernel<T><<<dim3((unsigned)((g.nx - 2 + BT - 1) / BT), zs), BT, 0, st>>>(b, L, (T)q1, (T)q2);
        neumann_x_moore_kernel<T><<<dim3((unsigned)((g.ny + BT - 1) / BT), zs), BT, 0, st>>>(b, L, (T)q1, (T)q2);
        *launches += 2;
    }
    return cudaGetLastError();
}

template <class T>
cudaError_t neumann_t(const Geom& g, int kxy, int kz, void* const* now, cudaStream_t st, int* launches)
{
    const BGeom b = bgeom(g);
    const Lv<T> L = level<T>(now);
    const unsigned zs = (unsigned)(g.hiz - g.loz);
    if (kxy == LAT_BC_NEUMANN && zs > 0) {
        neumann_y_kernel<T><<<dim3((unsigned)((g.nx - 2 + BT - 1) / BT), zs), BT, 0, st>>>(b, L);
        neumann_x_kernel<T><<<dim3((unsigned)((g.ny + BT - 1) / BT), zs), BT, 0, st>>>(b, L);
        *launches += 2;
    }
    if (kz == LAT_BC_NEUMANN) {
        const int ni = g.nz < g.nx ? g.nz : g.nx;
        neumann_z_kernel<T><<<dim3((unsigned)((g.ny + BT - 1) / BT), (unsigned)ni), BT, 0, st>>>(b, L, ni);
        *launches += 1;
    }
    return cudaGetLastError();
}

}  // namespace

size_t absorb_tt_bytes(const Geom& g, int elem)
{
    return (size_t)elem * 5 * (size_t)(2 * (g.nx + g.ny) - 4) * (size_t)(g.hiz - g.loz);
}

cudaError_t launch_neumann(const Geom& g, int model, double q1, double q2, int kxy, int kz, int elem, void* const* now,
                           cudaStream_t st, int* launches)
{
    if (model == LAT_MODEL_MOORE)
        return elem == 8 ? neumann_moore_t<double>(g, kxy, q1, q2, now, st, launches)
                         : neumann_moore_t<float>(g, kxy, q1, q2, now, st, launches);
    return elem == 8 ? neumann_t<double>(g, kxy, kz, now, st, launches)
                     : neumann_t<float>(g, kxy, kz, now, st, launches);
}

cudaError_t launch_absorb_tt(const Geom& g, int elem, void* const* now, void* const* past, void* tt, double dx,
                             double dy, double dz, double dt, cudaStream_t st)
{
    const BGeom b = bgeom(g);
    const BSpacing sp{dx, dy, dz, dt};
    const dim3 grid((unsigned)((b.P + BT - 1) / BT), (unsigned)(g.hiz - g.loz));
    if (elem == 8) absorb_tt_kernel<double><<<grid, BT, 0, st>>>(b, level<double>(now), level<double>(past), (double*)tt, sp);
    else absorb_tt_kernel<float><<<grid, BT, 0, st>>>(b, level<float>(now), level<float>(past), (float*)tt, sp);
    return cudaGetLastError();
}

cudaError_t launch_absorb_update(const Geom& g, int elem, void* const* now, void* const* past, const void* tt, double dt2,
                                 cudaStream_t st)
{
    const BGeom b = bgeom(g);
    const dim3 grid((unsigned)((b.P + BT - 1) / BT), (unsigned)(g.hiz - g.loz));
    if (elem == 8)
        absorb_update_kernel<double><<<grid, BT, 0, st>>>(b, level<double>(now), level<double>(past), (const double*)tt, dt2);
    else
        absorb_update_kernel<float><<<grid, BT, 0, st>>>(b, level<float>(now), level<float>(past), (const float*)tt, dt2);
    return cudaGetLastError();
}

}  // namespace lat
