// String detection on the "now" level of one scalar.
//
// 1. Bilinear face crossings (mpi_evolution.cpp:536-789, evolution.cpp:749-1004):
//    each site checks its three positive faces; each face's bilinear
//    interpolation of (Re phi, Im phi) is inverted through a quadratic.  The
//    reference appends roots to per-rank vectors; here a count pass, a scan of
//    block totals and a write pass put every crossing at its position in the
//    reference's order (sites in linear order; z-, y-, x-directed face; "+"
//    root before "-" root) with no sort.  All arithmetic is double precision in
//    the reference's order and this file is compiled with -fmad=false, so the
//    output is bit-identical to the reference on identical fields.
// 2. Plaquette winding (new, defined in include/lattice_gpu.h).
#include "lattice_internal.cuh"

namespace lat {

namespace {

constexpr int DB = 256;  // sites (threads) per detection block

struct Roots {
    int n;
    double s1[2], s2[2];
};

// One face: v00 at (u,w), v10 at (u+du,w), v01 at (u,w+dw), v11 at (u+du,w+dw).
__device__ __forceinline__ Roots face_roots(const double v00[2], const double v10[2], const double v01[2],
                                            const double v11[2], double u, double w, double du, double dw)
{
    double coeff1[2], coeff2[2], coeff3[2], coeff4[2];
#pragma unroll
    for (int comp = 0; comp < 2; ++comp) {
        coeff1[comp] = v11[comp] - v10[comp] - v01[comp] + v00[comp];
        coeff2[comp] = (w + dw) * (v10[comp] - v00[comp]) + w * (v01[comp] - v11[comp]);
        coeff3[comp] = (u + du) * (v01[comp] - v00[comp]) + u * (v10[comp] - v11[comp]);
        coeff4[comp] = (u + du) * ((w + dw) * v00[comp] - w * v01[comp]) - u * ((w + dw) * v10[comp] - w * v11[comp]);
    }
    const double a = coeff1[1] * coeff3[0] - coeff1[0] * coeff3[1];
    const double b = coeff1[1] * coeff4[0] + coeff2[1] * coeff3[0] - coeff1[0] * coeff4[1] - coeff2[0] * coeff3[1];
    const double c = coeff2[1] * coeff4[0] - coeff2[0] * coeff4[1];
    const double discrim = b * b - 4 * a * c;
    Roots r;
    r.n = 0;
    if (a == 0) {
        if (b != 0) {
            const double sol2 = -c / b;
            if (sol2 >= w && sol2 <= w + dw) {
                const double sol1 = -(coeff3[0] * sol2 + coeff4[0]) / (coeff1[0] * sol2 + coeff2[0]);
                if (sol1 >= u && sol1 <= u + du) { r.s1[r.n] = sol1; r.s2[r.n] = sol2; r.n++; }
            }
        }
    } else if (discrim >= 0) {
        const double sq = sqrt(discrim);
        double sol2 = (-b + sq) / (2 * a);
        if (sol2 >= w && sol2 <= w + dw) {
            const double sol1 = -(coeff3[0] * sol2 + coeff4[0]) / (coeff1[0] * sol2 + coeff2[0]);
            if (sol1 >= u && sol1 <= u + du) { r.s1[r.n] = sol1; r.s2[r.n] = sol2; r.n++; }
        }
        sol2 = (-b - sq) / (2 * a);
        if (sol2 >= w && sol2 <= w + dw) {
            const double sol1 = -(coeff3[0] * sol2 + coeff4[0]) / (coeff1[0] * sol2 + coeff2[0]);
            if (sol1 >= u && sol1 <= u + du) { r.s1[r.n] = sol1; r.s2[r.n] = sol2; r.n++; }
        }
    }
    return r;
}

struct SiteRoots {
    Roots zf, yf, xf;
    double x, y, z;
    int total;
};

template <class T>
__device__ __forceinline__ bool site_roots(const DetectArgs& a, const T* __restrict__ re, const T* __restrict__ im,
                                           long long sl, SiteRoots& out)
{
    const long long N = (long long)a.nx * a.syz;
    if (sl >= N) return false;
    const int s = (int)sl;
    const int i = s / a.syz;
    const int rem = s - i * a.syz;
    const int j = rem / a.nz;
    const int k = rem - j * a.nz;
    if (i < a.lox || i >= a.hix || j < a.loy || j >= a.hiy || k < a.loz || k >= a.hiz) return false;
    const int oxp = (i + 1 == a.nx) ? -(a.nx - 1) * a.syz : a.syz;
    const int oyp = (j + 1 == a.ny) ? -(a.ny - 1) * a.nz : a.nz;
    const int ozp = (k + 1 == a.nz) ? -(a.nz - 1) : 1;
    double v0[2], vx[2], vy[2], vz[2], vxy[2], vxz[2], vyz[2];
    v0[0] = (double)re[s];           v0[1] = (double)im[s];
    vx[0] = (double)re[s + oxp];     vx[1] = (double)im[s + oxp];
    vy[0] = (double)re[s + oyp];     vy[1] = (double)im[s + oyp];
    vz[0] = (double)re[s + ozp];     vz[1] = (double)im[s + ozp];
    vxy[0] = (double)re[s + oxp + oyp]; vxy[1] = (double)im[s + oxp + oyp];
    vxz[0] = (double)re[s + oxp + ozp]; vxz[1] = (double)im[s + oxp + ozp];
    vyz[0] = (double)re[s + oyp + ozp]; vyz[1] = (double)im[s + oyp + ozp];
    // physical coordinates (mpi_evolution.cpp:547-549)
    out.x = (double)(i - a.x0) * a.dx;
    out.y = (double)(j - a.y0) * a.dy;
    out.z = (double)(k - a.z0) * a.dz;
    out.zf = face_roots(v0, vx, vy, vxy, out.x, out.y, a.dx, a.dy);   // z-directed face (x,y)
    out.yf = face_roots(v0, vx, vz, vxz, out.x, out.z, a.dx, a.dz);   // y-directed face (x,z)
    out.xf = face_roots(v0, vy, vz, vyz, out.y, out.z, a.dy, a.dz);   // x-directed face (y,z)
    out.total = out.zf.n + out.yf.n + out.xf.n;
    return true;
}

__device__ __forceinline__ int block_exclusive_scan(int v, int* total)
{
    __shared__ int warp_sums[DB / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_sums[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        int ws = (lane < DB / 32) ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, ws, o);
            if (lane >= o) ws += t;
        }
        if (lane < DB / 32) warp_sums[lane] = ws;  // inclusive over warps
    }
    __syncthreads();
    const int warp_base = wid ? warp_sums[wid - 1] : 0;
    if (total) *total = warp_sums[DB / 32 - 1];
    return warp_base + incl - v;
}

template <class T>
__global__ void __launch_bounds__(DB) detect_count_kernel(const DetectArgs a, const T* __restrict__ re,
                                                          const T* __restrict__ im, long long* block_totals)
{
    SiteRoots r;
    const long long sl = (long long)blockIdx.x * DB + threadIdx.x;
    const int cnt = site_roots<T>(a, re, im, sl, r) ? r.total : 0;
    int total;
    block_exclusive_scan(cnt, &total);
    if (threadIdx.x == 0) block_totals[blockIdx.x] = total;
}

template <class T>
__global__ void __launch_bounds__(DB) detect_write_kernel(const DetectArgs a, const T* __restrict__ re,
                                                          const T* __restrict__ im, const long long* block_offsets,
                                                          double* xyz, long long cap)
{
    SiteRoots r;
    const long long sl = (long long)blockIdx.x * DB + threadIdx.x;
    const bool ok = site_roots<T>(a, re, im, sl, r);
    const int cnt = ok ? r.total : 0;
    long long pos = block_offsets[blockIdx.x] + block_exclusive_scan(cnt, nullptr);
    if (!ok) return;
    auto emit = [&](double x, double y, double z) {
        if (pos < cap) {
            xyz[3 * pos + 0] = x;
            xyz[3 * pos + 1] = y;
            xyz[3 * pos + 2] = z;
        }
        ++pos;
    };
    for (int q = 0; q < r.zf.n; ++q) emit(r.zf.s1[q], r.zf.s2[q], r.z);
    for (int q = 0; q < r.yf.n; ++q) emit(r.yf.s1[q], r.y, r.yf.s2[q]);
    for (int q = 0; q < r.xf.n; ++q) emit(r.x, r.xf.s1[q], r.xf.s2[q]);
}

// Exclusive scan of block totals in place (one block); *total = grand total.
__global__ void __launch_bounds__(1024) scan_totals_kernel(long long* v, int n, long long* total)
{
    __shared__ long long chunk_sum[1024];
    const int t = threadIdx.x;
    const int per = (n + 1023) / 1024;
    const int b = t * per, e = min(n, b + per);
    long long s = 0;
    for (int q = b; q < e; ++q) s += v[q];
    chunk_sum[t] = s;
    __syncthreads();
    if (t == 0) {
        long long run = 0;
        for (int q = 0; q < 1024; ++q) {
            const long long c = chunk_sum[q];
            chunk_sum[q] = run;
            run += c;
        }
        *total = run;
    }
    __syncthreads();
    long long run = chunk_sum[t];
    for (int q = b; q < e; ++q) {
        const long long c = v[q];
        v[q] = run;
        run += c;
    }
}

// ---------------------------------------------------------------------------
// plaquette winding
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ int edge_cross(T ax, T ay, T bx, T by)
{
    T cr;
    if constexpr (sizeof(T) == 8) cr = __dsub_rn(__dmul_rn(ax, by), __dmul_rn(ay, bx));
    else cr = __fsub_rn(__fmul_rn(ax, by), __fmul_rn(ay, bx));
    if (ay <= 0) {
        if (by > 0 && cr > 0) return 1;
    } else {
        if (by <= 0 && cr < 0) return -1;
    }
    return 0;
}

template <class T>
__global__ void __launch_bounds__(DB) winding_kernel(const DetectArgs a, int open_axes, const T* __restrict__ re,
                                                     const T* __restrict__ im, int8_t* out,
                                                     unsigned long long* abs_sum)
{
    const long long N = (long long)a.nx * a.syz;
    const long long sl = (long long)blockIdx.x * DB + threadIdx.x;
    int tot = 0;
    if (sl < N) {
        const int s = (int)sl;
        const int i = s / a.syz;
        const int rem = s - i * a.syz;
        const int j = rem / a.nz;
        const int k = rem - j * a.nz;
        const int oxp = (i + 1 == a.nx) ? -(a.nx - 1) * a.syz : a.syz;
        const int oyp = (j + 1 == a.ny) ? -(a.ny - 1) * a.nz : a.nz;
        const int ozp = (k + 1 == a.nz) ? -(a.nz - 1) : 1;
        // corners counter-clockwise about +d (include/lattice_gpu.h)
        const int cs[3][4] = {{s, s + oyp, s + oyp + ozp, s + ozp},
                              {s, s + ozp, s + ozp + oxp, s + oxp},
                              {s, s + oxp, s + oxp + oyp, s + oyp}};
        // a face is valid unless it wraps around a non-periodic axis (bit 0: x/y, bit 1: z)
        const bool xin = !(open_axes & 1) || i + 1 < a.nx, yin = !(open_axes & 1) || j + 1 < a.ny;
        const bool zin = !(open_axes & 2) || k + 1 < a.nz;
        const bool valid[3] = {yin && zin, zin && xin, xin && yin};
        T vr[3][4], vi[3][4];
#pragma unroll
        for (int d = 0; d < 3; ++d)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                vr[d][e] = re[cs[d][e]];
                vi[d][e] = im[cs[d][e]];
            }
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            int w = 0;
            if (valid[d]) {
#pragma unroll
                for (int e = 0; e < 4; ++e) w += edge_cross<T>(vr[d][e], vi[d][e], vr[d][(e + 1) & 3], vi[d][(e + 1) & 3]);
            }
            if (out) out[(long long)d * N + s] = (int8_t)w;
            tot += w < 0 ? -w : w;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) tot += __shfl_down_sync(0xffffffffu, tot, o);
    __shared__ int ws[DB / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = tot;
    __syncthreads();
    if (threadIdx.x == 0) {
        int b = 0;
        for (int w = 0; w < DB / 32; ++w) b += ws[w];
        if (b) atomicAdd(abs_sum, (unsigned long long)b);
    }
}

inline unsigned nblocks_of(const DetectArgs& a) { return (unsigned)(((long long)a.nx * a.syz + DB - 1) / DB); }

}  // namespace

int detect_block_sites() { return DB; }

cudaError_t launch_detect_count_f64(const DetectArgs& a, const double* re, const double* im, long long* bt, int nb,
                                    cudaStream_t st)
{
    detect_count_kernel<double><<<nb, DB, 0, st>>>(a, re, im, bt);
    return cudaGetLastError();
}
cudaError_t launch_detect_count_f32(const DetectArgs& a, const float* re, const float* im, long long* bt, int nb,
                                    cudaStream_t st)
{
    detect_count_kernel<float><<<nb, DB, 0, st>>>(a, re, im, bt);
    return cudaGetLastError();
}
cudaError_t launch_scan_totals(long long* bt, int nb, long long* total, cudaStream_t st)
{
    scan_totals_kernel<<<1, 1024, 0, st>>>(bt, nb, total);
    return cudaGetLastError();
}
cudaError_t launch_detect_write_f64(const DetectArgs& a, const double* re, const double* im, const long long* bo, int nb,
                                    double* xyz, long long cap, cudaStream_t st)
{
    detect_write_kernel<double><<<nb, DB, 0, st>>>(a, re, im, bo, xyz, cap);
    return cudaGetLastError();
}
cudaError_t launch_detect_write_f32(const DetectArgs& a, const float* re, const float* im, const long long* bo, int nb,
                                    double* xyz, long long cap, cudaStream_t st)
{
    detect_write_kernel<float><<<nb, DB, 0, st>>>(a, re, im, bo, xyz, cap);
    return cudaGetLastError();
}
cudaError_t launch_winding_f64(const DetectArgs& a, int open_axes, const double* re, const double* im, int8_t* out,
                               unsigned long long* abs_sum, cudaStream_t st)
{
    winding_kernel<double><<<nblocks_of(a), DB, 0, st>>>(a, open_axes, re, im, out, abs_sum);
    return cudaGetLastError();
}
cudaError_t launch_winding_f32(const DetectArgs& a, int open_axes, const float* re, const float* im, int8_t* out,
                               unsigned long long* abs_sum, cudaStream_t st)
{
    winding_kernel<float><<<nblocks_of(a), DB, 0, st>>>(a, open_axes, re, im, out, abs_sum);
    return cudaGetLastError();
}

}  // namespace lat
