// String initial conditions built from a straight-string radial profile
// (the table singleSemiAnalytic writes), evaluated per site on the GPU.
//
// The reference builds them on the host, one site after another, and writes
// them as text (initialConditions.cpp) or keeps them in memory (ic_func.cpp
// for ic_w_evolution).  Every site is independent given the table, so here
// one thread evaluates one site, reading the profile through L1/L2 (160 KB at
// the reference's 20001 points): HBM sees only the field writes.
//
// Boosted string (initialConditions.cpp:710-992, ic_func.cpp:685-964): two
// passes.  Pass 1 writes the t = 0 fields and A_t, the time component the
// Lorentz boost gives the gauge field.  Pass 2 writes the t = dt fields,
// gauge-transformed back to A_t = 0 with the centred (one-sided on the faces)
// differences of A_t.  Compiled with -fmad=false: the operations, their order
// and the IEEE sqrt/division are the reference's, so the t = 0 level differs
// from it only where its pow(x, 2) is not x*x (glibc is within an ulp of the
// correctly rounded square, which x*x is) and the t = dt level also by the
// last bits of cos/sin.
#include <cmath>
#include <string>

#include "lattice_handle.hpp"

namespace lat {

namespace {

// the straight-string table on the device
struct Profile {
    const double* S0;   // |phi|
    const double* S1;   // A_theta
    long long m;
    double a;           // spacing
    double winding;
    double g;
};

struct BoostArgs {
    int nx, ny, nz, x0, y0, z0;
    double dx, dy, dz, dt, g;
    double v1x, v1y, v1z, vsq, gamma;
    Profile pr;
    int form;
};

// initialConditions.cpp:756-782; off the table (or at its last point) |phi| = 1, A = n/g
__device__ int profile_at(const Profile& q, double d, double& phiMag, double& AMag)
{
    const double a = q.a;
    const long long p = (long long)round(d / a);
    if (p == 0) {
        phiMag = (q.S0[p + 1] * d - q.S0[p] * (d - a)) / a;
        AMag = (q.S1[p + 1] * d - q.S1[p] * (d - a)) / a;
        return 0;
    }
    if (p + 1 < q.m) {
        const double pa = (double)p * a, pp = (double)(p + 1) * a, pm = (double)(p - 1) * a;
        phiMag = (q.S0[p - 1] * (d - pa) * (d - pp) - 2 * q.S0[p] * (d - pm) * (d - pp) + q.S0[p + 1] * (d - pm) * (d - pa))
               / (2 * a * a);
        AMag = (q.S1[p - 1] * (d - pa) * (d - pp) - 2 * q.S1[p] * (d - pm) * (d - pp) + q.S1[p + 1] * (d - pm) * (d - pa))
             / (2 * a * a);
        return 0;
    }
    phiMag = 1;
    AMag = q.g == 0 ? 0 : q.winding / q.g;
    return 1;
}

// the string's fields at stationary-frame position (xs, ys)
__device__ int string_fields(const BoostArgs& q, double xs, double ys, double& re, double& im, double& Ax, double& Ay)
{
    const double distance = sqrt(xs * xs + ys * ys);
    double phiMag, AMag;
    const int off = profile_at(q.pr, distance, phiMag, AMag);
    if (xs == 0) {
        re = 0;
        Ay = 0;
    } else {
        re = phiMag * xs / distance;
        Ay = AMag * xs / (distance * distance);
    }
    if (ys == 0) {
        im = 0;
        Ax = 0;
    } else {
        im = phiMag * ys / distance;
        Ax = -AMag * ys / (distance * distance);
    }
    return off;
}

template <class T>
struct Out5 {
    T* c[5];
};

__device__ __forceinline__ void site_of(long long s, const BoostArgs& q, int& i, int& j, int& k)
{
    k = (int)(s % q.nz);
    const long long r = s / q.nz;
    j = (int)(r % q.ny);
    i = (int)(r / q.ny);
}

// sites off the table are rare (a table far shorter than the lattice's diagonal)
__device__ __forceinline__ void count_off(unsigned long long* off, int n)
{
    if (n) atomicAdd(off, 1ull);
}

// t = 0 (initialConditions.cpp:735-807; zb is taken with dy there, :745)
template <class T>
__global__ void boost_t0_kernel(BoostArgs q, long long N, Out5<T> o, double* At, unsigned long long* off)
{
    for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < N; s += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        site_of(s, q, i, j, k);
        const double xb = (i - q.x0) * q.dx, yb = (j - q.y0) * q.dy, zb = (k - q.z0) * q.dy;
        const double xs = xb + (q.gamma - 1) * (q.v1x * xb + q.v1y * yb + q.v1z * zb) * q.v1x / q.vsq;
        const double ys = yb + (q.gamma - 1) * (q.v1x * xb + q.v1y * yb + q.v1z * zb) * q.v1y / q.vsq;
        double re, im, Ax, Ay;
        const int n = string_fields(q, xs, ys, re, im, Ax, Ay);
        count_off(off, n);
        At[s] = -q.gamma * (q.v1x * Ax + q.v1y * Ay);
        const double A0 = Ax + (q.gamma - 1) * (q.v1x * Ax + q.v1y * Ay) * q.v1x / q.vsq;
        const double A1 = Ay + (q.gamma - 1) * (q.v1x * Ax + q.v1y * Ay) * q.v1y / q.vsq;
        const double A2 = (q.gamma - 1) * (q.v1x * Ax + q.v1y * Ay) * q.v1z / q.vsq;
        o.c[0][s] = (T)re;
        o.c[1][s] = (T)im;
        o.c[2][s] = (T)(q.dx * q.g * A0);
        o.c[3][s] = (T)(q.dy * q.g * A1);
        o.c[4][s] = (T)(q.dz * q.g * A2);
    }
}

// t = dt and the gauge transformation to A_t = 0 (initialConditions.cpp:818-988
// for LAT_IC_FORM_FILE, ic_func.cpp:811-961 for LAT_IC_FORM_INPROCESS)
template <class T>
__global__ void boost_t1_kernel(BoostArgs q, long long N, Out5<T> o, const double* __restrict__ At,
                                unsigned long long* off)
{
    const long long sy = q.nz, sx = (long long)q.ny * q.nz;
    for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < N; s += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        site_of(s, q, i, j, k);
        const double xb = (i - q.x0) * q.dx, yb = (j - q.y0) * q.dy, zb = (k - q.z0) * q.dz;
        const double xs =
            xb + (q.gamma - 1) * (q.v1x * xb + q.v1y * yb + q.v1z * zb) * q.v1x / q.vsq - q.gamma * q.v1x * q.dt;
        const double ys =
            yb + (q.gamma - 1) * (q.v1x * xb + q.v1y * yb + q.v1z * zb) * q.v1y / q.vsq - q.gamma * q.v1y * q.dt;
        double re, im, Ax, Ay;
        const int n = string_fields(q, xs, ys, re, im, Ax, Ay);
        count_off(off, n);
        double dAx, dAy, dAz, qx, qy, qz;
        if (i == 0) { dAx = At[s + sx] - At[s]; qx = q.dx; }
        else if (i == q.nx - 1) { dAx = At[s] - At[s - sx]; qx = q.dx; }
        else { dAx = At[s + sx] - At[s - sx]; qx = 2 * q.dx; }
        if (j == 0) { dAy = At[s + sy] - At[s]; qy = q.dy; }
        else if (j == q.ny - 1) { dAy = At[s] - At[s - sy]; qy = q.dy; }
        else { dAy = At[s + sy] - At[s - sy]; qy = 2 * q.dy; }
        if (k == 0) { dAz = At[s + 1] - At[s]; qz = q.dz; }
        else if (k == q.nz - 1) { dAz = At[s] - At[s - 1]; qz = q.dz; }
        else { dAz = At[s + 1] - At[s - 1]; qz = 2 * q.dz; }
        const double tx = (q.gamma - 1) * (q.v1x * Ax + q.v1y * Ay);
        double th0, th1, th2;
        if (q.form == LAT_IC_FORM_INPROCESS) {
            th0 = q.dx * q.g * (Ax + tx * q.v1x / q.vsq);
            th1 = q.dy * q.g * (Ay + tx * q.v1y / q.vsq);
            th2 = q.dz * q.g * (tx * q.v1z / q.vsq);
            th0 += -q.dx * q.g * q.dt * dAx / qx;
            th1 += -q.dy * q.g * q.dt * dAy / qy;
            th2 += -q.dz * q.g * q.dt * dAz / qz;
        } else {
            double A0 = Ax + tx * q.v1x / q.vsq;
            double A1 = Ay + tx * q.v1y / q.vsq;
            double A2 = tx * q.v1z / q.vsq;
            A0 += -q.dt * dAx / qx;
            A1 += -q.dt * dAy / qy;
            A2 += -q.dt * dAz / qz;
            th0 = q.dx * q.g * A0;
            th1 = q.dy * q.g * A1;
            th2 = q.dz * q.g * A2;
        }
        const double ang = -q.g * q.dt * At[s];
        double sn, cs;
        sincos(ang, &sn, &cs);
        o.c[0][s] = (T)(cs * re - sn * im);
        o.c[1][s] = (T)(cs * im + sn * re);
        o.c[2][s] = (T)th0;
        o.c[3][s] = (T)th1;
        o.c[4][s] = (T)th2;
    }
}

template <class T>
Out5<T> slots_of(lat_handle* h, int t)
{
    Out5<T> o;
    for (int c = 0; c < 5; ++c) o.c[c] = (T*)h->slot(c, t);
    return o;
}

}  // namespace

}  // namespace lat

using namespace lat;

extern "C" int lat_boost_ic_device(lat_handle* h, const lat_string_profile* prof, const lat_boost_ic* b,
                                   int64_t* off_table)
{
    if (!h || !prof || !b || !prof->phi || !prof->A) {
        set_error("lat_boost_ic_device: null argument");
        return LAT_ERR_INVALID;
    }
    const lat_params& p = h->p;
    if (p.model != LAT_MODEL_AH) {
        set_error("lat_boost_ic_device: Abelian-Higgs handles only");
        return LAT_ERR_INVALID;
    }
    if (p.nx < 2 || p.ny < 2 || p.nz < 2) {
        set_error("lat_boost_ic_device: every side must be at least 2 (one-sided differences on the faces)");
        return LAT_ERR_INVALID;
    }
    if (prof->m < 2 || !(prof->h > 0)) {
        set_error("lat_boost_ic_device: the profile needs m >= 2 points and h > 0");
        return LAT_ERR_INVALID;
    }
    if (b->form != LAT_IC_FORM_FILE && b->form != LAT_IC_FORM_INPROCESS) {
        set_error("lat_boost_ic_device: form must be LAT_IC_FORM_FILE or LAT_IC_FORM_INPROCESS");
        return LAT_ERR_INVALID;
    }
    // the reference's own expressions for |v|^2 and gamma, on the host with the
    // same libm (initialConditions.cpp:730-734)
    const double vsq = std::pow(b->v[0], 2) + std::pow(b->v[1], 2) + std::pow(b->v[2], 2);
    if (!(vsq > 0 && vsq < 1)) {
        set_error("lat_boost_ic_device: need 0 < |v| < 1");
        return LAT_ERR_INVALID;
    }
    BoostArgs q;
    q.nx = (int)p.nx;
    q.ny = (int)p.ny;
    q.nz = (int)p.nz;
    q.x0 = (q.nx - 1) / 2;
    q.y0 = (q.ny - 1) / 2;
    q.z0 = (q.nz - 1) / 2;
    q.dx = p.dx;
    q.dy = p.dy;
    q.dz = p.dz;
    q.dt = p.dt;
    q.g = p.g;
    q.v1x = b->v[0];
    q.v1y = b->v[1];
    q.v1z = b->v[2];
    q.vsq = vsq;
    q.gamma = 1 / std::sqrt(1 - vsq);
    q.pr.m = prof->m;
    q.pr.a = prof->h;
    q.pr.winding = prof->winding;
    q.pr.g = p.g;
    q.form = b->form;

    cudaError_t e = cudaSetDevice(h->device);
    const size_t tab = sizeof(double) * (size_t)prof->m;
    const size_t need = 2 * tab + sizeof(double) * (size_t)h->N + 64;
    char* scratch = nullptr;
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&scratch, need, h->stream);
    if (e != cudaSuccess) {
        set_error(std::string("lat_boost_ic_device: ") + cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? LAT_ERR_NOMEM : LAT_ERR_CUDA;
    }
    double* S0 = (double*)scratch;
    double* S1 = S0 + prof->m;
    double* At = S1 + prof->m;
    unsigned long long* off = (unsigned long long*)(At + h->N);
    q.pr.S0 = S0;
    q.pr.S1 = S1;
    unsigned long long off_host = 0;
    e = cudaMemcpyAsync(S0, prof->phi, tab, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(S1, prof->A, tab, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(off, 0, sizeof(unsigned long long), h->stream);
    const int threads = 256;
    long long blocks = ((long long)h->N + threads - 1) / threads;
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (e == cudaSuccess) {
        const long long N = h->N;
        if (h->elem == 8) {
            boost_t0_kernel<double><<<(unsigned)blocks, threads, 0, h->stream>>>(q, N, slots_of<double>(h, 0), At, off);
            boost_t1_kernel<double><<<(unsigned)blocks, threads, 0, h->stream>>>(q, N, slots_of<double>(h, 1), At, off);
        } else {
            boost_t0_kernel<float><<<(unsigned)blocks, threads, 0, h->stream>>>(q, N, slots_of<float>(h, 0), At, off);
            boost_t1_kernel<float><<<(unsigned)blocks, threads, 0, h->stream>>>(q, N, slots_of<float>(h, 1), At, off);
        }
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&off_host, off, sizeof(off_host), cudaMemcpyDeviceToHost, h->stream);
    const cudaError_t ef = cudaFreeAsync(scratch, h->stream);
    if (e == cudaSuccess) e = ef;
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) {
        set_error(std::string("lat_boost_ic_device: ") + cudaGetErrorString(e));
        return LAT_ERR_CUDA;
    }
    h->n = 0;
    h->bc_level = -1;
    h->div_valid = false;
    h->launches += 2;
    if (off_table) *off_table = (int64_t)off_host;
    return LAT_OK;
}

// ---------------------------------------------------------------------------
// Loop collision (initialConditions.cpp:994-1716).  Per level three kernels:
//   A: per site, the four boosted strings' fields, each pair's product with
//      its imaginary part tapered to zero on the faces (magnitude kept), and
//      the links theta = d*g*(A1 + A2); at t = 0 also the four A_t fields;
//   B: each pair divided by the linear interpolant of its magnitude across
//      one pair of periodic faces (pair 1 over y, pair 2 over x);
//   C: the same over the other faces (pair 1 over z, pair 2 over y), and the
//      product of the two pairs -> phi.
// B and C read whole boundary planes of the previous pass, hence the
// separate launches.  Scratch: A_t (4N), the pass outputs (2 x 4N) doubles.
// ---------------------------------------------------------------------------
namespace lat {

namespace {

struct LcBoost {
    double v[3], vsq, gamma;
};

struct LcArgs {
    int nx, ny, nz, x0, y0, z0;
    double dx, dy, dz, dt, g;
    LcBoost B[4];        // 1s, 1a, 2s, 2a
    double sf[4][2];     // rest-frame positions (lab-frame ones in ic_func's form)
    Profile pr;
    int older;           // ic_func.cpp's form: boosted one-forms keep only the boost term
};

// (a + i b)/d as std::complex builds it from `a + ci*b` and `/ d`
__device__ __forceinline__ void lc_unit(double a, double b, double d, double& re, double& im)
{
    re = (0.0 * b + a) / d;
    im = b / d;
}

__device__ __forceinline__ double lc_sq(double x) { return x * x; }

// initialConditions.cpp:1061-1330 (t = 0) and 1430-1690 (t = dt) for one site;
// with q.older, ic_func.cpp:1006-1250 and 1365-1621
__device__ int lc_site(const LcArgs& q, int t, int i, int j, int k, long long s, double* At, long long N,
                       double P0[4], double th[3])
{
    const double xb = (i - q.x0) * q.dx, yb = (j - q.y0) * q.dy, zb = (k - q.z0) * q.dy;   // zb with dy
    double pos[4][2];   // (ys1s, zs1s), (ys1a, zs1a), (xs2s, ys2s), (xs2a, ys2a)
#pragma unroll
    for (int w = 0; w < 4; ++w) {
        const LcBoost& b = q.B[w];
        const double c0 = w < 2 ? yb : xb, c1 = w < 2 ? zb : yb;
        if (b.vsq == 0) {
            pos[w][0] = c0;
            pos[w][1] = c1;
            continue;
        }
        const double dot = b.v[0] * xb + b.v[1] * yb + b.v[2] * zb;
        // pair 1 projects on v[1], v[2]; pair 2 on v[0], v[1], except that the
        // reference projects the anti-string's x on v[1] (:1085, :1460)
        const int e0 = w < 2 ? 1 : (w == 3 ? 1 : 0), e1 = w < 2 ? 2 : 1;
        pos[w][0] = c0 + (b.gamma - 1) * dot * b.v[e0] / b.vsq;
        pos[w][1] = c1 + (b.gamma - 1) * dot * b.v[e1] / b.vsq;
        if (t) {
            const int f0 = w < 2 ? 1 : 0;
            pos[w][0] -= b.gamma * b.v[f0] * q.dt;
            pos[w][1] -= b.gamma * b.v[f0 + 1] * q.dt;
        }
    }
    // offsets from each string: pair 1 (y, z), pair 2 (x, y)
    double off0[4], off1[4], d[4], pm[4], am[4];
    int off = 0;
#pragma unroll
    for (int w = 0; w < 4; ++w) {
        off0[w] = pos[w][0] - q.sf[w][0];
        off1[w] = pos[w][1] - q.sf[w][1];
        d[w] = sqrt(lc_sq(off0[w]) + lc_sq(off1[w]));
        off += profile_at(q.pr, d[w], pm[w], am[w]);
    }
    double u[4][2];
    lc_unit(-off1[0], off0[0], d[0], u[0][0], u[0][1]);   // 1s: (-(z - z1s), y - y1s)
    lc_unit(off1[1], off0[1], d[1], u[1][0], u[1][1]);    // 1a: (z - z1a, y - y1a)
    lc_unit(off0[2], off1[2], d[2], u[2][0], u[2][1]);    // 2s: (x - x2s, y - y2s)
    lc_unit(-off0[3], off1[3], d[3], u[3][0], u[3][1]);   // 2a: (-(x - x2a), y - y2a)
    if (t) {
#pragma unroll
        for (int w = 0; w < 4; ++w) {
            double sn, cs;
            sincos(q.g * q.dt * At[w * N + s], &sn, &cs);
            const double gr = -(0.0 * sn) + cs, gi = -sn;
            const double a = u[w][0], b = u[w][1];
            u[w][0] = a * gr - b * gi;
            u[w][1] = a * gi + b * gr;
        }
    }
    double ph[4][2], A[4][3];
    // x-directed pair: A has y, z components
    A[0][0] = 0;
    if (off1[0] == 0) { ph[0][0] = 0; A[0][1] = 0; }
    else { ph[0][0] = pm[0] * u[0][0]; A[0][1] = -am[0] * off1[0] / lc_sq(d[0]); }
    if (off0[0] == 0) { ph[0][1] = 0; A[0][2] = 0; }
    else { ph[0][1] = pm[0] * u[0][1]; A[0][2] = am[0] * off0[0] / lc_sq(d[0]); }
    A[1][0] = 0;
    if (off1[1] == 0) { ph[1][0] = 0; A[1][1] = 0; }
    else { ph[1][0] = pm[1] * u[1][0]; A[1][1] = am[1] * off1[1] / lc_sq(d[1]); }
    if (off0[1] == 0) { ph[1][1] = 0; A[1][2] = 0; }
    else { ph[1][1] = pm[1] * u[1][1]; A[1][2] = -am[1] * off0[1] / lc_sq(d[1]); }
    // z-directed pair: A has x, y components
    A[2][2] = 0;
    if (off0[2] == 0) { ph[2][0] = 0; A[2][1] = 0; }
    else { ph[2][0] = pm[2] * u[2][0]; A[2][1] = am[2] * off0[2] / lc_sq(d[2]); }
    if (off1[2] == 0) { ph[2][1] = 0; A[2][0] = 0; }
    else { ph[2][1] = pm[2] * u[2][1]; A[2][0] = -am[2] * off1[2] / lc_sq(d[2]); }
    A[3][2] = 0;
    if (off0[3] == 0) { ph[3][0] = 0; A[3][1] = 0; }
    else { ph[3][0] = pm[3] * u[3][0]; A[3][1] = -am[3] * off0[3] / lc_sq(d[3]); }
    if (off1[3] == 0) { ph[3][1] = 0; A[3][0] = 0; }
    else { ph[3][1] = pm[3] * u[3][1]; A[3][0] = am[3] * off1[3] / lc_sq(d[3]); }
    // Lorentz transformation of the one-forms
    double Ap[4][3];
#pragma unroll
    for (int w = 0; w < 4; ++w) {
        const LcBoost& b = q.B[w];
        const double dotA = w < 2 ? b.v[1] * A[w][1] + b.v[2] * A[w][2] : b.v[0] * A[w][0] + b.v[1] * A[w][1];
#pragma unroll
        for (int cc = 0; cc < 3; ++cc) {
            const double boost = (b.gamma - 1) * dotA * b.v[cc] / b.vsq;
            // ic_func.cpp:1195-1196, 1229-1230: the boost term alone (|v| > 0 there)
            Ap[w][cc] = q.older ? boost : (b.vsq == 0 ? A[w][cc] : A[w][cc] + boost);
        }
        if (!t) At[w * N + s] = -b.gamma * dotA;
    }
    if (t) {
        // gauge shift to A_t = 0 with periodic centred differences (:1618-1640)
        const int ip = (i + 1 + q.nx) % q.nx, im = (i - 1 + q.nx) % q.nx;
        const int jp = (j + 1 + q.ny) % q.ny, jm = (j - 1 + q.ny) % q.ny;
        const int kp = (k + 1 + q.nz) % q.nz, km = (k - 1 + q.nz) % q.nz;
        const long long sxp = ((long long)ip * q.ny + j) * q.nz + k, sxm = ((long long)im * q.ny + j) * q.nz + k;
        const long long syp = ((long long)i * q.ny + jp) * q.nz + k, sym = ((long long)i * q.ny + jm) * q.nz + k;
        const long long szp = ((long long)i * q.ny + j) * q.nz + kp, szm = ((long long)i * q.ny + j) * q.nz + km;
#pragma unroll
        for (int w = 0; w < 4; ++w) {
            const double* a = At + w * N;
            Ap[w][0] += -q.dt * (a[sxp] - a[sxm]) / (2 * q.dx);
            Ap[w][1] += -q.dt * (a[syp] - a[sym]) / (2 * q.dy);
            Ap[w][2] += -q.dt * (a[szp] - a[szm]) / (2 * q.dz);
        }
    }
    double Asum[2][3];
#pragma unroll
    for (int pair = 0; pair < 2; ++pair) {
        const double* a = ph[2 * pair];
        const double* b = ph[2 * pair + 1];
        double p0 = a[0] * b[0] - a[1] * b[1];
        double p1 = a[1] * b[0] + a[0] * b[1];
        const double pf = pair == 0 ? (1 - lc_sq(yb / (q.y0 * q.dy))) * (1 - lc_sq(zb / (q.z0 * q.dz)))
                                    : (1 - lc_sq(xb / (q.x0 * q.dx))) * (1 - lc_sq(yb / (q.y0 * q.dy)));
        if (lc_sq(p0) + lc_sq(p1 * pf) == 0) {
            p0 = p1;
            p1 = 0;
        } else {
            const double nf = sqrt((lc_sq(p0) + lc_sq(p1)) / (lc_sq(p0) + lc_sq(p1 * pf)));
            p0 = nf * p0;
            p1 = nf * pf * p1;
        }
        P0[2 * pair] = p0;
        P0[2 * pair + 1] = p1;
#pragma unroll
        for (int cc = 0; cc < 3; ++cc) Asum[pair][cc] = (Ap[2 * pair][cc] + Ap[2 * pair + 1][cc]) * pf;
    }
    th[0] = q.dx * q.g * (Asum[0][0] + Asum[1][0]);
    th[1] = q.dy * q.g * (Asum[0][1] + Asum[1][1]);
    th[2] = q.dz * q.g * (Asum[0][2] + Asum[1][2]);
    return off;
}

template <class T>
__global__ void lc_pass_a(LcArgs q, int t, long long N, double* At, double* P0, T* th0, T* th1, T* th2,
                          unsigned long long* off)
{
    for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < N; s += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(s % q.nz);
        const long long r = s / q.nz;
        const int j = (int)(r % q.ny), i = (int)(r / q.ny);
        double v4[4], th[3];
        if (lc_site(q, t, i, j, k, s, At, N, v4, th)) atomicAdd(off, 1ull);
#pragma unroll
        for (int w = 0; w < 4; ++w) P0[w * N + s] = v4[w];
        th0[s] = (T)th[0];
        th1[s] = (T)th[1];
        th2[s] = (T)th[2];
    }
}

__device__ __forceinline__ double lc_mag(const double* re, const double* im, long long s)
{
    return sqrt(lc_sq(re[s]) + lc_sq(im[s]));
}

// initialConditions.cpp:1336-1372 (pass B) and 1376-1414 (pass C, which also
// multiplies the pairs)
template <class T, bool LAST>
__global__ void lc_pass_bc(LcArgs q, long long N, const double* __restrict__ Pin, double* Pout, T* phr, T* phi)
{
    const double *r1 = Pin, *i1 = Pin + N, *r2 = Pin + 2 * N, *i2 = Pin + 3 * N;
    for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < N; s += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(s % q.nz);
        const long long r = s / q.nz;
        const int j = (int)(r % q.ny), i = (int)(r / q.ny);
        const long long row = ((long long)i * q.ny + j) * q.nz;
        const double xb = (i - q.x0) * q.dx, yb = (j - q.y0) * q.dy, zb = (k - q.z0) * q.dz;
        double m1t, m1b, m2t, m2b, w1, w2;
        if (!LAST) {
            // pair 1 across y, pair 2 across x
            m1t = lc_mag(r1, i1, ((long long)i * q.ny + (q.ny - 1)) * q.nz + k);
            m1b = lc_mag(r1, i1, ((long long)i * q.ny) * q.nz + k);
            m2t = lc_mag(r2, i2, ((long long)(q.nx - 1) * q.ny + j) * q.nz + k);
            m2b = lc_mag(r2, i2, ((long long)j) * q.nz + k);
            w1 = (m1t - m1b) * (yb + q.y0 * q.dy) / (2 * q.y0 * q.dy) + m1b;
            w2 = (m2t - m2b) * (xb + q.x0 * q.dx) / (2 * q.x0 * q.dx) + m2b;
        } else {
            // pair 1 across z, pair 2 across y
            m1t = lc_mag(r1, i1, row + (q.nz - 1));
            m1b = lc_mag(r1, i1, row);
            m2t = lc_mag(r2, i2, ((long long)i * q.ny + (q.ny - 1)) * q.nz + k);
            m2b = lc_mag(r2, i2, ((long long)i * q.ny) * q.nz + k);
            w1 = (m1t - m1b) * (zb + q.z0 * q.dz) / (2 * q.z0 * q.dz) + m1b;
            w2 = (m2t - m2b) * (yb + q.y0 * q.dy) / (2 * q.y0 * q.dy) + m2b;
        }
        const double a0 = r1[s] / w1, a1 = i1[s] / w1, b0 = r2[s] / w2, b1 = i2[s] / w2;
        if (!LAST) {
            Pout[s] = a0;
            Pout[N + s] = a1;
            Pout[2 * N + s] = b0;
            Pout[3 * N + s] = b1;
        } else {
            phr[s] = (T)(a0 * b0 - a1 * b1);
            phi[s] = (T)(a0 * b1 + a1 * b0);
        }
    }
}

template <class T>
cudaError_t lc_launch(lat_handle* h, const LcArgs& q, double* At, double* P0, double* P1, unsigned long long* off)
{
    const int threads = 128;
    long long blocks = ((long long)h->N + threads - 1) / threads;
    if (blocks > 152 * 32) blocks = 152 * 32;
    const long long N = h->N;
    for (int t = 0; t < 2; ++t) {
        T* sl[5];
        for (int c = 0; c < 5; ++c) sl[c] = (T*)h->slot(c, t);
        lc_pass_a<T><<<(unsigned)blocks, threads, 0, h->stream>>>(q, t, N, At, P0, sl[2], sl[3], sl[4], off);
        lc_pass_bc<T, false><<<(unsigned)blocks, threads, 0, h->stream>>>(q, N, P0, P1, nullptr, nullptr);
        lc_pass_bc<T, true><<<(unsigned)blocks, threads, 0, h->stream>>>(q, N, P1, nullptr, sl[0], sl[1]);
    }
    return cudaGetLastError();
}

void lc_boost_init(LcBoost& b, const double v[3])
{
    b.v[0] = v[0];
    b.v[1] = v[1];
    b.v[2] = v[2];
    b.vsq = std::pow(v[0], 2) + std::pow(v[1], 2) + std::pow(v[2], 2);
    b.gamma = 1 / std::sqrt(1 - b.vsq);
}

}  // namespace

}  // namespace lat

namespace lat {
namespace {

// Both loop-collision forms; `older` selects ic_func.cpp's.
int loop_collision_device(const char* who, lat_handle* h, const lat_string_profile* prof,
                          const lat_loop_collision_ic* c, int64_t* off_table, bool older)
{
    const std::string name(who);
    if (!h || !prof || !c || !prof->phi || !prof->A) {
        set_error(name + ": null argument");
        return LAT_ERR_INVALID;
    }
    const lat_params& p = h->p;
    if (p.model != LAT_MODEL_AH) {
        set_error(name + ": Abelian-Higgs handles only");
        return LAT_ERR_INVALID;
    }
    if (p.nx < 3 || p.ny < 3 || p.nz < 3) {
        set_error(name + ": every side must be at least 3");
        return LAT_ERR_INVALID;
    }
    if (prof->m < 2 || !(prof->h > 0)) {
        set_error(name + ": the profile needs m >= 2 points and h > 0");
        return LAT_ERR_INVALID;
    }
    LcArgs q;
    q.older = older ? 1 : 0;
    q.nx = (int)p.nx;
    q.ny = (int)p.ny;
    q.nz = (int)p.nz;
    q.x0 = (q.nx - 1) / 2;
    q.y0 = (q.ny - 1) / 2;
    q.z0 = (q.nz - 1) / 2;
    q.dx = p.dx;
    q.dy = p.dy;
    q.dz = p.dz;
    q.dt = p.dt;
    q.g = p.g;
    const double* vel[4] = {c->v1s, c->v1a, c->v2s, c->v2a};
    const double* pos[4] = {c->pos1s, c->pos1a, c->pos2s, c->pos2a};
    for (int w = 0; w < 4; ++w) {
        lc_boost_init(q.B[w], vel[w]);
        if (!(q.B[w].vsq < 1)) {
            set_error(name + ": every |v| must be below 1");
            return LAT_ERR_INVALID;
        }
        if (older && !(q.B[w].vsq > 0)) {
            // ic_func.cpp divides by |v|^2 with no branch for a string at rest
            set_error(name + ": every string must move (0 < |v| < 1)");
            return LAT_ERR_INVALID;
        }
        // rest-frame positions (initialConditions.cpp:1030-1046), on the host with
        // the reference's operations; ic_func's form measures from the given
        // lab-frame positions (ic_func.cpp:1034-1037)
        const LcBoost& b = q.B[w];
        if (b.vsq == 0 || older) {
            q.sf[w][0] = pos[w][0];
            q.sf[w][1] = pos[w][1];
        } else {
            const int e = w < 2 ? 1 : 0;
            const double dot = b.v[e] * pos[w][0] + b.v[e + 1] * pos[w][1];
            q.sf[w][0] = pos[w][0] + (b.gamma - 1) * dot * b.v[e] / b.vsq;
            q.sf[w][1] = pos[w][1] + (b.gamma - 1) * dot * b.v[e + 1] / b.vsq;
        }
    }
    q.pr.m = prof->m;
    q.pr.a = prof->h;
    q.pr.winding = prof->winding;
    q.pr.g = p.g;

    cudaError_t e = cudaSetDevice(h->device);
    const size_t tab = sizeof(double) * (size_t)prof->m;
    const size_t need = 2 * tab + sizeof(double) * 12 * (size_t)h->N + 64;
    char* scratch = nullptr;
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&scratch, need, h->stream);
    if (e != cudaSuccess) {
        set_error(name + ": " + cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? LAT_ERR_NOMEM : LAT_ERR_CUDA;
    }
    double* S0 = (double*)scratch;
    double* S1 = S0 + prof->m;
    double* At = S1 + prof->m;
    double* P0 = At + 4 * h->N;
    double* P1 = P0 + 4 * h->N;
    unsigned long long* off = (unsigned long long*)(P1 + 4 * h->N);
    q.pr.S0 = S0;
    q.pr.S1 = S1;
    unsigned long long off_host = 0;
    e = cudaMemcpyAsync(S0, prof->phi, tab, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(S1, prof->A, tab, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(off, 0, sizeof(unsigned long long), h->stream);
    if (e == cudaSuccess) e = h->elem == 8 ? lc_launch<double>(h, q, At, P0, P1, off) : lc_launch<float>(h, q, At, P0, P1, off);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&off_host, off, sizeof(off_host), cudaMemcpyDeviceToHost, h->stream);
    const cudaError_t ef = cudaFreeAsync(scratch, h->stream);
    if (e == cudaSuccess) e = ef;
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) {
        set_error(name + ": " + cudaGetErrorString(e));
        return LAT_ERR_CUDA;
    }
    h->n = 0;
    h->bc_level = -1;
    h->div_valid = false;
    h->launches += 6;
    if (off_table) *off_table = (int64_t)off_host;
    return LAT_OK;
}

}  // namespace
}  // namespace lat

extern "C" int lat_loop_collision_ic_device(lat_handle* h, const lat_string_profile* prof,
                                            const lat_loop_collision_ic* c, int64_t* off_table)
{
    return lat::loop_collision_device("lat_loop_collision_ic_device", h, prof, c, off_table, false);
}

extern "C" int lat_icfunc_loop_collision_ic_device(lat_handle* h, const lat_string_profile* prof,
                                                   const lat_loop_collision_ic* c, int64_t* off_table)
{
    return lat::loop_collision_device("lat_icfunc_loop_collision_ic_device", h, prof, c, off_table, true);
}

// ---------------------------------------------------------------------------
// Perturbed straight strings (initialConditions.cpp:113-668): one level of
// fields, written into both slots.
//   "simple sine" (:488-668): per site, the straight string offset along x by
//     eps*sin(Omega z)/Omega, Omega = 2 pi/(dz (nz-1)).
//   "NG sine" (:113-486): a Nambu-Goto sine wave.  Per (x, z) column with
//     z >= 0 a golden-section search (to 1e-6 in the string parameter, every
//     trial point's z(sigma) a 1001-point trapezoid integral) finds the
//     closest string point; the sites of the column follow from it, and the
//     reference mirrors them onto the columns with z < 0.  Here one thread
//     searches one column, and a second kernel evaluates every site from the
//     column whose write the reference's loop leaves last (its own, or the
//     mirrored one), so the result does not depend on an order of writes.
// The arithmetic follows the reference operation by operation (this unit is
// compiled with -fmad=false; pow(v, 2) is v*v, the correctly rounded square),
// with CUDA's sin, cos and sqrt.
// ---------------------------------------------------------------------------
namespace lat {

namespace {

constexpr int NG_NELLIP = 1001;  // N_ellipint (initialConditions.cpp:45)
constexpr double NG_TOL = 1e-6;  // tol (:44)

// both slots of the five components: c[0..4] slot 0, c[5..9] slot 1
template <class T>
struct Out10 {
    T* c[10];
};

struct SineArgs {
    int nx, ny, nz, x0, y0, z0;
    double dx, dy, dz, g, eps, Omega, pi, gr;
    Profile pr;
};

__device__ __forceinline__ double sq(double v) { return v * v; }

// z(sigma)*Omega: trapezoid rule with the phase shifted by -pi/2 (:189-198)
__device__ double ng_ellip(const SineArgs& q, double sigma)
{
    double e = 0;
    for (int j = 0; j < NG_NELLIP; j++) {
        const double trap_fac = (j == 0 || j == NG_NELLIP - 1) ? 0.5 : 1;
        const double theta = j * q.Omega * sigma / (NG_NELLIP - 1) - q.pi / 2;
        e += trap_fac * sqrt(1 - sq(q.eps * sin(theta))) * q.Omega * sigma / (NG_NELLIP - 1);
    }
    return e;
}

__device__ double ng_dist2(const SineArgs& q, double sigma, double x, double z)
{
    const double e = ng_ellip(q, sigma);
    return sq(x - q.eps * cos(q.Omega * sigma - q.pi / 2) / q.Omega) + sq(z - e / q.Omega);
}

// one column (i, k = z0 + kk): xs, zs, xs_sigma, zs_sigma, paraVecMag, normal_dist
__global__ void ng_column_kernel(const SineArgs q, double* __restrict__ col, int ncol)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncol) return;
    const int i = c % q.nx, k = q.z0 + c / q.nx;
    const double x = (i - q.x0) * q.dx, z = (k - q.z0) * q.dz;
    double a = -2 * q.pi / q.Omega, b = 2 * q.pi / q.Omega;
    double sigma1 = b - (b - a) / q.gr, sigma2 = a + (b - a) / q.gr;
    double d1 = ng_dist2(q, sigma1, x, z), d2 = ng_dist2(q, sigma2, x, z);
    double tolTest = 1, sigma = 0;
    while (tolTest > NG_TOL) {  // (b - a) shrinks by 1/gr per pass: ends after ~40 passes
        if (d1 < d2) b = sigma2;
        else a = sigma1;
        sigma1 = b - (b - a) / q.gr;
        sigma2 = a + (b - a) / q.gr;
        d1 = ng_dist2(q, sigma1, x, z);
        d2 = ng_dist2(q, sigma2, x, z);
        tolTest = b - a;
        if (tolTest <= NG_TOL) sigma = d1 > d2 ? sigma2 : sigma1;
    }
    const double xs = q.eps * cos(q.Omega * sigma - q.pi / 2) / q.Omega;
    const double zs = ng_ellip(q, sigma) / q.Omega;
    const double xs_sigma = -q.eps * sin(q.Omega * sigma - q.pi / 2);
    const double zs_sigma = sqrt(1 - sq(q.eps * sin(q.Omega * sigma - q.pi / 2)));
    const double paraVecMag = sqrt(sq(xs_sigma) + sq(zs_sigma));
    col[0 * (size_t)ncol + c] = xs;
    col[1 * (size_t)ncol + c] = zs;
    col[2 * (size_t)ncol + c] = xs_sigma;
    col[3 * (size_t)ncol + c] = zs_sigma;
    col[4 * (size_t)ncol + c] = paraVecMag;
    col[5 * (size_t)ncol + c] = (zs_sigma * (x - xs) - xs_sigma * (z - zs)) / paraVecMag;
}

// the reference's direct values at (i, j, k), k >= z0 (:438-467): phi0, phi1, A0, A1, A2
__device__ int ng_direct(const SineArgs& q, const double* __restrict__ col, int ncol, int i, int j, int k, double v[5])
{
    const int c = (k - q.z0) * q.nx + i;
    const double xs = col[c], zs = col[(size_t)ncol + c], xs_sigma = col[2 * (size_t)ncol + c];
    const double zs_sigma = col[3 * (size_t)ncol + c], paraVecMag = col[4 * (size_t)ncol + c];
    const double normal_dist = col[5 * (size_t)ncol + c];
    const double x = (i - q.x0) * q.dx, y = (j - q.y0) * q.dy, z = (k - q.z0) * q.dz;
    const double distance = sqrt(sq(x - xs) + sq(y) + sq(z - zs));
    double phiMag, AMag;
    const int off = profile_at(q.pr, distance, phiMag, AMag);
    if (normal_dist == 0) {
        v[0] = 0;
        v[3] = 0;
    } else {
        v[0] = phiMag * normal_dist / distance;
        v[3] = AMag * normal_dist / sq(distance);
    }
    if (y == 0) {
        v[1] = 0;
        v[2] = 0;
        v[4] = 0;
    } else {
        v[1] = phiMag * y / distance;
        v[2] = -AMag * zs_sigma * y / (sq(distance) * paraVecMag);
        v[4] = AMag * xs_sigma * y / (sq(distance) * paraVecMag);
    }
    return off;
}

// Site (i, j, k) as the reference leaves it.  Its loop over k >= z0 (outer),
// i, j writes (i, j, k) and then the mirror site (nx-1-i, j, nz-1-k) with
// phi0 and A1 negated (A2 onto (nx-1-i, j, nz-2-k), negated, for k < nz-1).
// A site gets at most one direct and one mirrored write per field; the later
// in loop order, (k, i, direct before mirror), stays.
template <class T>
__global__ void ng_fill_kernel(const SineArgs q, const double* __restrict__ col, int ncol, long long N, Out10<T> o,
                               unsigned long long* off)
{
    for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < N; s += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(s % q.nz);
        const long long r = s / q.nz;
        const int j = (int)(r % q.ny), i = (int)(r / q.ny);
        double dv[5] = {0, 0, 0, 0, 0}, mv[5];
        const bool direct = k >= q.z0;
        if (direct) count_off(off, ng_direct(q, col, ncol, i, j, k, dv));
        double out[5] = {0, 0, 0, 0, 0};
        // phi0, phi1, A0, A1: direct at key (k, i); mirror from column (nx-1-i, nz-1-k) at key (nz-1-k, nx-1-i)
        const int km = q.nz - 1 - k, im = q.nx - 1 - i;
        const bool mirror = km >= q.z0;
        const bool mirror_last = mirror && (!direct || km > k || (km == k && im >= i));
        if (mirror_last) {
            ng_direct(q, col, ncol, im, j, km, mv);
            out[0] = -mv[0];
            out[1] = mv[1];
            out[2] = mv[2];
            out[3] = -mv[3];
        } else if (direct) {
            out[0] = dv[0];
            out[1] = dv[1];
            out[2] = dv[2];
            out[3] = dv[3];
        }
        // A2: mirror from column (nx-1-i, nz-2-k), written while k_src <= nz-2
        const int k2 = q.nz - 2 - k;
        const bool mirror2 = k2 >= q.z0;
        if (mirror2 && (!direct || k2 > k || (k2 == k && im >= i))) {
            ng_direct(q, col, ncol, im, j, k2, mv);
            out[4] = -mv[4];
        } else if (direct) {
            out[4] = dv[4];
        }
        // link columns d*g*A (:482-486), both slots
        const double v5[5] = {out[0], out[1], q.dx * q.g * out[2], q.dy * q.g * out[3], q.dz * q.g * out[4]};
#pragma unroll
        for (int c = 0; c < 5; ++c) {
            o.c[c][s] = (T)v5[c];
            o.c[5 + c][s] = (T)v5[c];
        }
    }
}

template <class T>
__global__ void simple_sine_kernel(const SineArgs q, long long N, Out10<T> o, unsigned long long* off)
{
    for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < N; s += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(s % q.nz);
        const long long r = s / q.nz;
        const int j = (int)(r % q.ny), i = (int)(r / q.ny);
        const double x = (i - q.x0) * q.dx, y = (j - q.y0) * q.dy, z = (k - q.z0) * q.dz;
        const double xdist = x - q.eps * sin(q.Omega * z) / q.Omega;
        const double distance = sqrt(xdist * xdist + y * y);
        double phiMag, AMag, ph0, ph1, A0, A1;
        count_off(off, profile_at(q.pr, distance, phiMag, AMag));
        if (xdist == 0) {
            ph0 = 0;
            A1 = 0;
        } else {
            ph0 = phiMag * xdist / distance;
            A1 = AMag * xdist / sq(distance);
        }
        if (y == 0) {
            ph1 = 0;
            A0 = 0;
        } else {
            ph1 = phiMag * y / distance;
            A0 = -AMag * y / sq(distance);
        }
        const double v5[5] = {ph0, ph1, q.dx * q.g * A0, q.dy * q.g * A1, q.dz * q.g * 0.0};
#pragma unroll
        for (int c = 0; c < 5; ++c) {
            o.c[c][s] = (T)v5[c];
            o.c[5 + c][s] = (T)v5[c];
        }
    }
}

}  // namespace

}  // namespace lat

namespace lat {

namespace {

template <class T>
Out10<T> both_slots(lat_handle* h)
{
    Out10<T> o;
    for (int t = 0; t < 2; ++t)
        for (int c = 0; c < 5; ++c) o.c[5 * t + c] = (T*)h->slot(c, t);
    return o;
}

template <class T>
void sine_launch(lat_handle* h, const SineArgs& q, bool ng, const double* col, int ncol, unsigned long long* off)
{
    const int threads = 256;
    long long blocks = ((long long)h->N + threads - 1) / threads;
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (ng) ng_fill_kernel<T><<<(unsigned)blocks, threads, 0, h->stream>>>(q, col, ncol, h->N, both_slots<T>(h), off);
    else simple_sine_kernel<T><<<(unsigned)blocks, threads, 0, h->stream>>>(q, h->N, both_slots<T>(h), off);
}

// Shared by the two sine families: checks, the table on the device, the
// launches, the off-table count.
int sine_ic_device(lat_handle* h, const lat_string_profile* prof, double eps, int64_t* off_table, bool ng,
                   const char* fn)
{
    if (!h || !prof || !prof->phi || !prof->A) {
        set_error(std::string(fn) + ": null argument");
        return LAT_ERR_INVALID;
    }
    const lat_params& p = h->p;
    if (p.model != LAT_MODEL_AH) {
        set_error(std::string(fn) + ": Abelian-Higgs handles only");
        return LAT_ERR_INVALID;
    }
    if (p.nx < 2 || p.ny < 2 || p.nz < 2 || prof->m < 2 || !(prof->h > 0)) {
        set_error(std::string(fn) + ": sides >= 2, a profile of m >= 2 points and h > 0");
        return LAT_ERR_INVALID;
    }
    if (!(eps >= 0 && eps < 1)) {
        set_error(std::string(fn) + ": eps must lie in [0, 1)");
        return LAT_ERR_INVALID;
    }
    SineArgs q;
    q.nx = (int)p.nx;
    q.ny = (int)p.ny;
    q.nz = (int)p.nz;
    q.x0 = (q.nx - 1) / 2;
    q.y0 = (q.ny - 1) / 2;
    q.z0 = (q.nz - 1) / 2;
    q.dx = p.dx;
    q.dy = p.dy;
    q.dz = p.dz;
    q.g = p.g;
    q.eps = eps;
    q.pi = 4 * std::atan(1.0);           // initialConditions.cpp:40
    q.gr = 0.5 * (1 + std::sqrt(5.0));   // :50
    if (ng) {
        // Omega of a string periodic over dz*nz (:143-160), on the host with the reference's libm
        double e = 0;
        for (int j = 0; j < NG_NELLIP; j++) {
            const double trap_fac = (j == 0 || j == NG_NELLIP - 1) ? 0.5 : 1;
            const double theta = j * 2 * q.pi / (NG_NELLIP - 1);
            e += trap_fac * std::sqrt(1 - std::pow(eps * std::sin(theta), 2)) * 2 * q.pi / (NG_NELLIP - 1);
        }
        q.Omega = e / (p.dz * (double)p.nz);
    } else {
        q.Omega = 2 * q.pi / (p.dz * (double)(p.nz - 1));   // :510
    }
    q.pr.m = prof->m;
    q.pr.a = prof->h;
    q.pr.winding = prof->winding;
    q.pr.g = p.g;
    const int ncol = ng ? q.nx * (q.nz - q.z0) : 0;

    cudaError_t e = cudaSetDevice(h->device);
    const size_t tab = sizeof(double) * (size_t)prof->m;
    const size_t need = 2 * tab + sizeof(double) * 6 * (size_t)ncol + 64;
    char* scratch = nullptr;
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&scratch, need, h->stream);
    if (e != cudaSuccess) {
        set_error(std::string(fn) + ": " + cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? LAT_ERR_NOMEM : LAT_ERR_CUDA;
    }
    double* S0 = (double*)scratch;
    double* S1 = S0 + prof->m;
    double* col = S1 + prof->m;
    unsigned long long* off = (unsigned long long*)(col + 6 * (size_t)ncol);
    q.pr.S0 = S0;
    q.pr.S1 = S1;
    unsigned long long off_host = 0;
    e = cudaMemcpyAsync(S0, prof->phi, tab, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(S1, prof->A, tab, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(off, 0, sizeof(unsigned long long), h->stream);
    if (e == cudaSuccess) {
        if (ng) ng_column_kernel<<<(ncol + 127) / 128, 128, 0, h->stream>>>(q, col, ncol);
        if (h->elem == 8) sine_launch<double>(h, q, ng, col, ncol, off);
        else sine_launch<float>(h, q, ng, col, ncol, off);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&off_host, off, sizeof(off_host), cudaMemcpyDeviceToHost, h->stream);
    const cudaError_t ef = cudaFreeAsync(scratch, h->stream);
    if (e == cudaSuccess) e = ef;
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) {
        set_error(std::string(fn) + ": " + cudaGetErrorString(e));
        return LAT_ERR_CUDA;
    }
    h->n = 0;
    h->bc_level = -1;
    h->div_valid = false;
    h->launches += ng ? 2 : 1;
    if (off_table) *off_table = (int64_t)off_host;
    return LAT_OK;
}

}  // namespace

}  // namespace lat

extern "C" int lat_ng_sine_ic_device(lat_handle* h, const lat_string_profile* prof, double eps, int64_t* off_table)
{
    return lat::sine_ic_device(h, prof, eps, off_table, true, "lat_ng_sine_ic_device");
}

extern "C" int lat_simple_sine_ic_device(lat_handle* h, const lat_string_profile* prof, double eps,
                                         int64_t* off_table)
{
    return lat::sine_ic_device(h, prof, eps, off_table, false, "lat_simple_sine_ic_device");
}
