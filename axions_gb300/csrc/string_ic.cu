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

struct BoostArgs {
    int nx, ny, nz, x0, y0, z0;
    double dx, dy, dz, dt, g;
    double v1x, v1y, v1z, vsq, gamma;
    const double* S0;   // |phi| table (device)
    const double* S1;   // A table (device)
    long long m;
    double a;           // table spacing
    double winding;
    int form;
};

// initialConditions.cpp:756-782; off the table (or at its last point) |phi| = 1, A = n/g
__device__ int profile_at(const BoostArgs& q, double d, double& phiMag, double& AMag)
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
    const int off = profile_at(q, distance, phiMag, AMag);
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
    q.m = prof->m;
    q.a = prof->h;
    q.winding = prof->winding;
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
    q.S0 = S0;
    q.S1 = S1;
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
