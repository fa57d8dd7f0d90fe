// Random-phase initial conditions generated on the device.
//
// The reference draws one phase per site from std::mt19937 in linear order
// (mpi_evolution.cpp:287-312); lat_random_phase_ic() reproduces that sequence on
// the host, which costs tens of nanoseconds per site and an upload.  For
// ensembles and served jobs, where the reference's exact sequence is not
// needed, lat_random_phase_ic_device() draws the phases on the GPU with the
// counter-based generator Philox-4x32-10 (Salmon, Moraes, Dror and Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC11): site s uses counter
// (s, 0, 0, 0) and key (seed low, seed high) and takes its phase(s) from the
// four 32-bit outputs.  Same physics as the reference IC: phi = eta*e^{i phase},
// phase uniform in [0, 2 pi), both time levels equal, link phases zero.
#include <cmath>
#include <string>

#include "lattice_handle.hpp"

namespace lat {

namespace {

__host__ __device__ inline void philox_round(uint32_t c[4], const uint32_t k[2])
{
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    const uint32_t n0 = hi1 ^ c[1] ^ k[0];
    const uint32_t n2 = hi0 ^ c[3] ^ k[1];
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
}

__host__ __device__ inline void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1)
{
    uint32_t k[2] = {k0, k1};
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k[0] += 0x9E3779B9u;
            k[1] += 0xBB67AE85u;
        }
        philox_round(c, k);
    }
}

// 53-bit uniform in [0, 1) from two 32-bit words
__host__ __device__ inline double u01(uint32_t a, uint32_t b)
{
    return (double)(((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6)) * (1.0 / 9007199254740992.0);
}

template <class T>
__global__ void phase_ic_kernel(int64_t N, uint32_t k0, uint32_t k1, int independent, double eta, double eta2,
                                int moore, T* now_re1, T* now_im1, T* past_re1, T* past_im1, T* now_re2, T* now_im2,
                                T* past_re2, T* past_im2)
{
    const double two_pi = 2.0 * 3.14159265358979323846;
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < N; s += (int64_t)gridDim.x * blockDim.x) {
        uint32_t c[4] = {(uint32_t)s, (uint32_t)((uint64_t)s >> 32), 0u, 0u};
        philox4x32_10(c, k0, k1);
        const double ph1 = two_pi * u01(c[0], c[1]);
        double sn, cs;
        sincos(ph1, &sn, &cs);
        now_re1[s] = past_re1[s] = (T)(eta * cs);
        now_im1[s] = past_im1[s] = (T)(eta * sn);
        if (moore) {
            const double ph2 = independent ? two_pi * u01(c[2], c[3]) : ph1;
            sincos(ph2, &sn, &cs);
            now_re2[s] = past_re2[s] = (T)(eta2 * cs);
            now_im2[s] = past_im2[s] = (T)(eta2 * sn);
        }
    }
}

}  // namespace

// Host copy of the generator, for checks.
void philox4x32_10_host(uint32_t c[4], uint32_t k0, uint32_t k1) { philox4x32_10(c, k0, k1); }

}  // namespace lat

using namespace lat;

extern "C" {

int lat_random_phase_ic_device(lat_handle* h, uint64_t seed, int32_t independent)
{
    if (!h) {
        set_error("lat_random_phase_ic_device: null handle");
        return LAT_ERR_INVALID;
    }
    cudaError_t e = cudaSetDevice(h->device);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->fields, 0, (size_t)h->ncomp * 2 * (size_t)h->N * h->elem, h->stream);
    if (e != cudaSuccess) {
        set_error(std::string("lat_random_phase_ic_device: ") + cudaGetErrorString(e));
        return LAT_ERR_CUDA;
    }
    h->n = 0;
    h->bc_level = -1;  // new values: their Neumann layer is not set yet
    h->div_valid = false;
    const int tNow = 1, tPast = 0;  // level 0: now in slot 1, past in slot 0
    const int moore = h->p.model == LAT_MODEL_MOORE;
    const int threads = 256;
    int64_t blocks = (h->N + threads - 1) / threads;
    if (blocks > 152 * 64) blocks = 152 * 64;
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    if (h->elem == 8) {
        auto sl = [&](int c, int t) { return (double*)h->slot(c, t); };
        phase_ic_kernel<double><<<(unsigned)blocks, threads, 0, h->stream>>>(
            h->N, k0, k1, independent, h->p.eta, h->p.eta2, moore, sl(0, tNow), sl(1, tNow), sl(0, tPast), sl(1, tPast),
            moore ? sl(2, tNow) : nullptr, moore ? sl(3, tNow) : nullptr, moore ? sl(2, tPast) : nullptr,
            moore ? sl(3, tPast) : nullptr);
    } else {
        auto sl = [&](int c, int t) { return (float*)h->slot(c, t); };
        phase_ic_kernel<float><<<(unsigned)blocks, threads, 0, h->stream>>>(
            h->N, k0, k1, independent, h->p.eta, h->p.eta2, moore, sl(0, tNow), sl(1, tNow), sl(0, tPast), sl(1, tPast),
            moore ? sl(2, tNow) : nullptr, moore ? sl(3, tNow) : nullptr, moore ? sl(2, tPast) : nullptr,
            moore ? sl(3, tPast) : nullptr);
    }
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) {
        set_error(std::string("lat_random_phase_ic_device: ") + cudaGetErrorString(e));
        return LAT_ERR_CUDA;
    }
    h->launches += 1;
    return LAT_OK;
}

// Philox-4x32-10 on the host (the generator of lat_random_phase_ic_device), for
// callers that want to check or reproduce device ICs.
int lat_philox4x32_10(const uint32_t counter[4], const uint32_t key[2], uint32_t out[4])
{
    if (!counter || !key || !out) {
        set_error("lat_philox4x32_10: null argument");
        return LAT_ERR_INVALID;
    }
    uint32_t c[4] = {counter[0], counter[1], counter[2], counter[3]};
    philox4x32_10_host(c, key[0], key[1]);
    for (int q = 0; q < 4; ++q) out[q] = c[q];
    return LAT_OK;
}

}  // extern "C"
