// Deterministic reduction of per-block diagnostic partials, the
// double <-> float conversions of the FP32 path, and lat_dtrig_eval (the FP64
// step's sine and cosine on given arguments, for checks).
#include <string>

#include "dtrig.cuh"
#include "lattice_handle.hpp"

namespace lat {

namespace {

// One block sums the (energy, |G|) pairs of all blocks: every thread walks a
// fixed strided subset with Neumaier compensation, then a fixed tree combines
// the threads.  The result does not depend on timing, only on the grid.
__global__ void __launch_bounds__(1024) finalize_kernel(const double* __restrict__ partials, int nblocks,
                                                        double* __restrict__ out)
{
    __shared__ double se[1024], sg[1024];
    double e = 0, ce = 0, g = 0, cg = 0;
    for (int b = threadIdx.x; b < nblocks; b += 1024) {
        const double x = partials[2 * b], y = partials[2 * b + 1];
        double t = e + x;
        ce += (fabs(e) >= fabs(x)) ? (e - t) + x : (x - t) + e;
        e = t;
        t = g + y;
        cg += (fabs(g) >= fabs(y)) ? (g - t) + y : (y - t) + g;
        g = t;
    }
    se[threadIdx.x] = e + ce;
    sg[threadIdx.x] = g + cg;
    __syncthreads();
    for (int w = 512; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            se[threadIdx.x] += se[threadIdx.x + w];
            sg[threadIdx.x] += sg[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = se[0];
        out[1] = sg[0];
    }
}

__global__ void d2f_kernel(const double* __restrict__ in, float* __restrict__ out, int64_t n)
{
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        out[q] = (float)in[q];
}

__global__ void f2d_kernel(const float* __restrict__ in, double* __restrict__ out, int64_t n)
{
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        out[q] = (double)in[q];
}

// the FP64 step's dsin/dsincos and CUDA's sin/cos on the same arguments
__global__ void dtrig_kernel(const double* __restrict__ x, int64_t n, double* __restrict__ out)
{
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const double v = x[q];
        double s, c;
        dsincos(v, &s, &c);
        out[q] = dsin(v);
        out[n + q] = s;
        out[2 * n + q] = c;
        out[3 * n + q] = ::sin(v);
        out[4 * n + q] = ::cos(v);
    }
}

inline unsigned grid_for(int64_t n)
{
    int64_t b = (n + 255) / 256;
    if (b > 152 * 32) b = 152 * 32;
    return (unsigned)(b < 1 ? 1 : b);
}

}  // namespace

cudaError_t launch_finalize(const double* partials, int nblocks, double* out, cudaStream_t st)
{
    finalize_kernel<<<1, 1024, 0, st>>>(partials, nblocks, out);
    return cudaGetLastError();
}

cudaError_t launch_d2f(const double* in, float* out, int64_t n, cudaStream_t st)
{
    d2f_kernel<<<grid_for(n), 256, 0, st>>>(in, out, n);
    return cudaGetLastError();
}

cudaError_t launch_f2d(const float* in, double* out, int64_t n, cudaStream_t st)
{
    f2d_kernel<<<grid_for(n), 256, 0, st>>>(in, out, n);
    return cudaGetLastError();
}

}  // namespace lat

using namespace lat;

extern "C" int lat_dtrig_eval(const double* x, int64_t n, double* out)
{
    if (!x || !out || n < 0 || n > ((int64_t)1 << 26)) {
        set_error("lat_dtrig_eval: null pointer or n outside [0, 2^26]");
        return LAT_ERR_INVALID;
    }
    if (n == 0) return LAT_OK;
    double* d = nullptr;
    cudaError_t e = cudaMalloc((void**)&d, sizeof(double) * 6 * (size_t)n);
    if (e == cudaSuccess) e = cudaMemcpy(d, x, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        dtrig_kernel<<<grid_for(n), 256>>>(d, n, d + n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, d + n, sizeof(double) * 5 * (size_t)n, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) {
        set_error(std::string("lat_dtrig_eval: ") + cudaGetErrorString(e));
        return LAT_ERR_CUDA;
    }
    return LAT_OK;
}
