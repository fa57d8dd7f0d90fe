// Asynchronous snapshots of the current level (lat_snapshot_*).
//
// The reference writes |phi|^2 volumes and final fields from host arrays in the
// middle of its step loop (evolution.cpp:1423-1441, mooreEvol.cpp:700-718).
// Here the values are staged on the device by the handle's stream (so the
// level is read before any later step overwrites its slot) and copied to the
// caller's buffer on a second stream, overlapped with the steps that follow.
// Compiled with -fmad=false: |phi|^2 is re*re + im*im rounded as the reference's
// pow(re,2) + pow(im,2).
#include <cuda_runtime.h>

#include <string>

#include "lattice_handle.hpp"

namespace lat {
namespace {

template <class T>
__global__ void magnitude_kernel(const T* __restrict__ re, const T* __restrict__ im, double* __restrict__ out,
                                 int64_t n)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double a = (double)re[i], b = (double)im[i];
    out[i] = a * a + b * b;
}

__global__ void widen_kernel(const float* __restrict__ in, double* __restrict__ out, int64_t n)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (double)in[i];
}

int fail_cuda(const char* what, cudaError_t e)
{
    set_error(std::string("snapshot: ") + what + ": " + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? LAT_ERR_NOMEM : LAT_ERR_CUDA;
}

#define SN_CK(call)                                      \
    do {                                                 \
        const cudaError_t e_ = (call);                   \
        if (e_ != cudaSuccess) return fail_cuda(#call, e_); \
    } while (0)

int64_t cols_of(const lat_handle* h, int32_t kind)
{
    if (kind == LAT_SNAP_MAGNITUDE) return h->p.model == LAT_MODEL_MOORE ? 2 : 1;
    if (kind == LAT_SNAP_LEVEL) return h->ncomp;
    return -1;
}

}  // namespace
}  // namespace lat

extern "C" {

int64_t lat_snapshot_doubles(const lat_handle* h, int32_t kind)
{
    if (!h) return LAT_ERR_INVALID;
    const int64_t c = lat::cols_of(h, kind);
    return c < 0 ? (int64_t)LAT_ERR_INVALID : c * h->N;
}

int lat_snapshot_wait(lat_handle* h)
{
    using namespace lat;
    if (!h) {
        set_error("lat_snapshot_wait: null handle");
        return LAT_ERR_INVALID;
    }
    if (!h->snap_pending) return LAT_OK;
    SN_CK(cudaSetDevice(h->device));
    h->snap_pending = false;
    SN_CK(cudaEventSynchronize(h->snap_copied));
    return LAT_OK;
}

int lat_snapshot_begin(lat_handle* h, int32_t kind, double* dst)
{
    using namespace lat;
    if (!h || !dst || cols_of(h, kind) < 0) {
        set_error("lat_snapshot_begin: null handle or destination, or unknown kind");
        return LAT_ERR_INVALID;
    }
    int rc = lat_snapshot_wait(h);  // the staging buffer is free again
    if (rc) return rc;
    SN_CK(cudaSetDevice(h->device));
    if (!h->snap_stream) {
        SN_CK(cudaStreamCreateWithFlags(&h->snap_stream, cudaStreamNonBlocking));
        SN_CK(cudaEventCreateWithFlags(&h->snap_staged, cudaEventDisableTiming));
        SN_CK(cudaEventCreateWithFlags(&h->snap_copied, cudaEventDisableTiming));
    }
    const int64_t cols = cols_of(h, kind), N = h->N;
    const size_t bytes = sizeof(double) * (size_t)cols * (size_t)N;
    if (bytes > h->snap_cap) {
        if (h->snap_dev) {
            cudaFree(h->snap_dev);
            h->bytes -= (int64_t)h->snap_cap;
            h->snap_dev = nullptr;
            h->snap_cap = 0;
        }
        SN_CK(cudaMalloc(&h->snap_dev, bytes));
        h->snap_cap = bytes;
        h->bytes += (int64_t)bytes;
    }
    const int tNow = (int)((h->n + 1) % 2);
    const int tb = 256;
    const unsigned blocks = (unsigned)((N + tb - 1) / tb);
    for (int64_t c = 0; c < cols; ++c) {
        double* out = h->snap_dev + c * N;
        if (kind == LAT_SNAP_MAGNITUDE) {
            const int re = (int)(2 * c), im = (int)(2 * c + 1);
            if (h->elem == 8)
                magnitude_kernel<double><<<blocks, tb, 0, h->stream>>>((const double*)h->slot(re, tNow),
                                                                       (const double*)h->slot(im, tNow), out, N);
            else
                magnitude_kernel<float><<<blocks, tb, 0, h->stream>>>((const float*)h->slot(re, tNow),
                                                                      (const float*)h->slot(im, tNow), out, N);
            ++h->launches;
        } else if (h->elem == 8) {
            SN_CK(cudaMemcpyAsync(out, h->slot((int)c, tNow), sizeof(double) * (size_t)N, cudaMemcpyDeviceToDevice,
                                  h->stream));
        } else {
            widen_kernel<<<blocks, tb, 0, h->stream>>>((const float*)h->slot((int)c, tNow), out, N);
            ++h->launches;
        }
    }
    SN_CK(cudaGetLastError());
    SN_CK(cudaEventRecord(h->snap_staged, h->stream));
    SN_CK(cudaStreamWaitEvent(h->snap_stream, h->snap_staged, 0));
    SN_CK(cudaMemcpyAsync(dst, h->snap_dev, bytes, cudaMemcpyDeviceToHost, h->snap_stream));
    SN_CK(cudaEventRecord(h->snap_copied, h->snap_stream));
    h->snap_pending = true;
    return LAT_OK;
}

void* lat_host_alloc(int64_t bytes)
{
    void* p = nullptr;
    if (bytes <= 0 || cudaMallocHost(&p, (size_t)bytes) != cudaSuccess) {
        lat::set_error("lat_host_alloc: cudaMallocHost failed");
        return nullptr;
    }
    return p;
}

void lat_host_free(void* ptr)
{
    if (ptr) cudaFreeHost(ptr);
}

}  // extern "C"
