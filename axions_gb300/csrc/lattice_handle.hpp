// The lattice handle behind the opaque `lat_handle` of the C ABI; shared by
// the translation units that step lattices (lattice_api.cu, batch.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "lattice_internal.cuh"

struct lat_handle {
    lat_params p;
    int ncomp = 0;
    int64_t N = 0;
    size_t elem = 8;
    lat::Geom geom;
    int device = 0;
    cudaStream_t own = nullptr;
    cudaStream_t stream = nullptr;
    int64_t n = 0;             // TimeStep of the "now" level
    bool div_valid = false;    // divbuf holds the divergence of the past level
    // device memory
    void* fields = nullptr;    // [ncomp][2][N]
    void* divbuf = nullptr;    // [N]
    double* links = nullptr;   // two-pass FP64 link data [ah_link_slots()][N]
    size_t links_bytes = 0;
    bool recip = false;        // every spacing is a power of two: exact reciprocals
    int chunk = 32;            // x-planes per CTA of the tiled FP32 kernel
    double* partials = nullptr;
    int nblocks = 0;           // capacity of `partials` in (energy, |G|) pairs
    double* diag_dev = nullptr;
    int64_t diag_cap = 0;
    double* staging = nullptr;  // [N] doubles (FP32 handles)
    long long* det_blocks = nullptr;
    long long* det_total = nullptr;
    int det_nb = 0;
    double* det_xyz = nullptr;
    int64_t det_cap = 0;
    int8_t* wind = nullptr;
    unsigned long long* wind_sum = nullptr;
    lat::ChainBuffers chain;   // string-length buffers
    int64_t bc_level = -1;     // the level whose Neumann layer has been set
    void* btt = nullptr;       // absorbing layer's second time derivatives
    size_t btt_bytes = 0;
    // asynchronous snapshots (snapshot.cu)
    double* snap_dev = nullptr;          // staged copy of the level, [cols][N] doubles
    size_t snap_cap = 0;                 // bytes of snap_dev
    cudaStream_t snap_stream = nullptr;  // device-to-host copies
    cudaEvent_t snap_staged = nullptr;   // staging done (handle stream)
    cudaEvent_t snap_copied = nullptr;   // copy done (snap_stream)
    bool snap_pending = false;
    int64_t bytes = 0;
    int64_t launches = 0;      // kernels launched by this handle

    char* slot(int comp, int t) const { return (char*)fields + ((size_t)comp * 2 + (size_t)t) * (size_t)N * elem; }
};
