// Abelian-Higgs FP64 steps that allocate no device memory.
//
// lat_step() keeps its per-site link data (cos/sin of the link phases and the
// plaquette sines, see ah_twopass.cuh) in a buffer the handle allocates.
// Some callers cannot let a library allocate: a host application that owns all
// device memory through its own pool or a fixed budget and embeds the step in
// its own solver loop, or a tight stepping loop that cannot pay for
// cudaMalloc's implicit synchronisation of the whole device.  For them
// lat_ah_step_f64_noalloc() runs the same two-pass step (strict FP64, the
// reference's rounding) on fields the caller owns, with the link data in the
// fixed array below.  The array is part of the library image: every GPU that
// loads the library holds it (LAT_NOALLOC_MAX_SITES * 15 doubles = 31.5 MiB)
// until the process exits.
//
// This file is compiled with -fmad=false like the other strict FP64 kernels.
#include <cmath>
#include <mutex>
#include <string>

#include "ah_twopass.cuh"

namespace lat {

namespace {

constexpr long long kMaxSites = LAT_NOALLOC_MAX_SITES;
constexpr int kMaxDevices = 64;

// Link data of the calls below: L_COUNT slots of kMaxSites doubles.  Shared by
// every call on a device and left holding the last call's values; pass 1
// overwrites every slot the update reads before it is read, so nothing has to
// be cleared between calls.
static __device__ __align__(256) double g_noalloc_links[L_COUNT * kMaxSites];

std::mutex g_mu;
double* g_links_addr[kMaxDevices] = {};

// Device address of g_noalloc_links on the current device.  The name of a
// __device__ variable in host code is only a host-side stand-in, so the
// address is looked up once per device, with that device current.
int links_address(double** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        set_error(std::string("lat_ah_step_f64_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
        return LAT_ERR_NODEVICE;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("lat_ah_step_f64_noalloc: device ordinal out of range");
        return LAT_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_links_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_links);
        if (e != cudaSuccess || !p) {
            set_error(std::string("lat_ah_step_f64_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            return LAT_ERR_CUDA;
        }
        g_links_addr[dev] = static_cast<double*>(p);
    }
    *out = g_links_addr[dev];
    return LAT_OK;
}

}  // namespace

}  // namespace lat

using namespace lat;

extern "C" int lat_ah_step_f64_noalloc(const lat_params* p, double* fields, int64_t time_step, int32_t nsteps,
                                       void* stream)
{
    if (!p || !fields || nsteps < 0 || time_step < 0) {
        set_error("lat_ah_step_f64_noalloc: null pointer or negative count");
        return LAT_ERR_INVALID;
    }
    if (p->abi_version != LAT_ABI_VERSION || p->model != LAT_MODEL_AH || p->precision != LAT_F64 ||
        (p->bc != LAT_BC_PERIODIC && p->bc != LAT_BC_FIXED) ||
        p->bc_z < LAT_BCZ_AS_XY || p->bc_z > LAT_BCZ_NEUMANN ||
        (bc_z_kind(*p) != LAT_BC_PERIODIC && bc_z_kind(*p) != LAT_BC_FIXED)) {
        set_error("lat_ah_step_f64_noalloc: needs an Abelian-Higgs LAT_F64 parameter block");
        return LAT_ERR_INVALID;
    }
    const int64_t mn = (p->bc == LAT_BC_FIXED || bc_z_kind(*p) == LAT_BC_FIXED) ? 3 : 2;
    if (p->nx < mn || p->ny < mn || p->nz < mn || !(p->dx > 0 && p->dy > 0 && p->dz > 0 && p->dt > 0)) {
        set_error("lat_ah_step_f64_noalloc: bad lattice sides or spacings");
        return LAT_ERR_INVALID;
    }
    const int64_t N = p->nx * p->ny * p->nz;
    if (N > kMaxSites) {
        set_error("lat_ah_step_f64_noalloc: " + std::to_string(N) + " sites exceed the fixed scratch of " +
                  std::to_string(kMaxSites) + " sites (LAT_NOALLOC_MAX_SITES); use a lattice handle instead");
        return LAT_ERR_INVALID;
    }
    double* links = nullptr;
    int rc = links_address(&links);
    if (rc) return rc;

    const Geom g = make_geom(*p);
    auto pow2 = [](double v) {
        int e;
        return std::frexp(v, &e) == 0.5;
    };
    const bool recip = pow2(p->dx) && pow2(p->dy) && pow2(p->dz);
    DiagOut d = {};
    d.write = 1;
    d.energy_form = p->energy_form;
    cudaStream_t st = (cudaStream_t)stream;
    for (int32_t q = 0; q < nsteps; ++q) {
        const int64_t n = time_step + q;
        const int tNow = (int)((n + 1) % 2), tPast = (int)(n % 2);
        Fields<double, 5> f;
        for (int c = 0; c < 5; ++c) {
            f.now[c] = fields + ((size_t)c * 2 + (size_t)tNow) * (size_t)N;
            f.past[c] = fields + ((size_t)c * 2 + (size_t)tPast) * (size_t)N;
        }
        cudaError_t e = launch_ah_twopass<true>(g, f, links, make_coef(*p, n), d, false, recip, st);
        if (e != cudaSuccess) {
            set_error(std::string("lat_ah_step_f64_noalloc: launch: ") + cudaGetErrorString(e));
            return LAT_ERR_CUDA;
        }
    }
    return LAT_OK;
}
