// Abelian-Higgs FP64 steps that allocate no device memory.
//
// lat_step() keeps its per-site link data (cos/sin of the link phases and the
// plaquette sines, see ah_twopass.cuh) in a buffer the handle allocates.
// Some callers cannot let a library allocate: a host application that owns all
// device memory through its own pool or a fixed budget and embeds the step in
// its own solver loop, or a tight stepping loop that cannot pay for
// cudaMalloc's implicit synchronisation of the whole device.  For them
// lat_ah_step_f64_noalloc() runs the same two-pass step, with the same
// launchers and therefore the same doubles as lat_step on a handle of the same
// precision (LAT_F64 or LAT_F64_FAST), on fields the caller owns, with the link
// data in the fixed array below.  The array is part of the library image:
// every GPU that loads the library holds it (LAT_NOALLOC_MAX_SITES * 15
// doubles = 31.5 MiB) until the process exits.
#include <cuda.h>

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

// The device address of g_noalloc_links belongs to the context the module was
// loaded into.  It is looked up once per context: the cache below is keyed on
// the device ordinal and the current context's ID, which the driver never
// reuses within a process.  A cudaDeviceReset (a new primary context) or a
// caller's own driver-API context made current therefore gets its own lookup.
struct AddrCache {
    unsigned long long ctx_id;
    double* addr;
};
std::mutex g_mu;
AddrCache g_cache[kMaxDevices] = {};

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// ID of the context current on this thread; false when there is none yet or
// the driver does not provide the calls.  The driver's entry points are
// fetched through the runtime, so the library does not link libcuda itself.
bool current_context_id(unsigned long long* id)
{
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<CtxGetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(f);
    });
    if (!get_current || !get_id) return false;
    CUcontext ctx = nullptr;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return false;
    return get_id(ctx, id) == CUDA_SUCCESS;
}

// Device address of g_noalloc_links in the current context.  The name of a
// __device__ variable in host code is only a host-side stand-in, so the
// address is asked of the runtime, with the caller's device current.
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
    unsigned long long id = 0;
    bool have_id = current_context_id(&id);
    std::lock_guard<std::mutex> lock(g_mu);
    if (have_id && g_cache[dev].addr && g_cache[dev].ctx_id == id) {
        *out = g_cache[dev].addr;
        return LAT_OK;
    }
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_links);
    if (e != cudaSuccess || !p) {
        set_error(std::string("lat_ah_step_f64_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        return LAT_ERR_CUDA;
    }
    // the lookup made the device's primary context current if none was
    if (!have_id) have_id = current_context_id(&id);
    g_cache[dev] = have_id ? AddrCache{id, static_cast<double*>(p)} : AddrCache{0, nullptr};
    *out = static_cast<double*>(p);
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
    int rc = validate_params(p);
    if (rc) return rc;
    if (p->model != LAT_MODEL_AH || (p->precision != LAT_F64 && p->precision != LAT_F64_FAST) ||
        p->kernel_variant != 0 || p->bc > LAT_BC_FIXED || bc_z_kind(*p) > LAT_BC_FIXED) {
        set_error("lat_ah_step_f64_noalloc: needs an Abelian-Higgs LAT_F64 or LAT_F64_FAST parameter block "
                  "with periodic or fixed walls and kernel_variant 0");
        return LAT_ERR_INVALID;
    }
    const int64_t N = p->nx * p->ny * p->nz;
    if (N > kMaxSites) {
        set_error("lat_ah_step_f64_noalloc: " + std::to_string(N) + " sites exceed the fixed scratch of " +
                  std::to_string(kMaxSites) + " sites (LAT_NOALLOC_MAX_SITES); use a lattice handle instead");
        return LAT_ERR_INVALID;
    }
    double* links = nullptr;
    if ((rc = links_address(&links))) return rc;

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
        const StepCoef cf = make_coef(*p, n);
        const cudaError_t e = p->precision == LAT_F64_FAST
                                  ? launch_ah_twopass_fast(g, f, links, cf, d, false, recip, st)
                                  : launch_ah_twopass_strict(g, f, links, cf, d, false, recip, st);
        if (e != cudaSuccess) {
            set_error(std::string("lat_ah_step_f64_noalloc: launch: ") + cudaGetErrorString(e));
            return LAT_ERR_CUDA;
        }
    }
    return LAT_OK;
}
