// C ABI of liblattice_gpu.so (include/lattice_gpu.h): handle management,
// state transfer and the per-step orchestration that replaces the body of the
// reference's time-step loop (mpi_evolution.cpp:354-985 and its relatives).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "lattice_handle.hpp"
#include "lattice_internal.cuh"

namespace lat {

thread_local std::string g_err;
void set_error(const std::string& m) { g_err = m; }

int bc_z_kind(const lat_params& p)
{
    switch (p.bc_z) {
    case LAT_BCZ_PERIODIC: return LAT_BC_PERIODIC;
    case LAT_BCZ_FIXED: return LAT_BC_FIXED;
    case LAT_BCZ_NEUMANN: return LAT_BC_NEUMANN;
    default: return p.bc;
    }
}

// evolution.cpp:166-186: a periodic axis evolves every site, any other kind
// its interior (Neumann and absorbing layers are set or evolved separately)
Geom make_geom(const lat_params& p)
{
    Geom g;
    g.nx = (int)p.nx;
    g.ny = (int)p.ny;
    g.nz = (int)p.nz;
    g.syz = g.ny * g.nz;
    const bool pxy = p.bc == LAT_BC_PERIODIC, pz = bc_z_kind(p) == LAT_BC_PERIODIC;
    g.lox = g.loy = pxy ? 0 : 1;
    g.hix = pxy ? g.nx : g.nx - 1;
    g.hiy = pxy ? g.ny : g.ny - 1;
    g.loz = pz ? 0 : 1;
    g.hiz = pz ? g.nz : g.nz - 1;
    return g;
}

// Coefficients of step n, each evaluated like the reference expression it
// stands for (mpi_evolution.cpp:356-368,412-501; evolution.cpp:377-427).
StepCoef make_coef(const lat_params& p, int64_t n)
{
    StepCoef c;
    c.dx2 = p.dx * p.dx;
    c.dy2 = p.dy * p.dy;
    c.dz2 = p.dz * p.dz;
    c.dt = p.dt;
    c.dt2 = p.dt * p.dt;
    c.halfLambda = 0.5 * p.lambda;
    c.etaSq = p.eta * p.eta;
    c.halfLambda2 = 0.5 * p.lambda2;
    c.eta2Sq = p.eta2 * p.eta2;
    c.halfLambda12 = 0.5 * p.lambda12;
    c.m2gg = -2 * p.g * p.g;
    const double time = p.tau0 + n * p.dt;  // conformal time, mpi_evolution.cpp:356
    const double damp = (n < p.damped_nt) ? p.dampFac : 0;
    c.damp = damp;
    c.fric = damp + p.alpha * p.scaling / time;
    c.q1 = p.q1;
    c.q2 = p.q2;
    c.dx = p.dx;
    c.dy = p.dy;
    c.dz = p.dz;
    c.g = p.g;
    c.gdtdx = p.g * p.dt * p.dx;
    c.gdtdy = p.g * p.dt * p.dy;
    c.gdtdz = p.g * p.dt * p.dz;
    const double gxy = p.g * p.dx * p.dy, gxz = p.g * p.dx * p.dz, gyz = p.g * p.dy * p.dz;
    c.gxy2 = gxy * gxy;
    c.gxz2 = gxz * gxz;
    c.gyz2 = gyz * gyz;
    c.dV = p.dx * p.dy * p.dz;
    c.quarterLambda = 0.25 * p.lambda;
    c.quarterLambda2 = 0.25 * p.lambda2;
    c.halfLambda12e = 0.5 * p.lambda12;
    c.twog = 2 * p.g;
    c.inv_dx2 = 1.0 / c.dx2;
    c.inv_dy2 = 1.0 / c.dy2;
    c.inv_dz2 = 1.0 / c.dz2;
    c.inv_dt = 1.0 / p.dt;
    c.inv_dx = 1.0 / p.dx;
    c.inv_dy = 1.0 / p.dy;
    c.inv_dz = 1.0 / p.dz;
    c.inv_g = p.g != 0 ? 1.0 / p.g : 0.0;
    c.inv_gdtdx = c.gdtdx != 0 ? 1.0 / c.gdtdx : 0.0;
    c.inv_gdtdy = c.gdtdy != 0 ? 1.0 / c.gdtdy : 0.0;
    c.inv_gdtdz = c.gdtdz != 0 ? 1.0 / c.gdtdz : 0.0;
    c.inv_gxy2 = c.gxy2 != 0 ? 1.0 / c.gxy2 : 0.0;
    c.inv_gxz2 = c.gxz2 != 0 ? 1.0 / c.gxz2 : 0.0;
    c.inv_gyz2 = c.gyz2 != 0 ? 1.0 / c.gyz2 : 0.0;
    c.iso = (p.dx == p.dy && p.dx == p.dz) ? 1.0 : 0.0;
    c.fric_dt = c.fric / p.dt;
    return c;
}

}  // namespace lat

using namespace lat;


#define LAT_CK(call)                                                                             \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess) {                                                                 \
            set_error(std::string(#call) + ": " + cudaGetErrorString(e_));                       \
            return e_ == cudaErrorMemoryAllocation ? LAT_ERR_NOMEM                               \
                   : (e_ == cudaErrorNoDevice || e_ == cudaErrorInsufficientDriver ||            \
                      e_ == cudaErrorNoKernelImageForDevice) ? LAT_ERR_NODEVICE : LAT_ERR_CUDA;  \
        }                                                                                        \
    } while (0)

// a kernel launch: checked and counted
#define LAT_CKL(call)      \
    do {                   \
        LAT_CK(call);      \
        ++h->launches;     \
    } while (0)

#define LAT_REQUIRE(cond, msg)       \
    do {                             \
        if (!(cond)) {               \
            set_error(msg);          \
            return LAT_ERR_INVALID;  \
        }                            \
    } while (0)

static int dev_alloc(lat_handle* h, void** ptr, size_t bytes)
{
    LAT_CK(cudaMalloc(ptr, bytes));
    h->bytes += (int64_t)bytes;
    return LAT_OK;
}

static void dev_free(lat_handle* h, void** ptr, size_t bytes)
{
    if (*ptr) {
        cudaFree(*ptr);
        h->bytes -= (int64_t)bytes;
        *ptr = nullptr;
    }
}

extern "C" {

const char* lat_version(void) { return "axions_gb300 lattice 1.0 (sm_103a)"; }

const char* lat_last_error(void) { return g_err.c_str(); }

int lat_params_init(lat_params* p, int32_t model)
{
    LAT_REQUIRE(p, "lat_params_init: null");
    LAT_REQUIRE(model == LAT_MODEL_AH || model == LAT_MODEL_MOORE, "lat_params_init: unknown model");
    std::memset(p, 0, sizeof(*p));
    p->abi_version = LAT_ABI_VERSION;
    p->model = model;
    p->precision = LAT_F64;
    p->bc = LAT_BC_PERIODIC;
    p->nx = p->ny = p->nz = 1001;
    p->dx = p->dy = p->dz = 0.25;
    p->dt = 0.05;
    p->damped_nt = 200;
    p->dampFac = 0.5;
    p->alpha = 3;
    p->scaling = 1;
    p->tau0 = 1;
    p->energy_form = LAT_ENERGY_MPI;
    p->moore_current = LAT_MOORE_CURRENT_PLAIN;
    if (model == LAT_MODEL_AH) {  // mpi_evolution.cpp:28-30
        p->lambda = 1;
        p->eta = 1;
        p->g = 0 * std::sqrt(0.5 * p->lambda);
        p->q1 = 1;
    } else {  // moore_mpi_evolution.cpp:28-35
        p->lambda = 1;
        p->lambda2 = 1;
        p->lambda12 = 0;
        p->eta = 1;
        p->eta2 = 1;
        p->q1 = 2;
        p->q2 = p->q1 - 1;
        p->g = std::sqrt(0.5 * p->lambda * std::pow(p->eta, 2) / (p->q1 * p->q1 + p->q2 * p->q2));
    }
    return LAT_OK;
}

}  // extern "C"

// Checks shared by every entry point that takes a parameter block (also the
// allocation-free step, noalloc.cu).
int lat::validate_params(const lat_params* p)
{
    LAT_REQUIRE(p, "null params");
    LAT_REQUIRE(p->abi_version == LAT_ABI_VERSION, "lat_params.abi_version mismatch");
    LAT_REQUIRE(p->model == LAT_MODEL_AH || p->model == LAT_MODEL_MOORE, "unknown model");
    LAT_REQUIRE(p->precision == LAT_F64 || p->precision == LAT_F32 || p->precision == LAT_F64_FAST,
                "unknown precision");
    LAT_REQUIRE(p->kernel_variant == 0 || p->kernel_variant == 1 ||
                    ((p->kernel_variant == 2 || p->kernel_variant == 3) && p->precision == LAT_F32),
                "unknown kernel_variant (2 and 3 are for FP32 only)");
    LAT_REQUIRE(p->bc >= LAT_BC_PERIODIC && p->bc <= LAT_BC_ABSORBING, "unknown boundary condition");
    LAT_REQUIRE(p->bc_z >= LAT_BCZ_AS_XY && p->bc_z <= LAT_BCZ_NEUMANN, "unknown bc_z");
    const int kz = bc_z_kind(*p);
    LAT_REQUIRE(kz != LAT_BC_ABSORBING, "absorbing boundaries are for x and y only (set bc_z)");
    // mooreEvol.cpp:114-160 has Neumann x/y walls; its absorbing code is not written (:42, :402)
    LAT_REQUIRE(p->model == LAT_MODEL_AH || ((p->bc <= LAT_BC_NEUMANN) && kz <= LAT_BC_FIXED),
                "the Moore model provides periodic, fixed or Neumann x/y and periodic or fixed z boundaries");
    // the reference's z-Neumann pass runs over x planes i < nz (evolution.cpp:250): beyond nx it
    // would leave the array
    LAT_REQUIRE(kz != LAT_BC_NEUMANN || p->nz <= p->nx, "a Neumann z boundary needs nz <= nx");
    const int64_t mxy = p->bc == LAT_BC_PERIODIC ? 2 : 3, mz = kz == LAT_BC_PERIODIC ? 2 : 3;
    LAT_REQUIRE(p->nx >= mxy && p->ny >= mxy && p->nz >= mz, "lattice sides too small for the boundary condition");
    LAT_REQUIRE(p->nx <= 65535 + (p->bc == LAT_BC_PERIODIC ? 0 : 2), "nx above 65535 (grid z-dimension limit)");
    // each product is formed only once its factors are known to keep it in int64
    LAT_REQUIRE(p->ny < ((int64_t)1 << 31) && p->nz < ((int64_t)1 << 31) && p->ny * p->nz < ((int64_t)1 << 31) - 1 &&
                    p->nx * (p->ny * p->nz) < ((int64_t)1 << 31) - 1,
                "nx*ny*nz must be below 2^31");
    LAT_REQUIRE(p->dx > 0 && p->dy > 0 && p->dz > 0 && p->dt > 0, "spacings and dt must be positive");
    LAT_REQUIRE(std::isfinite(p->tau0) && p->tau0 > 0, "tau0 must be positive");
    LAT_REQUIRE(p->energy_form == LAT_ENERGY_EVOLUTION || p->energy_form == LAT_ENERGY_MPI, "unknown energy_form");
    LAT_REQUIRE(p->moore_current == LAT_MOORE_CURRENT_PLAIN || p->moore_current == LAT_MOORE_CURRENT_CHARGE,
                "unknown moore_current");
    return LAT_OK;
}

extern "C" {

static int validate(const lat_params* p) { return validate_params(p); }

// Device bytes lat_create allocates for `p` (the same terms as below).
static int64_t footprint(const lat_params& p)
{
    const int64_t N = p.nx * p.ny * p.nz;
    const int64_t elem = p.precision == LAT_F32 ? 4 : 8;
    const int64_t ncomp = p.model == LAT_MODEL_MOORE ? 7 : 5;
    int64_t b = ncomp * 2 * N * elem + N * elem;  // fields, divbuf
    if (p.model == LAT_MODEL_AH && elem == 8 && p.kernel_variant == 0) b += 8 * (int64_t)ah_link_slots() * N;
    const dim3 gr = site_grid(make_geom(p));
    b += 16 * (int64_t)gr.x * gr.y * gr.z;        // partials
    b += (int64_t)sizeof(long long) + (int64_t)sizeof(unsigned long long);
    return b;
}

int64_t lat_footprint_bytes(const lat_params* p)
{
    int rc = validate(p);
    if (rc) return rc;
    return footprint(*p);
}

int lat_create(const lat_params* p, lat_handle** out)
{
    int rc = validate(p);
    if (rc) return rc;
    LAT_REQUIRE(out, "lat_create: null out");
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        set_error(std::string("no CUDA device: ") + cudaGetErrorString(e));
        return LAT_ERR_NODEVICE;
    }
    lat_handle* h = new lat_handle();
    h->p = *p;
    h->ncomp = p->model == LAT_MODEL_MOORE ? 7 : 5;
    h->N = p->nx * p->ny * p->nz;
    h->elem = p->precision == LAT_F32 ? 4 : 8;
    auto pow2 = [](double v) {
        int e;
        return std::frexp(v, &e) == 0.5;
    };
    h->recip = pow2(p->dx) && pow2(p->dy) && pow2(p->dz);
    h->geom = make_geom(*p);
    h->chunk = default_chunk(*p);
    cudaGetDevice(&h->device);
    auto fail = [&](int code) {
        lat_destroy(h);
        return code;
    };
    if (cudaStreamCreateWithFlags(&h->own, cudaStreamNonBlocking) != cudaSuccess) {
        set_error("cudaStreamCreate failed");
        delete h;
        return LAT_ERR_CUDA;
    }
    h->stream = h->own;
    if ((rc = dev_alloc(h, &h->fields, (size_t)h->ncomp * 2 * h->N * h->elem))) return fail(rc);
    if ((rc = dev_alloc(h, &h->divbuf, (size_t)h->N * h->elem))) return fail(rc);
    if (p->model == LAT_MODEL_AH && h->elem == 8 && p->kernel_variant == 0) {
        h->links_bytes = sizeof(double) * (size_t)ah_link_slots() * (size_t)h->N;
        if ((rc = dev_alloc(h, (void**)&h->links, h->links_bytes))) return fail(rc);
    }
    const dim3 gr = site_grid(h->geom);
    h->nblocks = (int)(gr.x * gr.y * gr.z);
    if ((rc = dev_alloc(h, (void**)&h->partials, sizeof(double) * 2 * (size_t)h->nblocks))) return fail(rc);
    if ((rc = dev_alloc(h, (void**)&h->det_total, sizeof(long long)))) return fail(rc);
    if ((rc = dev_alloc(h, (void**)&h->wind_sum, sizeof(unsigned long long)))) return fail(rc);
    if (cudaMemsetAsync(h->fields, 0, (size_t)h->ncomp * 2 * h->N * h->elem, h->stream) != cudaSuccess ||
        cudaStreamSynchronize(h->stream) != cudaSuccess) {
        set_error("initial memset failed");
        return fail(LAT_ERR_CUDA);
    }
    *out = h;
    return LAT_OK;
}

}  // extern "C"

namespace lat {

// Give an existing lattice new parameters of the same shape (model,
// precision, boundaries, sides, kernels): the serving loop reuses idle
// lattices this way instead of freeing and allocating device memory.  The
// state is left as is; TimeStep restarts at 0.
int reconfigure_handle(lat_handle* h, const lat_params* p)
{
    int rc = validate(p);
    if (rc) return rc;
    LAT_REQUIRE(h, "reconfigure: null handle");
    LAT_REQUIRE(p->model == h->p.model && p->precision == h->p.precision && p->bc == h->p.bc && p->bc_z == h->p.bc_z && p->nx == h->p.nx &&
                    p->ny == h->p.ny && p->nz == h->p.nz && p->kernel_variant == h->p.kernel_variant,
                "reconfigure: different shape");
    h->p = *p;
    h->n = 0;
    h->bc_level = -1;  // new values: their Neumann layer is not set yet
    h->div_valid = false;
    auto pow2 = [](double v) {
        int e;
        return std::frexp(v, &e) == 0.5;
    };
    h->recip = pow2(p->dx) && pow2(p->dy) && pow2(p->dz);
    return LAT_OK;
}

}  // namespace lat

extern "C" {

int lat_destroy(lat_handle* h)
{
    if (!h) return LAT_OK;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    cudaFree(h->fields);
    cudaFree(h->divbuf);
    cudaFree(h->links);
    cudaFree(h->partials);
    cudaFree(h->diag_dev);
    cudaFree(h->staging);
    cudaFree(h->det_blocks);
    cudaFree(h->det_total);
    cudaFree(h->det_xyz);
    cudaFree(h->wind);
    cudaFree(h->wind_sum);
    chain_buffers_release(h->chain, nullptr);
    cudaFree(h->btt);
    if (h->snap_pending) cudaEventSynchronize(h->snap_copied);
    cudaFree(h->snap_dev);
    if (h->snap_staged) cudaEventDestroy(h->snap_staged);
    if (h->snap_copied) cudaEventDestroy(h->snap_copied);
    if (h->snap_stream) cudaStreamDestroy(h->snap_stream);
    if (h->own) cudaStreamDestroy(h->own);
    delete h;
    return LAT_OK;
}

int lat_set_stream(lat_handle* h, void* stream)
{
    LAT_REQUIRE(h, "null handle");
    h->stream = stream ? (cudaStream_t)stream : h->own;
    return LAT_OK;
}

int lat_get_params(const lat_handle* h, lat_params* out)
{
    LAT_REQUIRE(h && out, "null argument");
    *out = h->p;
    return LAT_OK;
}

int lat_num_components(const lat_handle* h) { return h ? h->ncomp : LAT_ERR_INVALID; }
int64_t lat_time_step(const lat_handle* h) { return h ? h->n : LAT_ERR_INVALID; }
int64_t lat_device_bytes(const lat_handle* h) { return h ? h->bytes : LAT_ERR_INVALID; }
int64_t lat_kernel_launches(const lat_handle* h) { return h ? h->launches : LAT_ERR_INVALID; }

static int ensure_staging(lat_handle* h)
{
    if (!h->staging) return dev_alloc(h, (void**)&h->staging, sizeof(double) * (size_t)h->N);
    return LAT_OK;
}

static int upload_level(lat_handle* h, const double* src, int t)
{
    for (int c = 0; c < h->ncomp; ++c) {
        const double* s = src + (size_t)c * h->N;
        if (h->elem == 8) {
            LAT_CK(cudaMemcpyAsync(h->slot(c, t), s, sizeof(double) * h->N, cudaMemcpyHostToDevice, h->stream));
        } else {
            LAT_CK(cudaMemcpyAsync(h->staging, s, sizeof(double) * h->N, cudaMemcpyHostToDevice, h->stream));
            LAT_CKL(launch_d2f(h->staging, (float*)h->slot(c, t), h->N, h->stream));
        }
    }
    return LAT_OK;
}

static int download_level(lat_handle* h, double* dst, int t)
{
    for (int c = 0; c < h->ncomp; ++c) {
        double* d = dst + (size_t)c * h->N;
        if (h->elem == 8) {
            LAT_CK(cudaMemcpyAsync(d, h->slot(c, t), sizeof(double) * h->N, cudaMemcpyDeviceToHost, h->stream));
        } else {
            LAT_CKL(launch_f2d((const float*)h->slot(c, t), h->staging, h->N, h->stream));
            LAT_CK(cudaMemcpyAsync(d, h->staging, sizeof(double) * h->N, cudaMemcpyDeviceToHost, h->stream));
        }
    }
    return LAT_OK;
}

int lat_set_state(lat_handle* h, const double* now, const double* past, int64_t time_step)
{
    LAT_REQUIRE(h && now && past, "lat_set_state: null argument");
    LAT_REQUIRE(time_step >= 0, "lat_set_state: negative time step");
    LAT_CK(cudaSetDevice(h->device));
    int rc;
    if (h->elem == 4 && (rc = ensure_staging(h))) return rc;
    h->n = time_step;
    h->bc_level = -1;  // new values: their Neumann layer is not set yet
    const int tNow = (int)((time_step + 1) % 2), tPast = (int)(time_step % 2);
    if ((rc = upload_level(h, now, tNow))) return rc;
    if (past == now) {
        // one level for both (a stationary start, mpi_evolution.cpp:155-162):
        // it crosses the host link once and is copied on the device
        for (int c = 0; c < h->ncomp; ++c)
            LAT_CK(cudaMemcpyAsync(h->slot(c, tPast), h->slot(c, tNow), (size_t)h->elem * h->N,
                                   cudaMemcpyDeviceToDevice, h->stream));
    } else if ((rc = upload_level(h, past, tPast))) {
        return rc;
    }
    LAT_CK(cudaStreamSynchronize(h->stream));
    h->div_valid = false;
    return LAT_OK;
}

int lat_get_state(lat_handle* h, double* now, double* past)
{
    LAT_REQUIRE(h, "lat_get_state: null handle");
    LAT_CK(cudaSetDevice(h->device));
    int rc;
    if (h->elem == 4 && (rc = ensure_staging(h))) return rc;
    const int tNow = (int)((h->n + 1) % 2), tPast = (int)(h->n % 2);
    if (now && (rc = download_level(h, now, tNow))) return rc;
    if (past && (rc = download_level(h, past, tPast))) return rc;
    LAT_CK(cudaStreamSynchronize(h->stream));
    return LAT_OK;
}

// One step of the loop body.  diag: compute energy/Gauss of the now level
// into diag_dst[0..1] (device); store_div: keep div(theta) of the now level
// for the next step's Gauss term.
// Neumann layers of the current level (evolution.cpp:194-265), set once per
// level before anything reads it as the reference's loop body does after its
// boundary step: the step, diagnostics, detection, winding, string length.
// get_state and snapshots see the level as stored (the reference's dumps of a
// new level are written before its boundary step).
static int ensure_boundaries(lat_handle* h)
{
    const int kxy = h->p.bc, kz = bc_z_kind(h->p);
    if ((kxy != LAT_BC_NEUMANN && kz != LAT_BC_NEUMANN) || h->bc_level == h->n) return LAT_OK;
    const int tNow = (int)((h->n + 1) % 2);
    void* now[7];
    for (int c = 0; c < h->ncomp; ++c) now[c] = h->slot(c, tNow);
    int nl = 0;
    LAT_CK(launch_neumann(h->geom, h->p.model, h->p.q1, h->p.q2, kxy, kz, (int)h->elem, now, h->stream, &nl));
    h->launches += nl;
    h->bc_level = h->n;
    return LAT_OK;
}

static int do_step(lat_handle* h, bool diag, bool store_div, double* diag_dst, bool write = true)
{
    const lat_params& p = h->p;
    const int tNow = (int)((h->n + 1) % 2), tPast = (int)(h->n % 2);
    int rc = ensure_boundaries(h);
    if (rc) return rc;
    const bool absorb = write && p.bc == LAT_BC_ABSORBING;
    void* nowv[5];
    void* pastv[5];
    if (absorb) {
        for (int c = 0; c < 5; ++c) {
            nowv[c] = h->slot(c, tNow);
            pastv[c] = h->slot(c, tPast);
        }
        const size_t need = absorb_tt_bytes(h->geom, (int)h->elem);
        if (need > h->btt_bytes) {
            dev_free(h, &h->btt, h->btt_bytes);
            h->btt_bytes = 0;
            if ((rc = dev_alloc(h, &h->btt, need))) return rc;
            h->btt_bytes = need;
        }
        // before the interior step overwrites the past level these read
        LAT_CKL(launch_absorb_tt(h->geom, (int)h->elem, nowv, pastv, h->btt, p.dx, p.dy, p.dz, p.dt, h->stream));
    }
    const StepCoef cf = make_coef(p, h->n);
    DiagOut d;
    d.partials = h->partials;
    d.divbuf = h->divbuf;
    d.use_div = 1;
    d.store_div = store_div ? 1 : 0;
    d.energy_form = p.energy_form;
    d.charge_current = p.moore_current == LAT_MOORE_CURRENT_CHARGE;
    d.write = write ? 1 : 0;
    const int th0 = h->ncomp - 3;
    // divergence of the past level's theta for this step's Gauss term
    if (diag && p.g != 0 && !h->div_valid) {
        if (h->elem == 8)
            LAT_CKL(launch_divergence_f64(h->geom, (const double*)h->slot(th0, tPast), (const double*)h->slot(th0 + 1, tPast),
                                         (const double*)h->slot(th0 + 2, tPast), cf, (double*)h->divbuf, h->stream));
        else
            LAT_CKL(launch_divergence_f32(h->geom, (const float*)h->slot(th0, tPast), (const float*)h->slot(th0 + 1, tPast),
                                         (const float*)h->slot(th0 + 2, tPast), cf, (float*)h->divbuf, h->stream));
    }
    int tiled_used = 0;  // CTAs of the x-marching FP32 step, if it ran
    if (p.model == LAT_MODEL_AH) {
        if (h->elem == 8) {
            Fields<double, 5> f;
            for (int c = 0; c < 5; ++c) {
                f.now[c] = (const double*)h->slot(c, tNow);
                f.past[c] = (double*)h->slot(c, tPast);
            }
            if (h->links) {
                LAT_CK(p.precision == LAT_F64_FAST
                           ? launch_ah_twopass_fast(h->geom, f, h->links, cf, d, diag, h->recip, h->stream)
                           : launch_ah_twopass_strict(h->geom, f, h->links, cf, d, diag, h->recip, h->stream));
                h->launches += 2;
            } else {
                LAT_CKL(launch_ah_step_f64(h->geom, f, cf, d, diag, h->stream));
            }
        } else {
            Fields<float, 5> f;
            for (int c = 0; c < 5; ++c) {
                f.now[c] = (const float*)h->slot(c, tNow);
                f.past[c] = (float*)h->slot(c, tPast);
            }
            if (p.kernel_variant != 1)
                LAT_CKL(launch_ah_tiled_f32(h->geom, f, cf, d, diag, h->chunk, h->stream, p.kernel_variant, &tiled_used));
            else LAT_CKL(launch_ah_step_f32(h->geom, f, cf, d, diag, h->stream));
        }
    } else {
        if (h->elem == 8) {
            Fields<double, 7> f;
            for (int c = 0; c < 7; ++c) {
                f.now[c] = (const double*)h->slot(c, tNow);
                f.past[c] = (double*)h->slot(c, tPast);
            }
            LAT_CKL(launch_moore_step_f64(h->geom, f, cf, d, diag, h->stream));
        } else {
            Fields<float, 7> f;
            for (int c = 0; c < 7; ++c) {
                f.now[c] = (const float*)h->slot(c, tNow);
                f.past[c] = (float*)h->slot(c, tPast);
            }
            if (p.kernel_variant != 1)
                LAT_CKL(launch_moore_tiled_f32(h->geom, f, cf, d, diag, h->chunk, h->stream, p.kernel_variant, &tiled_used));
            else LAT_CKL(launch_moore_step_f32(h->geom, f, cf, d, diag, h->stream));
        }
    }
    if (absorb) LAT_CKL(launch_absorb_update(h->geom, (int)h->elem, nowv, pastv, h->btt, p.dt * p.dt, h->stream));
    if (diag) {
        // partials written by the step: one per CTA of the kernel that ran
        const int used = tiled_used > 0 ? tiled_used : h->nblocks;
        LAT_CKL(launch_finalize(h->partials, used, diag_dst, h->stream));
    }
    if (write) {
        h->n += 1;
        h->div_valid = store_div;
    } else if (diag && p.g != 0) {
        h->div_valid = true;  // the divergence of the past level was computed above and is unchanged
    }
    return LAT_OK;
}

static int64_t evolved_sites(const lat_handle* h)
{
    const Geom& g = h->geom;
    return (int64_t)(g.hix - g.lox) * (g.hiy - g.loy) * (g.hiz - g.loz);
}

static int ensure_diag(lat_handle* h, int64_t entries)
{
    if (entries <= h->diag_cap) return LAT_OK;
    dev_free(h, (void**)&h->diag_dev, sizeof(double) * 2 * (size_t)h->diag_cap);
    h->diag_cap = 0;
    int rc = dev_alloc(h, (void**)&h->diag_dev, sizeof(double) * 2 * (size_t)entries);
    if (rc) return rc;
    h->diag_cap = entries;
    return LAT_OK;
}

int lat_step(lat_handle* h, int32_t nsteps)
{
    LAT_REQUIRE(h && nsteps >= 0, "lat_step: bad argument");
    LAT_CK(cudaSetDevice(h->device));
    for (int32_t q = 0; q < nsteps; ++q) {
        int rc = do_step(h, false, false, nullptr);
        if (rc) return rc;
    }
    LAT_CK(cudaStreamSynchronize(h->stream));
    return LAT_OK;
}

int lat_step_diag(lat_handle* h, lat_diag* out)
{
    LAT_REQUIRE(h && out, "lat_step_diag: null argument");
    LAT_CK(cudaSetDevice(h->device));
    int rc = ensure_diag(h, 1);
    if (rc) return rc;
    const int64_t n = h->n;
    if ((rc = do_step(h, true, h->p.g != 0, h->diag_dev))) return rc;
    double v[2];
    LAT_CK(cudaMemcpyAsync(v, h->diag_dev, sizeof(v), cudaMemcpyDeviceToHost, h->stream));
    LAT_CK(cudaStreamSynchronize(h->stream));
    out->energy = v[0];
    out->gauss_abs_sum = v[1];
    out->sites = evolved_sites(h);
    out->time_step = n;
    return LAT_OK;
}

// The loop of lat_advance.
static int advance_impl(lat_handle* h, int32_t nsteps, int32_t diag_every, lat_diag* out, int64_t cap,
                        int64_t* count)
{
    int64_t ndiag = 0;
    if (diag_every > 0) {
        int64_t want = 0;
        for (int64_t n = h->n; n < h->n + nsteps; ++n) want += (n % diag_every == 0);
        want = want < cap ? want : cap;
        int rc = ensure_diag(h, want > 0 ? want : 1);
        if (rc) return rc;
    }
    std::vector<int64_t> steps;
    for (int32_t q = 0; q < nsteps; ++q) {
        const int64_t n = h->n;
        const bool diag = diag_every > 0 && n % diag_every == 0 && ndiag < cap;
        const bool next = diag_every > 0 && (n + 1) % diag_every == 0;
        const bool store = next && h->p.g != 0;
        int rc = do_step(h, diag, store, diag ? h->diag_dev + 2 * ndiag : nullptr, true);
        if (rc) return rc;
        if (diag) {
            steps.push_back(n);
            ++ndiag;
        }
    }
    if (ndiag > 0) {
        std::vector<double> v(2 * (size_t)ndiag);
        LAT_CK(cudaMemcpyAsync(v.data(), h->diag_dev, sizeof(double) * v.size(), cudaMemcpyDeviceToHost, h->stream));
        LAT_CK(cudaStreamSynchronize(h->stream));
        const int64_t sites = evolved_sites(h);
        for (int64_t q = 0; q < ndiag; ++q) {
            out[q].energy = v[2 * q];
            out[q].gauss_abs_sum = v[2 * q + 1];
            out[q].sites = sites;
            out[q].time_step = steps[q];
        }
    } else {
        LAT_CK(cudaStreamSynchronize(h->stream));
    }
    if (count) *count = ndiag;
    return LAT_OK;
}

int lat_advance(lat_handle* h, int32_t nsteps, int32_t diag_every, lat_diag* out, int64_t cap, int64_t* count)
{
    LAT_REQUIRE(h && nsteps >= 0 && diag_every >= 0, "lat_advance: bad argument");
    LAT_REQUIRE(diag_every == 0 || (out && cap >= 0), "lat_advance: diagnostics requested without output");
    LAT_CK(cudaSetDevice(h->device));
    return advance_impl(h, nsteps, diag_every, out, cap, count);
}

// The three calls in one.  Overlapping the copies with the first and the
// last step on a second stream (uploads during the first link pass, the final
// past level's download during the last step) ran 5-10 % slower than the
// calls in sequence on GB300 (Grace host link), so the calls run in sequence.
int lat_run(lat_handle* h, const double* now, const double* past, int64_t time_step, int32_t nsteps,
            int32_t diag_every, lat_diag* out, int64_t cap, int64_t* count, double* now_out, double* past_out)
{
    LAT_REQUIRE(h && now && past, "lat_run: null argument");
    LAT_REQUIRE(time_step >= 0 && nsteps >= 0 && diag_every >= 0, "lat_run: bad argument");
    LAT_REQUIRE(diag_every == 0 || (out && cap >= 0), "lat_run: diagnostics requested without output");
    int rc;
    if ((rc = lat_set_state(h, now, past, time_step))) return rc;
    if ((rc = advance_impl(h, nsteps, diag_every, out, cap, count))) return rc;
    return (now_out || past_out) ? lat_get_state(h, now_out, past_out) : LAT_OK;
}

int lat_diagnostics(lat_handle* h, lat_diag* out)
{
    LAT_REQUIRE(h && out, "lat_diagnostics: null argument");
    LAT_CK(cudaSetDevice(h->device));
    int rc = ensure_diag(h, 1);
    if (rc) return rc;
    if ((rc = do_step(h, true, false, h->diag_dev, false))) return rc;
    double v[2];
    LAT_CK(cudaMemcpyAsync(v, h->diag_dev, sizeof(v), cudaMemcpyDeviceToHost, h->stream));
    LAT_CK(cudaStreamSynchronize(h->stream));
    out->energy = v[0];
    out->gauss_abs_sum = v[1];
    out->sites = evolved_sites(h);
    out->time_step = h->n;
    return LAT_OK;
}

static DetectArgs detect_args(const lat_handle* h)
{
    DetectArgs a;
    const Geom& g = h->geom;
    a.nx = g.nx;
    a.ny = g.ny;
    a.nz = g.nz;
    a.syz = g.syz;
    a.lox = g.lox;
    a.loy = g.loy;
    a.loz = g.loz;
    a.hix = g.hix;
    a.hiy = g.hiy;
    a.hiz = g.hiz;
    a.dx = h->p.dx;
    a.dy = h->p.dy;
    a.dz = h->p.dz;
    a.x0 = (int)(0.5 * (g.nx - 1));  // mpi_evolution.cpp:131-133
    a.y0 = (int)(0.5 * (g.ny - 1));
    a.z0 = (int)(0.5 * (g.nz - 1));
    return a;
}

// count the crossings of `field` on the current level (block totals scanned in place)
static int detect_count(lat_handle* h, int32_t field, int64_t* total_out)
{
    int rc0 = ensure_boundaries(h);
    if (rc0) return rc0;
    const DetectArgs a = detect_args(h);
    const int tNow = (int)((h->n + 1) % 2);
    const int nb = (int)((h->N + detect_block_sites() - 1) / detect_block_sites());
    if (nb > h->det_nb) {
        dev_free(h, (void**)&h->det_blocks, sizeof(long long) * (size_t)h->det_nb);
        h->det_nb = 0;
        int rc = dev_alloc(h, (void**)&h->det_blocks, sizeof(long long) * (size_t)nb);
        if (rc) return rc;
        h->det_nb = nb;
    }
    const void* re = h->slot(2 * field, tNow);
    const void* im = h->slot(2 * field + 1, tNow);
    if (h->elem == 8) LAT_CKL(launch_detect_count_f64(a, (const double*)re, (const double*)im, h->det_blocks, nb, h->stream));
    else LAT_CKL(launch_detect_count_f32(a, (const float*)re, (const float*)im, h->det_blocks, nb, h->stream));
    LAT_CKL(launch_scan_totals(h->det_blocks, nb, h->det_total, h->stream));
    long long total = 0;
    LAT_CK(cudaMemcpyAsync(&total, h->det_total, sizeof(total), cudaMemcpyDeviceToHost, h->stream));
    LAT_CK(cudaStreamSynchronize(h->stream));
    *total_out = total;
    return LAT_OK;
}

// write the first nw crossings (after detect_count) into h->det_xyz
static int detect_write(lat_handle* h, int32_t field, int64_t nw)
{
    if (nw <= 0) return LAT_OK;
    if (nw > h->det_cap) {
        dev_free(h, (void**)&h->det_xyz, sizeof(double) * 3 * (size_t)h->det_cap);
        h->det_cap = 0;
        int rc = dev_alloc(h, (void**)&h->det_xyz, sizeof(double) * 3 * (size_t)nw);
        if (rc) return rc;
        h->det_cap = nw;
    }
    const DetectArgs a = detect_args(h);
    const int tNow = (int)((h->n + 1) % 2);
    const int nb = (int)((h->N + detect_block_sites() - 1) / detect_block_sites());
    const void* re = h->slot(2 * field, tNow);
    const void* im = h->slot(2 * field + 1, tNow);
    if (h->elem == 8)
        LAT_CKL(launch_detect_write_f64(a, (const double*)re, (const double*)im, h->det_blocks, nb, h->det_xyz, nw, h->stream));
    else
        LAT_CKL(launch_detect_write_f32(a, (const float*)re, (const float*)im, h->det_blocks, nb, h->det_xyz, nw, h->stream));
    return LAT_OK;
}

int lat_detect_crossings(lat_handle* h, int32_t field, double* xyz, int64_t cap, int64_t* count)
{
    LAT_REQUIRE(h && count, "lat_detect_crossings: null argument");
    LAT_REQUIRE(field == LAT_FIELD_PHI1 || (field == LAT_FIELD_PHI2 && h->p.model == LAT_MODEL_MOORE),
                "lat_detect_crossings: bad field");
    LAT_REQUIRE(cap >= 0 && (xyz || cap == 0), "lat_detect_crossings: bad capacity");
    LAT_CK(cudaSetDevice(h->device));
    int64_t total = 0;
    int rc = detect_count(h, field, &total);
    if (rc) return rc;
    *count = total;
    const int64_t nw = total < cap ? total : cap;
    if (nw > 0) {
        if ((rc = detect_write(h, field, nw))) return rc;
        LAT_CK(cudaMemcpyAsync(xyz, h->det_xyz, sizeof(double) * 3 * (size_t)nw, cudaMemcpyDeviceToHost, h->stream));
        LAT_CK(cudaStreamSynchronize(h->stream));
    }
    if (xyz && total > cap) {
        set_error("lat_detect_crossings: capacity smaller than the number of crossings");
        return LAT_ERR_CAPACITY;
    }
    return LAT_OK;
}

int lat_string_length(lat_handle* h, int32_t field, int32_t split, int32_t method, double* L0, double* L1,
                      int64_t* count)
{
    LAT_REQUIRE(h && L0 && L1, "lat_string_length: null argument");
    LAT_REQUIRE(field == LAT_FIELD_PHI1 || (field == LAT_FIELD_PHI2 && h->p.model == LAT_MODEL_MOORE),
                "lat_string_length: bad field");
    LAT_REQUIRE(method >= LAT_CHAIN_AUTO && method <= LAT_CHAIN_EXHAUSTIVE, "lat_string_length: bad method");
    const bool periodic = h->p.bc == LAT_BC_PERIODIC && bc_z_kind(h->p) == LAT_BC_PERIODIC;
    LAT_REQUIRE(method != LAT_CHAIN_HASH || periodic, "lat_string_length: the hash needs a periodic lattice");
    LAT_CK(cudaSetDevice(h->device));
    *L0 = *L1 = 0.0;
    int64_t total = 0;
    int rc = detect_count(h, field, &total);
    if (rc) return rc;
    if (count) *count = total;
    if (total == 0) return LAT_OK;
    if ((rc = detect_write(h, field, total))) return rc;
    if (method == LAT_CHAIN_AUTO) method = periodic ? LAT_CHAIN_HASH : LAT_CHAIN_EXHAUSTIVE;
    const ChainGeom g = make_chain_geom(h->p, total);
    double out[2];
    rc = chain_length_run(g, h->det_xyz, total, split, method, h->chain, &h->bytes, h->stream, out, &h->launches);
    if (rc) return rc;
    *L0 = out[0];
    *L1 = out[1];
    return LAT_OK;
}

int lat_winding(lat_handle* h, int32_t field, int8_t* out, int64_t* abs_sum)
{
    LAT_REQUIRE(h, "lat_winding: null handle");
    LAT_REQUIRE(field == LAT_FIELD_PHI1 || (field == LAT_FIELD_PHI2 && h->p.model == LAT_MODEL_MOORE),
                "lat_winding: bad field");
    LAT_CK(cudaSetDevice(h->device));
    if (out && !h->wind) {
        int rc = dev_alloc(h, (void**)&h->wind, (size_t)3 * h->N);
        if (rc) return rc;
    }
    int rcb = ensure_boundaries(h);
    if (rcb) return rcb;
    const DetectArgs a = detect_args(h);
    const int tNow = (int)((h->n + 1) % 2);
    const void* re = h->slot(2 * field, tNow);
    const void* im = h->slot(2 * field + 1, tNow);
    LAT_CK(cudaMemsetAsync(h->wind_sum, 0, sizeof(unsigned long long), h->stream));
    int8_t* dst = out ? h->wind : nullptr;
    const int open_axes = (h->p.bc != LAT_BC_PERIODIC ? 1 : 0) | (bc_z_kind(h->p) != LAT_BC_PERIODIC ? 2 : 0);
    if (h->elem == 8)
        LAT_CKL(launch_winding_f64(a, open_axes, (const double*)re, (const double*)im, dst, h->wind_sum, h->stream));
    else
        LAT_CKL(launch_winding_f32(a, open_axes, (const float*)re, (const float*)im, dst, h->wind_sum, h->stream));
    unsigned long long tot = 0;
    LAT_CK(cudaMemcpyAsync(&tot, h->wind_sum, sizeof(tot), cudaMemcpyDeviceToHost, h->stream));
    if (out) LAT_CK(cudaMemcpyAsync(out, h->wind, (size_t)3 * h->N, cudaMemcpyDeviceToHost, h->stream));
    LAT_CK(cudaStreamSynchronize(h->stream));
    if (abs_sum) *abs_sum = (int64_t)tot;
    return LAT_OK;
}

}  // extern "C"
