// Internal declarations shared by the CUDA translation units of
// liblattice_gpu.so.  Not part of the C ABI (that is include/lattice_gpu.h).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/lattice_gpu.h"

namespace lat {

// ---------------------------------------------------------------------------
// geometry of the evolved region
// ---------------------------------------------------------------------------
struct Geom {
    int nx, ny, nz;       // lattice sides
    int syz;              // ny*nz
    int lox, loy, loz;    // first evolved index per axis (0 periodic, 1 otherwise)
    int hix, hiy, hiz;    // one past the last evolved index per axis
};

// thread-block shape of the site kernels: 32 along z (coalesced), 8 along y
constexpr int BZ = 32;
constexpr int BY = 8;
constexpr int BLOCK = BZ * BY;

inline dim3 site_grid(const Geom& g)
{
    return dim3((unsigned)((g.hiz - g.loz + BZ - 1) / BZ), (unsigned)((g.hiy - g.loy + BY - 1) / BY),
                (unsigned)(g.hix - g.lox));
}

// ---------------------------------------------------------------------------
// per-step coefficients.  Each is the exact double the reference evaluates
// (same operands, same order), so an FP64 kernel reproduces its arithmetic.
// ---------------------------------------------------------------------------
// Field list of the step coefficients (X-macro), so that the FP32 kernels get
// native-float copies instead of converting doubles at every use.
#define LAT_COEF_FIELDS(X)                                                   \
    X(dx2) X(dy2) X(dz2)                 /* dx*dx ...                      */ \
    X(dt) X(dt2)                         /* dt, dt*dt                      */ \
    X(halfLambda) X(etaSq)               /* 0.5*lambda, eta*eta            */ \
    X(halfLambda2) X(eta2Sq)             /* 0.5*lambda2, eta2*eta2 (Moore) */ \
    X(halfLambda12)                      /* 0.5*lambda12 (Moore)           */ \
    X(m2gg)                              /* (-2*g)*g                       */ \
    X(fric)                              /* damp + alpha*scaling/tau       */ \
    X(damp)                              /* dampFac or 0                   */ \
    X(q1) X(q2)                          /* Moore charges                  */ \
    X(dx) X(dy) X(dz) X(g)                                                    \
    X(gdtdx) X(gdtdy) X(gdtdz)           /* (g*dt)*dmu                     */ \
    X(gxy2) X(gxz2) X(gyz2)              /* ((g*dx)*dy)^2 ...              */ \
    X(dV)                                /* (dx*dy)*dz                     */ \
    X(quarterLambda) X(quarterLambda2) X(halfLambda12e)                       \
    X(twog)                              /* 2*g                            */ \
    X(inv_dx2) X(inv_dy2) X(inv_dz2) X(inv_dt) X(inv_dx) X(inv_dy) X(inv_dz) X(inv_g) \
    X(inv_gdtdx) X(inv_gdtdy) X(inv_gdtdz) X(inv_gxy2) X(inv_gxz2) X(inv_gyz2) \
    X(iso)                               /* 1 when dx == dy == dz, else 0 */      \
    X(fric_dt)                           /* fric / dt (fused FP64 step)    */

template <class R>
struct StepCoefT {
#define LAT_COEF_DECL(name) R name;
    LAT_COEF_FIELDS(LAT_COEF_DECL)
#undef LAT_COEF_DECL
};
using StepCoef = StepCoefT<double>;

template <class R>
inline StepCoefT<R> coef_as(const StepCoef& c)
{
    StepCoefT<R> o;
#define LAT_COEF_CAST(name) o.name = (R)c.name;
    LAT_COEF_FIELDS(LAT_COEF_CAST)
#undef LAT_COEF_CAST
    return o;
}

StepCoef make_coef(const lat_params& p, int64_t n);
// LAT_OK or LAT_ERR_INVALID (with the message set) for a parameter block
int validate_params(const lat_params* p);
Geom make_geom(const lat_params& p);
// LAT_BC_* of the z axis (bc_z, or the same as bc)
int bc_z_kind(const lat_params& p);

// Kernel argument block: base pointers of the two slots of every component.
template <class T, int NC>
struct Fields {
    const T* __restrict__ now[NC];
    T* past[NC];
};

struct DiagOut {
    double* partials;    // [2 * nblocks]: energy, |G| per block (or nullptr)
    void* divbuf;        // divergence of theta at one level, [N] of T
    int use_div;         // the diagnostic reads divbuf as the past-level divergence
    int store_div;       // write the now-level divergence into divbuf
    int energy_form;     // LAT_ENERGY_*
    int charge_current;  // Moore: q-weighted current
    int write;           // 0: diagnostics only, the state is left unchanged
};

// launchers (one translation unit per model/precision)
cudaError_t launch_ah_step_f64(const Geom&, const Fields<double, 5>&, const StepCoef&, const DiagOut&, bool diag,
                               cudaStream_t);
cudaError_t launch_ah_step_f32(const Geom&, const Fields<float, 5>&, const StepCoef&, const DiagOut&, bool diag,
                               cudaStream_t);
cudaError_t launch_moore_step_f64(const Geom&, const Fields<double, 7>&, const StepCoef&, const DiagOut&, bool diag,
                                  cudaStream_t);
cudaError_t launch_moore_step_f32(const Geom&, const Fields<float, 7>&, const StepCoef&, const DiagOut&, bool diag,
                                  cudaStream_t);
// two-pass FP64 Abelian-Higgs step (link data in L, [15][N] doubles)
int ah_link_slots();
cudaError_t launch_ah_twopass_strict(const Geom&, const Fields<double, 5>&, double* L, const StepCoef&, const DiagOut&,
                                     bool diag, bool recip, cudaStream_t);
cudaError_t launch_ah_twopass_fast(const Geom&, const Fields<double, 5>&, double* L, const StepCoef&, const DiagOut&,
                                   bool diag, bool recip, cudaStream_t);
// x-planes per CTA of the tiled FP32 step for a new handle (tuned value of the
// shape if known in this process, else a heuristic); tune.cu
int default_chunk(const lat_params& p);
// x-planes per work item of a lattice stepped in a batch (its shape only)
int batch_chunk(const Geom& g);
// number of CTAs (and diagnostic partials) of the tiled FP32 step
int tiled_blocks(const Geom&, int chunk);
// x-marching FP32 steps, `chunk` x-planes per CTA.  variant 0: the pair step
// (two z-sites per thread, pair_step.cuh) where the layout allows it, else the
// tiled step (tiled_step.cuh); 2: the tiled step with one-element staging
// copies; 3: the tiled step with 16-byte staging where allowed.  *blocks
// receives the CTAs (diagnostic partials) of the kernel launched.
cudaError_t launch_ah_tiled_f32(const Geom&, const Fields<float, 5>&, const StepCoef&, const DiagOut&, bool diag,
                                int chunk, cudaStream_t, int variant, int* blocks);
cudaError_t launch_moore_tiled_f32(const Geom&, const Fields<float, 7>&, const StepCoef&, const DiagOut&, bool diag,
                                   int chunk, cudaStream_t, int variant, int* blocks);
// divergence of theta on one level into divbuf (used when no previous step stored it)
cudaError_t launch_divergence_f64(const Geom&, const double* thx, const double* thy, const double* thz,
                                  const StepCoef&, double* out, cudaStream_t);
cudaError_t launch_divergence_f32(const Geom&, const float* thx, const float* thy, const float* thz,
                                  const StepCoef&, float* out, cudaStream_t);

// Neumann and absorbing boundaries (boundary.cu); `now`/`past` are the five
// component slots of a level, elem the bytes per value
cudaError_t launch_neumann(const Geom&, int model, double q1, double q2, int kxy, int kz, int elem,
                           void* const* now, cudaStream_t, int* launches);
size_t absorb_tt_bytes(const Geom&, int elem);
cudaError_t launch_absorb_tt(const Geom&, int elem, void* const* now, void* const* past, void* tt, double dx,
                             double dy, double dz, double dt, cudaStream_t);
cudaError_t launch_absorb_update(const Geom&, int elem, void* const* now, void* const* past, const void* tt,
                                 double dt2, cudaStream_t);

// deterministic sum of per-block partials into out[0..1] (energy, |G|)
cudaError_t launch_finalize(const double* partials, int nblocks, double* out, cudaStream_t);

// conversions between the double host layout and FP32 device fields
cudaError_t launch_d2f(const double* in, float* out, int64_t n, cudaStream_t);
cudaError_t launch_f2d(const float* in, double* out, int64_t n, cudaStream_t);

// detection
struct DetectArgs {
    int nx, ny, nz, syz, lox, loy, loz, hix, hiy, hiz;
    double dx, dy, dz;
    int x0, y0, z0;
};
int detect_block_sites();
cudaError_t launch_detect_count_f64(const DetectArgs&, const double* re, const double* im, long long* block_totals,
                                    int nblocks, cudaStream_t);
cudaError_t launch_detect_count_f32(const DetectArgs&, const float* re, const float* im, long long* block_totals,
                                    int nblocks, cudaStream_t);
cudaError_t launch_scan_totals(long long* block_totals, int nblocks, long long* total, cudaStream_t);
cudaError_t launch_detect_write_f64(const DetectArgs&, const double* re, const double* im, const long long* block_offsets,
                                    int nblocks, double* xyz, long long cap, cudaStream_t);
cudaError_t launch_detect_write_f32(const DetectArgs&, const float* re, const float* im, const long long* block_offsets,
                                    int nblocks, double* xyz, long long cap, cudaStream_t);
cudaError_t launch_winding_f64(const DetectArgs&, int open_axes, const double* re, const double* im, int8_t* out,
                               unsigned long long* abs_sum, cudaStream_t);
cudaError_t launch_winding_f32(const DetectArgs&, int open_axes, const float* re, const float* im, int8_t* out,
                               unsigned long long* abs_sum, cudaStream_t);

// ---------------------------------------------------------------------------
// string length by greedy chaining of crossings (string_length.cu)
// ---------------------------------------------------------------------------
struct ChainGeom {
    double L[3];          // n*d: box side
    double half[3];       // (0.5*n)*d: minimum-image threshold
    double quarter[3];    // (0.25*n)*d: half-side of the inner (L0) box
    double lo[3];         // -x0*d: lower edge of crossing coordinates
    double w[3];          // hash cell width (>= the cutoff radius)
    int nb[3];            // hash cells per axis
    int periodic[3];      // minimum image per axis (x, y from bc; z from bc_z)
    double cutoff;        // (dx*dx + dy*dy + dz*dz)^2, compared with squared distances
    double root_cutoff;   // sqrt(cutoff): the closing length the reference adds
    int nnb;              // distinct neighbour-cell offsets
    signed char off[27][3];
};

ChainGeom make_chain_geom(const lat_params& p, int64_t M);
// points lie in the box the hash covers (finite, within [lo, lo+L] per axis)
bool chain_points_in_box(const ChainGeom& g, const double* xyz_host, int64_t M);
// device buffers of the chaining, kept between calls (grown as needed)
struct ChainBuffers {
    void* ws = nullptr;
    size_t ws_bytes = 0;
    void* edges = nullptr;  // links between crossings
    size_t edge_bytes = 0;
};
void chain_buffers_release(ChainBuffers& b, int64_t* held);
// Chaining of the M crossings at d_xyz (device, [M][3]).  method: LAT_CHAIN_HASH
// or LAT_CHAIN_EXHAUSTIVE.  Buffers grow as needed (`held`, may be NULL, counts
// their bytes).  out[0..1] = L0, L1 (host).  Returns a LAT_* status.
int chain_length_run(const ChainGeom& g, const double* d_xyz, int64_t M, int split, int method, ChainBuffers& buf,
                     int64_t* held, cudaStream_t st, double* out, int64_t* launches);

// error reporting
void set_error(const std::string& msg);

}  // namespace lat
