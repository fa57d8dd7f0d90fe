/*
 * lattice_gpu.h — C ABI of the GB300 lattice-evolution library (liblattice_gpu.so).
 *
 * The reference (sjcott/Axions) has no library boundary: its hot path is the
 * body of the time-step loop inside main() of four programs.  Each entry point
 * below names the loop-body fragment it replaces (reference file:line).  The
 * C++ drop-in programs (in axions_gb300/host/) and the Python mirror
 * (axions_gb300/lattice.py) call only these functions.
 *
 * Conventions
 *   - Every function returns int status: LAT_OK (0) or a negative LAT_ERR_*.
 *     lat_last_error() returns a message for the calling thread's last error.
 *     No C++ exception crosses this boundary and no device code traps.
 *   - Device memory is owned by the handle.  Host buffers are owned by the
 *     caller and copied synchronously (the call returns when the copy is done).
 *   - Field layout on the host is the reference's: one contiguous array per
 *     component, sites in linear order (i*ny + j)*nz + k (z fastest), i.e. the
 *     `pos` of calcInd() in mpi_evolution.cpp:62 and Array(..,i,j,k) in
 *     array.cpp:66-94.  Component order:
 *        Abelian-Higgs: phi_re, phi_im, theta_x, theta_y, theta_z   (5)
 *        Moore:         phi1_re, phi1_im, phi2_re, phi2_im,
 *                       theta_x, theta_y, theta_z                    (7)
 *     theta_mu is the link phase g*d_mu*A_mu (ic.txt columns,
 *     initialConditions.cpp:539).
 *   - Time levels follow the reference's two-slot scheme: at time step n the
 *     "now" level is slot (n+1)%2 and the "past" level slot n%2
 *     (mpi_evolution.cpp:370-371); a step writes the new level into the past
 *     slot in place (mpi_evolution.cpp:432,499-501).
 *   - One host thread per handle.  Handles are independent of one another.
 */
#ifndef AXIONS_LATTICE_GPU_H
#define AXIONS_LATTICE_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LAT_ABI_VERSION 1

/* status codes */
#define LAT_OK             0
#define LAT_ERR_INVALID   -1  /* bad argument or parameter combination      */
#define LAT_ERR_NOMEM     -2  /* device or host allocation failed            */
#define LAT_ERR_CUDA      -3  /* CUDA runtime error                          */
#define LAT_ERR_TIMEOUT   -4  /* a bounded device wait gave up               */
#define LAT_ERR_CAPACITY  -5  /* caller buffer too small (count still valid) */
#define LAT_ERR_STATE     -6  /* call not valid in the handle's state        */
#define LAT_ERR_NODEVICE  -7  /* no CUDA device / kernel image not loadable  */

/* models */
#define LAT_MODEL_AH     0   /* Abelian-Higgs: evolution.cpp, mpi_evolution.cpp       */
#define LAT_MODEL_MOORE  1   /* two scalars: mooreEvol.cpp, moore_mpi_evolution.cpp  */

/* precision of the stored fields and of the step arithmetic */
#define LAT_F64 0            /* the reference's arithmetic                          */
#define LAT_F32 1            /* FP32 fields and step; energy/Gauss sums stay FP64   */
#define LAT_F64_FAST 2       /* FP64 fields; fused multiply-adds and a corrected
                                reciprocal for /dt (each operation within an ulp of
                                LAT_F64's); not bit-identical to the reference's order */

/* boundary handling: `bc` for the x and y axes (the reference's xyBC), `bc_z`
 * for z (zBC; 0 = the same as bc) */
#define LAT_BC_PERIODIC  0   /* periodic (mpi_evolution.cpp:385-405)                         */
#define LAT_BC_FIXED     1   /* only interior sites evolve; the outer layer of sites is
                                held fixed (evolution.cpp:166-186 with xyBC/zBC "fixed";
                                mooreEvol.cpp:187-189,672-692)                               */
#define LAT_BC_NEUMANN   2   /* interior sites evolve; before each step the outer layer of
                                the current level is set from the next layer in, phi
                                transported along the link (evolution.cpp:194-265; the z
                                pass covers x planes i < nz as the reference's does).
                                Moore (mooreEvol.cpp:114-160): x and y only, phi_a along
                                q_a*theta                                                    */
#define LAT_BC_ABSORBING 3   /* x and y only: the outer layer evolves with the one-sided
                                first-order absorbing updates of evolution.cpp:446-691 (and
                                the whole layer is updated, :1375-1402). Abelian-Higgs only  */
#define LAT_BCZ_AS_XY     0  /* bc_z values */
#define LAT_BCZ_PERIODIC  1
#define LAT_BCZ_FIXED     2
#define LAT_BCZ_NEUMANN   3

/* energy density variants (diagnostics) */
#define LAT_ENERGY_EVOLUTION 0  /* evolution.cpp:322-334,398-427 and mooreEvol.cpp:341-391:
                                   gauge kinetic term (dtheta/(g*dt*dmu))^2/2, zero if g==0  */
#define LAT_ENERGY_MPI       1  /* mpi_evolution.cpp:509-532, moore_mpi_evolution.cpp:558-588:
                                   gauge kinetic term (dtheta/dt)^2/2, always included      */

/* gauge current of the Moore model */
#define LAT_MOORE_CURRENT_PLAIN  0  /* j1 + j2 without charges (moore_mpi_evolution.cpp:498-515) */
#define LAT_MOORE_CURRENT_CHARGE 1  /* q1*j1 + q2*j2 (mooreEvol.cpp:295-312)                     */

/* which scalar a detection call looks at */
#define LAT_FIELD_PHI1 0     /* phi (AH) or phi1 (Moore) */
#define LAT_FIELD_PHI2 1     /* phi2 (Moore only)        */

/*
 * Parameters.  Names and meaning follow the reference's compile-time
 * constants (mpi_evolution.cpp:15-60, moore_mpi_evolution.cpp:15-65,
 * evolution.cpp:23-58, mooreEvol.cpp:19-42).  lat_params_init() fills the
 * defaults of mpi_evolution.cpp (AH) or moore_mpi_evolution.cpp (Moore).
 */
typedef struct lat_params {
    int32_t abi_version;   /* must be LAT_ABI_VERSION                                   */
    int32_t model;         /* LAT_MODEL_*                                                */
    int32_t precision;     /* LAT_F64 / LAT_F32                                          */
    int32_t bc;            /* LAT_BC_*                                                   */
    int64_t nx, ny, nz;    /* lattice sides; nx*ny*nz < 2^31                             */
    double dx, dy, dz, dt;
    double lambda;         /* AH lambda; Moore lambda1                                   */
    double eta;            /* AH eta;    Moore eta1                                      */
    double lambda2;        /* Moore only                                                 */
    double eta2;           /* Moore only                                                 */
    double lambda12;       /* Moore only: cross coupling                                 */
    double g;              /* gauge coupling                                             */
    double q1, q2;         /* Moore charges (reference: const int)                       */
    int32_t damped_nt;     /* damping applies while TimeStep < damped_nt                 */
    int32_t moore_current; /* LAT_MOORE_CURRENT_*                                        */
    double dampFac;        /* damping coefficient while damped                           */
    double alpha;          /* PRS friction factor on the scalars                         */
    double scaling;        /* scale-factor power; friction = alpha*scaling/tau           */
    double tau0;           /* conformal time at step 0: tau = tau0 + TimeStep*dt (=1)    */
    int32_t energy_form;   /* LAT_ENERGY_*                                               */
    int32_t kernel_variant;/* 0: default kernels; 1: one-pass stencils (for checks);
                              2 (FP32): the tiled step staging one element per copy
                              instead of 16-byte row chunks (for checks)                 */
    int32_t bc_z;          /* LAT_BCZ_*: boundary of the z axis (0: the same as bc)        */
    int32_t reserved_i;
    double reserved[3];
} lat_params;

typedef struct lat_handle lat_handle;

/* Result of one diagnostic step: energy of the level before the update and the
 * Gauss-law deviation summed over the evolved sites (the reference's
 * deviationParameter before its normalisation, evolution.cpp:419,1404-1408). */
typedef struct lat_diag {
    double energy;         /* sum over evolved sites of rho*dx*dy*dz                     */
    double gauss_abs_sum;  /* sum over evolved sites of |G|  (0 when g == 0)             */
    int64_t sites;         /* number of evolved sites summed over                        */
    int64_t time_step;     /* TimeStep the values belong to                              */
} lat_diag;

/* ---- library ---------------------------------------------------------------- */
const char* lat_version(void);
const char* lat_last_error(void);

/* Fill reference defaults for a model.  Replaces the const blocks
 * mpi_evolution.cpp:15-60 / moore_mpi_evolution.cpp:15-65. */
int lat_params_init(lat_params* p, int32_t model);

/* Host-side seeded random-phase initial condition, both levels equal, theta=0.
 * Replaces mpi_evolution.cpp:287-312 (AH) and moore_mpi_evolution.cpp:293-323
 * (Moore): mt19937(seed), uniform_real_distribution<double>(0, 2*pi), one draw
 * per site in linear order, phi = eta*(cos, sin).  For Moore, independent != 0
 * draws phi1's phase then phi2's phase per site from the same stream (an
 * extension; the reference gives both scalars the same phase,
 * moore_mpi_evolution.cpp:309-313).  `fields` is [ncomp][nx*ny*nz]. */
int lat_random_phase_ic(const lat_params* p, uint32_t seed, int32_t independent,
                        double* fields);

/* ---- lattice handle ----------------------------------------------------------- */
/* Allocate the two-level state of one lattice on the current CUDA device.
 * Replaces the field vectors of mpi_evolution.cpp:94 (no halo: the whole
 * lattice is resident and the periodic wrap is done in-kernel). */
int lat_create(const lat_params* p, lat_handle** out);
int lat_destroy(lat_handle* h);

/* Launch all work of this handle on `stream` (a cudaStream_t); NULL restores
 * the handle's own stream. */
int lat_set_stream(lat_handle* h, void* stream);

int lat_get_params(const lat_handle* h, lat_params* out);
int lat_num_components(const lat_handle* h);
int64_t lat_time_step(const lat_handle* h);
/* bytes of device memory the handle holds */
int64_t lat_device_bytes(const lat_handle* h);
/* number of CUDA kernels this handle has launched so far (for benchmarks that
 * report their launch count; no counterpart in the reference) */
int64_t lat_kernel_launches(const lat_handle* h);

/* Upload the state: `now` is the level at TimeStep `time_step`, `past` the one
 * before (for a stationary start pass the same array twice, as
 * mpi_evolution.cpp:155-162 does: it is then uploaded once and copied on the
 * device).  Each is [ncomp][nx*ny*nz] doubles; FP32 handles convert on the
 * device.  Replaces the IC load mpi_evolution.cpp:143-285. */
int lat_set_state(lat_handle* h, const double* now, const double* past, int64_t time_step);
/* Download the state; either pointer may be NULL. */
int lat_get_state(lat_handle* h, double* now, double* past);

/* Advance `nsteps` leapfrog steps without diagnostics.  Replaces the per-site
 * EoM + in-place update of mpi_evolution.cpp:381-501 (AH) and
 * moore_mpi_evolution.cpp:405-550 (Moore), and the halo exchange
 * mpi_evolution.cpp:925-943, which is not needed on one resident lattice. */
int lat_step(lat_handle* h, int32_t nsteps);

/* One step that also returns the energy and Gauss deviation of the level it
 * starts from.  Replaces evolution.cpp:273-431 + 1384-1408 and
 * mooreEvol.cpp:187-395 + 672-692 (one step of the loop with its valsPerLoop
 * values). */
int lat_step_diag(lat_handle* h, lat_diag* out);

/* Run `nsteps` steps; at every step n with n % diag_every == 0 (diag_every > 0)
 * record a lat_diag into `out` (capacity `cap` entries, `*count` = entries
 * written).  Diagnostics stay on the device until the end of the call. */
int lat_advance(lat_handle* h, int32_t nsteps, int32_t diag_every,
                lat_diag* out, int64_t cap, int64_t* count);

/* A whole run from host state to host state: lat_set_state(now, past,
 * time_step), lat_advance(nsteps, diag_every, out, cap, count) and
 * lat_get_state(now_out, past_out) in one call, with the same results bit for
 * bit (now_out or past_out may be NULL; past == now for a stationary start).
 * Replaces a run of the reference program: the initial conditions read or
 * drawn at mpi_evolution.cpp:231-312, then the loop at 354-985.  Synchronous:
 * the host buffers may be reused when it returns. */
int lat_run(lat_handle* h, const double* now, const double* past, int64_t time_step,
            int32_t nsteps, int32_t diag_every, lat_diag* out, int64_t cap, int64_t* count,
            double* now_out, double* past_out);

/* Diagnostics of the current level without stepping (read-only). */
int lat_diagnostics(lat_handle* h, lat_diag* out);

/* Bilinear string-crossing detection on the current ("now") level of one
 * scalar.  Replaces mpi_evolution.cpp:536-789 (+ the gather :795-888) and
 * evolution.cpp:723-1016.  Writes `*count` crossings as xyz triples
 * (x0,y0,z0,x1,...) in the reference's order: sites in linear order, and per
 * site the z-directed face, the y-directed face, the x-directed face, each with
 * its "+sqrt" root before its "-sqrt" root.  Coordinates are (i - x0)*dx with
 * x0 = int((nx-1)/2) (mpi_evolution.cpp:131-133,547-549).  If cap is too small
 * the first `cap` triples are written, *count holds the full count and the call
 * returns LAT_ERR_CAPACITY.  xyz may be NULL with cap 0 to query the count. */
int lat_detect_crossings(lat_handle* h, int32_t field, double* xyz, int64_t cap,
                         int64_t* count);

/* Integer winding of the scalar's phase around every plaquette of the current
 * level (no counterpart in the reference, which has only the bilinear
 * detection above; followString.cpp:1-262 is an unfinished fragment).
 * out (may be NULL) is int8 [3][nx*ny*nz]: out[d*N + s] is the winding (-1, 0
 * or +1) of the face with normal d (0=x, 1=y, 2=z) whose lowest corner is site
 * s, traversed counter-clockwise about +d:
 *   d=x: s, s+y, s+y+z, s+z    d=y: s, s+z, s+z+x, s+x    d=z: s, s+x, s+x+y, s+y
 * Each edge a->b contributes the signed crossing of the ray Re>0, Im=0 decided
 * by the sign of Re(a)Im(b) - Im(a)Re(b) (products rounded separately, no FMA),
 * so results are bit-exact between host and device.  *abs_sum (may be NULL)
 * is the sum of |winding| over all faces.  With LAT_BC_FIXED faces that leave
 * the lattice are 0. */
int lat_winding(lat_handle* h, int32_t field, int8_t* out, int64_t* abs_sum);

/* Total string length by greedy chaining of crossings; replaces
 * ic_w_evolution.cpp:961-1087 (stringLength[0], stringLength[1]).
 * From the current crossing the nearest remaining one whose squared distance
 * is <= (dx^2+dy^2+dz^2)^2 is next (the last of equally near ones wins); its
 * distance is added.  Per axis the separation |a-b| is used when it is at most
 * half the box, else box-|a-b| on a periodic lattice and 0 on a fixed one (as
 * the reference does).  With none in reach the chain closes onto its first
 * crossing if that is in reach, adding sqrt((dx^2+dy^2+dz^2)^2) as the
 * reference does, and restarts at the lowest remaining index.  With split != 0
 * a step counts to *L0 when the crossing it leaves lies in the central box
 * |x| <= nx*dx/4 (same for y, z) and to *L1 otherwise; with split == 0 all goes
 * to *L0.  The result equals the reference's bit for bit on the same crossing
 * list.  method: LAT_CHAIN_HASH walks the linked components of a periodic
 * lattice in parallel through a cell hash; LAT_CHAIN_EXHAUSTIVE is one thread
 * block testing every remaining crossing per step (any lattice; the fixed-wall
 * rule above links crossings across the box, so fixed lattices use it);
 * LAT_CHAIN_AUTO picks. */
#define LAT_CHAIN_AUTO        0
#define LAT_CHAIN_HASH        1
#define LAT_CHAIN_EXHAUSTIVE  2

/* Crossings of scalar `field` on the current level (as lat_detect_crossings,
 * kept on the device) chained as above.  count (may be NULL) = crossings. */
int lat_string_length(lat_handle* h, int32_t field, int32_t split, int32_t method, double* L0, double* L1,
                      int64_t* count);

/* The same chaining for M host crossings xyz[3*M] on the geometry of p (nx..nz,
 * dx..dz, bc), on the current CUDA device.  LAT_CHAIN_HASH needs a periodic
 * lattice and every point inside the box ((i-x0)*dx coordinates). */
int lat_string_length_points(const lat_params* p, const double* xyz, int64_t M, int32_t split, int32_t method,
                             double* L0, double* L1);

/* Bound of the device-side waits of LAT_CHAIN_EXHAUSTIVE (the grid barrier of
 * its cooperative walk, which stands in for the reference's OpenMP region per
 * step, ic_w_evolution.cpp:985-1040): a wait polls at most `polls` times
 * (0: the default, 2^24 polls, about a second), then the walk stops and the
 * call returns LAT_ERR_TIMEOUT with the device still usable.
 * missing_arrivals > 0 makes every barrier wait for that many arrivals that
 * never come, so that a test can make the bound run out; 0 in normal use.
 * Process-wide; affects later calls. */
int lat_set_chain_wait(int64_t polls, int32_t missing_arrivals);

/* ---- asynchronous snapshots ------------------------------------------------------
 * The reference writes its field dumps (gifData |phi|^2 volumes,
 * evolution.cpp:1423-1441, mooreEvol.cpp:700-718; finalField) from host arrays
 * inside the step loop, so the loop waits for every dump.  A snapshot copies
 * the current level to host memory while later steps run:
 *   LAT_SNAP_MAGNITUDE  |phi|^2 per site, re*re + im*im in double ([N] doubles;
 *                       Moore: [2][N], |phi1|^2 then |phi2|^2)
 *   LAT_SNAP_LEVEL      the whole level, [ncomp][N] doubles (lat_get_state's
 *                       `now` layout)
 * lat_snapshot_begin stages the values on the handle's stream (before any step
 * issued afterwards) and starts their copy into `dst` (lat_snapshot_doubles
 * doubles) on a separate stream.  With `dst` from lat_host_alloc (pinned) the
 * call returns at once and the copy overlaps the following steps; with
 * ordinary memory it returns when the copy is done.  lat_snapshot_wait blocks
 * until `dst` holds the values.  One snapshot is in flight per handle: a new
 * begin first waits for the previous copy. */
#define LAT_SNAP_MAGNITUDE 0
#define LAT_SNAP_LEVEL     1
int64_t lat_snapshot_doubles(const lat_handle* h, int32_t kind);
int lat_snapshot_begin(lat_handle* h, int32_t kind, double* dst);
int lat_snapshot_wait(lat_handle* h);

/* Page-locked host memory for snapshot destinations (NULL on failure), and its
 * release.  For callers that do not link the CUDA runtime themselves. */
void* lat_host_alloc(int64_t bytes);
void lat_host_free(void* ptr);

/* ---- device-side random-phase IC ------------------------------------------------
 * The physics of lat_random_phase_ic (phi = eta*e^{i phase}, phase uniform in
 * [0, 2 pi), both levels equal, theta = 0, TimeStep 0) drawn on the GPU with
 * the counter-based generator Philox-4x32-10: site s uses counter (s, 0, 0, 0)
 * and key (seed & 0xffffffff, seed >> 32); its phase is 2 pi times the 53-bit
 * uniform of outputs 0 and 1 (for Moore with independent != 0, phi2's phase
 * comes from outputs 2 and 3).  Not the reference's mt19937 sequence: for
 * ensembles and served jobs, where reproducing it is not needed.  No
 * counterpart in the reference. */
int lat_random_phase_ic_device(lat_handle* h, uint64_t seed, int32_t independent);

/* ---- string initial conditions from a straight-string profile --------------------
 * The radial profile of a static straight string of winding n, as
 * singleSemiAnalytic.cpp writes it to SOR_Fields.txt: phi[i] = |phi|(r_i),
 * A[i] = A_theta(r_i), r_i = i*h.  The reference's families read it with
 * second-order interpolation about the nearest point (first order at r < h/2,
 * initialConditions.cpp:760-774).  A site farther out than the table's last
 * interior point takes |phi| = 1, A = n/g (0 for g = 0), as the reference does
 * off its table; the reference also reads one entry past its table when the
 * nearest point is the last one, which here counts as off the table. */
typedef struct lat_string_profile {
    const double* phi;   /* m host values */
    const double* A;     /* m host values */
    int64_t m;           /* >= 2 */
    double h;            /* > 0 */
    double winding;      /* n */
} lat_string_profile;

/* the two roundings of the reference's boost family: initialConditions.cpp
 * builds A and writes d*g*A; ic_func.cpp (the in-process IC of ic_w_evolution)
 * writes theta = d*g*(...) and adds the gauge shift to theta */
#define LAT_IC_FORM_FILE      0
#define LAT_IC_FORM_INPROCESS 1

typedef struct lat_boost_ic {
    double v[3];         /* boost velocity, |v| < 1, not 0 */
    int32_t form;        /* LAT_IC_FORM_* */
    int32_t reserved;
} lat_boost_ic;

/* A z-directed straight string at the lattice centre, Lorentz-boosted with
 * velocity v (initialConditions.cpp:710-992, ic_func.cpp:685-964): the fields
 * at t = 0 go to the past slot and those at t = dt (with the gauge
 * transformation back to temporal gauge) to the current slot; time step 0.
 * Uses the handle's sizes (each >= 2), spacings, dt and g.  `off_table` (may
 * be null) receives the number of site evaluations beyond the profile table.
 * Abelian-Higgs handles only. */
int lat_boost_ic_device(lat_handle* h, const lat_string_profile* prof, const lat_boost_ic* b, int64_t* off_table);

/* Two string/anti-string pairs set up to collide and form loops
 * (initialConditions.cpp:994-1716, ic_type "loop collision"): an x-directed
 * pair at (y, z) = pos1s, pos1a moving with v1s, v1a and a z-directed pair at
 * (x, y) = pos2s, pos2a moving with v2s, v2a (|v| < 1; 0 leaves a string at
 * rest).  Each pair's product field has its imaginary part tapered to zero on
 * the faces (magnitude kept), is divided by linear interpolants of its
 * magnitude across the periodic faces (two passes), and the two pairs are
 * multiplied.  Both levels: t = 0 into the past slot, t = dt (boosted
 * positions, gauge rotation of phi and the periodic centred gauge shift of A)
 * into the current slot; time step 0.  Sides >= 3.  The reference reads four
 * uninitialised link components at t = dt (A1s[0], A1a[0], A2s[2], A2a[2]
 * are only set in the t = 0 loop's private copies); here they are 0, their
 * t = 0 value.  Abelian-Higgs handles only. */
typedef struct lat_loop_collision_ic {
    double pos1s[2], pos1a[2];   /* (y, z) of the x-directed string, anti-string */
    double pos2s[2], pos2a[2];   /* (x, y) of the z-directed string, anti-string */
    double v1s[3], v1a[3], v2s[3], v2a[3];
} lat_loop_collision_ic;

int lat_loop_collision_ic_device(lat_handle* h, const lat_string_profile* prof, const lat_loop_collision_ic* c,
                                 int64_t* off_table);
/* The older loop collision of ic_func.cpp:966-1720, which ic_w_evolution
 * builds in process (ic_func.cpp:25 ships with ic_type "loop collision";
 * positions and velocities of ic_func.cpp:61-72).  The same steps and outputs
 * as lat_loop_collision_ic_device, except that:
 *   - each string's distance is measured from the given position as it stands
 *     (initialConditions.cpp first maps it to the string's rest frame);
 *   - each string's boosted one-form keeps only the boost term
 *     (gamma-1)(v.A)v/|v|^2 (ic_func.cpp:1195-1196, 1229-1230, 1539-1542);
 *   - every string must move: 0 < |v| < 1 (the form divides by |v|^2).
 * ic_func.cpp declares A1s with two elements and stores its z component in
 * A1s[2] (:973, :1100); here that component is a third element, which is what
 * the reference's own build computes (its ic_w_evolution output after three
 * steps matches bit for bit).  Abelian-Higgs handles only; sides >= 3. */
int lat_icfunc_loop_collision_ic_device(lat_handle* h, const lat_string_profile* prof,
                                        const lat_loop_collision_ic* c, int64_t* off_table);
/* Straight strings perturbed by a sine wave of amplitude eps in [0, 1) (the
 * value the reference reads from standard input), built on the device from
 * the profile table into both slots of an Abelian-Higgs handle (one level, as
 * the reference's Data/ic.txt); time step 0.  Sides >= 2.
 *   lat_ng_sine_ic_device     "NG sine", initialConditions.cpp:113-486: a
 *       Nambu-Goto sine wave along z, Omega set so that it is periodic over
 *       dz*nz; per (x, z) column with z >= 0 a golden-section search to 1e-6
 *       for the closest string point; the z < 0 half mirrored as the
 *       reference's loop leaves it.
 *   lat_simple_sine_ic_device "simple sine", :488-668: the straight string
 *       offset along x by eps*sin(Omega z)/Omega, Omega = 2 pi/(dz (nz-1)).
 * off_table (may be null) receives the evaluations beyond the table. */
int lat_ng_sine_ic_device(lat_handle* h, const lat_string_profile* prof, double eps, int64_t* off_table);
int lat_simple_sine_ic_device(lat_handle* h, const lat_string_profile* prof, double eps, int64_t* off_table);

/* The generator on the host (checks, reproduction of device ICs). */
int lat_philox4x32_10(const uint32_t counter[4], const uint32_t key[2], uint32_t out[4]);

/* The FP64 step's sine and cosine (a table-driven reduction to |r| <= pi/512,
 * within about two ulps) evaluated on the current device at n host arguments x, for
 * checks: out (5*n doubles, host) receives sin(x) from the sine alone, then
 * sin(x) and cos(x) from the joint sincos, then CUDA's sin(x) and cos(x).
 * No counterpart in the reference, whose step calls libm's sin and cos
 * (mpi_evolution.cpp:418-487).  n <= 2^26. */
int lat_dtrig_eval(const double* x, int64_t n, double* out);

/* ---- tuning of the tiled FP32 step ------------------------------------------------
 * chunk = x-planes each CTA of the tiled FP32 step marches through.  New
 * handles start with the value tuned for their shape in this process (or
 * loaded from a cache file), else with a heuristic.  lat_autotune times the
 * candidates on a scratch lattice of the same shape (the handle's state is
 * untouched), applies the fastest and remembers it.  No counterpart in the
 * reference. */
typedef struct lat_tuning {
    int32_t chunk;
    int32_t candidates;    /* candidates timed by lat_autotune (0: not tuned) */
    double ms_per_step;    /* measured time of the chosen candidate */
} lat_tuning;
int lat_autotune(lat_handle* h, int32_t trial_steps, lat_tuning* out);
int lat_get_tuning(const lat_handle* h, lat_tuning* out);
int lat_set_tuning(lat_handle* h, const lat_tuning* t);
int lat_tune_cache_save(const char* path);
int lat_tune_cache_load(const char* path);   /* returns the number of entries loaded */

/* Device bytes lat_create would allocate for p (negative status if p is invalid);
 * used for admission by HBM footprint.  No counterpart in the reference. */
int64_t lat_footprint_bytes(const lat_params* p);

/* ---- batches: many lattices advanced by the same launches ----------------------
 * The reference runs one lattice per program invocation; an ensemble of
 * independent lattices (different seeds, couplings, sizes, models) is a loop of
 * runs.  A batch advances all its lattices together: each step is one
 * persistent kernel over the tiles of every lattice, and nsteps of them are one
 * CUDA graph.  Lattices are ordinary FP32 handles (LAT_F32): state transfer,
 * detection and winding keep working on each handle between batch calls.  A
 * lattice's results are bitwise the same alone, in any mix and through
 * lat_step/lat_advance on its own handle. */
typedef struct lat_batch lat_batch;
int lat_batch_create(int32_t max_jobs, lat_batch** out);          /* max_jobs <= 256 */
int lat_batch_destroy(lat_batch* b);                               /* handles are not freed */
/* Add a lattice; it advances until its TimeStep reaches stop_step and records
 * a lat_diag every diag_every steps (0: none).  Returns its slot (>= 0). */
int lat_batch_add(lat_batch* b, lat_handle* h, int32_t diag_every, int64_t stop_step);
int lat_batch_remove(lat_batch* b, lat_handle* h);
int lat_batch_size(const lat_batch* b);
/* x-planes per work item for every lattice of the batch (clamped to its x
   extent); 0 restores the default, which depends on each lattice's shape only
   (64, or 16 for x extents up to 32, clamped to the extent).  Only the
   partial sums of the diagnostics depend on it. */
int lat_batch_set_chunk(lat_batch* b, int32_t chunk);
int64_t lat_batch_kernel_launches(const lat_batch* b);
/* Advance every lattice by up to nsteps (not past its stop_step).  Returns the
 * number of lattices that have not reached their stop_step. */
int lat_batch_advance(lat_batch* b, int32_t nsteps);
/* Move the diagnostics recorded for h so far into out (oldest first). */
int lat_batch_take_diags(lat_batch* b, lat_handle* h, lat_diag* out, int64_t cap, int64_t* count);

/* ---- serving: a job queue with continuous batching ------------------------------
 * The reference runs one job per program invocation (run_mpi_evol.sh,
 * submit_job.sh).  A server owns a worker thread and one batch.  Jobs are
 * admitted in arrival order while their device footprint (lat_footprint_bytes)
 * fits hbm_budget_bytes, get a device random-phase IC
 * (lat_random_phase_ic_device) and join the batch; the batch advances
 * tick_steps steps at a time, jobs arriving meanwhile join at the next tick and
 * finished jobs leave.  Fields stay on the device for a job's whole life.  A
 * job's results are the same whatever else runs beside it.  Served jobs run
 * the FP32 path.  No counterpart in the reference. */
typedef struct lat_server lat_server;
typedef struct lat_server_config {
    int64_t hbm_budget_bytes;   /* device memory the running (and pooled) lattices may hold */
    int32_t tick_steps;         /* steps per batch call (one CUDA graph)                   */
    int32_t max_running;        /* jobs on the device at once, <= 256                      */
} lat_server_config;
typedef struct lat_job_spec {
    lat_params params;          /* precision LAT_F32                                       */
    uint64_t seed;              /* device IC seed                                          */
    int32_t nsteps;             /* steps to run from TimeStep 0                           */
    int32_t diag_every;         /* record energy/Gauss every diag_every steps (0: none)    */
    int32_t independent;        /* Moore: independent phases for phi2                      */
    int32_t winding_at_end;     /* compute sum |winding| of phi (phi1) at the end          */
} lat_job_spec;
typedef struct lat_job_result {
    int64_t job_id;
    int32_t status;             /* 0 queued, 1 running, 2 done, < 0 failed (LAT_ERR_*)     */
    int32_t ndiag;              /* diagnostics recorded (lat_server_diags)                 */
    double submit_s, start_s, end_s;  /* seconds since the server started                   */
    double final_energy;        /* diagnostics of the final level                          */
    double final_gauss;
    int64_t winding_abs;        /* sum |winding| of the final level, if requested          */
    int64_t site_updates;       /* nx*ny*nz*nsteps                                         */
} lat_job_result;
typedef struct lat_server_stats {
    int64_t submitted, queued, running, done, failed;
    int64_t site_updates, ticks;
    int64_t running_bytes, pooled_bytes, peak_bytes;
    double busy_s, wall_s;
} lat_server_stats;
int lat_server_create(const lat_server_config* cfg, lat_server** out);
int lat_server_submit(lat_server* s, const lat_job_spec* spec, int64_t* job_id);
int lat_server_poll(lat_server* s, int64_t job_id, lat_job_result* out);
int lat_server_wait(lat_server* s, int64_t job_id, double timeout_s, lat_job_result* out);
int lat_server_diags(lat_server* s, int64_t job_id, lat_diag* out, int64_t cap, int64_t* count);
int lat_server_get_stats(lat_server* s, lat_server_stats* out);
/* Drops queued jobs, lets running ones finish, frees everything. */
int lat_server_destroy(lat_server* s);

/* ---- stepping without allocation ---------------------------------------------- */
/* Largest lattice (sites) lat_ah_step_f64_noalloc accepts: 64^3. */
#define LAT_NOALLOC_MAX_SITES 262144

/* Advance `nsteps` Abelian-Higgs FP64 steps on fields the caller owns, without
 * allocating any device memory: the same kernels and the same doubles as
 * lat_step on a handle with the same parameters (p->precision LAT_F64 or
 * LAT_F64_FAST, kernel_variant 0, periodic or fixed walls).  No counterpart in
 * the reference: it exists for callers that cannot let a library allocate,
 * e.g. a host application that owns all device memory through its own pool or
 * a fixed budget, or a tight stepping loop that cannot afford cudaMalloc's
 * synchronisation of the device.
 *   fields     device pointer, [5 components][2 slots][nx*ny*nz] doubles in the
 *              reference's slot layout (slot (n+1)%2 holds level n, slot n%2
 *              level n-1; mpi_evolution.cpp:62,370-371); updated in place.
 *   time_step  the TimeStep of the first step (its now level).
 *   stream     cudaStream_t to launch on (NULL: the default stream).  The call
 *              only enqueues work; synchronise the stream before reading.
 * The step's per-site scratch (link data) lives in a fixed array inside the
 * library, LAT_NOALLOC_MAX_SITES*15 doubles (31.5 MiB), held by every GPU that
 * loads the library until the process exits.  Larger lattices are rejected
 * with LAT_ERR_INVALID.  The first call in a CUDA context (per device, and
 * again after cudaDeviceReset or in another context the caller makes current)
 * looks up that array's device address; make that call before any stream
 * capture.  All calls on a device share the array, so calls whose work
 * overlaps on the GPU (different streams, threads or processes sharing the
 * context) race; serialise them. */
int lat_ah_step_f64_noalloc(const lat_params* p, double* fields, int64_t time_step, int32_t nsteps,
                            void* stream);

#ifdef __cplusplus
}
#endif

#endif /* AXIONS_LATTICE_GPU_H */
