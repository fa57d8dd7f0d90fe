/*
 * lattice_oracle.h — CPU restatement of the reference's lattice hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This code is the checker for the CUDA library:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
 * The product (liblattice_gpu.so and the drop-in programs) never links it.
 *
 * Parity: pinned against the reference itself.  oracle/ref/build_ref.py
 * compiles the reference programs from their own sources (single-rank MPI
 * stub, 17-digit output); tests/golden/make_golden.py runs them and stores
 * their outputs as fixtures; tests/test_oracle_golden.py checks this
 * restatement against those fixtures.
 *
 * State layout (same as the reference's calcInd, mpi_evolution.cpp:62):
 *   st[(comp*2 + slot)*N + pos], pos = (i*ny + j)*nz + k, slot = time-level
 *   parity; at TimeStep n, tNow = (n+1)%2 and tPast = n%2.
 *   Components as in include/lattice_gpu.h (AH: 5, Moore: 7).
 */
#ifndef AXIONS_LATTICE_ORACLE_H
#define AXIONS_LATTICE_ORACLE_H

#include <stdint.h>
#include "../include/lattice_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* mt19937 + uniform_real_distribution<double>(0, 2*pi) as libstdc++ computes
 * them (generate_canonical with two 32-bit draws).  Used by
 * mpi_evolution.cpp:290-312. */
typedef struct orc_mt19937 { uint32_t mt[624]; int idx; } orc_mt19937;
void orc_mt_seed(orc_mt19937* g, uint32_t seed);
uint32_t orc_mt_next(orc_mt19937* g);
double orc_uniform_0_2pi(orc_mt19937* g);

/* random-phase IC into a full state (both slots equal, theta = 0) */
int orc_random_phase_ic(const lat_params* p, uint32_t seed, int independent, double* st);

/* set the number of OpenMP threads used by step/diagnostics (<=0: default) */
void orc_set_threads(int n);
int orc_get_threads(void);

/* Neumann boundaries (bc or bc_z LAT_BC_NEUMANN) of level n, in place
 * (evolution.cpp:194-265).  orc_step applies them first; a caller that reads
 * level n as the reference's loop body does after its boundary step (crossing
 * detection) applies them before.  Idempotent. */
int orc_apply_boundaries(const lat_params* p, double* st, int64_t n);

/* One leapfrog step at TimeStep n, in place.  If diag != NULL the
 * diagnostics of the level n (before the update) are computed first. */
int orc_step(const lat_params* p, double* st, int64_t n, lat_diag* diag);

/* diagnostics of level n without stepping */
int orc_diagnostics(const lat_params* p, const double* st, int64_t n, lat_diag* diag);

/* bilinear crossings of scalar `field` on level n (tNow slot) */
int orc_detect(const lat_params* p, const double* st, int64_t n, int field,
               double* xyz, int64_t cap, int64_t* count);

/* plaquette winding of scalar `field` on level n, out = int8[3][N] (may be NULL) */
int orc_winding(const lat_params* p, const double* st, int64_t n, int field,
                int8_t* out, int64_t* abs_sum);

/* ic_func.cpp's "random" IC (minstd_rand, uniform in [-1, 1] per component) */
int orc_icfunc_random_ic(const lat_params* p, uint32_t seed, double* st);

/* Boosted straight-string IC (initialConditions.cpp:710-992 for
 * LAT_IC_FORM_FILE, ic_func.cpp:685-964 for LAT_IC_FORM_INPROCESS) into a
 * full AH state: slot 0 = t 0, slot 1 = t dt.  Returns the number of site
 * evaluations beyond the profile table, or -1 for bad arguments. */
int64_t orc_boost_ic(const lat_params* p, const lat_string_profile* prof, const lat_boost_ic* b, double* st);

/* Loop-collision IC (initialConditions.cpp:994-1716) into a full AH state:
 * slot 0 = t 0, slot 1 = t dt.  Returns the number of evaluations beyond the
 * profile table, or -1 for bad arguments. */
int64_t orc_loop_collision_ic(const lat_params* p, const lat_string_profile* prof, const lat_loop_collision_ic* c,
                              double* st);
int64_t orc_icfunc_loop_collision_ic(const lat_params* p, const lat_string_profile* prof,
                                     const lat_loop_collision_ic* c, double* st);

/* Perturbed straight strings of initialConditions.cpp into both slots of a
 * full AH state: "NG sine" (:113-486, a Nambu-Goto sine wave: per (x, z)
 * column a golden-section search for the closest string point, fields
 * reflected across z = 0) and "simple sine" (:488-668, the straight string
 * offset along x by eps*sin(Omega z)/Omega).  eps is the amplitude the
 * reference reads from standard input.  Return the number of evaluations
 * beyond the profile table, or -1 for bad arguments. */
int64_t orc_ng_sine_ic(const lat_params* p, const lat_string_profile* prof, double eps, double* st);
int64_t orc_simple_sine_ic(const lat_params* p, const lat_string_profile* prof, double eps, double* st);
/* the NG-sine pieces: Omega of the lattice, and one column's string point
 * (xs, zs, xs_sigma, zs_sigma, paraVecMag, normal_dist) */
double orc_ng_omega(double eps, double dz, int64_t nz);
void orc_ng_column(double eps, double Omega, double x, double z, double* out);

/* Test only: move the step's sin/cos results by one ulp for a fraction frac of
 * the arguments (0 = the reference's values), to measure how far one-ulp
 * differences carry through the dynamics. */
void orc_set_trig_perturbation(double frac);

/* total string length by greedy chaining of crossings, ic_w_evolution.cpp:961-1087 */
int orc_string_length(const lat_params* p, const double* xyz, int64_t M, int split, double* L0, double* L1);

#ifdef __cplusplus
}
#endif
#endif
