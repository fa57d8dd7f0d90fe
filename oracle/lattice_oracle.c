/*
 * lattice_oracle.c — CPU restatement of the reference's lattice hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker for the CUDA library; see the header).
 *
 * Every expression keeps the reference's operation order, so that with
 * -ffp-contract=off and the same libm this file reproduces the reference's
 * doubles bit for bit (checked against fixtures made by running the reference;
 * tests/test_oracle_golden.py).  pow(x,2) is written x*x, which is what g++ -O3
 * emits for the reference's pow(x,2).
 */
#include "lattice_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------- */
/* RNG: mt19937 (Matsumoto & Nishimura 1998) and libstdc++'s                  */
/* generate_canonical<double,53> / uniform_real_distribution                  */
/* ------------------------------------------------------------------------- */

void orc_mt_seed(orc_mt19937* g, uint32_t seed)
{
    g->mt[0] = seed;
    for (int i = 1; i < 624; ++i)
        g->mt[i] = 1812433253u * (g->mt[i - 1] ^ (g->mt[i - 1] >> 30)) + (uint32_t)i;
    g->idx = 624;
}

static void orc_mt_twist(orc_mt19937* g)
{
    for (int i = 0; i < 624; ++i) {
        uint32_t y = (g->mt[i] & 0x80000000u) | (g->mt[(i + 1) % 624] & 0x7fffffffu);
        uint32_t v = g->mt[(i + 397) % 624] ^ (y >> 1);
        if (y & 1u) v ^= 0x9908b0dfu;
        g->mt[i] = v;
    }
    g->idx = 0;
}

uint32_t orc_mt_next(orc_mt19937* g)
{
    if (g->idx >= 624) orc_mt_twist(g);
    uint32_t y = g->mt[g->idx++];
    y ^= (y >> 11);
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= (y >> 18);
    return y;
}

/* uniform_real_distribution<double>(0, 2*pi) with pi = 4*atan(1)
 * (mpi_evolution.cpp:12,291): u = (g1 + g2*2^32) / 2^64, clamped below 1,
 * value = u*(b - a) + a. */
double orc_uniform_0_2pi(orc_mt19937* g)
{
    double sum = 0.0;
    double tmp = 1.0;
    sum += (double)orc_mt_next(g) * tmp;
    tmp *= 4294967296.0;
    sum += (double)orc_mt_next(g) * tmp;
    tmp *= 4294967296.0;
    double u = sum / tmp;
    if (u >= 1.0) u = nextafter(1.0, 0.0);
    const double pi = 4.0 * atan(1.0);
    const double b = 2 * pi, a = 0.0;
    return u * (b - a) + a;
}

static int ncomp_of(const lat_params* p) { return p->model == LAT_MODEL_MOORE ? 7 : 5; }

int orc_random_phase_ic(const lat_params* p, uint32_t seed, int independent, double* st)
{
    const int64_t N = p->nx * p->ny * p->nz;
    const int nc = ncomp_of(p);
    memset(st, 0, sizeof(double) * (size_t)nc * 2 * (size_t)N);
    orc_mt19937 g;
    orc_mt_seed(&g, seed);
    for (int64_t s = 0; s < N; ++s) {
        double phase = orc_uniform_0_2pi(&g);
        double ph2 = phase;
        if (p->model == LAT_MODEL_MOORE && independent) ph2 = orc_uniform_0_2pi(&g);
        double v[4];
        v[0] = p->eta * cos(phase);
        v[1] = p->eta * sin(phase);
        int ns = 2;
        if (p->model == LAT_MODEL_MOORE) {
            v[2] = p->eta2 * cos(ph2);
            v[3] = p->eta2 * sin(ph2);
            ns = 4;
        }
        for (int c = 0; c < ns; ++c) {
            st[((int64_t)c * 2 + 0) * N + s] = v[c];
            st[((int64_t)c * 2 + 1) * N + s] = v[c];
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------- */
/* threads                                                                    */
/* ------------------------------------------------------------------------- */
static int g_threads = 0;
void orc_set_threads(int n) { g_threads = n; }
int orc_get_threads(void)
{
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------- */
/* geometry                                                                   */
/* ------------------------------------------------------------------------- */
typedef struct {
    int64_t nx, ny, nz, N, syz;
    int lox, loy, loz, hix, hiy, hiz;   /* evolved region: [lo, hi) per axis */
    int kxy, kz;                        /* LAT_BC_* of the x/y axes and of z */
} geo_t;

/* the boundary kind of z: bc_z, or the same as bc */
static int z_kind(const lat_params* p)
{
    switch (p->bc_z) {
    case LAT_BCZ_PERIODIC: return LAT_BC_PERIODIC;
    case LAT_BCZ_FIXED: return LAT_BC_FIXED;
    case LAT_BCZ_NEUMANN: return LAT_BC_NEUMANN;
    default: return p->bc;
    }
}

/* evolution.cpp:166-186: every non-periodic axis evolves its interior */
static geo_t make_geo(const lat_params* p)
{
    geo_t g;
    g.nx = p->nx; g.ny = p->ny; g.nz = p->nz;
    g.N = g.nx * g.ny * g.nz;
    g.syz = g.ny * g.nz;
    g.kxy = p->bc;
    g.kz = z_kind(p);
    const int pxy = g.kxy == LAT_BC_PERIODIC, pz = g.kz == LAT_BC_PERIODIC;
    g.lox = g.loy = pxy ? 0 : 1;
    g.hix = pxy ? (int)g.nx : (int)g.nx - 1;
    g.hiy = pxy ? (int)g.ny : (int)g.ny - 1;
    g.loz = pz ? 0 : 1;
    g.hiz = pz ? (int)g.nz : (int)g.nz - 1;
    return g;
}

static inline int64_t wrapp(int64_t a, int64_t n) { return a + 1 == n ? 0 : a + 1; }
static inline int64_t wrapm(int64_t a, int64_t n) { return a == 0 ? n - 1 : a - 1; }
static inline int64_t site(const geo_t* g, int64_t i, int64_t j, int64_t k) { return (i * g->ny + j) * g->nz + k; }

/* friction coefficient and damping of step n (mpi_evolution.cpp:356-368) */
static void friction_of(const lat_params* p, int64_t n, double* damp, double* fric)
{
    double time = p->tau0 + n * p->dt;
    *damp = (n < p->damped_nt) ? p->dampFac : 0;
    *fric = *damp + p->alpha * p->scaling / time;
}

#define ST(c, t, s) st[((int64_t)(c) * 2 + (t)) * N + (s)]

/* ------------------------------------------------------------------------- */
/* Abelian-Higgs step: mpi_evolution.cpp:381-501 (== evolution.cpp:273-373 + */
/* 1384-1402 for the fields).  Components: 0,1 = phi; 2,3,4 = theta_x,y,z.     */
/* ------------------------------------------------------------------------- */
/* ------------------------------------------------------------------------- */
/* Neumann boundaries of the now level, in place (evolution.cpp:194-265): the  */
/* y faces (x interior), then the x faces (all y), then the z faces, theta     */
/* copied from the next layer in and phi transported along its link.  The z    */
/* pass runs over x planes i < nz (and i < nx) as the reference's loop does.   */
/* ------------------------------------------------------------------------- */
#define TH(m, t, s) ST(2 + (m), t, s)
#define PH(c, t, s) ST(c, t, s)

/* Sensitivity probe (test infrastructure): with orc_set_trig_perturbation(f)
 * and f > 0, the sine and cosine of the step, the diagnostics and the
 * boundaries return glibc's value moved by one ulp for a fraction f of their
 * arguments (chosen by a hash of the argument's bits, so the choice does not
 * depend on threads or order).  f = 0 (the default) leaves every value as the
 * reference's. */
static double g_trig_perturb = 0.0;
void orc_set_trig_perturbation(double frac) { g_trig_perturb = frac; }
static inline double trig_bump(double x, double y)
{
    uint64_t z;
    memcpy(&z, &x, 8);
    z += 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    z ^= z >> 31;
    if ((double)(z >> 11) * (1.0 / 9007199254740992.0) >= g_trig_perturb) return y;
    return nextafter(y, (z & 1) ? INFINITY : -INFINITY);
}
static inline double psin(double x) { const double y = sin(x); return g_trig_perturb > 0 ? trig_bump(x, y) : y; }
static inline double pcos(double x) { const double y = cos(x); return g_trig_perturb > 0 ? trig_bump(x, y) : y; }

static void neumann_pair(double* st, int64_t N, int tNow, int mu, int64_t b0, int64_t i0, int64_t b1, int64_t i1)
{
    const int c[2] = {1, -1};
    for (int m = 0; m < 3; ++m) {
        TH(m, tNow, b0) = TH(m, tNow, i0);
        TH(m, tNow, b1) = TH(m, tNow, i1);
    }
    for (int comp = 0; comp < 2; ++comp) {
        const int oc = comp + c[comp];
        const double cc = (double)c[comp];
        PH(comp, tNow, b0) = pcos(TH(mu, tNow, b0)) * PH(comp, tNow, i0) + cc * psin(TH(mu, tNow, b0)) * PH(oc, tNow, i0);
        PH(comp, tNow, b1) = pcos(TH(mu, tNow, i1)) * PH(comp, tNow, i1) - cc * psin(TH(mu, tNow, i1)) * PH(oc, tNow, i1);
    }
}

/* Moore: phi_a transported along q_a * theta (mooreEvol.cpp:114-160); components
 * phi1 (0, 1), phi2 (2, 3), theta (4, 5, 6) */
static void neumann_pair_moore(const lat_params* p, double* st, int64_t N, int tNow, int mu, int64_t b0, int64_t i0,
                               int64_t b1, int64_t i1)
{
    const int c[2] = {1, -1};
    for (int m = 0; m < 3; ++m) {
        ST(4 + m, tNow, b0) = ST(4 + m, tNow, i0);
        ST(4 + m, tNow, b1) = ST(4 + m, tNow, i1);
    }
    for (int comp = 0; comp < 2; ++comp) {
        const double cc = (double)c[comp];
        for (int a = 0; a < 2; ++a) {
            const double q = a == 0 ? p->q1 : p->q2;
            const int f = 2 * a + comp, o = 2 * a + comp + c[comp];
            ST(f, tNow, b0) = pcos(q * ST(4 + mu, tNow, b0)) * ST(f, tNow, i0) + cc * psin(q * ST(4 + mu, tNow, b0)) * ST(o, tNow, i0);
            ST(f, tNow, b1) = pcos(q * ST(4 + mu, tNow, i1)) * ST(f, tNow, i1) - cc * psin(q * ST(4 + mu, tNow, i1)) * ST(o, tNow, i1);
        }
    }
}

int orc_apply_boundaries(const lat_params* p, double* st, int64_t n)
{
    if (!p || !st) return LAT_ERR_INVALID;
    const geo_t G = make_geo(p);
    const int64_t N = G.N;
    const int tNow = (int)((n + 1) % 2);
    const int64_t nx = G.nx, ny = G.ny, nz = G.nz;
    if (p->model == LAT_MODEL_MOORE) {
        if (G.kxy == LAT_BC_NEUMANN) {
            for (int64_t i = 1; i < nx - 1; ++i)
                for (int64_t k = G.loz; k < G.hiz; ++k)
                    neumann_pair_moore(p, st, N, tNow, 1, site(&G, i, 0, k), site(&G, i, 1, k), site(&G, i, ny - 1, k),
                                       site(&G, i, ny - 2, k));
            for (int64_t j = 0; j < ny; ++j)
                for (int64_t k = G.loz; k < G.hiz; ++k)
                    neumann_pair_moore(p, st, N, tNow, 0, site(&G, 0, j, k), site(&G, 1, j, k), site(&G, nx - 1, j, k),
                                       site(&G, nx - 2, j, k));
        }
        return 0;
    }
    if (G.kxy == LAT_BC_NEUMANN) {
        for (int64_t i = 1; i < nx - 1; ++i)
            for (int64_t k = G.loz; k < G.hiz; ++k)
                neumann_pair(st, N, tNow, 1, site(&G, i, 0, k), site(&G, i, 1, k), site(&G, i, ny - 1, k),
                             site(&G, i, ny - 2, k));
        for (int64_t j = 0; j < ny; ++j)
            for (int64_t k = G.loz; k < G.hiz; ++k)
                neumann_pair(st, N, tNow, 0, site(&G, 0, j, k), site(&G, 1, j, k), site(&G, nx - 1, j, k),
                             site(&G, nx - 2, j, k));
    }
    if (G.kz == LAT_BC_NEUMANN) {
        const int64_t ni = nz < nx ? nz : nx;
        for (int64_t i = 0; i < ni; ++i)
            for (int64_t j = 0; j < ny; ++j)
                neumann_pair(st, N, tNow, 2, site(&G, i, j, 0), site(&G, i, j, 1), site(&G, i, j, nz - 1),
                             site(&G, i, j, nz - 2));
    }
    return 0;
}

/* ------------------------------------------------------------------------- */
/* absorbing x/y boundaries (evolution.cpp:446-691): second time derivatives  */
/* of the outer layer from one-sided first-order formulas, into btt[5][N]     */
/* (boundary sites only); written before the interior update overwrites the  */
/* past level it reads.                                                       */
/* ------------------------------------------------------------------------- */
/* covariant second difference along mu at s (neighbours sp, sm) */
static double cov2(const double* st, int64_t N, int tNow, int comp, int mu, int64_t s, int64_t sp, int64_t sm, double d)
{
    const int c[2] = {1, -1};
    const int oc = comp + c[comp];
    const double cc = (double)c[comp];
    return (pcos(TH(mu, tNow, s)) * PH(comp, tNow, sp) + cc * psin(TH(mu, tNow, s)) * PH(oc, tNow, sp) - 2 * PH(comp, tNow, s)
            + pcos(TH(mu, tNow, sm)) * PH(comp, tNow, sm) - cc * psin(TH(mu, tNow, sm)) * PH(oc, tNow, sm)) / (d * d);
}

/* one-sided time-space difference at the low face: s0 boundary, s1 = s0 + mu */
static double near_ts(const double* st, int64_t N, int tNow, int tPast, int comp, int mu, int64_t s0, int64_t s1,
                      double dt, double d)
{
    const int c[2] = {1, -1};
    const int oc = comp + c[comp];
    const double cc = (double)c[comp];
    return (pcos(TH(mu, tNow, s0)) * PH(comp, tNow, s1) + cc * psin(TH(mu, tNow, s0)) * PH(oc, tNow, s1) - PH(comp, tNow, s0)
            - pcos(TH(mu, tPast, s0)) * PH(comp, tPast, s1) - cc * psin(TH(mu, tPast, s0)) * PH(oc, tPast, s1)
            + PH(comp, tPast, s0)) / (dt * d);
}

/* at the high face: s0 boundary, s1 = s0 - mu; the past cos reads the link at sc
 * (s1, except at the (nx-1, ny-1) corner's x term, evolution.cpp:656) */
static double far_ts(const double* st, int64_t N, int tNow, int tPast, int comp, int mu, int64_t s0, int64_t s1,
                     int64_t sc, double dt, double d)
{
    const int c[2] = {1, -1};
    const int oc = comp + c[comp];
    const double cc = (double)c[comp];
    return (PH(comp, tNow, s0) - pcos(TH(mu, tNow, s1)) * PH(comp, tNow, s1) + cc * psin(TH(mu, tNow, s1)) * PH(oc, tNow, s1)
            - PH(comp, tPast, s0) + pcos(TH(mu, tPast, sc)) * PH(comp, tPast, s1)
            - cc * psin(TH(mu, tPast, s1)) * PH(oc, tPast, s1)) / (dt * d);
}

static double th2(const double* st, int64_t N, int tNow, int m, int64_t sp, int64_t s, int64_t sm, double d)
{
    return (TH(m, tNow, sp) - 2 * TH(m, tNow, s) + TH(m, tNow, sm)) / (d * d);
}

static double th_near(const double* st, int64_t N, int tNow, int tPast, int m, int64_t s0, int64_t s1, double dt, double d)
{
    return (TH(m, tNow, s1) - TH(m, tNow, s0) - TH(m, tPast, s1) + TH(m, tPast, s0)) / (dt * d);
}

static double th_far(const double* st, int64_t N, int tNow, int tPast, int m, int64_t s0, int64_t s1, double dt, double d)
{
    return (TH(m, tNow, s0) - TH(m, tNow, s1) - TH(m, tPast, s0) + TH(m, tPast, s1)) / (dt * d);
}

#define BTT(c, s) btt[(int64_t)(c) * N + (s)]

static void absorb_tt(const lat_params* p, const double* st, int64_t n, double* btt)
{
    const geo_t G = make_geo(p);
    const int64_t N = G.N, nx = G.nx, ny = G.ny, nz = G.nz;
    const int tNow = (int)((n + 1) % 2), tPast = (int)(n % 2);
    const double dx = p->dx, dy = p->dy, dz = p->dz, dt = p->dt;
    for (int64_t k = G.loz; k < G.hiz; ++k) {
        const int64_t kp = (k + 1) % nz, km = (k - 1 + nz) % nz;
        /* x faces (evolution.cpp:447-509) */
        for (int64_t j = 1; j < ny - 1; ++j) {
            const int64_t a = site(&G, 0, j, k), b = site(&G, nx - 1, j, k);
            for (int comp = 0; comp < 2; ++comp) {
                double yy = cov2(st, N, tNow, comp, 1, a, site(&G, 0, j + 1, k), site(&G, 0, j - 1, k), dy);
                double zz = cov2(st, N, tNow, comp, 2, a, site(&G, 0, j, kp), site(&G, 0, j, km), dz);
                double tx = near_ts(st, N, tNow, tPast, comp, 0, a, site(&G, 1, j, k), dt, dx);
                BTT(comp, a) = tx + 0.5 * (yy + zz);
                yy = cov2(st, N, tNow, comp, 1, b, site(&G, nx - 1, j + 1, k), site(&G, nx - 1, j - 1, k), dy);
                zz = cov2(st, N, tNow, comp, 2, b, site(&G, nx - 1, j, kp), site(&G, nx - 1, j, km), dz);
                const int64_t b1 = site(&G, nx - 2, j, k);
                tx = far_ts(st, N, tNow, tPast, comp, 0, b, b1, b1, dt, dx);
                BTT(comp, b) = -tx + 0.5 * (yy + zz);
            }
            for (int m = 0; m < 3; ++m) {
                double yy = th2(st, N, tNow, m, site(&G, 0, j + 1, k), a, site(&G, 0, j - 1, k), dy);
                double zz = th2(st, N, tNow, m, site(&G, 0, j, kp), a, site(&G, 0, j, km), dz);
                double tx = th_near(st, N, tNow, tPast, m, a, site(&G, 1, j, k), dt, dx);
                BTT(2 + m, a) = tx + 0.5 * (yy + zz);
                yy = th2(st, N, tNow, m, site(&G, nx - 1, j + 1, k), b, site(&G, nx - 1, j - 1, k), dy);
                zz = th2(st, N, tNow, m, site(&G, nx - 1, j, kp), b, site(&G, nx - 1, j, km), dz);
                tx = th_far(st, N, tNow, tPast, m, b, site(&G, nx - 2, j, k), dt, dx);
                BTT(2 + m, b) = -tx + 0.5 * (yy + zz);
            }
        }
        /* y faces (:511-573) */
        for (int64_t i = 1; i < nx - 1; ++i) {
            const int64_t a = site(&G, i, 0, k), b = site(&G, i, ny - 1, k);
            for (int comp = 0; comp < 2; ++comp) {
                double xx = cov2(st, N, tNow, comp, 0, a, site(&G, i + 1, 0, k), site(&G, i - 1, 0, k), dx);
                double zz = cov2(st, N, tNow, comp, 2, a, site(&G, i, 0, kp), site(&G, i, 0, km), dz);
                double ty = near_ts(st, N, tNow, tPast, comp, 1, a, site(&G, i, 1, k), dt, dy);
                BTT(comp, a) = ty + 0.5 * (xx + zz);
                xx = cov2(st, N, tNow, comp, 0, b, site(&G, i + 1, ny - 1, k), site(&G, i - 1, ny - 1, k), dx);
                zz = cov2(st, N, tNow, comp, 2, b, site(&G, i, ny - 1, kp), site(&G, i, ny - 1, km), dz);
                const int64_t b1 = site(&G, i, ny - 2, k);
                ty = far_ts(st, N, tNow, tPast, comp, 1, b, b1, b1, dt, dy);
                BTT(comp, b) = -ty + 0.5 * (xx + zz);
            }
            for (int m = 0; m < 3; ++m) {
                double xx = th2(st, N, tNow, m, site(&G, i + 1, 0, k), a, site(&G, i - 1, 0, k), dx);
                double zz = th2(st, N, tNow, m, site(&G, i, 0, kp), a, site(&G, i, 0, km), dz);
                double ty = th_near(st, N, tNow, tPast, m, a, site(&G, i, 1, k), dt, dy);
                BTT(2 + m, a) = ty + 0.5 * (xx + zz);
                xx = th2(st, N, tNow, m, site(&G, i + 1, ny - 1, k), b, site(&G, i - 1, ny - 1, k), dx);
                zz = th2(st, N, tNow, m, site(&G, i, ny - 1, kp), b, site(&G, i, ny - 1, km), dz);
                ty = th_far(st, N, tNow, tPast, m, b, site(&G, i, ny - 2, k), dt, dy);
                BTT(2 + m, b) = -ty + 0.5 * (xx + zz);
            }
        }
        /* corners (:575-689) */
        const int64_t c00 = site(&G, 0, 0, k), c01 = site(&G, 0, ny - 1, k);
        const int64_t c10 = site(&G, nx - 1, 0, k), c11 = site(&G, nx - 1, ny - 1, k);
        for (int comp = 0; comp < 2; ++comp) {
            double zz = cov2(st, N, tNow, comp, 2, c00, site(&G, 0, 0, kp), site(&G, 0, 0, km), dz);
            double tx = near_ts(st, N, tNow, tPast, comp, 0, c00, site(&G, 1, 0, k), dt, dx);
            double ty = near_ts(st, N, tNow, tPast, comp, 1, c00, site(&G, 0, 1, k), dt, dy);
            BTT(comp, c00) = (zz + 2 * (tx + ty)) / 3;
            zz = cov2(st, N, tNow, comp, 2, c01, site(&G, 0, ny - 1, kp), site(&G, 0, ny - 1, km), dz);
            tx = near_ts(st, N, tNow, tPast, comp, 0, c01, site(&G, 1, ny - 1, k), dt, dx);
            int64_t s1 = site(&G, 0, ny - 2, k);
            ty = far_ts(st, N, tNow, tPast, comp, 1, c01, s1, s1, dt, dy);
            BTT(comp, c01) = (zz + 2 * (tx - ty)) / 3;
            zz = cov2(st, N, tNow, comp, 2, c10, site(&G, nx - 1, 0, kp), site(&G, nx - 1, 0, km), dz);
            s1 = site(&G, nx - 2, 0, k);
            tx = far_ts(st, N, tNow, tPast, comp, 0, c10, s1, s1, dt, dx);
            ty = near_ts(st, N, tNow, tPast, comp, 1, c10, site(&G, nx - 1, 1, k), dt, dy);
            BTT(comp, c10) = (zz - 2 * (tx - ty)) / 3;
            zz = cov2(st, N, tNow, comp, 2, c11, site(&G, nx - 1, ny - 1, kp), site(&G, nx - 1, ny - 1, km), dz);
            tx = far_ts(st, N, tNow, tPast, comp, 0, c11, site(&G, nx - 2, ny - 1, k), c11, dt, dx);
            s1 = site(&G, nx - 1, ny - 2, k);
            ty = far_ts(st, N, tNow, tPast, comp, 1, c11, s1, s1, dt, dy);
            BTT(comp, c11) = (zz - 2 * (tx + ty)) / 3;
        }
        for (int m = 0; m < 3; ++m) {
            double zz = th2(st, N, tNow, m, site(&G, 0, 0, kp), c00, site(&G, 0, 0, km), dz);
            double tx = th_near(st, N, tNow, tPast, m, c00, site(&G, 1, 0, k), dt, dx);
            double ty = th_near(st, N, tNow, tPast, m, c00, site(&G, 0, 1, k), dt, dy);
            BTT(2 + m, c00) = (zz + 2 * (tx + ty)) / 3;
            zz = th2(st, N, tNow, m, site(&G, 0, ny - 1, kp), c01, site(&G, 0, ny - 1, km), dz);
            tx = th_near(st, N, tNow, tPast, m, c01, site(&G, 1, ny - 1, k), dt, dx);
            ty = th_far(st, N, tNow, tPast, m, c01, site(&G, 0, ny - 2, k), dt, dy);
            BTT(2 + m, c01) = (zz + 2 * (tx - ty)) / 3;
            zz = th2(st, N, tNow, m, site(&G, nx - 1, 0, kp), c10, site(&G, nx - 1, 0, km), dz);
            tx = th_far(st, N, tNow, tPast, m, c10, site(&G, nx - 2, 0, k), dt, dx);
            ty = th_near(st, N, tNow, tPast, m, c10, site(&G, nx - 1, 1, k), dt, dy);
            BTT(2 + m, c10) = (zz - 2 * (tx - ty)) / 3;
            zz = th2(st, N, tNow, m, site(&G, nx - 1, ny - 1, kp), c11, site(&G, nx - 1, ny - 1, km), dz);
            tx = th_far(st, N, tNow, tPast, m, c11, site(&G, nx - 2, ny - 1, k), dt, dx);
            ty = th_far(st, N, tNow, tPast, m, c11, site(&G, nx - 1, ny - 2, k), dt, dy);
            BTT(2 + m, c11) = (zz - 2 * (tx + ty)) / 3;
        }
    }
}

/* the outer x/y layer's update with btt (evolution.cpp:1375-1402) */
static void absorb_update(const lat_params* p, double* st, int64_t n, const double* btt)
{
    const geo_t G = make_geo(p);
    const int64_t N = G.N, nx = G.nx, ny = G.ny;
    const int tNow = (int)((n + 1) % 2), tPast = (int)(n % 2);
    const double dt = p->dt;
    for (int64_t i = 0; i < nx; ++i)
        for (int64_t j = 0; j < ny; ++j) {
            if (i != 0 && i != nx - 1 && j != 0 && j != ny - 1) continue;
            for (int64_t k = G.loz; k < G.hiz; ++k) {
                const int64_t s = site(&G, i, j, k);
                for (int c = 0; c < 5; ++c)
                    ST(c, tPast, s) = 2 * ST(c, tNow, s) - ST(c, tPast, s) + dt * dt * BTT(c, s);
            }
        }
}

#undef TH
#undef PH

static void ah_update(const lat_params* p, double* st, int64_t n)
{
    const geo_t G = make_geo(p);
    const int64_t N = G.N;
    const int tNow = (int)((n + 1) % 2), tPast = (int)(n % 2);
    double* btt = NULL;
    if (G.kxy == LAT_BC_ABSORBING) {
        btt = (double*)calloc((size_t)(5 * N), sizeof(double));
        if (btt) absorb_tt(p, st, n, btt);
    }
    double damp, fric;
    friction_of(p, n, &damp, &fric);
    const double dx = p->dx, dy = p->dy, dz = p->dz, dt = p->dt;
    const double lambda = p->lambda, eta = p->eta, g = p->g;
    const int c[2] = {1, -1};

#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
    for (int64_t i = G.lox; i < G.hix; ++i) {
        const int64_t ip = wrapp(i, G.nx), im = wrapm(i, G.nx);
        for (int64_t j = G.loy; j < G.hiy; ++j) {
            const int64_t jp = wrapp(j, G.ny), jm = wrapm(j, G.ny);
            for (int64_t k = G.loz; k < G.hiz; ++k) {
                const int64_t kp = wrapp(k, G.nz), km = wrapm(k, G.nz);
                const int64_t s = site(&G, i, j, k);
                const int64_t ipx = site(&G, ip, j, k), imx = site(&G, im, j, k);
                const int64_t ipy = site(&G, i, jp, k), imy = site(&G, i, jm, k);
                const int64_t ipz = site(&G, i, j, kp), imz = site(&G, i, j, km);
                const int64_t ipxmy = site(&G, ip, jm, k), ipxmz = site(&G, ip, j, km);
                const int64_t imxpy = site(&G, im, jp, k), ipymz = site(&G, i, jp, km);
                const int64_t imxpz = site(&G, im, j, kp), imypz = site(&G, i, jm, kp);

                double phiMagSqr = ST(0, tNow, s) * ST(0, tNow, s) + ST(1, tNow, s) * ST(1, tNow, s);
                for (int comp = 0; comp < 2; ++comp) {
                    const int oc = comp + c[comp];
                    const double cc = (double)c[comp];
                    double phixx = (pcos(ST(2, tNow, s)) * ST(comp, tNow, ipx) + cc * psin(ST(2, tNow, s)) * ST(oc, tNow, ipx) - 2 * ST(comp, tNow, s)
                                    + pcos(ST(2, tNow, imx)) * ST(comp, tNow, imx) - cc * psin(ST(2, tNow, imx)) * ST(oc, tNow, imx)) / (dx * dx);
                    double phiyy = (pcos(ST(3, tNow, s)) * ST(comp, tNow, ipy) + cc * psin(ST(3, tNow, s)) * ST(oc, tNow, ipy) - 2 * ST(comp, tNow, s)
                                    + pcos(ST(3, tNow, imy)) * ST(comp, tNow, imy) - cc * psin(ST(3, tNow, imy)) * ST(oc, tNow, imy)) / (dy * dy);
                    double phizz = (pcos(ST(4, tNow, s)) * ST(comp, tNow, ipz) + cc * psin(ST(4, tNow, s)) * ST(oc, tNow, ipz) - 2 * ST(comp, tNow, s)
                                    + pcos(ST(4, tNow, imz)) * ST(comp, tNow, imz) - cc * psin(ST(4, tNow, imz)) * ST(oc, tNow, imz)) / (dz * dz);
                    double phitt = phixx + phiyy + phizz - 0.5 * lambda * (phiMagSqr - eta * eta) * ST(comp, tNow, s);
                    if (fric != 0) {
                        double phit = (ST(comp, tNow, s) - ST(comp, tPast, s)) / dt;
                        phitt = phitt - fric * phit;
                    }
                    ST(comp, tPast, s) = 2 * ST(comp, tNow, s) - ST(comp, tPast, s) + dt * dt * phitt;
                }

                double curx = pcos(ST(2, tNow, s)) * (ST(1, tNow, s) * ST(0, tNow, ipx) - ST(0, tNow, s) * ST(1, tNow, ipx))
                            + psin(ST(2, tNow, s)) * (ST(0, tNow, s) * ST(0, tNow, ipx) + ST(1, tNow, s) * ST(1, tNow, ipx));
                double cury = pcos(ST(3, tNow, s)) * (ST(1, tNow, s) * ST(0, tNow, ipy) - ST(0, tNow, s) * ST(1, tNow, ipy))
                            + psin(ST(3, tNow, s)) * (ST(0, tNow, s) * ST(0, tNow, ipy) + ST(1, tNow, s) * ST(1, tNow, ipy));
                double curz = pcos(ST(4, tNow, s)) * (ST(1, tNow, s) * ST(0, tNow, ipz) - ST(0, tNow, s) * ST(1, tNow, ipz))
                            + psin(ST(4, tNow, s)) * (ST(0, tNow, s) * ST(0, tNow, ipz) + ST(1, tNow, s) * ST(1, tNow, ipz));

                double Fxy_y = (psin(ST(2, tNow, s) + ST(3, tNow, ipx) - ST(2, tNow, ipy) - ST(3, tNow, s))
                              - psin(ST(2, tNow, imy) + ST(3, tNow, ipxmy) - ST(2, tNow, s) - ST(3, tNow, imy))) / (dy * dy);
                double Fxz_z = (psin(ST(2, tNow, s) + ST(4, tNow, ipx) - ST(2, tNow, ipz) - ST(4, tNow, s))
                              - psin(ST(2, tNow, imz) + ST(4, tNow, ipxmz) - ST(2, tNow, s) - ST(4, tNow, imz))) / (dz * dz);
                double Fyx_x = (psin(ST(3, tNow, s) + ST(2, tNow, ipy) - ST(3, tNow, ipx) - ST(2, tNow, s))
                              - psin(ST(3, tNow, imx) + ST(2, tNow, imxpy) - ST(3, tNow, s) - ST(2, tNow, imx))) / (dx * dx);
                double Fyz_z = (psin(ST(3, tNow, s) + ST(4, tNow, ipy) - ST(3, tNow, ipz) - ST(4, tNow, s))
                              - psin(ST(3, tNow, imz) + ST(4, tNow, ipymz) - ST(3, tNow, s) - ST(4, tNow, imz))) / (dz * dz);
                double Fzx_x = (psin(ST(4, tNow, s) + ST(2, tNow, ipz) - ST(4, tNow, ipx) - ST(2, tNow, s))
                              - psin(ST(4, tNow, imx) + ST(2, tNow, imxpz) - ST(4, tNow, s) - ST(2, tNow, imx))) / (dx * dx);
                double Fzy_y = (psin(ST(4, tNow, s) + ST(3, tNow, ipz) - ST(4, tNow, ipy) - ST(3, tNow, s))
                              - psin(ST(4, tNow, imy) + ST(3, tNow, imypz) - ST(4, tNow, s) - ST(3, tNow, imy))) / (dy * dy);

                double tt[3];
                tt[0] = -2 * g * g * curx - Fxy_y - Fxz_z;
                tt[1] = -2 * g * g * cury - Fyx_x - Fyz_z;
                tt[2] = -2 * g * g * curz - Fzx_x - Fzy_y;
                if (damp != 0) {
                    for (int m = 0; m < 3; ++m) {
                        double thetat = (ST(2 + m, tNow, s) - ST(2 + m, tPast, s)) / dt;
                        tt[m] = tt[m] - damp * thetat;
                    }
                }
                for (int m = 0; m < 3; ++m)
                    ST(2 + m, tPast, s) = 2 * ST(2 + m, tNow, s) - ST(2 + m, tPast, s) + dt * dt * tt[m];
            }
        }
    }
    if (btt) {
        absorb_update(p, st, n, btt);
        free(btt);
    }
}

/* Abelian-Higgs diagnostics of level n: evolution.cpp:294-427 (energy, Gauss)
 * or, for LAT_ENERGY_MPI, mpi_evolution.cpp:509-532 (energy). */
static void ah_diag(const lat_params* p, const double* st, int64_t n, lat_diag* out)
{
    const geo_t G = make_geo(p);
    const int64_t N = G.N;
    const int tNow = (int)((n + 1) % 2), tPast = (int)(n % 2);
    const double dx = p->dx, dy = p->dy, dz = p->dz, dt = p->dt;
    const double lambda = p->lambda, eta = p->eta, g = p->g;
    const int c[2] = {1, -1};
    const int mpi_form = p->energy_form == LAT_ENERGY_MPI;
    double energy = 0, dev = 0;

#pragma omp parallel for schedule(static) reduction(+:energy,dev) num_threads(orc_get_threads())
    for (int64_t i = G.lox; i < G.hix; ++i) {
        const int64_t ip = wrapp(i, G.nx), im = wrapm(i, G.nx);
        for (int64_t j = G.loy; j < G.hiy; ++j) {
            const int64_t jp = wrapp(j, G.ny), jm = wrapm(j, G.ny);
            for (int64_t k = G.loz; k < G.hiz; ++k) {
                const int64_t kp = wrapp(k, G.nz), km = wrapm(k, G.nz);
                const int64_t s = site(&G, i, j, k);
                const int64_t ipx = site(&G, ip, j, k), imx = site(&G, im, j, k);
                const int64_t ipy = site(&G, i, jp, k), imy = site(&G, i, jm, k);
                const int64_t ipz = site(&G, i, j, kp), imz = site(&G, i, j, km);
                double phiMagSqr = ST(0, tNow, s) * ST(0, tNow, s) + ST(1, tNow, s) * ST(1, tNow, s);
                double phit[2], phix[2], phiy[2], phiz[2];
                for (int comp = 0; comp < 2; ++comp) {
                    const int oc = comp + c[comp];
                    const double cc = (double)c[comp];
                    phit[comp] = (ST(comp, tNow, s) - ST(comp, tPast, s)) / dt;
                    phix[comp] = (ST(comp, tNow, s) - pcos(ST(2, tNow, imx)) * ST(comp, tNow, imx) + cc * psin(ST(2, tNow, imx)) * ST(oc, tNow, imx)) / dx;
                    phiy[comp] = (ST(comp, tNow, s) - pcos(ST(3, tNow, imy)) * ST(comp, tNow, imy) + cc * psin(ST(3, tNow, imy)) * ST(oc, tNow, imy)) / dy;
                    phiz[comp] = (ST(comp, tNow, s) - pcos(ST(4, tNow, imz)) * ST(comp, tNow, imz) + cc * psin(ST(4, tNow, imz)) * ST(oc, tNow, imz)) / dz;
                }
                double Pxy = ST(2, tNow, s) + ST(3, tNow, ipx) - ST(2, tNow, ipy) - ST(3, tNow, s);
                double Pxz = ST(2, tNow, s) + ST(4, tNow, ipx) - ST(2, tNow, ipz) - ST(4, tNow, s);
                double Pyz = ST(3, tNow, s) + ST(4, tNow, ipy) - ST(3, tNow, ipz) - ST(4, tNow, s);
                double gauss = 0, thetaDotCont = 0, FCont = 0;
                if (mpi_form) {
                    double t0 = (ST(2, tNow, s) - ST(2, tPast, s)) / dt;
                    double t1 = (ST(3, tNow, s) - ST(3, tPast, s)) / dt;
                    double t2 = (ST(4, tNow, s) - ST(4, tPast, s)) / dt;
                    thetaDotCont = 0.5 * (t0 * t0 + t1 * t1 + t2 * t2);
                    double gxy = g * dx * dy, gxz = g * dx * dz, gyz = g * dy * dz;
                    FCont = (1 - pcos(Pxy)) / (gxy * gxy) + (1 - pcos(Pxz)) / (gxz * gxz) + (1 - pcos(Pyz)) / (gyz * gyz);
                }
                if (g != 0) {
                    double divNow = (ST(2, tNow, s) - ST(2, tNow, imx)) / (dx * dx) + (ST(3, tNow, s) - ST(3, tNow, imy)) / (dy * dy)
                                  + (ST(4, tNow, s) - ST(4, tNow, imz)) / (dz * dz);
                    double divPast = (ST(2, tPast, s) - ST(2, tPast, imx)) / (dx * dx) + (ST(3, tPast, s) - ST(3, tPast, imy)) / (dy * dy)
                                   + (ST(4, tPast, s) - ST(4, tPast, imz)) / (dz * dz);
                    double divThetat = (divNow - divPast) / dt;
                    gauss = divThetat / g - 2 * g * (ST(1, tNow, s) * phit[0] - ST(0, tNow, s) * phit[1]);
                    if (!mpi_form) {
                        double t0 = (ST(2, tNow, s) - ST(2, tPast, s)) / (g * dt * dx);
                        double t1 = (ST(3, tNow, s) - ST(3, tPast, s)) / (g * dt * dy);
                        double t2 = (ST(4, tNow, s) - ST(4, tPast, s)) / (g * dt * dz);
                        thetaDotCont = 0.5 * (t0 * t0 + t1 * t1 + t2 * t2);
                        double gxy = g * dx * dy, gxz = g * dx * dz, gyz = g * dy * dz;
                        double Fxy = (1 - pcos(Pxy)) / (gxy * gxy);
                        double Fxz = (1 - pcos(Pxz)) / (gxz * gxz);
                        double Fyz = (1 - pcos(Pyz)) / (gyz * gyz);
                        FCont = Fxy + Fxz + Fyz;
                    }
                } else if (!mpi_form) {
                    thetaDotCont = 0;
                    FCont = 0;
                }
                double pm = phiMagSqr - eta * eta;
                double ed = phit[0] * phit[0] + phit[1] * phit[1] + phix[0] * phix[0] + phix[1] * phix[1] + phiy[0] * phiy[0]
                          + phiy[1] * phiy[1] + phiz[0] * phiz[0] + phiz[1] * phiz[1] + thetaDotCont + FCont + 0.25 * lambda * (pm * pm);
                if (mpi_form) energy += ed * dx * dy * dz;
                else energy += dx * dy * dz * ed;
                dev += fabs(gauss);
            }
        }
    }
    out->energy = energy;
    out->gauss_abs_sum = dev;
    out->sites = (int64_t)(G.hix - G.lox) * (G.hiy - G.loy) * (G.hiz - G.loz);
    out->time_step = n;
}

/* ------------------------------------------------------------------------- */
/* Moore model: moore_mpi_evolution.cpp:405-550 (periodic, friction, current  */
/* without q) and mooreEvol.cpp:187-337 + 672-692 (fixed, q-weighted current). */
/* Components: 0,1 = phi1; 2,3 = phi2; 4,5,6 = theta_x,y,z.                    */
/* ------------------------------------------------------------------------- */
#define PH(f, comp) ((f) * 2 + (comp))   /* f = 0 (phi1) / 1 (phi2) */
#define TH(m) (4 + (m))

static void moore_update(const lat_params* p, double* st, int64_t n)
{
    const geo_t G = make_geo(p);
    const int64_t N = G.N;
    const int tNow = (int)((n + 1) % 2), tPast = (int)(n % 2);
    double damp, fric;
    friction_of(p, n, &damp, &fric);
    const double dx = p->dx, dy = p->dy, dz = p->dz, dt = p->dt;
    const double l1 = p->lambda, l2 = p->lambda2, l12 = p->lambda12, e1 = p->eta, e2 = p->eta2, g = p->g;
    const double q[2] = {p->q1, p->q2};
    const int charge = p->moore_current == LAT_MOORE_CURRENT_CHARGE;
    const int c[2] = {1, -1};

#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
    for (int64_t i = G.lox; i < G.hix; ++i) {
        const int64_t ip = wrapp(i, G.nx), im = wrapm(i, G.nx);
        for (int64_t j = G.loy; j < G.hiy; ++j) {
            const int64_t jp = wrapp(j, G.ny), jm = wrapm(j, G.ny);
            for (int64_t k = G.loz; k < G.hiz; ++k) {
                const int64_t kp = wrapp(k, G.nz), km = wrapm(k, G.nz);
                const int64_t s = site(&G, i, j, k);
                const int64_t ipx = site(&G, ip, j, k), imx = site(&G, im, j, k);
                const int64_t ipy = site(&G, i, jp, k), imy = site(&G, i, jm, k);
                const int64_t ipz = site(&G, i, j, kp), imz = site(&G, i, j, km);
                const int64_t ipxmy = site(&G, ip, jm, k), ipxmz = site(&G, ip, j, km);
                const int64_t imxpy = site(&G, im, jp, k), ipymz = site(&G, i, jp, km);
                const int64_t imxpz = site(&G, im, j, kp), imypz = site(&G, i, jm, kp);
                const int64_t nb[3][2] = {{ipx, imx}, {ipy, imy}, {ipz, imz}};
                const double d2[3] = {dx * dx, dy * dy, dz * dz};

                double mag[2];
                for (int f = 0; f < 2; ++f)
                    mag[f] = ST(PH(f, 0), tNow, s) * ST(PH(f, 0), tNow, s) + ST(PH(f, 1), tNow, s) * ST(PH(f, 1), tNow, s);
                for (int comp = 0; comp < 2; ++comp) {
                    const int oc = comp + c[comp];
                    const double cc = (double)c[comp];
                    for (int f = 0; f < 2; ++f) {
                        const double qf = q[f];
                        double lap[3];
                        for (int m = 0; m < 3; ++m) {
                            const int64_t pp = nb[m][0], mm = nb[m][1];
                            lap[m] = (pcos(qf * ST(TH(m), tNow, s)) * ST(PH(f, comp), tNow, pp) + cc * psin(qf * ST(TH(m), tNow, s)) * ST(PH(f, oc), tNow, pp)
                                      - 2 * ST(PH(f, comp), tNow, s)
                                      + pcos(qf * ST(TH(m), tNow, mm)) * ST(PH(f, comp), tNow, mm) - cc * psin(qf * ST(TH(m), tNow, mm)) * ST(PH(f, oc), tNow, mm)) / d2[m];
                        }
                        double pot = (f == 0) ? (0.5 * l1 * (mag[0] - e1 * e1) + 0.5 * l12 * (mag[1] - e2 * e2))
                                              : (0.5 * l2 * (mag[1] - e2 * e2) + 0.5 * l12 * (mag[0] - e1 * e1));
                        double phitt = lap[0] + lap[1] + lap[2] - pot * ST(PH(f, comp), tNow, s);
                        if (fric != 0) {
                            double phit = (ST(PH(f, comp), tNow, s) - ST(PH(f, comp), tPast, s)) / dt;
                            phitt = phitt - fric * phit;
                        }
                        ST(PH(f, comp), tPast, s) = 2 * ST(PH(f, comp), tNow, s) - ST(PH(f, comp), tPast, s) + dt * dt * phitt;
                    }
                }

                double cur[3];
                for (int m = 0; m < 3; ++m) {
                    const int64_t pp = nb[m][0];
                    double cf[2];
                    for (int f = 0; f < 2; ++f) {
                        const double qf = q[f];
                        double v = pcos(qf * ST(TH(m), tNow, s)) * (ST(PH(f, 1), tNow, s) * ST(PH(f, 0), tNow, pp) - ST(PH(f, 0), tNow, s) * ST(PH(f, 1), tNow, pp))
                                 + psin(qf * ST(TH(m), tNow, s)) * (ST(PH(f, 0), tNow, s) * ST(PH(f, 0), tNow, pp) + ST(PH(f, 1), tNow, s) * ST(PH(f, 1), tNow, pp));
                        cf[f] = charge ? qf * v : v;
                    }
                    cur[m] = cf[0] + cf[1];
                }

                double Fxy_y = (psin(ST(TH(0), tNow, s) + ST(TH(1), tNow, ipx) - ST(TH(0), tNow, ipy) - ST(TH(1), tNow, s))
                              - psin(ST(TH(0), tNow, imy) + ST(TH(1), tNow, ipxmy) - ST(TH(0), tNow, s) - ST(TH(1), tNow, imy))) / (dy * dy);
                double Fxz_z = (psin(ST(TH(0), tNow, s) + ST(TH(2), tNow, ipx) - ST(TH(0), tNow, ipz) - ST(TH(2), tNow, s))
                              - psin(ST(TH(0), tNow, imz) + ST(TH(2), tNow, ipxmz) - ST(TH(0), tNow, s) - ST(TH(2), tNow, imz))) / (dz * dz);
                double Fyx_x = (psin(ST(TH(1), tNow, s) + ST(TH(0), tNow, ipy) - ST(TH(1), tNow, ipx) - ST(TH(0), tNow, s))
                              - psin(ST(TH(1), tNow, imx) + ST(TH(0), tNow, imxpy) - ST(TH(1), tNow, s) - ST(TH(0), tNow, imx))) / (dx * dx);
                double Fyz_z = (psin(ST(TH(1), tNow, s) + ST(TH(2), tNow, ipy) - ST(TH(1), tNow, ipz) - ST(TH(2), tNow, s))
                              - psin(ST(TH(1), tNow, imz) + ST(TH(2), tNow, ipymz) - ST(TH(1), tNow, s) - ST(TH(2), tNow, imz))) / (dz * dz);
                double Fzx_x = (psin(ST(TH(2), tNow, s) + ST(TH(0), tNow, ipz) - ST(TH(2), tNow, ipx) - ST(TH(0), tNow, s))
                              - psin(ST(TH(2), tNow, imx) + ST(TH(0), tNow, imxpz) - ST(TH(2), tNow, s) - ST(TH(0), tNow, imx))) / (dx * dx);
                double Fzy_y = (psin(ST(TH(2), tNow, s) + ST(TH(1), tNow, ipz) - ST(TH(2), tNow, ipy) - ST(TH(1), tNow, s))
                              - psin(ST(TH(2), tNow, imy) + ST(TH(1), tNow, imypz) - ST(TH(2), tNow, s) - ST(TH(1), tNow, imy))) / (dy * dy);

                double tt[3];
                tt[0] = -2 * g * g * cur[0] - Fxy_y - Fxz_z;
                tt[1] = -2 * g * g * cur[1] - Fyx_x - Fyz_z;
                tt[2] = -2 * g * g * cur[2] - Fzx_x - Fzy_y;
                if (damp != 0) {
                    for (int m = 0; m < 3; ++m) {
                        double thetat = (ST(TH(m), tNow, s) - ST(TH(m), tPast, s)) / dt;
                        tt[m] = tt[m] - damp * thetat;
                    }
                }
                for (int m = 0; m < 3; ++m)
                    ST(TH(m), tPast, s) = 2 * ST(TH(m), tNow, s) - ST(TH(m), tPast, s) + dt * dt * tt[m];
            }
        }
    }
}

/* Moore diagnostics: mooreEvol.cpp:339-391 (energy + Gauss with charges) or
 * moore_mpi_evolution.cpp:558-588 (LAT_ENERGY_MPI energy). */
static void moore_diag(const lat_params* p, const double* st, int64_t n, lat_diag* out)
{
    const geo_t G = make_geo(p);
    const int64_t N = G.N;
    const int tNow = (int)((n + 1) % 2), tPast = (int)(n % 2);
    const double dx = p->dx, dy = p->dy, dz = p->dz, dt = p->dt;
    const double l1 = p->lambda, l2 = p->lambda2, l12 = p->lambda12, e1 = p->eta, e2 = p->eta2, g = p->g;
    const double q[2] = {p->q1, p->q2};
    const int c[2] = {1, -1};
    const int mpi_form = p->energy_form == LAT_ENERGY_MPI;
    double energy = 0, dev = 0;

#pragma omp parallel for schedule(static) reduction(+:energy,dev) num_threads(orc_get_threads())
    for (int64_t i = G.lox; i < G.hix; ++i) {
        const int64_t ip = wrapp(i, G.nx), im = wrapm(i, G.nx);
        for (int64_t j = G.loy; j < G.hiy; ++j) {
            const int64_t jp = wrapp(j, G.ny), jm = wrapm(j, G.ny);
            for (int64_t k = G.loz; k < G.hiz; ++k) {
                const int64_t kp = wrapp(k, G.nz), km = wrapm(k, G.nz);
                const int64_t s = site(&G, i, j, k);
                const int64_t ipx = site(&G, ip, j, k), imx = site(&G, im, j, k);
                const int64_t ipy = site(&G, i, jp, k), imy = site(&G, i, jm, k);
                const int64_t ipz = site(&G, i, j, kp), imz = site(&G, i, j, km);
                const int64_t mmv[3] = {imx, imy, imz};
                const double dd[3] = {dx, dy, dz};
                double mag[2];
                for (int f = 0; f < 2; ++f)
                    mag[f] = ST(PH(f, 0), tNow, s) * ST(PH(f, 0), tNow, s) + ST(PH(f, 1), tNow, s) * ST(PH(f, 1), tNow, s);
                double pt[2][2], pd[2][3][2];
                for (int comp = 0; comp < 2; ++comp) {
                    const int oc = comp + c[comp];
                    const double cc = (double)c[comp];
                    for (int f = 0; f < 2; ++f) {
                        const double qf = q[f];
                        pt[f][comp] = (ST(PH(f, comp), tNow, s) - ST(PH(f, comp), tPast, s)) / dt;
                        for (int m = 0; m < 3; ++m) {
                            const int64_t mm = mmv[m];
                            pd[f][m][comp] = (ST(PH(f, comp), tNow, s) - pcos(qf * ST(TH(m), tNow, mm)) * ST(PH(f, comp), tNow, mm)
                                              + cc * psin(qf * ST(TH(m), tNow, mm)) * ST(PH(f, oc), tNow, mm)) / dd[m];
                        }
                    }
                }
                double Pxy = ST(TH(0), tNow, s) + ST(TH(1), tNow, ipx) - ST(TH(0), tNow, ipy) - ST(TH(1), tNow, s);
                double Pxz = ST(TH(0), tNow, s) + ST(TH(2), tNow, ipx) - ST(TH(0), tNow, ipz) - ST(TH(2), tNow, s);
                double Pyz = ST(TH(1), tNow, s) + ST(TH(2), tNow, ipy) - ST(TH(1), tNow, ipz) - ST(TH(2), tNow, s);
                double gauss = 0, thetaDotCont = 0, FCont = 0;
                if (mpi_form) {
                    double t0 = (ST(TH(0), tNow, s) - ST(TH(0), tPast, s)) / dt;
                    double t1 = (ST(TH(1), tNow, s) - ST(TH(1), tPast, s)) / dt;
                    double t2 = (ST(TH(2), tNow, s) - ST(TH(2), tPast, s)) / dt;
                    thetaDotCont = 0.5 * (t0 * t0 + t1 * t1 + t2 * t2);
                    double gxy = g * dx * dy, gxz = g * dx * dz, gyz = g * dy * dz;
                    FCont = (1 - pcos(Pxy)) / (gxy * gxy) + (1 - pcos(Pxz)) / (gxz * gxz) + (1 - pcos(Pyz)) / (gyz * gyz);
                }
                if (g != 0) {
                    double divNow = (ST(TH(0), tNow, s) - ST(TH(0), tNow, imx)) / (dx * dx) + (ST(TH(1), tNow, s) - ST(TH(1), tNow, imy)) / (dy * dy)
                                  + (ST(TH(2), tNow, s) - ST(TH(2), tNow, imz)) / (dz * dz);
                    double divPast = (ST(TH(0), tPast, s) - ST(TH(0), tPast, imx)) / (dx * dx) + (ST(TH(1), tPast, s) - ST(TH(1), tPast, imy)) / (dy * dy)
                                   + (ST(TH(2), tPast, s) - ST(TH(2), tPast, imz)) / (dz * dz);
                    double divThetat = (divNow - divPast) / dt;
                    gauss = divThetat / g - 2 * g * (q[0] * (ST(PH(0, 1), tNow, s) * pt[0][0] - ST(PH(0, 0), tNow, s) * pt[0][1])
                                                   + q[1] * (ST(PH(1, 1), tNow, s) * pt[1][0] - ST(PH(1, 0), tNow, s) * pt[1][1]));
                    if (!mpi_form) {
                        double t0 = (ST(TH(0), tNow, s) - ST(TH(0), tPast, s)) / (g * dt * dx);
                        double t1 = (ST(TH(1), tNow, s) - ST(TH(1), tPast, s)) / (g * dt * dy);
                        double t2 = (ST(TH(2), tNow, s) - ST(TH(2), tPast, s)) / (g * dt * dz);
                        thetaDotCont = 0.5 * (t0 * t0 + t1 * t1 + t2 * t2);
                        double gxy = g * dx * dy, gxz = g * dx * dz, gyz = g * dy * dz;
                        double Fxy = (1 - pcos(Pxy)) / (gxy * gxy);
                        double Fxz = (1 - pcos(Pxz)) / (gxz * gxz);
                        double Fyz = (1 - pcos(Pyz)) / (gyz * gyz);
                        FCont = Fxy + Fxz + Fyz;
                    }
                }
                double m1 = mag[0] - e1 * e1, m2 = mag[1] - e2 * e2;
                double ed = pt[0][0] * pt[0][0] + pt[0][1] * pt[0][1] + pd[0][0][0] * pd[0][0][0] + pd[0][0][1] * pd[0][0][1]
                          + pd[0][1][0] * pd[0][1][0] + pd[0][1][1] * pd[0][1][1] + pd[0][2][0] * pd[0][2][0] + pd[0][2][1] * pd[0][2][1]
                          + pt[1][0] * pt[1][0] + pt[1][1] * pt[1][1] + pd[1][0][0] * pd[1][0][0] + pd[1][0][1] * pd[1][0][1]
                          + pd[1][1][0] * pd[1][1][0] + pd[1][1][1] * pd[1][1][1] + pd[1][2][0] * pd[1][2][0] + pd[1][2][1] * pd[1][2][1]
                          + thetaDotCont + FCont + 0.25 * l1 * (m1 * m1) + 0.25 * l2 * (m2 * m2) + 0.5 * l12 * m1 * m2;
                if (mpi_form) energy += ed * dx * dy * dz;
                else energy += dx * dy * dz * ed;
                dev += fabs(gauss);
            }
        }
    }
    out->energy = energy;
    out->gauss_abs_sum = dev;
    out->sites = (int64_t)(G.hix - G.lox) * (G.hiy - G.loy) * (G.hiz - G.loz);
    out->time_step = n;
}

int orc_diagnostics(const lat_params* p, const double* st, int64_t n, lat_diag* diag)
{
    if (!p || !st || !diag) return LAT_ERR_INVALID;
    if (p->model == LAT_MODEL_MOORE) moore_diag(p, st, n, diag);
    else ah_diag(p, st, n, diag);
    return 0;
}

int orc_step(const lat_params* p, double* st, int64_t n, lat_diag* diag)
{
    if (!p || !st) return LAT_ERR_INVALID;
    orc_apply_boundaries(p, st, n);  /* evolution.cpp:194-265: before the derivatives */
    if (diag) orc_diagnostics(p, st, n, diag);
    if (p->model == LAT_MODEL_MOORE) moore_update(p, st, n);
    else ah_update(p, st, n);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* bilinear crossing detection: mpi_evolution.cpp:536-789                     */
/* ------------------------------------------------------------------------- */
typedef struct { double* xyz; int64_t cap, count; } sink_t;

static void push(sink_t* o, double x, double y, double z)
{
    if (o->count < o->cap) {
        o->xyz[3 * o->count + 0] = x;
        o->xyz[3 * o->count + 1] = y;
        o->xyz[3 * o->count + 2] = z;
    }
    o->count++;
}

/* One face.  v00 = phi at the corner (u, w), v10 at (u+du, w), v01 at (u, w+dw),
 * v11 at (u+du, w+dw), per component.  Solutions: sol1 along u, sol2 along w.
 * emit(sol1, sol2) maps back to (x,y,z). */
static int face_roots(const double v00[2], const double v10[2], const double v01[2], const double v11[2],
                      double u, double w, double du, double dw, double s1[2], double s2[2])
{
    double coeff1[2], coeff2[2], coeff3[2], coeff4[2];
    for (int comp = 0; comp < 2; ++comp) {
        coeff1[comp] = v11[comp] - v10[comp] - v01[comp] + v00[comp];
        coeff2[comp] = (w + dw) * (v10[comp] - v00[comp]) + w * (v01[comp] - v11[comp]);
        coeff3[comp] = (u + du) * (v01[comp] - v00[comp]) + u * (v10[comp] - v11[comp]);
        coeff4[comp] = (u + du) * ((w + dw) * v00[comp] - w * v01[comp]) - u * ((w + dw) * v10[comp] - w * v11[comp]);
    }
    double a = coeff1[1] * coeff3[0] - coeff1[0] * coeff3[1];
    double b = coeff1[1] * coeff4[0] + coeff2[1] * coeff3[0] - coeff1[0] * coeff4[1] - coeff2[0] * coeff3[1];
    double c = coeff2[1] * coeff4[0] - coeff2[0] * coeff4[1];
    double discrim = b * b - 4 * a * c;
    int nroot = 0;
    if (a == 0) {
        if (b != 0) {
            double sol2 = -c / b;
            if (sol2 >= w && sol2 <= w + dw) {
                double sol1 = -(coeff3[0] * sol2 + coeff4[0]) / (coeff1[0] * sol2 + coeff2[0]);
                if (sol1 >= u && sol1 <= u + du) { s1[nroot] = sol1; s2[nroot] = sol2; nroot++; }
            }
        }
    } else if (discrim >= 0) {
        double sol2 = (-b + sqrt(discrim)) / (2 * a);
        if (sol2 >= w && sol2 <= w + dw) {
            double sol1 = -(coeff3[0] * sol2 + coeff4[0]) / (coeff1[0] * sol2 + coeff2[0]);
            if (sol1 >= u && sol1 <= u + du) { s1[nroot] = sol1; s2[nroot] = sol2; nroot++; }
        }
        sol2 = (-b - sqrt(discrim)) / (2 * a);
        if (sol2 >= w && sol2 <= w + dw) {
            double sol1 = -(coeff3[0] * sol2 + coeff4[0]) / (coeff1[0] * sol2 + coeff2[0]);
            if (sol1 >= u && sol1 <= u + du) { s1[nroot] = sol1; s2[nroot] = sol2; nroot++; }
        }
    }
    return nroot;
}

int orc_detect(const lat_params* p, const double* st, int64_t n, int field,
               double* xyz, int64_t cap, int64_t* count)
{
    if (!p || !st || !count) return LAT_ERR_INVALID;
    if (field != 0 && !(field == 1 && p->model == LAT_MODEL_MOORE)) return LAT_ERR_INVALID;
    const geo_t G = make_geo(p);
    const int64_t N = G.N;
    const int tNow = (int)((n + 1) % 2);
    const int c0 = 2 * field;
    const double dx = p->dx, dy = p->dy, dz = p->dz;
    const int64_t x0 = (int64_t)(0.5 * (G.nx - 1)), y0 = (int64_t)(0.5 * (G.ny - 1)), z0 = (int64_t)(0.5 * (G.nz - 1));
    sink_t o = {xyz, xyz ? cap : 0, 0};
    for (int64_t i = G.lox; i < G.hix; ++i) {
        const int64_t ip = wrapp(i, G.nx);
        const double x = (double)(i - x0) * dx;
        for (int64_t j = G.loy; j < G.hiy; ++j) {
            const int64_t jp = wrapp(j, G.ny);
            const double y = (double)(j - y0) * dy;
            for (int64_t k = G.loz; k < G.hiz; ++k) {
                const int64_t kp = wrapp(k, G.nz);
                const double z = (double)(k - z0) * dz;
                const int64_t s = site(&G, i, j, k);
                const int64_t ipx = site(&G, ip, j, k), ipy = site(&G, i, jp, k), ipz = site(&G, i, j, kp);
                const int64_t ipxpy = site(&G, ip, jp, k), ipxpz = site(&G, ip, j, kp), ipypz = site(&G, i, jp, kp);
                double v0[2], vx[2], vy[2], vz[2], vxy[2], vxz[2], vyz[2];
                for (int comp = 0; comp < 2; ++comp) {
                    v0[comp] = ST(c0 + comp, tNow, s);
                    vx[comp] = ST(c0 + comp, tNow, ipx);
                    vy[comp] = ST(c0 + comp, tNow, ipy);
                    vz[comp] = ST(c0 + comp, tNow, ipz);
                    vxy[comp] = ST(c0 + comp, tNow, ipxpy);
                    vxz[comp] = ST(c0 + comp, tNow, ipxpz);
                    vyz[comp] = ST(c0 + comp, tNow, ipypz);
                }
                double s1[2], s2[2];
                int nr;
                /* z-directed face: u = x, w = y */
                nr = face_roots(v0, vx, vy, vxy, x, y, dx, dy, s1, s2);
                for (int r = 0; r < nr; ++r) push(&o, s1[r], s2[r], z);
                /* y-directed face: u = x, w = z */
                nr = face_roots(v0, vx, vz, vxz, x, z, dx, dz, s1, s2);
                for (int r = 0; r < nr; ++r) push(&o, s1[r], y, s2[r]);
                /* x-directed face: u = y, w = z */
                nr = face_roots(v0, vy, vz, vyz, y, z, dy, dz, s1, s2);
                for (int r = 0; r < nr; ++r) push(&o, x, s1[r], s2[r]);
            }
        }
    }
    *count = o.count;
    return (xyz && o.count > cap) ? LAT_ERR_CAPACITY : 0;
}

/* ------------------------------------------------------------------------- */
/* plaquette winding (new; definition in include/lattice_gpu.h)              */
/* ------------------------------------------------------------------------- */
static int edge_cross(double ax, double ay, double bx, double by)
{
    /* volatile keeps the two products separately rounded */
    volatile double p1 = ax * by;
    volatile double p2 = ay * bx;
    double cr = p1 - p2;
    if (ay <= 0) { if (by > 0 && cr > 0) return 1; }
    else { if (by <= 0 && cr < 0) return -1; }
    return 0;
}

int orc_winding(const lat_params* p, const double* st, int64_t n, int field,
                int8_t* out, int64_t* abs_sum)
{
    if (!p || !st) return LAT_ERR_INVALID;
    if (field != 0 && !(field == 1 && p->model == LAT_MODEL_MOORE)) return LAT_ERR_INVALID;
    const geo_t G = make_geo(p);
    const int64_t N = G.N;
    const int tNow = (int)((n + 1) % 2);
    const int c0 = 2 * field;
    const int pxy = G.kxy == LAT_BC_PERIODIC, pz = G.kz == LAT_BC_PERIODIC;
    int64_t tot = 0;
    if (out) memset(out, 0, (size_t)(3 * N));
    for (int64_t i = 0; i < G.nx; ++i) {
        const int64_t ip = wrapp(i, G.nx);
        for (int64_t j = 0; j < G.ny; ++j) {
            const int64_t jp = wrapp(j, G.ny);
            for (int64_t k = 0; k < G.nz; ++k) {
                const int64_t kp = wrapp(k, G.nz);
                const int64_t s = site(&G, i, j, k);
                /* corner lists per normal d */
                int64_t cs[3][4] = {
                    {s, site(&G, i, jp, k), site(&G, i, jp, kp), site(&G, i, j, kp)},
                    {s, site(&G, i, j, kp), site(&G, ip, j, kp), site(&G, ip, j, k)},
                    {s, site(&G, ip, j, k), site(&G, ip, jp, k), site(&G, i, jp, k)}};
                /* a face is valid unless it wraps around a non-periodic axis */
                const int xin = pxy || i + 1 < G.nx, yin = pxy || j + 1 < G.ny, zin = pz || k + 1 < G.nz;
                const int valid[3] = {yin && zin, zin && xin, xin && yin};
                for (int d = 0; d < 3; ++d) {
                    if (!valid[d]) continue;
                    int w = 0;
                    for (int e = 0; e < 4; ++e) {
                        const int64_t a = cs[d][e], b = cs[d][(e + 1) & 3];
                        w += edge_cross(ST(c0, tNow, a), ST(c0 + 1, tNow, a), ST(c0, tNow, b), ST(c0 + 1, tNow, b));
                    }
                    if (out) out[d * N + s] = (int8_t)w;
                    tot += w < 0 ? -w : w;
                }
            }
        }
    }
    if (abs_sum) *abs_sum = tot;
    return 0;
}

/* ------------------------------------------------------------------------- */
/* ic_func.cpp:647-683 random IC: minstd_rand(seed) (Park-Miller, multiplier */
/* 48271, modulus 2^31-1) and uniform_real_distribution<double>(-1, 1) as     */
/* libstdc++ computes it (generate_canonical from two draws).  Per site in    */
/* linear order: phi_re, phi_im, then (if g != 0) theta_mu = d_mu * u.  Both  */
/* time levels equal.                                                         */
/* ------------------------------------------------------------------------- */
typedef struct { uint64_t x; } orc_minstd;

static uint32_t minstd_next(orc_minstd* g)
{
    g->x = (g->x * 48271u) % 2147483647u;
    return (uint32_t)g->x;
}

static double minstd_uniform_m1_1(orc_minstd* g)
{
    const long double r = 2147483646.0L;  /* max - min + 1 */
    double sum = 0.0, tmp = 1.0;
    sum += (double)(minstd_next(g) - 1u) * tmp;
    tmp = (double)((long double)tmp * r);
    sum += (double)(minstd_next(g) - 1u) * tmp;
    tmp = (double)((long double)tmp * r);
    double u = sum / tmp;
    if (u >= 1.0) u = nextafter(1.0, 0.0);
    return u * (1.0 - (-1.0)) + (-1.0);
}

int orc_icfunc_random_ic(const lat_params* p, uint32_t seed, double* st)
{
    if (!p || !st || p->model != LAT_MODEL_AH) return LAT_ERR_INVALID;
    const int64_t N = p->nx * p->ny * p->nz;
    memset(st, 0, sizeof(double) * 5 * 2 * (size_t)N);
    orc_minstd g;
    g.x = seed % 2147483647u;
    if (g.x == 0) g.x = 1;
    for (int64_t s = 0; s < N; ++s) {
        double v[5] = {0, 0, 0, 0, 0};
        v[0] = minstd_uniform_m1_1(&g);
        v[1] = minstd_uniform_m1_1(&g);
        if (p->g != 0) {
            v[2] = p->dx * minstd_uniform_m1_1(&g);
            v[3] = p->dy * minstd_uniform_m1_1(&g);
            v[4] = p->dz * minstd_uniform_m1_1(&g);
        }
        for (int c = 0; c < 5; ++c) {
            st[((int64_t)c * 2 + 0) * N + s] = v[c];
            st[((int64_t)c * 2 + 1) * N + s] = v[c];
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------- */
/* total string length by greedy chaining of crossings                        */
/* (ic_w_evolution.cpp:961-1087), single-thread semantics: from the current   */
/* point, the nearest remaining point within (dx^2+dy^2+dz^2)^2 (compared     */
/* with the squared distance; the last of equally near points wins) is the     */
/* next; its distance is added; when none is left in reach, the distance to    */
/* the first point of the chain is checked and, if within reach, the cutoff's  */
/* square root is added (as the reference does), and a new chain starts at     */
/* the first remaining point.  Per-axis minimum image only for periodic axes.  */
/* With split, lengths are added to L0 when the current point lies in the     */
/* central quarter-box, else to L1.  O(M^2), like the reference.              */
/* ------------------------------------------------------------------------- */
static double chain_dist2(const double* a, const double* b, double bx, double by, double bz, int pxy, int pz)
{
    double d = 0, t;
    t = fabs(a[0] - b[0]);
    if (t <= 0.5 * bx) d = (a[0] - b[0]) * (a[0] - b[0]);
    else if (pxy) d = (bx - t) * (bx - t);
    t = fabs(a[1] - b[1]);
    if (t <= 0.5 * by) d += (a[1] - b[1]) * (a[1] - b[1]);
    else if (pxy) d += (by - t) * (by - t);
    t = fabs(a[2] - b[2]);
    if (t <= 0.5 * bz) d += (a[2] - b[2]) * (a[2] - b[2]);
    else if (pz) d += (bz - t) * (bz - t);
    return d;
}

int orc_string_length(const lat_params* p, const double* xyz, int64_t M, int split, double* L0, double* L1)
{
    if (!p || (!xyz && M) || !L0 || !L1) return LAT_ERR_INVALID;
    const double dx = p->dx, dy = p->dy, dz = p->dz;
    const double bx = p->nx * dx, by = p->ny * dy, bz = p->nz * dz;
    const geo_t G = make_geo(p);
    const int pxy = G.kxy == LAT_BC_PERIODIC, pz = G.kz == LAT_BC_PERIODIC;
    const double c0 = dx * dx + dy * dy + dz * dz;
    const double cutoff = c0 * c0;
    *L0 = 0;
    *L1 = 0;
    if (M == 0) return 0;
    char* alive = (char*)malloc((size_t)M);
    if (!alive) return LAT_ERR_NOMEM;
    memset(alive, 1, (size_t)M);
    int64_t f = 0, first = 0;
    double begin[3] = {xyz[0], xyz[1], xyz[2]};
    for (int64_t it = 0; it < M; ++it) {
        double best = cutoff;
        int64_t bi = -1;
        for (int64_t j = 0; j < M; ++j) {
            if (!alive[j] || j == f) continue;
            const double d = chain_dist2(&xyz[3 * f], &xyz[3 * j], bx, by, bz, pxy, pz);
            if (d <= best) {
                best = d;
                bi = j;
            }
        }
        const double* cf = &xyz[3 * f];
        const int inner = cf[0] >= -0.25 * p->nx * dx && cf[0] <= 0.25 * p->nx * dx && cf[1] >= -0.25 * p->ny * dy &&
                          cf[1] <= 0.25 * p->ny * dy && cf[2] >= -0.25 * p->nz * dz && cf[2] <= 0.25 * p->nz * dz;
        if (bi >= 0) {
            if (split && !inner) *L1 += sqrt(best);
            else *L0 += sqrt(best);
            alive[f] = 0;
            f = bi;
        } else {
            const double d = chain_dist2(cf, begin, bx, by, bz, pxy, pz);
            if (d <= best) {
                if (split && !inner) *L1 += sqrt(best);
                else *L0 += sqrt(best);
            }
            alive[f] = 0;
            while (first < M && !alive[first]) ++first;
            if (first < M) {
                f = first;
                begin[0] = xyz[3 * f];
                begin[1] = xyz[3 * f + 1];
                begin[2] = xyz[3 * f + 2];
            }
        }
    }
    free(alive);
    return 0;
}


/* ---------------------------------------------------------------------------
 * Boosted straight-string IC, initialConditions.cpp:710-992 and
 * ic_func.cpp:685-964, restated with the reference's operation order and
 * libm calls (pow(x, 2) included).
 * ------------------------------------------------------------------------- */

/* |phi| and A_theta at distance d: initialConditions.cpp:756-782 (second
 * order about the nearest table point, first order next to r = 0); beyond the
 * table (and at its last point, where the reference reads one past its end)
 * |phi| = 1, A = n/g. */
static int profile_at(const lat_string_profile* pr, double g, double d, double* phiMag, double* AMag)
{
    const double a = pr->h;
    const int64_t p = (int64_t)round(d / a);
    const double* S0 = pr->phi;
    const double* S1 = pr->A;
    if (p == 0) {
        *phiMag = (S0[p + 1] * d - S0[p] * (d - a)) / a;
        *AMag = (S1[p + 1] * d - S1[p] * (d - a)) / a;
        return 0;
    }
    if (p + 1 < pr->m) {
        const double pa = (double)p * a, pp = (double)(p + 1) * a, pm = (double)(p - 1) * a;
        *phiMag = (S0[p - 1] * (d - pa) * (d - pp) - 2 * S0[p] * (d - pm) * (d - pp) + S0[p + 1] * (d - pm) * (d - pa))
                / (2 * a * a);
        *AMag = (S1[p - 1] * (d - pa) * (d - pp) - 2 * S1[p] * (d - pm) * (d - pp) + S1[p + 1] * (d - pm) * (d - pa))
              / (2 * a * a);
        return 0;
    }
    *phiMag = 1;
    *AMag = g == 0 ? 0 : pr->winding / g;
    return 1;
}

int64_t orc_boost_ic(const lat_params* p, const lat_string_profile* prof, const lat_boost_ic* b, double* st)
{
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    if (nx < 2 || ny < 2 || nz < 2 || !prof || prof->m < 2 || !(prof->h > 0) || !b) return -1;
    const int64_t N = (int64_t)nx * ny * nz;
    const double dx = p->dx, dy = p->dy, dz = p->dz, dt = p->dt, g = p->g;
    const double v1x = b->v[0], v1y = b->v[1], v1z = b->v[2];
    const double vMagSqr = pow(v1x, 2) + pow(v1y, 2) + pow(v1z, 2);
    if (!(vMagSqr > 0 && vMagSqr < 1)) return -1;
    const double gamma = 1 / sqrt(1 - vMagSqr);
    const int x0 = (nx - 1) / 2, y0 = (ny - 1) / 2, z0 = (nz - 1) / 2;
    double* At = (double*)malloc(sizeof(double) * (size_t)N);
    if (!At) return -1;
#define BST(c, t) (st + ((size_t)(c) * 2 + (t)) * (size_t)N)
    int64_t off = 0;
    /* t = 0 (zb uses dy, initialConditions.cpp:745) */
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                const int64_t s = ((int64_t)i * ny + j) * nz + k;
                const double xb = (i - x0) * dx, yb = (j - y0) * dy, zb = (k - z0) * dy;
                const double xs = xb + (gamma - 1) * (v1x * xb + v1y * yb + v1z * zb) * v1x / vMagSqr;
                const double ys = yb + (gamma - 1) * (v1x * xb + v1y * yb + v1z * zb) * v1y / vMagSqr;
                const double distance = sqrt(pow(xs, 2) + pow(ys, 2));
                double phiMag, AMag, Ax, Ay, re, im;
                off += profile_at(prof, g, distance, &phiMag, &AMag);
                if (xs == 0) { re = 0; Ay = 0; }
                else { re = phiMag * xs / distance; Ay = AMag * xs / pow(distance, 2); }
                if (ys == 0) { im = 0; Ax = 0; }
                else { im = phiMag * ys / distance; Ax = -AMag * ys / pow(distance, 2); }
                At[s] = -gamma * (v1x * Ax + v1y * Ay);
                const double A0 = Ax + (gamma - 1) * (v1x * Ax + v1y * Ay) * v1x / vMagSqr;
                const double A1 = Ay + (gamma - 1) * (v1x * Ax + v1y * Ay) * v1y / vMagSqr;
                const double A2 = (gamma - 1) * (v1x * Ax + v1y * Ay) * v1z / vMagSqr;
                BST(0, 0)[s] = re;
                BST(1, 0)[s] = im;
                BST(2, 0)[s] = dx * g * A0;
                BST(3, 0)[s] = dy * g * A1;
                BST(4, 0)[s] = dz * g * A2;
            }
    /* t = dt, then the gauge transformation that removes A_t (centred
     * differences inside, one-sided on the faces: no periodic wrap) */
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                const int64_t s = ((int64_t)i * ny + j) * nz + k;
                const double xb = (i - x0) * dx, yb = (j - y0) * dy, zb = (k - z0) * dz;
                const double xs = xb + (gamma - 1) * (v1x * xb + v1y * yb + v1z * zb) * v1x / vMagSqr - gamma * v1x * dt;
                const double ys = yb + (gamma - 1) * (v1x * xb + v1y * yb + v1z * zb) * v1y / vMagSqr - gamma * v1y * dt;
                const double distance = sqrt(pow(xs, 2) + pow(ys, 2));
                double phiMag, AMag, Ax, Ay, re, im;
                off += profile_at(prof, g, distance, &phiMag, &AMag);
                if (xs == 0) { re = 0; Ay = 0; }
                else { re = phiMag * xs / distance; Ay = AMag * xs / pow(distance, 2); }
                if (ys == 0) { im = 0; Ax = 0; }
                else { im = phiMag * ys / distance; Ax = -AMag * ys / pow(distance, 2); }
                const int64_t sy = (int64_t)nz, sx = (int64_t)ny * nz;
                double dAx, dAy, dAz;   /* At differences and their divisors */
                double qx, qy, qz;
                if (i == 0) { dAx = At[s + sx] - At[s]; qx = dx; }
                else if (i == nx - 1) { dAx = At[s] - At[s - sx]; qx = dx; }
                else { dAx = At[s + sx] - At[s - sx]; qx = 2 * dx; }
                if (j == 0) { dAy = At[s + sy] - At[s]; qy = dy; }
                else if (j == ny - 1) { dAy = At[s] - At[s - sy]; qy = dy; }
                else { dAy = At[s + sy] - At[s - sy]; qy = 2 * dy; }
                if (k == 0) { dAz = At[s + 1] - At[s]; qz = dz; }
                else if (k == nz - 1) { dAz = At[s] - At[s - 1]; qz = dz; }
                else { dAz = At[s + 1] - At[s - 1]; qz = 2 * dz; }
                const double tx = (gamma - 1) * (v1x * Ax + v1y * Ay);
                double th0, th1, th2;
                if (b->form == LAT_IC_FORM_INPROCESS) {
                    /* ic_func.cpp:901-951 */
                    th0 = dx * g * (Ax + tx * v1x / vMagSqr);
                    th1 = dy * g * (Ay + tx * v1y / vMagSqr);
                    th2 = dz * g * (tx * v1z / vMagSqr);
                    th0 += -dx * g * dt * dAx / qx;
                    th1 += -dy * g * dt * dAy / qy;
                    th2 += -dz * g * dt * dAz / qz;
                } else {
                    /* initialConditions.cpp:918-977 */
                    double A0 = Ax + tx * v1x / vMagSqr;
                    double A1 = Ay + tx * v1y / vMagSqr;
                    double A2 = tx * v1z / vMagSqr;
                    A0 += -dt * dAx / qx;
                    A1 += -dt * dAy / qy;
                    A2 += -dt * dAz / qz;
                    th0 = dx * g * A0;
                    th1 = dy * g * A1;
                    th2 = dz * g * A2;
                }
                const double ang = -g * dt * At[s];
                BST(0, 1)[s] = cos(ang) * re - sin(ang) * im;
                BST(1, 1)[s] = cos(ang) * im + sin(ang) * re;
                BST(2, 1)[s] = th0;
                BST(3, 1)[s] = th1;
                BST(4, 1)[s] = th2;
            }
#undef BST
    free(At);
    return off;
}

/* ---------------------------------------------------------------------------
 * Loop-collision IC, initialConditions.cpp:994-1716, restated with the
 * reference's operation order: pow(x, 2), std::complex<double> arithmetic
 * written out as libstdc++ performs it for finite values (double + complex
 * adds to the real part only, complex * complex = (ac - bd, ad + bc)).
 * ------------------------------------------------------------------------- */

typedef struct { double v[3]; double vsq, gamma; } lc_boost;

static void lc_boost_init(lc_boost* b, const double v[3])
{
    b->v[0] = v[0];
    b->v[1] = v[1];
    b->v[2] = v[2];
    b->vsq = pow(v[0], 2) + pow(v[1], 2) + pow(v[2], 2);
    b->gamma = 1 / sqrt(1 - b->vsq);
}

/* (a + i b)/d as std::complex builds it from `a + ci*b` and `/ d` */
static void lc_unit(double a, double b, double d, double* re, double* im)
{
    *re = (0.0 * b + a) / d;
    *im = b / d;
}

/* the per-site work of one level (initialConditions.cpp:1061-1330 at t = 0,
 * 1430-1690 at t = dt); At is written at t = 0 and read at t = dt.  older:
 * ic_func.cpp's form (:1006-1250 at t = 0, :1365-1621 at t = dt), whose boosted
 * one-forms keep only the boost term (:1195-1196, :1229-1230, :1539-1542) */
static int lc_site(const lat_params* p, const lat_string_profile* prof, const lat_loop_collision_ic* c,
                   const lc_boost B[4], const double sf[4][2], int t, int i, int j, int k, double* At[4],
                   double P0[4], double th[3], int older)
{
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    const int x0 = (nx - 1) / 2, y0 = (ny - 1) / 2, z0 = (nz - 1) / 2;
    const double dx = p->dx, dy = p->dy, dz = p->dz, dt = p->dt, g = p->g;
    const int64_t s = ((int64_t)i * ny + j) * nz + k;
    const double xb = (i - x0) * dx, yb = (j - y0) * dy, zb = (k - z0) * dy;   /* zb with dy: :1067,:1442 */
    const lc_boost *b1s = &B[0], *b1a = &B[1], *b2s = &B[2], *b2a = &B[3];
    double ys1s, zs1s, ys1a, zs1a, xs2s, ys2s, xs2a, ys2a;
#define DOT(b) ((b)->v[0] * xb + (b)->v[1] * yb + (b)->v[2] * zb)
    if (b1s->vsq == 0) { ys1s = yb; zs1s = zb; }
    else {
        ys1s = yb + (b1s->gamma - 1) * DOT(b1s) * b1s->v[1] / b1s->vsq;
        zs1s = zb + (b1s->gamma - 1) * DOT(b1s) * b1s->v[2] / b1s->vsq;
        if (t) { ys1s -= b1s->gamma * b1s->v[1] * dt; zs1s -= b1s->gamma * b1s->v[2] * dt; }
    }
    if (b1a->vsq == 0) { ys1a = yb; zs1a = zb; }
    else {
        ys1a = yb + (b1a->gamma - 1) * DOT(b1a) * b1a->v[1] / b1a->vsq;
        zs1a = zb + (b1a->gamma - 1) * DOT(b1a) * b1a->v[2] / b1a->vsq;
        if (t) { ys1a -= b1a->gamma * b1a->v[1] * dt; zs1a -= b1a->gamma * b1a->v[2] * dt; }
    }
    if (b2s->vsq == 0) { xs2s = xb; ys2s = yb; }
    else {
        xs2s = xb + (b2s->gamma - 1) * DOT(b2s) * b2s->v[0] / b2s->vsq;
        ys2s = yb + (b2s->gamma - 1) * DOT(b2s) * b2s->v[1] / b2s->vsq;
        if (t) { xs2s -= b2s->gamma * b2s->v[0] * dt; ys2s -= b2s->gamma * b2s->v[1] * dt; }
    }
    if (b2a->vsq == 0) { xs2a = xb; ys2a = yb; }
    else {
        /* the reference projects xs2a on v2a[1] (:1085, :1460) */
        xs2a = xb + (b2a->gamma - 1) * DOT(b2a) * b2a->v[1] / b2a->vsq;
        ys2a = yb + (b2a->gamma - 1) * DOT(b2a) * b2a->v[1] / b2a->vsq;
        if (t) { xs2a -= b2a->gamma * b2a->v[0] * dt; ys2a -= b2a->gamma * b2a->v[1] * dt; }
    }
#undef DOT
    /* x - y style subtraction is written `a - b; a -= c` above: the reference
     * computes (xb + boost) - gamma*v*dt, the same two roundings */
    double d[4], pm[4], am[4];
    d[0] = sqrt(pow(ys1s - sf[0][0], 2) + pow(zs1s - sf[0][1], 2));
    d[1] = sqrt(pow(ys1a - sf[1][0], 2) + pow(zs1a - sf[1][1], 2));
    d[2] = sqrt(pow(xs2s - sf[2][0], 2) + pow(ys2s - sf[2][1], 2));
    d[3] = sqrt(pow(xs2a - sf[3][0], 2) + pow(ys2a - sf[3][1], 2));
    int off = 0;
    for (int q = 0; q < 4; ++q) off += profile_at(prof, g, d[q], &pm[q], &am[q]);
    double u[4][2];
    lc_unit(-(zs1s - sf[0][1]), ys1s - sf[0][0], d[0], &u[0][0], &u[0][1]);
    lc_unit(zs1a - sf[1][1], ys1a - sf[1][0], d[1], &u[1][0], &u[1][1]);
    lc_unit(xs2s - sf[2][0], ys2s - sf[2][1], d[2], &u[2][0], &u[2][1]);
    lc_unit(-(xs2a - sf[3][0]), ys2a - sf[3][1], d[3], &u[3][0], &u[3][1]);
    if (t) {
        /* phi -> phi e^{-i g dt At(t=0)}: gRot = cos - ci*sin, then cUnit*gRot */
        for (int q = 0; q < 4; ++q) {
            const double x = g * dt * At[q][s];
            const double sn = sin(x), cs = cos(x);
            const double gr = -(0.0 * sn) + cs, gi = -sn;
            const double a = u[q][0], bq = u[q][1];
            u[q][0] = a * gr - bq * gi;
            u[q][1] = a * gi + bq * gr;
        }
    }
    double ph[4][2], A[4][3];
    /* x-directed string (y, z components of A); A1s[0] = A1a[0] = 0 */
    A[0][0] = 0;
    if (zs1s - sf[0][1] == 0) { ph[0][0] = 0; A[0][1] = 0; }
    else { ph[0][0] = pm[0] * u[0][0]; A[0][1] = -am[0] * (zs1s - sf[0][1]) / pow(d[0], 2); }
    if (ys1s - sf[0][0] == 0) { ph[0][1] = 0; A[0][2] = 0; }
    else { ph[0][1] = pm[0] * u[0][1]; A[0][2] = am[0] * (ys1s - sf[0][0]) / pow(d[0], 2); }
    A[1][0] = 0;
    if (zs1a - sf[1][1] == 0) { ph[1][0] = 0; A[1][1] = 0; }
    else { ph[1][0] = pm[1] * u[1][0]; A[1][1] = am[1] * (zs1a - sf[1][1]) / pow(d[1], 2); }
    if (ys1a - sf[1][0] == 0) { ph[1][1] = 0; A[1][2] = 0; }
    else { ph[1][1] = pm[1] * u[1][1]; A[1][2] = -am[1] * (ys1a - sf[1][0]) / pow(d[1], 2); }
    /* z-directed string (x, y components); A2s[2] = A2a[2] = 0 */
    A[2][2] = 0;
    if (xs2s - sf[2][0] == 0) { ph[2][0] = 0; A[2][1] = 0; }
    else { ph[2][0] = pm[2] * u[2][0]; A[2][1] = am[2] * (xs2s - sf[2][0]) / pow(d[2], 2); }
    if (ys2s - sf[2][1] == 0) { ph[2][1] = 0; A[2][0] = 0; }
    else { ph[2][1] = pm[2] * u[2][1]; A[2][0] = -am[2] * (ys2s - sf[2][1]) / pow(d[2], 2); }
    A[3][2] = 0;
    if (xs2a - sf[3][0] == 0) { ph[3][0] = 0; A[3][1] = 0; }
    else { ph[3][0] = pm[3] * u[3][0]; A[3][1] = -am[3] * (xs2a - sf[3][0]) / pow(d[3], 2); }
    if (ys2a - sf[3][1] == 0) { ph[3][1] = 0; A[3][0] = 0; }
    else { ph[3][1] = pm[3] * u[3][1]; A[3][0] = am[3] * (ys2a - sf[3][1]) / pow(d[3], 2); }
    /* Lorentz transformation of the one-forms (pair 1 dots v with A's y, z;
     * pair 2 with A's x, y) */
    double Ap[4][3];
    for (int cc = 0; cc < 3 && older; ++cc) {
        Ap[0][cc] = (b1s->gamma - 1) * (b1s->v[1] * A[0][1] + b1s->v[2] * A[0][2]) * b1s->v[cc] / b1s->vsq;
        Ap[1][cc] = (b1a->gamma - 1) * (b1a->v[1] * A[1][1] + b1a->v[2] * A[1][2]) * b1a->v[cc] / b1a->vsq;
        Ap[2][cc] = (b2s->gamma - 1) * (b2s->v[0] * A[2][0] + b2s->v[1] * A[2][1]) * b2s->v[cc] / b2s->vsq;
        Ap[3][cc] = (b2a->gamma - 1) * (b2a->v[0] * A[3][0] + b2a->v[1] * A[3][1]) * b2a->v[cc] / b2a->vsq;
    }
    for (int cc = 0; cc < 3 && !older; ++cc) {
        Ap[0][cc] = b1s->vsq == 0 ? A[0][cc]
                                  : A[0][cc] + (b1s->gamma - 1) * (b1s->v[1] * A[0][1] + b1s->v[2] * A[0][2]) * b1s->v[cc] / b1s->vsq;
        Ap[1][cc] = b1a->vsq == 0 ? A[1][cc]
                                  : A[1][cc] + (b1a->gamma - 1) * (b1a->v[1] * A[1][1] + b1a->v[2] * A[1][2]) * b1a->v[cc] / b1a->vsq;
        Ap[2][cc] = b2s->vsq == 0 ? A[2][cc]
                                  : A[2][cc] + (b2s->gamma - 1) * (b2s->v[0] * A[2][0] + b2s->v[1] * A[2][1]) * b2s->v[cc] / b2s->vsq;
        Ap[3][cc] = b2a->vsq == 0 ? A[3][cc]
                                  : A[3][cc] + (b2a->gamma - 1) * (b2a->v[0] * A[3][0] + b2a->v[1] * A[3][1]) * b2a->v[cc] / b2a->vsq;
    }
    if (!t) {
        At[0][s] = -b1s->gamma * (b1s->v[1] * A[0][1] + b1s->v[2] * A[0][2]);
        At[1][s] = -b1a->gamma * (b1a->v[1] * A[1][1] + b1a->v[2] * A[1][2]);
        At[2][s] = -b2s->gamma * (b2s->v[0] * A[2][0] + b2s->v[1] * A[2][1]);
        At[3][s] = -b2a->gamma * (b2a->v[0] * A[3][0] + b2a->v[1] * A[3][1]);
    } else {
        /* gauge shift to At = 0, periodic centred differences (:1618-1640) */
        const int ip = (i + 1 + nx) % nx, im = (i - 1 + nx) % nx;
        const int jp = (j + 1 + ny) % ny, jm = (j - 1 + ny) % ny;
        const int kp = (k + 1 + nz) % nz, km = (k - 1 + nz) % nz;
        const int64_t sxp = ((int64_t)ip * ny + j) * nz + k, sxm = ((int64_t)im * ny + j) * nz + k;
        const int64_t syp = ((int64_t)i * ny + jp) * nz + k, sym = ((int64_t)i * ny + jm) * nz + k;
        const int64_t szp = ((int64_t)i * ny + j) * nz + kp, szm = ((int64_t)i * ny + j) * nz + km;
        for (int q = 0; q < 4; ++q) Ap[q][0] += -dt * (At[q][sxp] - At[q][sxm]) / (2 * dx);
        for (int q = 0; q < 4; ++q) Ap[q][1] += -dt * (At[q][syp] - At[q][sym]) / (2 * dy);
        for (int q = 0; q < 4; ++q) Ap[q][2] += -dt * (At[q][szp] - At[q][szm]) / (2 * dz);
    }
    /* pair products, tapered imaginary parts, magnitude kept (:1234-1262) */
    double A1[3], A2[3];
    for (int pair = 0; pair < 2; ++pair) {
        const double* a = ph[2 * pair];
        const double* bq = ph[2 * pair + 1];
        double p0 = a[0] * bq[0] - a[1] * bq[1];
        double p1 = a[1] * bq[0] + a[0] * bq[1];
        const double pf = pair == 0 ? (1 - pow(yb / (y0 * dy), 2)) * (1 - pow(zb / (z0 * dz), 2))
                                    : (1 - pow(xb / (x0 * dx), 2)) * (1 - pow(yb / (y0 * dy), 2));
        if (pow(p0, 2) + pow(p1 * pf, 2) == 0) {
            p0 = p1;
            p1 = 0;
        } else {
            const double nf = sqrt((pow(p0, 2) + pow(p1, 2)) / (pow(p0, 2) + pow(p1 * pf, 2)));
            p0 = nf * p0;
            p1 = nf * pf * p1;
        }
        P0[2 * pair] = p0;
        P0[2 * pair + 1] = p1;
        double* Ad = pair == 0 ? A1 : A2;
        for (int cc = 0; cc < 3; ++cc) Ad[cc] = (Ap[2 * pair][cc] + Ap[2 * pair + 1][cc]) * pf;
    }
    th[0] = dx * g * (A1[0] + A2[0]);
    th[1] = dy * g * (A1[1] + A2[1]);
    th[2] = dz * g * (A1[2] + A2[2]);
    return off;
}

static double lc_mag(const double* re, const double* im, int64_t s)
{
    return sqrt(pow(re[s], 2) + pow(im[s], 2));
}

static int64_t lc_build(const lat_params* p, const lat_string_profile* prof, const lat_loop_collision_ic* c,
                        double* st, int older)
{
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    if (nx < 3 || ny < 3 || nz < 3 || !prof || prof->m < 2 || !(prof->h > 0) || !c) return -1;
    lc_boost B[4];
    lc_boost_init(&B[0], c->v1s);
    lc_boost_init(&B[1], c->v1a);
    lc_boost_init(&B[2], c->v2s);
    lc_boost_init(&B[3], c->v2a);
    for (int q = 0; q < 4; ++q)
        if (!(B[q].vsq < 1) || (older && !(B[q].vsq > 0))) return -1;
    /* positions in each string's rest frame (:1030-1046); ic_func's form
     * measures from the lab-frame positions (ic_func.cpp:1034-1037) */
    double sf[4][2];
    const double* pos[4] = {c->pos1s, c->pos1a, c->pos2s, c->pos2a};
    for (int q = 0; q < 4; ++q) {
        const lc_boost* b = &B[q];
        if (b->vsq == 0 || older) { sf[q][0] = pos[q][0]; sf[q][1] = pos[q][1]; continue; }
        const int i0 = q < 2 ? 1 : 0;   /* pair 1: (y, z) use v[1], v[2]; pair 2: (x, y) use v[0], v[1] */
        const double dot = b->v[i0] * pos[q][0] + b->v[i0 + 1] * pos[q][1];
        sf[q][0] = pos[q][0] + (b->gamma - 1) * dot * b->v[i0] / b->vsq;
        sf[q][1] = pos[q][1] + (b->gamma - 1) * dot * b->v[i0 + 1] / b->vsq;
    }
    const int64_t N = (int64_t)nx * ny * nz;
    double* buf = (double*)malloc(sizeof(double) * (size_t)N * 12);
    if (!buf) return -1;
    double* At[4] = {buf, buf + N, buf + 2 * N, buf + 3 * N};
    double* P0[4] = {buf + 4 * N, buf + 5 * N, buf + 6 * N, buf + 7 * N};   /* phi1_0 re, im; phi2_0 re, im */
    double* P1[4] = {buf + 8 * N, buf + 9 * N, buf + 10 * N, buf + 11 * N};
    const int x0 = (nx - 1) / 2, y0 = (ny - 1) / 2, z0 = (nz - 1) / 2;
    const double dx = p->dx, dy = p->dy, dz = p->dz;
    int64_t off = 0;
#define LST(cc, t) (st + ((size_t)(cc) * 2 + (t)) * (size_t)N)
#define IX(i, j, k) (((int64_t)(i) * ny + (j)) * nz + (k))
    for (int t = 0; t < 2; ++t) {
        for (int i = 0; i < nx; ++i)
            for (int j = 0; j < ny; ++j)
                for (int k = 0; k < nz; ++k) {
                    double v4[4], th[3];
                    off += lc_site(p, prof, c, B, sf, t, i, j, k, At, v4, th, older);
                    const int64_t s = IX(i, j, k);
                    for (int q = 0; q < 4; ++q) P0[q][s] = v4[q];
                    LST(2, t)[s] = th[0];
                    LST(3, t)[s] = th[1];
                    LST(4, t)[s] = th[2];
                }
        /* magnitudes made continuous across the periodic faces: pair 1 over y,
         * pair 2 over x (:1336-1372), then pair 1 over z, pair 2 over y
         * (:1376-1414) */
        for (int i = 0; i < nx; ++i)
            for (int j = 0; j < ny; ++j)
                for (int k = 0; k < nz; ++k) {
                    const double xb = (i - x0) * dx, yb = (j - y0) * dy;
                    const int64_t s = IX(i, j, k);
                    const double m1t = lc_mag(P0[0], P0[1], IX(i, ny - 1, k)), m1b = lc_mag(P0[0], P0[1], IX(i, 0, k));
                    const double m2t = lc_mag(P0[2], P0[3], IX(nx - 1, j, k)), m2b = lc_mag(P0[2], P0[3], IX(0, j, k));
                    const double i1 = (m1t - m1b) * (yb + y0 * dy) / (2 * y0 * dy) + m1b;
                    const double i2 = (m2t - m2b) * (xb + x0 * dx) / (2 * x0 * dx) + m2b;
                    P1[0][s] = P0[0][s] / i1;
                    P1[1][s] = P0[1][s] / i1;
                    P1[2][s] = P0[2][s] / i2;
                    P1[3][s] = P0[3][s] / i2;
                }
        for (int i = 0; i < nx; ++i)
            for (int j = 0; j < ny; ++j)
                for (int k = 0; k < nz; ++k) {
                    const double yb = (j - y0) * dy, zb = (k - z0) * dz;
                    const int64_t s = IX(i, j, k);
                    const double m1t = lc_mag(P1[0], P1[1], IX(i, j, nz - 1)), m1b = lc_mag(P1[0], P1[1], IX(i, j, 0));
                    const double m2t = lc_mag(P1[2], P1[3], IX(i, ny - 1, k)), m2b = lc_mag(P1[2], P1[3], IX(i, 0, k));
                    const double i1 = (m1t - m1b) * (zb + z0 * dz) / (2 * z0 * dz) + m1b;
                    const double i2 = (m2t - m2b) * (yb + y0 * dy) / (2 * y0 * dy) + m2b;
                    const double a0 = P1[0][s] / i1, a1 = P1[1][s] / i1;
                    const double b0 = P1[2][s] / i2, b1 = P1[3][s] / i2;
                    LST(0, t)[s] = a0 * b0 - a1 * b1;
                    LST(1, t)[s] = a0 * b1 + a1 * b0;
                }
    }
#undef LST
#undef IX
    free(buf);
    return off;
}

int64_t orc_loop_collision_ic(const lat_params* p, const lat_string_profile* prof, const lat_loop_collision_ic* c,
                              double* st)
{
    return lc_build(p, prof, c, st, 0);
}

/* ic_func.cpp:966-1720, the "loop collision" that ic_w_evolution builds in
 * process (ic_func.cpp:25): the same steps as initialConditions.cpp's except
 * that the strings sit at the given lab-frame positions, the boosted one-forms
 * keep only the boost term, and every velocity must be non-zero (the form
 * divides by |v|^2 with no v = 0 branch) */
int64_t orc_icfunc_loop_collision_ic(const lat_params* p, const lat_string_profile* prof,
                                     const lat_loop_collision_ic* c, double* st)
{
    return lc_build(p, prof, c, st, 1);
}

/* ---------------------------------------------------------------------------
 * Perturbed straight strings, initialConditions.cpp:113-668, restated with
 * the reference's operation order (pow(x, 2) as the reference calls it).
 * Both write one level of fields; here it goes into both slots.
 * ------------------------------------------------------------------------- */

#define NG_NELLIP 1001  /* N_ellipint, initialConditions.cpp:45 */
#define NG_TOL 1e-6     /* tol, :44 */

/* trapezoid rule for the string's z(sigma): E(Omega*sigma) with the phase
 * shifted by -pi/2 (initialConditions.cpp:189-198) */
static double ng_ellip(double eps, double Omega, double sigma)
{
    const double pi = 4 * atan(1.0);
    double e = 0;
    for (int j = 0; j < NG_NELLIP; j++) {
        const double trap_fac = (j == 0 || j == NG_NELLIP - 1) ? 0.5 : 1;
        const double theta = j * Omega * sigma / (NG_NELLIP - 1) - pi / 2;
        e += trap_fac * sqrt(1 - pow(eps * sin(theta), 2)) * Omega * sigma / (NG_NELLIP - 1);
    }
    return e;
}

static double ng_dist2(double eps, double Omega, double sigma, double x, double z)
{
    const double pi = 4 * atan(1.0);
    const double e = ng_ellip(eps, Omega, sigma);
    return pow(x - eps * cos(Omega * sigma - pi / 2) / Omega, 2) + pow(z - e / Omega, 2);
}

/* Omega for a string periodic over the z extent dz*nz (initialConditions.cpp:143-160) */
double orc_ng_omega(double eps, double dz, int64_t nz)
{
    const double pi = 4 * atan(1.0);
    double e = 0;
    for (int j = 0; j < NG_NELLIP; j++) {
        const double trap_fac = (j == 0 || j == NG_NELLIP - 1) ? 0.5 : 1;
        const double theta = j * 2 * pi / (NG_NELLIP - 1);
        e += trap_fac * sqrt(1 - pow(eps * sin(theta), 2)) * 2 * pi / (NG_NELLIP - 1);
    }
    return e / (dz * (double)nz);
}

/* golden-section search for the string parameter closest to (x, z)
 * (initialConditions.cpp:175-382) and the quantities the sites of column
 * (x, z) use: out = xs, zs, xs_sigma, zs_sigma, paraVecMag, normal_dist */
void orc_ng_column(double eps, double Omega, double x, double z, double* out)
{
    const double pi = 4 * atan(1.0);
    const double gr = 0.5 * (1 + sqrt(5.0));
    double a = -2 * pi / Omega, b = 2 * pi / Omega;
    double sigma1 = b - (b - a) / gr, sigma2 = a + (b - a) / gr;
    double d1 = ng_dist2(eps, Omega, sigma1, x, z), d2 = ng_dist2(eps, Omega, sigma2, x, z);
    double tolTest = 1, sigma = 0;
    while (tolTest > NG_TOL) {
        if (d1 < d2) b = sigma2;
        else a = sigma1;
        sigma1 = b - (b - a) / gr;
        sigma2 = a + (b - a) / gr;
        d1 = ng_dist2(eps, Omega, sigma1, x, z);
        d2 = ng_dist2(eps, Omega, sigma2, x, z);
        tolTest = b - a;
        if (tolTest <= NG_TOL) sigma = d1 > d2 ? sigma2 : sigma1;
    }
    const double xs = eps * cos(Omega * sigma - pi / 2) / Omega;
    const double zs = ng_ellip(eps, Omega, sigma) / Omega;
    const double xs_sigma = -eps * sin(Omega * sigma - pi / 2);
    const double zs_sigma = sqrt(1 - pow(eps * sin(Omega * sigma - pi / 2), 2));
    const double paraVecMag = sqrt(pow(xs_sigma, 2) + pow(zs_sigma, 2));
    out[0] = xs;
    out[1] = zs;
    out[2] = xs_sigma;
    out[3] = zs_sigma;
    out[4] = paraVecMag;
    out[5] = (zs_sigma * (x - xs) - xs_sigma * (z - zs)) / paraVecMag;
}

int64_t orc_ng_sine_ic(const lat_params* p, const lat_string_profile* prof, double eps, double* st)
{
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    if (nx < 2 || ny < 2 || nz < 2 || !prof || prof->m < 2 || !(prof->h > 0) || !(eps >= 0 && eps < 1)) return -1;
    const int64_t N = (int64_t)nx * ny * nz;
    const double dx = p->dx, dy = p->dy, dz = p->dz, g = p->g;
    const double Omega = orc_ng_omega(eps, dz, nz);
    const int x0 = (nx - 1) / 2, y0 = (ny - 1) / 2, z0 = (nz - 1) / 2;
    double* F[5];
    for (int c = 0; c < 5; ++c) F[c] = st + (size_t)c * 2 * N;   /* slot 0 first, copied to slot 1 below */
    for (int c = 0; c < 5; ++c) memset(F[c], 0, sizeof(double) * (size_t)N);
#define NIX(i, j, k) (((int64_t)(i) * ny + (j)) * nz + (k))
    int64_t off = 0;
    for (int k = z0; k < nz; k++) {
        const double z = (k - z0) * dz;
        for (int i = 0; i < nx; i++) {
            const double x = (i - x0) * dx;
            double col[6];
            orc_ng_column(eps, Omega, x, z, col);
            const double xs = col[0], zs = col[1], xs_sigma = col[2], zs_sigma = col[3], paraVecMag = col[4],
                         normal_dist = col[5];
            for (int j = 0; j < ny; j++) {
                const double y = (j - y0) * dy;
                const double distance = sqrt(pow(x - xs, 2) + pow(y, 2) + pow(z - zs, 2));
                double phiMag, AMag, ph0, ph1, A0, A1, A2;
                off += profile_at(prof, g, distance, &phiMag, &AMag);
                if (normal_dist == 0) { ph0 = 0; A1 = 0; }
                else { ph0 = phiMag * normal_dist / distance; A1 = AMag * normal_dist / pow(distance, 2); }
                if (y == 0) { ph1 = 0; A0 = 0; A2 = 0; }
                else {
                    ph1 = phiMag * y / distance;
                    A0 = -AMag * zs_sigma * y / (pow(distance, 2) * paraVecMag);
                    A2 = AMag * xs_sigma * y / (pow(distance, 2) * paraVecMag);
                }
                const int64_t s = NIX(i, j, k), r = NIX(nx - 1 - i, j, nz - 1 - k);
                F[0][s] = ph0;
                F[1][s] = ph1;
                F[2][s] = A0;
                F[3][s] = A1;
                F[4][s] = A2;
                /* reflection across z = 0 (initialConditions.cpp:470-477) */
                F[0][r] = -F[0][s];
                F[1][r] = F[1][s];
                F[2][r] = F[2][s];
                F[3][r] = -F[3][s];
                if (k != nz - 1) F[4][NIX(nx - 1 - i, j, nz - 2 - k)] = -F[4][s];
            }
        }
    }
#undef NIX
    /* link columns d*g*A (initialConditions.cpp:482-486) */
    for (int64_t s = 0; s < N; ++s) {
        F[2][s] = dx * g * F[2][s];
        F[3][s] = dy * g * F[3][s];
        F[4][s] = dz * g * F[4][s];
    }
    for (int c = 0; c < 5; ++c) memcpy(F[c] + N, F[c], sizeof(double) * (size_t)N);
    return off;
}

int64_t orc_simple_sine_ic(const lat_params* p, const lat_string_profile* prof, double eps, double* st)
{
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    if (nx < 2 || ny < 2 || nz < 2 || !prof || prof->m < 2 || !(prof->h > 0)) return -1;
    const int64_t N = (int64_t)nx * ny * nz;
    const double dx = p->dx, dy = p->dy, dz = p->dz, g = p->g;
    const double pi = 4 * atan(1.0);
    const double Omega = 2 * pi / (dz * (nz - 1));
    const int x0 = (nx - 1) / 2, y0 = (ny - 1) / 2, z0 = (nz - 1) / 2;
    int64_t off = 0;
    for (int i = 0; i < nx; i++) {
        const double x = (i - x0) * dx;
        for (int j = 0; j < ny; j++) {
            const double y = (j - y0) * dy;
            for (int k = 0; k < nz; k++) {
                const double z = (k - z0) * dz;
                const double xdist = x - eps * sin(Omega * z) / Omega;
                const double distance = sqrt(xdist * xdist + y * y);
                double phiMag, AMag, ph0, ph1, A0, A1, A2;
                off += profile_at(prof, g, distance, &phiMag, &AMag);
                if (xdist == 0) { ph0 = 0; A1 = 0; }
                else { ph0 = phiMag * xdist / distance; A1 = AMag * xdist / pow(distance, 2); }
                if (y == 0) { ph1 = 0; A0 = 0; A2 = 0; }
                else { ph1 = phiMag * y / distance; A0 = -AMag * y / pow(distance, 2); A2 = 0; }
                const int64_t s = ((int64_t)i * ny + j) * nz + k;
                const double v[5] = {ph0, ph1, dx * g * A0, dy * g * A1, dz * g * A2};
                for (int c = 0; c < 5; ++c) {
                    st[((size_t)c * 2) * N + s] = v[c];
                    st[((size_t)c * 2 + 1) * N + s] = v[c];
                }
            }
        }
    }
    return off;
}
