// Abelian-Higgs FP64 step in two passes.
//
// FP64 on GB300 runs at 1/64 of the FP32 rate, so the step is bound by FP64
// instructions, not by HBM: the one-pass kernel (ah_step.cuh) evaluates every
// link's sin/cos and every plaquette sine twice, once for each site that
// needs it (as the reference does, mpi_evolution.cpp:418-487).  Here pass 1
// evaluates them once per site into a scratch buffer ("link data") and pass 2
// performs the update (mpi_evolution.cpp:412-501) reading the link data of the
// site and of its three backward neighbours.  The extra HBM traffic
// (~200 B/site) is small next to the FP64 time it saves.
//
// STRICT = true keeps the reference's rounding operation by operation (the
// translation unit is compiled with -fmad=false); the link data are the very
// doubles the one-pass kernel computes, so the two paths agree bit for bit.
// STRICT = false (LAT_F64_FAST) lets the compiler fuse multiply-adds, divides
// by dt through a corrected reciprocal, and takes sin(P_yx) = -sin(P_xy)
// (likewise zx, zy): the same arithmetic to within an ulp per operation.
#pragma once

#include "site_common.cuh"

namespace lat {

// link-data slots ([slot][N], SoA)
enum LinkSlot {
    L_CX, L_SX, L_CY, L_SY, L_CZ, L_SZ,   // cos/sin of theta_mu at the site
    L_PXY, L_PXZ, L_PYZ,                    // sin of P_xy, P_xz, P_yz at the site
    L_PYX, L_PZX, L_PZY,                    // sin of P_yx, P_zx, P_zy (STRICT only)
    L_CPXY, L_CPXZ, L_CPYZ,                 // cos of P_xy, P_xz, P_yz (diagnostic steps)
    L_COUNT
};

// Base address of every link-data slot.  The host forms them from the
// buffer and the site count in 64-bit arithmetic: an int slot*N + s offset
// would pass 2^31 above 143,165,576 sites (15 slots), where a kernel would
// write at a wrapped offset.  Inside one slot the site index s < 2^31.
template <class P>
struct LinkSlotsT {
    P p[L_COUNT];
};
using LinkSlots = LinkSlotsT<double* __restrict__>;
using LinkSlotsC = LinkSlotsT<const double* __restrict__>;

inline LinkSlots link_slots(double* L, long long N)
{
    LinkSlots s;
    for (int q = 0; q < L_COUNT; ++q) s.p[q] = L + (size_t)q * (size_t)N;
    return s;
}

inline LinkSlotsC link_slots_c(const double* L, long long N)
{
    LinkSlotsC s;
    for (int q = 0; q < L_COUNT; ++q) s.p[q] = L + (size_t)q * (size_t)N;
    return s;
}

// a / b where b = spacing^2 or spacing: exact reciprocal multiply when every
// spacing is a power of two (then a*(1/b) == a/b for all a), else the IEEE
// quotient by cdiv from the host reciprocal.
template <bool RECIP>
__device__ __forceinline__ double sdiv(double a, double b, double inv_b)
{
    if constexpr (RECIP) return mul_pow2(a, inv_b);
    else return cdiv(a, b, inv_b);
}

// a / dt.  STRICT: the IEEE quotient by cdiv (two residual corrections from
// the host reciprocal; a zero dividend returns a * (1/b), the same +-0).
// Fast: q = a*r corrected by one residual step (Markstein), which returns the
// correctly rounded quotient except in rare cases where it is one ulp off.
template <bool STRICT>
__device__ __forceinline__ double tdiv(double a, double b, double inv_b)
{
    if constexpr (STRICT) return cdiv(a, b, inv_b);
    else {
        const double q = a * inv_b;
        const double r = fma(-q, b, a);
        return fma(r, inv_b, q);
    }
}

template <bool STRICT, bool DIAG>
__global__ void __launch_bounds__(BLOCK) ah_links_kernel(const Geom g, const double* __restrict__ TX,
                                                         const double* __restrict__ TY,
                                                         const double* __restrict__ TZ, const LinkSlots L)
{
    const int k = (int)(blockIdx.x * BZ + threadIdx.x);
    const int j = (int)(blockIdx.y * BY + threadIdx.y);
    const int i = (int)blockIdx.z;
    if (k >= g.nz || j >= g.ny) return;
    const Nbr n = make_nbr(g, i, j, k);
    const int s = n.s;
    const double tx = TX[s], ty = TY[s], tz = TZ[s];
    const double tyxp = TY[s + n.xp], tzxp = TZ[s + n.xp];
    const double txyp = TX[s + n.yp], tzyp = TZ[s + n.yp];
    const double txzp = TX[s + n.zp], tyzp = TY[s + n.zp];
    double sv, cv;
    dsincos(tx, &sv, &cv);
    L.p[L_CX][s] = cv;
    L.p[L_SX][s] = sv;
    dsincos(ty, &sv, &cv);
    L.p[L_CY][s] = cv;
    L.p[L_SY][s] = sv;
    dsincos(tz, &sv, &cv);
    L.p[L_CZ][s] = cv;
    L.p[L_SZ][s] = sv;
    // plaquette angles, summed in the reference's order (mpi_evolution.cpp:471-487)
    const double Pxy = tx + tyxp - txyp - ty;
    const double Pxz = tx + tzxp - txzp - tz;
    const double Pyz = ty + tzyp - tyzp - tz;
    if constexpr (DIAG) {
        dsincos(Pxy, &sv, &cv);
        L.p[L_PXY][s] = sv;
        L.p[L_CPXY][s] = cv;
        dsincos(Pxz, &sv, &cv);
        L.p[L_PXZ][s] = sv;
        L.p[L_CPXZ][s] = cv;
        dsincos(Pyz, &sv, &cv);
        L.p[L_PYZ][s] = sv;
        L.p[L_CPYZ][s] = cv;
    } else {
        L.p[L_PXY][s] = dsin(Pxy);
        L.p[L_PXZ][s] = dsin(Pxz);
        L.p[L_PYZ][s] = dsin(Pyz);
    }
    if constexpr (STRICT) {
        L.p[L_PYX][s] = dsin(ty + txyp - tyxp - tx);
        L.p[L_PZX][s] = dsin(tz + txzp - tzxp - tx);
        L.p[L_PZY][s] = dsin(tz + tyzp - tzyp - ty);
    }
}

template <bool STRICT, bool DIAG, bool RECIP>
__global__ void __launch_bounds__(BLOCK, 2) ah_update_kernel(const Geom g, const Fields<double, 5> f,
                                                          const LinkSlotsC L, const StepCoef c,
                                                          const DiagOut d)
{
    const int k = g.loz + (int)(blockIdx.x * BZ + threadIdx.x);
    const int j = g.loy + (int)(blockIdx.y * BY + threadIdx.y);
    const int i = g.lox + (int)blockIdx.z;
    double e_site = 0.0, g_site = 0.0;

    if (k < g.hiz && j < g.hiy) {
        const Nbr n = make_nbr(g, i, j, k);
        const int s = n.s;
        const int sxm = s + n.xm, sym_ = s + n.ym, szm = s + n.zm;
        const double* __restrict__ P0 = f.now[0];
        const double* __restrict__ P1 = f.now[1];

        const double p0 = P0[s], p1 = P1[s];
        const double p0xp = P0[s + n.xp], p1xp = P1[s + n.xp], p0xm = P0[sxm], p1xm = P1[sxm];
        const double p0yp = P0[s + n.yp], p1yp = P1[s + n.yp], p0ym = P0[sym_], p1ym = P1[sym_];
        const double p0zp = P0[s + n.zp], p1zp = P1[s + n.zp], p0zm = P0[szm], p1zm = P1[szm];
        const double q0 = f.past[0][s], q1 = f.past[1][s];
        const double tx = f.now[2][s], ty = f.now[3][s], tz = f.now[4][s];
        const double qx = f.past[2][s], qy = f.past[3][s], qz = f.past[4][s];

        const double cx = L.p[L_CX][s], sx = L.p[L_SX][s];
        const double cy = L.p[L_CY][s], sy = L.p[L_SY][s];
        const double cz = L.p[L_CZ][s], sz = L.p[L_SZ][s];
        const double cxm = L.p[L_CX][sxm], sxm_ = L.p[L_SX][sxm];
        const double cym = L.p[L_CY][sym_], sym = L.p[L_SY][sym_];
        const double czm = L.p[L_CZ][szm], szm_ = L.p[L_SZ][szm];
        const double sPxy = L.p[L_PXY][s], sPxz = L.p[L_PXZ][s], sPyz = L.p[L_PYZ][s];
        const double sPxy_m = L.p[L_PXY][sym_], sPxz_m = L.p[L_PXZ][szm], sPyz_m = L.p[L_PYZ][szm];
        double sPyx, sPzx, sPzy, sPyx_m, sPzx_m, sPzy_m;
        if constexpr (STRICT) {
            sPyx = L.p[L_PYX][s];
            sPzx = L.p[L_PZX][s];
            sPzy = L.p[L_PZY][s];
            sPyx_m = L.p[L_PYX][sxm];
            sPzx_m = L.p[L_PZX][sxm];
            sPzy_m = L.p[L_PZY][sym_];
        } else {
            sPyx = -sPxy;
            sPzx = -sPxz;
            sPzy = -sPyz;
            sPyx_m = -L.p[L_PXY][sxm];
            sPzx_m = -L.p[L_PXZ][sxm];
            sPzy_m = -L.p[L_PYZ][sym_];
        }

        const double twop0 = mul_pow2(p0, 2.0), twop1 = mul_pow2(p1, 2.0);  // 2 * p0, 2 * p1
        const double phiMagSqr = p0 * p0 + p1 * p1;
        const double pot = c.halfLambda * (phiMagSqr - c.etaSq);

        double tt0, tt1, curx, cury, curz;
        if constexpr (STRICT) {
            // covariant Laplacian (mpi_evolution.cpp:418-428), c = +1 then c = -1
            const double lap0 = sdiv<RECIP>(cx * p0xp + sx * p1xp - twop0 + cxm * p0xm - sxm_ * p1xm, c.dx2, c.inv_dx2)
                              + sdiv<RECIP>(cy * p0yp + sy * p1yp - twop0 + cym * p0ym - sym * p1ym, c.dy2, c.inv_dy2)
                              + sdiv<RECIP>(cz * p0zp + sz * p1zp - twop0 + czm * p0zm - szm_ * p1zm, c.dz2, c.inv_dz2);
            const double lap1 = sdiv<RECIP>(cx * p1xp - sx * p0xp - twop1 + cxm * p1xm + sxm_ * p0xm, c.dx2, c.inv_dx2)
                              + sdiv<RECIP>(cy * p1yp - sy * p0yp - twop1 + cym * p1ym + sym * p0ym, c.dy2, c.inv_dy2)
                              + sdiv<RECIP>(cz * p1zp - sz * p0zp - twop1 + czm * p1zm + szm_ * p0zm, c.dz2, c.inv_dz2);
            tt0 = lap0 - pot * p0;
            tt1 = lap1 - pot * p1;
            if (c.fric != 0) {
                tt0 = tt0 - c.fric * tdiv<STRICT>(p0 - q0, c.dt, c.inv_dt);
                tt1 = tt1 - c.fric * tdiv<STRICT>(p1 - q1, c.dt, c.inv_dt);
            }
            // gauge current (mpi_evolution.cpp:459-466)
            curx = cx * (p1 * p0xp - p0 * p1xp) + sx * (p0 * p0xp + p1 * p1xp);
            cury = cy * (p1 * p0yp - p0 * p1yp) + sy * (p0 * p0yp + p1 * p1yp);
            curz = cz * (p1 * p0zp - p0 * p1zp) + sz * (p0 * p0zp + p1 * p1zp);
        } else {
            // The same quantities with fewer FP64 instructions.  The forward
            // link-transported neighbour U_mu phi(x+mu), A = c phi0' + s phi1',
            // B = c phi1' - s phi0', enters both the Laplacian and the current:
            // j_mu = c (phi1 phi0' - phi0 phi1') + s (phi0 phi0' + phi1 phi1')
            //      = phi1 A - phi0 B.
            // With equal spacings the three directions are summed before one
            // scaling; friction uses fric/dt from the host.
            const double Ax = fma(sx, p1xp, cx * p0xp), Bx = fma(-sx, p0xp, cx * p1xp);
            const double Ay = fma(sy, p1yp, cy * p0yp), By = fma(-sy, p0yp, cy * p1yp);
            const double Az = fma(sz, p1zp, cz * p0zp), Bz = fma(-sz, p0zp, cz * p1zp);
            double lap0, lap1;
            if (c.iso != 0) {
                const double s0 = fma(-sxm_, p1xm, fma(cxm, p0xm, Ax)) + fma(-sym, p1ym, fma(cym, p0ym, Ay))
                                + fma(-szm_, p1zm, fma(czm, p0zm, Az));
                const double s1 = fma(sxm_, p0xm, fma(cxm, p1xm, Bx)) + fma(sym, p0ym, fma(cym, p1ym, By))
                                + fma(szm_, p0zm, fma(czm, p1zm, Bz));
                lap0 = sdiv<RECIP>(fma(-6.0, p0, s0), c.dx2, c.inv_dx2);
                lap1 = sdiv<RECIP>(fma(-6.0, p1, s1), c.dx2, c.inv_dx2);
            } else {
                lap0 = sdiv<RECIP>(fma(-sxm_, p1xm, fma(cxm, p0xm, Ax)) - twop0, c.dx2, c.inv_dx2)
                     + sdiv<RECIP>(fma(-sym, p1ym, fma(cym, p0ym, Ay)) - twop0, c.dy2, c.inv_dy2)
                     + sdiv<RECIP>(fma(-szm_, p1zm, fma(czm, p0zm, Az)) - twop0, c.dz2, c.inv_dz2);
                lap1 = sdiv<RECIP>(fma(sxm_, p0xm, fma(cxm, p1xm, Bx)) - twop1, c.dx2, c.inv_dx2)
                     + sdiv<RECIP>(fma(sym, p0ym, fma(cym, p1ym, By)) - twop1, c.dy2, c.inv_dy2)
                     + sdiv<RECIP>(fma(szm_, p0zm, fma(czm, p1zm, Bz)) - twop1, c.dz2, c.inv_dz2);
            }
            tt0 = fma(-pot, p0, lap0);
            tt1 = fma(-pot, p1, lap1);
            if (c.fric != 0) {
                tt0 = fma(-c.fric_dt, p0 - q0, tt0);
                tt1 = fma(-c.fric_dt, p1 - q1, tt1);
            }
            curx = fma(p1, Ax, -p0 * Bx);
            cury = fma(p1, Ay, -p0 * By);
            curz = fma(p1, Az, -p0 * Bz);
        }

        // lattice curl (mpi_evolution.cpp:471-487)
        const double Fxy_y = sdiv<RECIP>(sPxy - sPxy_m, c.dy2, c.inv_dy2);
        const double Fxz_z = sdiv<RECIP>(sPxz - sPxz_m, c.dz2, c.inv_dz2);
        const double Fyx_x = sdiv<RECIP>(sPyx - sPyx_m, c.dx2, c.inv_dx2);
        const double Fyz_z = sdiv<RECIP>(sPyz - sPyz_m, c.dz2, c.inv_dz2);
        const double Fzx_x = sdiv<RECIP>(sPzx - sPzx_m, c.dx2, c.inv_dx2);
        const double Fzy_y = sdiv<RECIP>(sPzy - sPzy_m, c.dy2, c.inv_dy2);

        double ttx = c.m2gg * curx - Fxy_y - Fxz_z;
        double tty = c.m2gg * cury - Fyx_x - Fyz_z;
        double ttz = c.m2gg * curz - Fzx_x - Fzy_y;
        if (c.damp != 0) {
            ttx = ttx - c.damp * tdiv<STRICT>(tx - qx, c.dt, c.inv_dt);
            tty = tty - c.damp * tdiv<STRICT>(ty - qy, c.dt, c.inv_dt);
            ttz = ttz - c.damp * tdiv<STRICT>(tz - qz, c.dt, c.inv_dt);
        }

        double divNow = 0;
        if (DIAG || d.store_div) {
            const double txm = f.now[2][sxm], tym = f.now[3][sym_], tzm = f.now[4][szm];
            divNow = sdiv<RECIP>(tx - txm, c.dx2, c.inv_dx2) + sdiv<RECIP>(ty - tym, c.dy2, c.inv_dy2)
                   + sdiv<RECIP>(tz - tzm, c.dz2, c.inv_dz2);
        }

        if constexpr (DIAG) {
            // energy density and Gauss deviation of the now level
            // (evolution.cpp:322-334,377-427; mpi_evolution.cpp:509-532).  Each
            // divisor other than dt occurs once per site, so cdiv's host
            // reciprocal replaces the division's own (the same doubles).
            const double cPxy = L.p[L_CPXY][s], cPxz = L.p[L_CPXZ][s], cPyz = L.p[L_CPYZ][s];
            const double pt0 = tdiv<STRICT>(p0 - q0, c.dt, c.inv_dt);
            const double pt1 = tdiv<STRICT>(p1 - q1, c.dt, c.inv_dt);
            const double px0 = sdiv<RECIP>(p0 - cxm * p0xm + sxm_ * p1xm, c.dx, c.inv_dx);
            const double px1 = sdiv<RECIP>(p1 - cxm * p1xm - sxm_ * p0xm, c.dx, c.inv_dx);
            const double py0 = sdiv<RECIP>(p0 - cym * p0ym + sym * p1ym, c.dy, c.inv_dy);
            const double py1 = sdiv<RECIP>(p1 - cym * p1ym - sym * p0ym, c.dy, c.inv_dy);
            const double pz0 = sdiv<RECIP>(p0 - czm * p0zm + szm_ * p1zm, c.dz, c.inv_dz);
            const double pz1 = sdiv<RECIP>(p1 - czm * p1zm - szm_ * p0zm, c.dz, c.inv_dz);
            double tdc = 0, fc = 0, gauss = 0;
            if (d.energy_form == LAT_ENERGY_MPI) {
                const double a0 = tdiv<true>(tx - qx, c.dt, c.inv_dt), a1 = tdiv<true>(ty - qy, c.dt, c.inv_dt),
                             a2 = tdiv<true>(tz - qz, c.dt, c.inv_dt);
                tdc = 0.5 * (a0 * a0 + a1 * a1 + a2 * a2);
                fc = cdiv(1 - cPxy, c.gxy2, c.inv_gxy2) + cdiv(1 - cPxz, c.gxz2, c.inv_gxz2)
                   + cdiv(1 - cPyz, c.gyz2, c.inv_gyz2);
            }
            if (c.g != 0) {
                const double divPast = reinterpret_cast<const double*>(d.divbuf)[s];
                const double divThetat = tdiv<true>(divNow - divPast, c.dt, c.inv_dt);
                gauss = cdiv(divThetat, c.g, c.inv_g) - c.twog * (p1 * pt0 - p0 * pt1);
                if (d.energy_form != LAT_ENERGY_MPI) {
                    const double a0 = cdiv(tx - qx, c.gdtdx, c.inv_gdtdx), a1 = cdiv(ty - qy, c.gdtdy, c.inv_gdtdy),
                                 a2 = cdiv(tz - qz, c.gdtdz, c.inv_gdtdz);
                    tdc = 0.5 * (a0 * a0 + a1 * a1 + a2 * a2);
                    const double Fxy = cdiv(1 - cPxy, c.gxy2, c.inv_gxy2);
                    const double Fxz = cdiv(1 - cPxz, c.gxz2, c.inv_gxz2);
                    const double Fyz = cdiv(1 - cPyz, c.gyz2, c.inv_gyz2);
                    fc = Fxy + Fxz + Fyz;
                }
            }
            const double pm = phiMagSqr - c.etaSq;
            const double ed = pt0 * pt0 + pt1 * pt1 + px0 * px0 + px1 * px1 + py0 * py0 + py1 * py1 + pz0 * pz0
                            + pz1 * pz1 + tdc + fc + c.quarterLambda * (pm * pm);
            if (d.energy_form == LAT_ENERGY_MPI) e_site = ed * c.dx * c.dy * c.dz;
            else e_site = c.dV * ed;
            g_site = fabs(gauss);
        }

        if (d.store_div) reinterpret_cast<double*>(d.divbuf)[s] = divNow;

        if (d.write) {  // in-place update of the past slot (mpi_evolution.cpp:432,499-501)
            f.past[0][s] = twop0 - q0 + c.dt2 * tt0;
            f.past[1][s] = twop1 - q1 + c.dt2 * tt1;
            f.past[2][s] = mul_pow2(tx, 2.0) - qx + c.dt2 * ttx;
            f.past[3][s] = mul_pow2(ty, 2.0) - qy + c.dt2 * tty;
            f.past[4][s] = mul_pow2(tz, 2.0) - qz + c.dt2 * ttz;
        }
    }
    if constexpr (DIAG) block_sum2_store(e_site, g_site, d.partials);
}

template <bool STRICT>
cudaError_t launch_ah_twopass(const Geom& g, const Fields<double, 5>& f, double* L, const StepCoef& c,
                              const DiagOut& d, bool diag, bool recip, cudaStream_t st)
{
    const long long N = (long long)g.nx * g.syz;
    const LinkSlots Lw = link_slots(L, N);
    const LinkSlotsC Lr = link_slots_c(L, N);
    Geom all = g;
    all.lox = all.loy = all.loz = 0;
    all.hix = g.nx;
    all.hiy = g.ny;
    all.hiz = g.nz;
    const dim3 block(BZ, BY);
    if (diag) ah_links_kernel<STRICT, true><<<site_grid(all), block, 0, st>>>(g, f.now[2], f.now[3], f.now[4], Lw);
    else ah_links_kernel<STRICT, false><<<site_grid(all), block, 0, st>>>(g, f.now[2], f.now[3], f.now[4], Lw);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const dim3 grid = site_grid(g);
    if (diag) {
        if (recip) ah_update_kernel<STRICT, true, true><<<grid, block, 0, st>>>(g, f, Lr, c, d);
        else ah_update_kernel<STRICT, true, false><<<grid, block, 0, st>>>(g, f, Lr, c, d);
    } else {
        if (recip) ah_update_kernel<STRICT, false, true><<<grid, block, 0, st>>>(g, f, Lr, c, d);
        else ah_update_kernel<STRICT, false, false><<<grid, block, 0, st>>>(g, f, Lr, c, d);
    }
    return cudaGetLastError();
}

}  // namespace lat
