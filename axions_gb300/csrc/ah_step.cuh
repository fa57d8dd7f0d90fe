// Abelian-Higgs leapfrog step: one fused stencil kernel per time step.
//
// Replaces the per-site loop body of mpi_evolution.cpp:381-501 (EoM of phi and
// the link phases theta, in-place update into the past slot) and, on
// diagnostic steps, the energy and Gauss terms of evolution.cpp:294-427.
// The update is in place and race-free: every thread reads neighbours only
// from the "now" slot, and the "past" slot only at its own site before writing
// it.  The FP64 instantiation keeps the reference's operation order operation
// by operation (this translation unit is compiled with -fmad=false), so the
// only differences to the reference are CUDA's sin/cos versus libm's.
#pragma once

#include "site_common.cuh"

namespace lat {

template <class T, bool DIAG>
__global__ void __launch_bounds__(BLOCK) ah_step_kernel(const Geom g, const Fields<T, 5> f, const StepCoefT<T> c,
                                                        const DiagOut d)
{
    using TR = Trig<T>;
    const int k = g.loz + (int)(blockIdx.x * BZ + threadIdx.x);
    const int j = g.loy + (int)(blockIdx.y * BY + threadIdx.y);
    const int i = g.lox + (int)blockIdx.z;
    double e_site = 0.0, g_site = 0.0;

    if (k < g.hiz && j < g.hiy) {
        const Nbr n = make_nbr(g, i, j, k);
        const int s = n.s;
        const T* __restrict__ P0 = f.now[0];
        const T* __restrict__ P1 = f.now[1];
        const T* __restrict__ TX = f.now[2];
        const T* __restrict__ TY = f.now[3];
        const T* __restrict__ TZ = f.now[4];

        const T dt2 = (T)c.dt2;

        // scalar field, now level, at the site and its six neighbours
        const T p0 = P0[s], p1 = P1[s];
        const T p0xp = P0[s + n.xp], p1xp = P1[s + n.xp], p0xm = P0[s + n.xm], p1xm = P1[s + n.xm];
        const T p0yp = P0[s + n.yp], p1yp = P1[s + n.yp], p0ym = P0[s + n.ym], p1ym = P1[s + n.ym];
        const T p0zp = P0[s + n.zp], p1zp = P1[s + n.zp], p0zm = P0[s + n.zm], p1zm = P1[s + n.zm];
        // past level at the site (read before it is overwritten)
        const T q0 = f.past[0][s], q1 = f.past[1][s];
        const T qx = f.past[2][s], qy = f.past[3][s], qz = f.past[4][s];

        // link phases
        const T tx = TX[s], ty = TY[s], tz = TZ[s];
        const T txm = TX[s + n.xm], tym = TY[s + n.ym], tzm = TZ[s + n.zm];
        T sx, cx, sy, cy, sz, cz, sxm, cxm, sym, cym, szm, czm;
        TR::sincos(tx, &sx, &cx);
        TR::sincos(ty, &sy, &cy);
        TR::sincos(tz, &sz, &cz);
        TR::sincos(txm, &sxm, &cxm);
        TR::sincos(tym, &sym, &cym);
        TR::sincos(tzm, &szm, &czm);

        const T phiMagSqr = p0 * p0 + p1 * p1;
        const T pot = (T)c.halfLambda * (phiMagSqr - (T)c.etaSq);

        // covariant Laplacian, component 0 (c = +1) and 1 (c = -1)
        // (mpi_evolution.cpp:418-428)
        T lap0 = qdiv<T>(cx * p0xp + sx * p1xp - 2 * p0 + cxm * p0xm - sxm * p1xm, c.dx2, c.inv_dx2)
               + qdiv<T>(cy * p0yp + sy * p1yp - 2 * p0 + cym * p0ym - sym * p1ym, c.dy2, c.inv_dy2)
               + qdiv<T>(cz * p0zp + sz * p1zp - 2 * p0 + czm * p0zm - szm * p1zm, c.dz2, c.inv_dz2);
        T lap1 = qdiv<T>(cx * p1xp - sx * p0xp - 2 * p1 + cxm * p1xm + sxm * p0xm, c.dx2, c.inv_dx2)
               + qdiv<T>(cy * p1yp - sy * p0yp - 2 * p1 + cym * p1ym + sym * p0ym, c.dy2, c.inv_dy2)
               + qdiv<T>(cz * p1zp - sz * p0zp - 2 * p1 + czm * p1zm + szm * p0zm, c.dz2, c.inv_dz2);
        T tt0 = lap0 - pot * p0;
        T tt1 = lap1 - pot * p1;
        if (c.fric != 0) {
            tt0 = tt0 - (T)c.fric * qdiv<T>(p0 - q0, c.dt, c.inv_dt);
            tt1 = tt1 - (T)c.fric * qdiv<T>(p1 - q1, c.dt, c.inv_dt);
        }

        // gauge current (mpi_evolution.cpp:459-466)
        const T curx = cx * (p1 * p0xp - p0 * p1xp) + sx * (p0 * p0xp + p1 * p1xp);
        const T cury = cy * (p1 * p0yp - p0 * p1yp) + sy * (p0 * p0yp + p1 * p1yp);
        const T curz = cz * (p1 * p0zp - p0 * p1zp) + sz * (p0 * p0zp + p1 * p1zp);

        // plaquette angles at the site and at the backward neighbours
        // (mpi_evolution.cpp:471-487)
        const T tyxp = TY[s + n.xp], tzxp = TZ[s + n.xp];
        const T txyp = TX[s + n.yp], tzyp = TZ[s + n.yp];
        const T txzp = TX[s + n.zp], tyzp = TY[s + n.zp];
        const T Pxy = tx + tyxp - txyp - ty;
        const T Pxz = tx + tzxp - txzp - tz;
        const T Pyx = ty + txyp - tyxp - tx;
        const T Pyz = ty + tzyp - tyzp - tz;
        const T Pzx = tz + txzp - tzxp - tx;
        const T Pzy = tz + tyzp - tzyp - ty;
        const T Pxy_m = TX[s + n.ym] + TY[s + n.xp + n.ym] - tx - tym;
        const T Pxz_m = TX[s + n.zm] + TZ[s + n.xp + n.zm] - tx - tzm;
        const T Pyx_m = TY[s + n.xm] + TX[s + n.xm + n.yp] - ty - txm;
        const T Pyz_m = TY[s + n.zm] + TZ[s + n.yp + n.zm] - ty - tzm;
        const T Pzx_m = TZ[s + n.xm] + TX[s + n.xm + n.zp] - tz - txm;
        const T Pzy_m = TZ[s + n.ym] + TY[s + n.ym + n.zp] - tz - tym;

        T sPxy, cPxy, sPxz, cPxz, sPyz, cPyz;
        if constexpr (DIAG) {
            TR::sincos(Pxy, &sPxy, &cPxy);
            TR::sincos(Pxz, &sPxz, &cPxz);
            TR::sincos(Pyz, &sPyz, &cPyz);
        } else {
            sPxy = TR::sin(Pxy);
            sPxz = TR::sin(Pxz);
            sPyz = TR::sin(Pyz);
        }
        const T Fxy_y = qdiv<T>(sPxy - TR::sin(Pxy_m), c.dy2, c.inv_dy2);
        const T Fxz_z = qdiv<T>(sPxz - TR::sin(Pxz_m), c.dz2, c.inv_dz2);
        const T Fyx_x = qdiv<T>(TR::sin(Pyx) - TR::sin(Pyx_m), c.dx2, c.inv_dx2);
        const T Fyz_z = qdiv<T>(sPyz - TR::sin(Pyz_m), c.dz2, c.inv_dz2);
        const T Fzx_x = qdiv<T>(TR::sin(Pzx) - TR::sin(Pzx_m), c.dx2, c.inv_dx2);
        const T Fzy_y = qdiv<T>(TR::sin(Pzy) - TR::sin(Pzy_m), c.dy2, c.inv_dy2);

        const T m2gg = (T)c.m2gg;
        T ttx = m2gg * curx - Fxy_y - Fxz_z;
        T tty = m2gg * cury - Fyx_x - Fyz_z;
        T ttz = m2gg * curz - Fzx_x - Fzy_y;
        if (c.damp != 0) {
            const T damp = (T)c.damp;
            ttx = ttx - damp * qdiv<T>(tx - qx, c.dt, c.inv_dt);
            tty = tty - damp * qdiv<T>(ty - qy, c.dt, c.inv_dt);
            ttz = ttz - damp * qdiv<T>(tz - qz, c.dt, c.inv_dt);
        }

        // divergence of theta on the now level (evolution.cpp:388-389)
        T divNow = 0;
        if (DIAG || d.store_div)
            divNow = qdiv<T>(tx - txm, c.dx2, c.inv_dx2) + qdiv<T>(ty - tym, c.dy2, c.inv_dy2)
                   + qdiv<T>(tz - tzm, c.dz2, c.inv_dz2);

        if constexpr (DIAG) {
            // energy density and Gauss deviation of the now level
            // (evolution.cpp:322-334,377-427; mpi_evolution.cpp:509-532)
            const T pt0 = qdiv<T>(p0 - q0, c.dt, c.inv_dt);
            const T pt1 = qdiv<T>(p1 - q1, c.dt, c.inv_dt);
            const T px0 = qdiv<T>(p0 - cxm * p0xm + sxm * p1xm, c.dx, c.inv_dx);
            const T px1 = qdiv<T>(p1 - cxm * p1xm - sxm * p0xm, c.dx, c.inv_dx);
            const T py0 = qdiv<T>(p0 - cym * p0ym + sym * p1ym, c.dy, c.inv_dy);
            const T py1 = qdiv<T>(p1 - cym * p1ym - sym * p0ym, c.dy, c.inv_dy);
            const T pz0 = qdiv<T>(p0 - czm * p0zm + szm * p1zm, c.dz, c.inv_dz);
            const T pz1 = qdiv<T>(p1 - czm * p1zm - szm * p0zm, c.dz, c.inv_dz);
            T tdc = 0, fc = 0, gauss = 0;
            if (d.energy_form == LAT_ENERGY_MPI) {
                const T a0 = qdiv<T>(tx - qx, c.dt, c.inv_dt);
                const T a1 = qdiv<T>(ty - qy, c.dt, c.inv_dt);
                const T a2 = qdiv<T>(tz - qz, c.dt, c.inv_dt);
                tdc = (T)0.5 * (a0 * a0 + a1 * a1 + a2 * a2);
                fc = qdiv<T>(1 - cPxy, c.gxy2, c.inv_gxy2) + qdiv<T>(1 - cPxz, c.gxz2, c.inv_gxz2)
                   + qdiv<T>(1 - cPyz, c.gyz2, c.inv_gyz2);
            }
            if (c.g != 0) {
                const T divPast = reinterpret_cast<const T*>(d.divbuf)[s];
                const T divThetat = qdiv<T>(divNow - divPast, c.dt, c.inv_dt);
                gauss = qdiv<T>(divThetat, c.g, c.inv_g) - (T)c.twog * (p1 * pt0 - p0 * pt1);
                if (d.energy_form != LAT_ENERGY_MPI) {
                    const T a0 = qdiv<T>(tx - qx, c.gdtdx, c.inv_gdtdx);
                    const T a1 = qdiv<T>(ty - qy, c.gdtdy, c.inv_gdtdy);
                    const T a2 = qdiv<T>(tz - qz, c.gdtdz, c.inv_gdtdz);
                    tdc = (T)0.5 * (a0 * a0 + a1 * a1 + a2 * a2);
                    const T Fxy = qdiv<T>(1 - cPxy, c.gxy2, c.inv_gxy2);
                    const T Fxz = qdiv<T>(1 - cPxz, c.gxz2, c.inv_gxz2);
                    const T Fyz = qdiv<T>(1 - cPyz, c.gyz2, c.inv_gyz2);
                    fc = Fxy + Fxz + Fyz;
                }
            }
            const T pm = phiMagSqr - (T)c.etaSq;
            const T ed = pt0 * pt0 + pt1 * pt1 + px0 * px0 + px1 * px1 + py0 * py0 + py1 * py1 + pz0 * pz0 + pz1 * pz1
                       + tdc + fc + (T)c.quarterLambda * (pm * pm);
            if (d.energy_form == LAT_ENERGY_MPI) e_site = (double)(ed * (T)c.dx * (T)c.dy * (T)c.dz);
            else e_site = (double)((T)c.dV * ed);
            g_site = (double)(gauss < 0 ? -gauss : gauss);
        }

        if (d.store_div) reinterpret_cast<T*>(d.divbuf)[s] = divNow;

        // in-place update of the past slot (mpi_evolution.cpp:432,499-501)
        if (d.write) {
            f.past[0][s] = leapfrog<T>(p0, q0, dt2, tt0);
            f.past[1][s] = leapfrog<T>(p1, q1, dt2, tt1);
            f.past[2][s] = leapfrog<T>(tx, qx, dt2, ttx);
            f.past[3][s] = leapfrog<T>(ty, qy, dt2, tty);
            f.past[4][s] = leapfrog<T>(tz, qz, dt2, ttz);
        }
    }

    if constexpr (DIAG) block_sum2_store(e_site, g_site, d.partials);
}

template <class T>
cudaError_t launch_ah_step_t(const Geom& g, const Fields<T, 5>& f, const StepCoef& c64, const DiagOut& d, bool diag,
                             cudaStream_t st)
{
    const StepCoefT<T> c = coef_as<T>(c64);
    const dim3 grid = site_grid(g);
    const dim3 block(BZ, BY);
    if (diag) ah_step_kernel<T, true><<<grid, block, 0, st>>>(g, f, c, d);
    else ah_step_kernel<T, false><<<grid, block, 0, st>>>(g, f, c, d);
    return cudaGetLastError();
}

// Divergence of theta of one level (evolution.cpp:388-391), for a diagnostic
// step whose previous step did not store it.  Read-only.
template <class T>
__global__ void __launch_bounds__(BLOCK) divergence_kernel(const Geom g, const T* __restrict__ TX,
                                                           const T* __restrict__ TY, const T* __restrict__ TZ,
                                                           const StepCoefT<T> c, T* __restrict__ out)
{
    const int k = g.loz + (int)(blockIdx.x * BZ + threadIdx.x);
    const int j = g.loy + (int)(blockIdx.y * BY + threadIdx.y);
    const int i = g.lox + (int)blockIdx.z;
    if (k >= g.hiz || j >= g.hiy) return;
    const Nbr n = make_nbr(g, i, j, k);
    const int s = n.s;
    out[s] = qdiv<T>(TX[s] - TX[s + n.xm], c.dx2, c.inv_dx2) + qdiv<T>(TY[s] - TY[s + n.ym], c.dy2, c.inv_dy2)
           + qdiv<T>(TZ[s] - TZ[s + n.zm], c.dz2, c.inv_dz2);
}

template <class T>
cudaError_t launch_divergence_t(const Geom& g, const T* tx, const T* ty, const T* tz, const StepCoef& c, T* out,
                                cudaStream_t st)
{
    divergence_kernel<T><<<site_grid(g), dim3(BZ, BY), 0, st>>>(g, tx, ty, tz, coef_as<T>(c), out);
    return cudaGetLastError();
}

}  // namespace lat
