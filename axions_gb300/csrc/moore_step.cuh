// Moore-model leapfrog step: two complex scalars phi1, phi2 with charges
// q1, q2 on one compact U(1) gauge field; one fused stencil kernel per step.
//
// Replaces moore_mpi_evolution.cpp:405-550 (periodic, friction, current
// without charges) and mooreEvol.cpp:187-337 + 672-692 (fixed boundaries,
// q-weighted current); diagnostics follow mooreEvol.cpp:339-391 or
// moore_mpi_evolution.cpp:558-588.  Same in-place scheme and operation order
// as the Abelian-Higgs kernel.
#pragma once

#include "site_common.cuh"

namespace lat {

template <class T, bool DIAG>
__global__ void __launch_bounds__(BLOCK) moore_step_kernel(const Geom g, const Fields<T, 7> f, const StepCoefT<T> c,
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
        const int pp[3] = {n.xp, n.yp, n.zp};
        const int mm[3] = {n.xm, n.ym, n.zm};
        const T d2[3] = {c.dx2, c.dy2, c.dz2};
        const T id2[3] = {c.inv_dx2, c.inv_dy2, c.inv_dz2};
        const T dd[3] = {c.dx, c.dy, c.dz};
        const T idd[3] = {c.inv_dx, c.inv_dy, c.inv_dz};
        const T q[2] = {(T)c.q1, (T)c.q2};
        const T dt2 = (T)c.dt2;
        const T* __restrict__ TH[3] = {f.now[4], f.now[5], f.now[6]};

        // scalars: v[f][comp], neighbours vp/vm[f][comp][axis]
        T v[2][2], vp[2][2][3], vm[2][2][3], qv[2][2];
#pragma unroll
        for (int fi = 0; fi < 2; ++fi)
#pragma unroll
            for (int comp = 0; comp < 2; ++comp) {
                const T* __restrict__ P = f.now[2 * fi + comp];
                v[fi][comp] = P[s];
                qv[fi][comp] = f.past[2 * fi + comp][s];
#pragma unroll
                for (int m = 0; m < 3; ++m) {
                    vp[fi][comp][m] = P[s + pp[m]];
                    vm[fi][comp][m] = P[s + mm[m]];
                }
            }
        T th[3], thm[3], qth[3];
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            th[m] = TH[m][s];
            thm[m] = TH[m][s + mm[m]];
            qth[m] = f.past[4 + m][s];
        }
        // link factors cos/sin(q_f * theta) at the site and the backward neighbour
        T cs[2][3], sn[2][3], csm[2][3], snm[2][3];
#pragma unroll
        for (int fi = 0; fi < 2; ++fi)
#pragma unroll
            for (int m = 0; m < 3; ++m) {
                TR::sincos(q[fi] * th[m], &sn[fi][m], &cs[fi][m]);
                TR::sincos(q[fi] * thm[m], &snm[fi][m], &csm[fi][m]);
            }

        T mag[2];
#pragma unroll
        for (int fi = 0; fi < 2; ++fi) mag[fi] = v[fi][0] * v[fi][0] + v[fi][1] * v[fi][1];
        const T pot[2] = {(T)c.halfLambda * (mag[0] - (T)c.etaSq) + (T)c.halfLambda12 * (mag[1] - (T)c.eta2Sq),
                          (T)c.halfLambda2 * (mag[1] - (T)c.eta2Sq) + (T)c.halfLambda12 * (mag[0] - (T)c.etaSq)};

        T acc[2][2];
#pragma unroll
        for (int fi = 0; fi < 2; ++fi) {
#pragma unroll
            for (int comp = 0; comp < 2; ++comp) {
                const int oc = 1 - comp;
                T lap[3];
#pragma unroll
                for (int m = 0; m < 3; ++m) {
                    // comp 0: c = +1, comp 1: c = -1 (moore_mpi_evolution.cpp:445-465)
                    T num;
                    if (comp == 0)
                        num = cs[fi][m] * vp[fi][0][m] + sn[fi][m] * vp[fi][1][m] - 2 * v[fi][0]
                            + csm[fi][m] * vm[fi][0][m] - snm[fi][m] * vm[fi][1][m];
                    else
                        num = cs[fi][m] * vp[fi][1][m] - sn[fi][m] * vp[fi][0][m] - 2 * v[fi][1]
                            + csm[fi][m] * vm[fi][1][m] + snm[fi][m] * vm[fi][0][m];
                    lap[m] = qdiv<T>(num, d2[m], id2[m]);
                    (void)oc;
                }
                T tt = lap[0] + lap[1] + lap[2] - pot[fi] * v[fi][comp];
                if (c.fric != 0) tt = tt - (T)c.fric * qdiv<T>(v[fi][comp] - qv[fi][comp], c.dt, c.inv_dt);
                acc[fi][comp] = tt;
            }
        }

        // gauge current (moore_mpi_evolution.cpp:498-515 / mooreEvol.cpp:295-312)
        T cur[3];
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            T cf[2];
#pragma unroll
            for (int fi = 0; fi < 2; ++fi) {
                const T val = cs[fi][m] * (v[fi][1] * vp[fi][0][m] - v[fi][0] * vp[fi][1][m])
                            + sn[fi][m] * (v[fi][0] * vp[fi][0][m] + v[fi][1] * vp[fi][1][m]);
                cf[fi] = d.charge_current ? q[fi] * val : val;
            }
            cur[m] = cf[0] + cf[1];
        }

        // plaquettes (identical to the Abelian-Higgs kernel)
        const T tx = th[0], ty = th[1], tz = th[2];
        const T txm = thm[0], tym = thm[1], tzm = thm[2];
        const T* __restrict__ TX = TH[0];
        const T* __restrict__ TY = TH[1];
        const T* __restrict__ TZ = TH[2];
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
        T tt[3];
        tt[0] = m2gg * cur[0] - Fxy_y - Fxz_z;
        tt[1] = m2gg * cur[1] - Fyx_x - Fyz_z;
        tt[2] = m2gg * cur[2] - Fzx_x - Fzy_y;
        if (c.damp != 0) {
#pragma unroll
            for (int m = 0; m < 3; ++m) tt[m] = tt[m] - (T)c.damp * qdiv<T>(th[m] - qth[m], c.dt, c.inv_dt);
        }

        T divNow = 0;
        if (DIAG || d.store_div)
            divNow = qdiv<T>(tx - txm, c.dx2, c.inv_dx2) + qdiv<T>(ty - tym, c.dy2, c.inv_dy2)
                   + qdiv<T>(tz - tzm, c.dz2, c.inv_dz2);

        if constexpr (DIAG) {
            T pt[2][2], pd[2][3][2];
#pragma unroll
            for (int fi = 0; fi < 2; ++fi) {
                pt[fi][0] = qdiv<T>(v[fi][0] - qv[fi][0], c.dt, c.inv_dt);
                pt[fi][1] = qdiv<T>(v[fi][1] - qv[fi][1], c.dt, c.inv_dt);
#pragma unroll
                for (int m = 0; m < 3; ++m) {
                    pd[fi][m][0] = qdiv<T>(v[fi][0] - csm[fi][m] * vm[fi][0][m] + snm[fi][m] * vm[fi][1][m], dd[m], idd[m]);
                    pd[fi][m][1] = qdiv<T>(v[fi][1] - csm[fi][m] * vm[fi][1][m] - snm[fi][m] * vm[fi][0][m], dd[m], idd[m]);
                }
            }
            T tdc = 0, fc = 0, gauss = 0;
            if (d.energy_form == LAT_ENERGY_MPI) {
                const T a0 = qdiv<T>(tx - qth[0], c.dt, c.inv_dt);
                const T a1 = qdiv<T>(ty - qth[1], c.dt, c.inv_dt);
                const T a2 = qdiv<T>(tz - qth[2], c.dt, c.inv_dt);
                tdc = (T)0.5 * (a0 * a0 + a1 * a1 + a2 * a2);
                fc = qdiv<T>(1 - cPxy, c.gxy2, c.inv_gxy2) + qdiv<T>(1 - cPxz, c.gxz2, c.inv_gxz2)
                   + qdiv<T>(1 - cPyz, c.gyz2, c.inv_gyz2);
            }
            if (c.g != 0) {
                const T divPast = reinterpret_cast<const T*>(d.divbuf)[s];
                const T divThetat = qdiv<T>(divNow - divPast, c.dt, c.inv_dt);
                gauss = qdiv<T>(divThetat, c.g, c.inv_g)
                      - (T)c.twog * (q[0] * (v[0][1] * pt[0][0] - v[0][0] * pt[0][1])
                                    + q[1] * (v[1][1] * pt[1][0] - v[1][0] * pt[1][1]));
                if (d.energy_form != LAT_ENERGY_MPI) {
                    const T a0 = qdiv<T>(tx - qth[0], c.gdtdx, c.inv_gdtdx);
                    const T a1 = qdiv<T>(ty - qth[1], c.gdtdy, c.inv_gdtdy);
                    const T a2 = qdiv<T>(tz - qth[2], c.gdtdz, c.inv_gdtdz);
                    tdc = (T)0.5 * (a0 * a0 + a1 * a1 + a2 * a2);
                    const T Fxy = qdiv<T>(1 - cPxy, c.gxy2, c.inv_gxy2);
                    const T Fxz = qdiv<T>(1 - cPxz, c.gxz2, c.inv_gxz2);
                    const T Fyz = qdiv<T>(1 - cPyz, c.gyz2, c.inv_gyz2);
                    fc = Fxy + Fxz + Fyz;
                }
            }
            const T m1 = mag[0] - (T)c.etaSq, m2 = mag[1] - (T)c.eta2Sq;
            const T ed = pt[0][0] * pt[0][0] + pt[0][1] * pt[0][1] + pd[0][0][0] * pd[0][0][0] + pd[0][0][1] * pd[0][0][1]
                       + pd[0][1][0] * pd[0][1][0] + pd[0][1][1] * pd[0][1][1] + pd[0][2][0] * pd[0][2][0]
                       + pd[0][2][1] * pd[0][2][1] + pt[1][0] * pt[1][0] + pt[1][1] * pt[1][1]
                       + pd[1][0][0] * pd[1][0][0] + pd[1][0][1] * pd[1][0][1] + pd[1][1][0] * pd[1][1][0]
                       + pd[1][1][1] * pd[1][1][1] + pd[1][2][0] * pd[1][2][0] + pd[1][2][1] * pd[1][2][1] + tdc + fc
                       + (T)c.quarterLambda * (m1 * m1) + (T)c.quarterLambda2 * (m2 * m2) + (T)c.halfLambda12e * m1 * m2;
            if (d.energy_form == LAT_ENERGY_MPI) e_site = (double)(ed * (T)c.dx * (T)c.dy * (T)c.dz);
            else e_site = (double)((T)c.dV * ed);
            g_site = (double)(gauss < 0 ? -gauss : gauss);
        }

        if (d.store_div) reinterpret_cast<T*>(d.divbuf)[s] = divNow;

        if (d.write) {
#pragma unroll
            for (int fi = 0; fi < 2; ++fi)
#pragma unroll
                for (int comp = 0; comp < 2; ++comp)
                    f.past[2 * fi + comp][s] = leapfrog<T>(v[fi][comp], qv[fi][comp], dt2, acc[fi][comp]);
#pragma unroll
            for (int m = 0; m < 3; ++m) f.past[4 + m][s] = leapfrog<T>(th[m], qth[m], dt2, tt[m]);
        }
    }

    if constexpr (DIAG) block_sum2_store(e_site, g_site, d.partials);
}

template <class T>
cudaError_t launch_moore_step_t(const Geom& g, const Fields<T, 7>& f, const StepCoef& c64, const DiagOut& d, bool diag,
                                cudaStream_t st)
{
    const StepCoefT<T> c = coef_as<T>(c64);
    const dim3 grid = site_grid(g);
    const dim3 block(BZ, BY);
    if (diag) moore_step_kernel<T, true><<<grid, block, 0, st>>>(g, f, c, d);
    else moore_step_kernel<T, false><<<grid, block, 0, st>>>(g, f, c, d);
    return cudaGetLastError();
}

}  // namespace lat
