// Abelian-Higgs FP32 step: one fused kernel per step, tiled in (y, z) and
// marching along x.
//
// The FP32 step is meant to run at HBM speed, so the one-pass kernel's
// redundant work has to go: it evaluates every link's sin/cos and every
// plaquette sine once for each site that uses it (18 per site, as the
// reference does, mpi_evolution.cpp:418-487).  Here a CTA owns a TZ x TY tile
// of (z, y) columns and marches along x.  For each x-plane:
//   * the now-level theta and phi of the tile plus a one-site halo are staged
//     in shared memory by cp.async, two planes ahead of the compute;
//   * every site of the tile plus the low y/z halo evaluates its link data once:
//     cos/sin of theta_x,y,z and the sines of the plaquettes P_xy, P_xz, P_yz
//     (sin P_yx = -sin P_xy etc.);
//   * the update reads the link data of its y- and z-backward neighbours from
//     shared memory and of its x-backward neighbour from registers carried
//     over from the previous plane.
// HBM traffic is the algorithmic 3 accesses per value: 60 B per site.  The
// arithmetic is FP32 with fused multiply-adds and reciprocals; energy and
// Gauss sums are accumulated in FP64.
#pragma once

#include <cuda_pipeline.h>

#include "site_common.cuh"

namespace lat {

constexpr int TT_Z = 32;            // tile width along z (one warp)
constexpr int TT_Y = 8;             // tile height along y (warps per CTA)
constexpr int TT_THREADS = TT_Z * TT_Y;
constexpr int TT_HZ = TT_Z + 2;     // staged plane: tile + 1-site halo on both sides
constexpr int TT_HY = TT_Y + 2;
constexpr int TT_LZ = TT_Z + 1;     // link data: tile + low halo
constexpr int TT_LY = TT_Y + 1;
constexpr int TT_STAGES = 3;        // planes i, i+1 in use, i+2 in flight

// link-data planes kept in shared memory for the y/z neighbours
enum { LS_CY, LS_SY, LS_CZ, LS_SZ, LS_PXY, LS_PXZ, LS_PYZ, LS_N };

template <class T>
struct TiledSmem {
    T th[TT_STAGES][3][TT_HY][TT_HZ];   // theta_x,y,z of a plane
    T ph[TT_STAGES][2][TT_HY][TT_HZ];   // phi_re, phi_im of a plane
    T L[LS_N][TT_LY][TT_LZ];            // link data of the current plane
    double red[2][TT_THREADS / 32];
};

__device__ __forceinline__ int wrap_idx(int a, int n)
{
    return a < 0 ? a + n : (a >= n ? a - n : a);
}

// Issue the asynchronous copy of plane `pi` (tile + halo) into stage `b`.
template <class T>
__device__ __forceinline__ void stage_plane(TiledSmem<T>& sm, int b, const Fields<T, 5>& f, const Geom& g, int pi,
                                            int j0, int k0)
{
    const int tid = threadIdx.y * TT_Z + threadIdx.x;
    const int base = pi * g.syz;
    for (int e = tid; e < TT_HY * TT_HZ; e += TT_THREADS) {
        const int hy = e / TT_HZ, hz = e - hy * TT_HZ;
        const int j = wrap_idx(j0 - 1 + hy, g.ny), k = wrap_idx(k0 - 1 + hz, g.nz);
        const int s = base + j * g.nz + k;
        __pipeline_memcpy_async(&sm.th[b][0][hy][hz], f.now[2] + s, sizeof(T));
        __pipeline_memcpy_async(&sm.th[b][1][hy][hz], f.now[3] + s, sizeof(T));
        __pipeline_memcpy_async(&sm.th[b][2][hy][hz], f.now[4] + s, sizeof(T));
        __pipeline_memcpy_async(&sm.ph[b][0][hy][hz], f.now[0] + s, sizeof(T));
        __pipeline_memcpy_async(&sm.ph[b][1][hy][hz], f.now[1] + s, sizeof(T));
    }
    __pipeline_commit();
}

template <class T, bool DIAG>
__global__ void __launch_bounds__(TT_THREADS, 2)
ah_tiled_kernel(const Geom g, const Fields<T, 5> f, const StepCoefT<T> c, const DiagOut d, const int chunk)
{
    using TR = Trig<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TiledSmem<T>& sm = *reinterpret_cast<TiledSmem<T>*>(smem_raw);

    const int tz = threadIdx.x, ty = threadIdx.y;
    const int k0 = g.lo + (int)blockIdx.x * TT_Z;
    const int j0 = g.lo + (int)blockIdx.y * TT_Y;
    const int ib = g.lo + (int)blockIdx.z * chunk;
    const int ie = min(ib + chunk, g.hix);
    const int k = k0 + tz, j = j0 + ty;
    const bool active = (k < g.hiz) && (j < g.hiy);
    const int kk = wrap_idx(k, g.nz), jj = wrap_idx(j, g.ny);   // in-range copy for loads
    const int hy = ty + 1, hz = tz + 1;                          // own position in the staged plane

    // a second link-data position for the low halo: row j0-1 (33 sites) and
    // column k0-1 (8 sites)
    const int tid = ty * TT_Z + tz;
    int ly2 = -1, lz2 = -1;
    if (tid < TT_LZ) { ly2 = 0; lz2 = tid; }
    else if (tid < TT_LZ + TT_Y) { ly2 = tid - TT_LZ + 1; lz2 = 0; }

    // ---- prologue: plane ib-1 (own column) and the first two staged planes
    const int im = wrap_idx(ib - 1, g.nx);
    T cxm, sxm, sPxy_xm, sPxz_xm, txm_prev, p0m, p1m;
    {
        const int s = (im * g.ny + jj) * g.nz + kk;
        const int sxp = (wrap_idx(ib, g.nx) * g.ny + jj) * g.nz + kk;
        const int syp = (im * g.ny + wrap_idx(jj + 1, g.ny)) * g.nz + kk;
        const int szp = (im * g.ny + jj) * g.nz + wrap_idx(kk + 1, g.nz);
        const T tx = f.now[2][s], ty_ = f.now[3][s], tz_ = f.now[4][s];
        TR::sincos(tx, &sxm, &cxm);
        sPxy_xm = TR::sin(tx + f.now[3][sxp] - f.now[2][syp] - ty_);
        sPxz_xm = TR::sin(tx + f.now[4][sxp] - f.now[2][szp] - tz_);
        txm_prev = tx;
        p0m = f.now[0][s];
        p1m = f.now[1][s];
    }
    int cur = 0;
    stage_plane<T>(sm, 0, f, g, wrap_idx(ib, g.nx), j0, k0);
    stage_plane<T>(sm, 1, f, g, wrap_idx(ib + 1, g.nx), j0, k0);

    double e_acc = 0.0, g_acc = 0.0;

    for (int i = ib; i < ie; ++i) {
        const int nxt = cur == 2 ? 0 : cur + 1;
        const int nn = nxt == 2 ? 0 : nxt + 1;
        // plane i+2 into the free stage while i and i+1 are used
        if (i + 1 < ie) stage_plane<T>(sm, nn, f, g, wrap_idx(i + 2, g.nx), j0, k0);
        else __pipeline_commit();
        __pipeline_wait_prior(1);  // planes i and i+1 have landed
        __syncthreads();

        // ---- link data of the tile site and, for some threads, a halo site
        auto links = [&](int ly, int lz, T& cyv, T& syv, T& czv, T& szv, T& sxy, T& sxz, T& syz, T* cxo, T* sxo,
                         T* cpo) {
            const T tx = sm.th[cur][0][ly][lz], tyv = sm.th[cur][1][ly][lz], tzv = sm.th[cur][2][ly][lz];
            const T tyxp = sm.th[nxt][1][ly][lz], tzxp = sm.th[nxt][2][ly][lz];
            const T txyp = sm.th[cur][0][ly + 1][lz], tzyp = sm.th[cur][2][ly + 1][lz];
            const T txzp = sm.th[cur][0][ly][lz + 1], tyzp = sm.th[cur][1][ly][lz + 1];
            TR::sincos(tyv, &syv, &cyv);
            TR::sincos(tzv, &szv, &czv);
            const T Pxy = tx + tyxp - txyp - tyv;
            const T Pxz = tx + tzxp - txzp - tzv;
            const T Pyz = tyv + tzyp - tyzp - tzv;
            if (cpo) {
                TR::sincos(Pxy, &sxy, &cpo[0]);
                TR::sincos(Pxz, &sxz, &cpo[1]);
                TR::sincos(Pyz, &syz, &cpo[2]);
            } else {
                sxy = TR::sin(Pxy);
                sxz = TR::sin(Pxz);
                syz = TR::sin(Pyz);
            }
            if (cxo) TR::sincos(tx, sxo, cxo);
        };
        T cx, sx, cy, sy, cz, sz, sPxy, sPxz, sPyz, cP[3];
        links(hy, hz, cy, sy, cz, sz, sPxy, sPxz, sPyz, &cx, &sx, DIAG ? cP : nullptr);
        sm.L[LS_CY][hy][hz] = cy;
        sm.L[LS_SY][hy][hz] = sy;
        sm.L[LS_CZ][hy][hz] = cz;
        sm.L[LS_SZ][hy][hz] = sz;
        sm.L[LS_PXY][hy][hz] = sPxy;
        sm.L[LS_PXZ][hy][hz] = sPxz;
        sm.L[LS_PYZ][hy][hz] = sPyz;
        if (ly2 >= 0) {
            T a0, a1, a2, a3, a4, a5, a6;
            links(ly2, lz2, a0, a1, a2, a3, a4, a5, a6, nullptr, nullptr, nullptr);
            sm.L[LS_CY][ly2][lz2] = a0;
            sm.L[LS_SY][ly2][lz2] = a1;
            sm.L[LS_CZ][ly2][lz2] = a2;
            sm.L[LS_SZ][ly2][lz2] = a3;
            sm.L[LS_PXY][ly2][lz2] = a4;
            sm.L[LS_PXZ][ly2][lz2] = a5;
            sm.L[LS_PYZ][ly2][lz2] = a6;
        }
        __syncthreads();

        const T p0 = sm.ph[cur][0][hy][hz], p1 = sm.ph[cur][1][hy][hz];
        const T tx = sm.th[cur][0][hy][hz], tyv = sm.th[cur][1][hy][hz], tzv = sm.th[cur][2][hy][hz];
        if (active) {
            const int s = (i * g.ny + j) * g.nz + k;
            const T q0 = f.past[0][s], q1 = f.past[1][s];
            const T qx = f.past[2][s], qy = f.past[3][s], qz = f.past[4][s];
            const T p0xp = sm.ph[nxt][0][hy][hz], p1xp = sm.ph[nxt][1][hy][hz];
            const T p0yp = sm.ph[cur][0][hy + 1][hz], p1yp = sm.ph[cur][1][hy + 1][hz];
            const T p0ym = sm.ph[cur][0][hy - 1][hz], p1ym = sm.ph[cur][1][hy - 1][hz];
            const T p0zp = sm.ph[cur][0][hy][hz + 1], p1zp = sm.ph[cur][1][hy][hz + 1];
            const T p0zm = sm.ph[cur][0][hy][hz - 1], p1zm = sm.ph[cur][1][hy][hz - 1];
            const T cym = sm.L[LS_CY][hy - 1][hz], sym = sm.L[LS_SY][hy - 1][hz];
            const T czm = sm.L[LS_CZ][hy][hz - 1], szm = sm.L[LS_SZ][hy][hz - 1];
            const T sPxy_ym = sm.L[LS_PXY][hy - 1][hz], sPyz_ym = sm.L[LS_PYZ][hy - 1][hz];
            const T sPxz_zm = sm.L[LS_PXZ][hy][hz - 1], sPyz_zm = sm.L[LS_PYZ][hy][hz - 1];

            const T phiMagSqr = p0 * p0 + p1 * p1;
            const T pot = c.halfLambda * (phiMagSqr - c.etaSq);
            T tt0 = (cx * p0xp + sx * p1xp - 2 * p0 + cxm * p0m - sxm * p1m) * c.inv_dx2
                  + (cy * p0yp + sy * p1yp - 2 * p0 + cym * p0ym - sym * p1ym) * c.inv_dy2
                  + (cz * p0zp + sz * p1zp - 2 * p0 + czm * p0zm - szm * p1zm) * c.inv_dz2 - pot * p0;
            T tt1 = (cx * p1xp - sx * p0xp - 2 * p1 + cxm * p1m + sxm * p0m) * c.inv_dx2
                  + (cy * p1yp - sy * p0yp - 2 * p1 + cym * p1ym + sym * p0ym) * c.inv_dy2
                  + (cz * p1zp - sz * p0zp - 2 * p1 + czm * p1zm + szm * p0zm) * c.inv_dz2 - pot * p1;
            if (c.fric != 0) {
                tt0 -= c.fric * (p0 - q0) * c.inv_dt;
                tt1 -= c.fric * (p1 - q1) * c.inv_dt;
            }
            const T curx = cx * (p1 * p0xp - p0 * p1xp) + sx * (p0 * p0xp + p1 * p1xp);
            const T cury = cy * (p1 * p0yp - p0 * p1yp) + sy * (p0 * p0yp + p1 * p1yp);
            const T curz = cz * (p1 * p0zp - p0 * p1zp) + sz * (p0 * p0zp + p1 * p1zp);
            // lattice curl with sin(P_yx) = -sin(P_xy), sin(P_zx) = -sin(P_xz), sin(P_zy) = -sin(P_yz)
            const T Fxy_y = (sPxy - sPxy_ym) * c.inv_dy2;
            const T Fxz_z = (sPxz - sPxz_zm) * c.inv_dz2;
            const T Fyx_x = (sPxy_xm - sPxy) * c.inv_dx2;
            const T Fyz_z = (sPyz - sPyz_zm) * c.inv_dz2;
            const T Fzx_x = (sPxz_xm - sPxz) * c.inv_dx2;
            const T Fzy_y = (sPyz_ym - sPyz) * c.inv_dy2;
            T ttx = c.m2gg * curx - Fxy_y - Fxz_z;
            T tty = c.m2gg * cury - Fyx_x - Fyz_z;
            T ttz = c.m2gg * curz - Fzx_x - Fzy_y;
            if (c.damp != 0) {
                ttx -= c.damp * (tx - qx) * c.inv_dt;
                tty -= c.damp * (tyv - qy) * c.inv_dt;
                ttz -= c.damp * (tzv - qz) * c.inv_dt;
            }
            T divNow = 0;
            if (DIAG || d.store_div) {
                const T tym = sm.th[cur][1][hy - 1][hz], tzm = sm.th[cur][2][hy][hz - 1];
                divNow = (tx - txm_prev) * c.inv_dx2 + (tyv - tym) * c.inv_dy2 + (tzv - tzm) * c.inv_dz2;
            }
            if constexpr (DIAG) {
                const T pt0 = (p0 - q0) * c.inv_dt, pt1 = (p1 - q1) * c.inv_dt;
                const T px0 = (p0 - cxm * p0m + sxm * p1m) * c.inv_dx, px1 = (p1 - cxm * p1m - sxm * p0m) * c.inv_dx;
                const T py0 = (p0 - cym * p0ym + sym * p1ym) * c.inv_dy, py1 = (p1 - cym * p1ym - sym * p0ym) * c.inv_dy;
                const T pz0 = (p0 - czm * p0zm + szm * p1zm) * c.inv_dz, pz1 = (p1 - czm * p1zm - szm * p0zm) * c.inv_dz;
                T tdc = 0, fc = 0, gauss = 0;
                if (d.energy_form == LAT_ENERGY_MPI) {
                    const T a0 = (tx - qx) * c.inv_dt, a1 = (tyv - qy) * c.inv_dt, a2 = (tzv - qz) * c.inv_dt;
                    tdc = (T)0.5 * (a0 * a0 + a1 * a1 + a2 * a2);
                    fc = (1 - cP[0]) * c.inv_gxy2 + (1 - cP[1]) * c.inv_gxz2 + (1 - cP[2]) * c.inv_gyz2;
                }
                if (c.g != 0) {
                    const T divPast = reinterpret_cast<const T*>(d.divbuf)[s];
                    gauss = (divNow - divPast) * c.inv_dt * c.inv_g - c.twog * (p1 * pt0 - p0 * pt1);
                    if (d.energy_form != LAT_ENERGY_MPI) {
                        const T a0 = (tx - qx) * c.inv_gdtdx, a1 = (tyv - qy) * c.inv_gdtdy, a2 = (tzv - qz) * c.inv_gdtdz;
                        tdc = (T)0.5 * (a0 * a0 + a1 * a1 + a2 * a2);
                        fc = (1 - cP[0]) * c.inv_gxy2 + (1 - cP[1]) * c.inv_gxz2 + (1 - cP[2]) * c.inv_gyz2;
                    }
                }
                const T pm = phiMagSqr - c.etaSq;
                const T ed = pt0 * pt0 + pt1 * pt1 + px0 * px0 + px1 * px1 + py0 * py0 + py1 * py1 + pz0 * pz0
                           + pz1 * pz1 + tdc + fc + c.quarterLambda * (pm * pm);
                e_acc += (double)(d.energy_form == LAT_ENERGY_MPI ? ed * c.dx * c.dy * c.dz : c.dV * ed);
                g_acc += (double)fabs(gauss);
            }
            if (d.store_div) reinterpret_cast<T*>(d.divbuf)[s] = divNow;
            if (d.write) {
                f.past[0][s] = leapfrog<T>(p0, q0, c.dt2, tt0);
                f.past[1][s] = leapfrog<T>(p1, q1, c.dt2, tt1);
                f.past[2][s] = leapfrog<T>(tx, qx, c.dt2, ttx);
                f.past[3][s] = leapfrog<T>(tyv, qy, c.dt2, tty);
                f.past[4][s] = leapfrog<T>(tzv, qz, c.dt2, ttz);
            }
        }
        // carry the x-backward data of the next plane
        cxm = cx;
        sxm = sx;
        sPxy_xm = sPxy;
        sPxz_xm = sPxz;
        txm_prev = tx;
        p0m = p0;
        p1m = p1;
        cur = nxt;
        __syncthreads();  // stage `cur` of this plane and L are reused next
    }
    __pipeline_wait_prior(0);

    if constexpr (DIAG) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            e_acc += __shfl_down_sync(0xffffffffu, e_acc, o);
            g_acc += __shfl_down_sync(0xffffffffu, g_acc, o);
        }
        if (tz == 0) {
            sm.red[0][ty] = e_acc;
            sm.red[1][ty] = g_acc;
        }
        __syncthreads();
        if (tid == 0) {
            double a = 0, b = 0;
            for (int w = 0; w < TT_Y; ++w) {
                a += sm.red[0][w];
                b += sm.red[1][w];
            }
            const int blk = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
            d.partials[2 * blk] = a;
            d.partials[2 * blk + 1] = b;
        }
    }
}

inline dim3 tiled_grid(const Geom& g, int chunk)
{
    return dim3((unsigned)((g.hiz - g.lo + TT_Z - 1) / TT_Z), (unsigned)((g.hiy - g.lo + TT_Y - 1) / TT_Y),
                (unsigned)((g.hix - g.lo + chunk - 1) / chunk));
}

template <class T>
cudaError_t launch_ah_tiled_t(const Geom& g, const Fields<T, 5>& f, const StepCoef& c64, const DiagOut& d, bool diag,
                              int chunk, cudaStream_t st)
{
    const StepCoefT<T> c = coef_as<T>(c64);
    const size_t smem = sizeof(TiledSmem<T>);
    if (smem > 48 * 1024) {  // opt in above the default dynamic shared-memory limit
        cudaFuncSetAttribute(ah_tiled_kernel<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(ah_tiled_kernel<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    }
    const dim3 grid = tiled_grid(g, chunk);
    const dim3 block(TT_Z, TT_Y);
    if (diag) ah_tiled_kernel<T, true><<<grid, block, smem, st>>>(g, f, c, d, chunk);
    else ah_tiled_kernel<T, false><<<grid, block, smem, st>>>(g, f, c, d, chunk);
    return cudaGetLastError();
}

}  // namespace lat
