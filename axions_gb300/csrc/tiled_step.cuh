// FP32 lattice step for NS complex scalars on one compact U(1) gauge field:
// one fused kernel per step, tiled in (y, z) and marching along x.
//   NS = 1: Abelian-Higgs (mpi_evolution.cpp:381-501, charge 1);
//   NS = 2: Moore model, charges q1, q2 (moore_mpi_evolution.cpp:405-550,
//           mooreEvol.cpp:191-337).
//
// The FP32 step is meant to run at HBM speed, so the one-pass kernel's
// redundant work has to go: the reference evaluates every link factor and
// every plaquette sine once for each site that uses it.  Here a CTA owns a
// TZ x TY tile of (z, y) columns and marches along x.  For each x-plane:
//   * the now-level theta and phi of the tile plus a one-site halo are staged
//     in shared memory by cp.async, two planes ahead of the compute, in
//     16-byte row chunks where the layout allows (periodic z, nz % 4 == 0);
//   * every site of the tile plus its low y/z halo evaluates its link data
//     once: e^{i q_f theta_mu} for each scalar f and direction mu, and the
//     sines of the plaquettes P_xy, P_xz, P_yz (sin P_yx = -sin P_xy etc.);
//   * the update reads the link data of its y- and z-backward neighbours from
//     shared memory and of its x-backward neighbour from registers carried
//     over from the previous plane.
// HBM traffic is the algorithmic 3 accesses per value (60 B/site AH, 84 B/site
// Moore).  The arithmetic is FP32 with fused multiply-adds and reciprocals;
// energy and Gauss sums are accumulated in FP64.
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
constexpr int TT_PZ = 40;           // staged row pitch (elements): 160 B, rows start on 16-byte boundaries
constexpr int TT_C0 = 3;            // column of staged position hz = 0 (z = k0 - 1); z = k0 is column 4
constexpr int TT_NQ = TT_PZ / 4;    // 16-byte chunks of a staged row

// link data kept in shared memory for the y/z neighbours:
// per scalar f: cos/sin(q_f theta_y), cos/sin(q_f theta_z); then sin P_xy, P_xz, P_yz
template <int NS>
struct LinkIdx {
    static constexpr __host__ __device__ int cy(int f) { return 4 * f; }
    static constexpr __host__ __device__ int sy(int f) { return 4 * f + 1; }
    static constexpr __host__ __device__ int cz(int f) { return 4 * f + 2; }
    static constexpr __host__ __device__ int sz(int f) { return 4 * f + 3; }
    static constexpr int pxy = 4 * NS, pxz = 4 * NS + 1, pyz = 4 * NS + 2, count = 4 * NS + 3;
};

template <class T, int NS>
struct TiledSmem {
    T th[TT_STAGES][3][TT_HY][TT_PZ];       // theta_x,y,z of a plane; position (hy, hz) at [hy][hz + TT_C0]
    T ph[TT_STAGES][2 * NS][TT_HY][TT_PZ];  // scalar components of a plane
    T L[LinkIdx<NS>::count][TT_LY][TT_LZ];  // link data of the current plane
    double red[2][TT_THREADS / 32];
};

// Charges of the scalars: qpow[f] != 0 means q_f is that small integer and
// e^{i q theta} is formed as a power of e^{i theta}; otherwise sincos(q*theta).
template <class T>
struct Charges {
    T q[2];
    int qpow[2];
    int charge_current;  // Moore: q-weighted current (mooreEvol.cpp) or not
};

__device__ __forceinline__ int wrap_idx(int a, int n)
{
    return a < 0 ? a + n : (a >= n ? a - n : a);
}

// e^{i q theta} from e^{i theta} = (c, s): repeated complex multiplication.
template <class T>
__device__ __forceinline__ void cpow(T c, T s, int q, T& cq, T& sq)
{
    T rc = c, rs = s;
    const int n = q < 0 ? -q : q;
    for (int m = 1; m < n; ++m) {
        const T t = rc * c - rs * s;
        rs = rc * s + rs * c;
        rc = t;
    }
    cq = rc;
    sq = q < 0 ? -rs : rs;
}

template <class T>
__device__ __forceinline__ void charged(T theta, T c1, T s1, const Charges<T>& ch, int f, T& cq, T& sq)
{
    if (ch.qpow[f] == 1) {
        cq = c1;
        sq = s1;
    } else if (ch.qpow[f] != 0) {
        cpow<T>(c1, s1, ch.qpow[f], cq, sq);
    } else {
        Trig<T>::sincos(ch.q[f] * theta, &sq, &cq);
    }
}

// Issue the asynchronous copy of plane `pi` (tile + halo) into stage `b`,
// one element per copy.  The staged positions are spread evenly over the
// CTA's threads (no warp copies more than two), so no warp arrives late at
// the barrier.  Only the positions the tile's in-range sites use are copied:
// rows j0-1 .. j0+wy and columns k0-1 .. k0+wz (wy, wz the in-range rows and
// columns of the tile), whose indices wrap at most once.
template <class T, int NS>
__device__ __forceinline__ void stage_plane(TiledSmem<T, NS>& sm, int b, const Fields<T, 2 * NS + 3>& f, const Geom& g,
                                            int pi, int j0, int k0, int wy, int wz)
{
    const int tid = threadIdx.y * TT_Z + threadIdx.x;
    const int base = pi * g.syz;
    for (int q = tid; q < TT_HY * TT_HZ; q += TT_THREADS) {
        const int hy = q / TT_HZ, hz = q - hy * TT_HZ;
        if (hy > wy + 1 || hz > wz + 1) continue;
        const int s = base + wrap_idx(j0 - 1 + hy, g.ny) * g.nz + wrap_idx(k0 - 1 + hz, g.nz);
#pragma unroll
        for (int m = 0; m < 3; ++m) __pipeline_memcpy_async(&sm.th[b][m][hy][hz + TT_C0], f.now[2 * NS + m] + s, sizeof(T));
#pragma unroll
        for (int c = 0; c < 2 * NS; ++c) __pipeline_memcpy_async(&sm.ph[b][c][hy][hz + TT_C0], f.now[c] + s, sizeof(T));
    }
    __pipeline_commit();
}

// 16-byte staging (FP32, periodic z, nz a multiple of 4, 16-byte aligned
// fields): a staged row is TT_NQ chunks of 4 elements, chunk cq holding
// z = k0-4+4cq .. k0-1+4cq, which wrap as one piece because nz and the chunk
// start are multiples of 4.  Threads 64..163 (warps 2-5; warps 0 and 1 carry
// the halo link data) own one (row, chunk) pair each and copy it for every
// component.  vec_plan() gives a thread's plane-independent source offset and
// its destination in a staged component, or dst = -1.
struct VecPlan {
    int off;  // row * nz + z within a plane
    int dst;  // hy * TT_PZ + 4 * cq, or -1
};

__device__ __forceinline__ VecPlan vec_plan(const Geom& g, int j0, int k0, int wy, int wz)
{
    VecPlan vp{0, -1};
    const int p = threadIdx.y * TT_Z + threadIdx.x - 2 * 32;
    if (p >= 0 && p < TT_HY * TT_NQ) {
        const int hy = p / TT_NQ, cq = p - hy * TT_NQ;
        // rows j0-1 .. j0+wy; columns k0-1 .. k0+wz are chunks 0 .. 1 + wz/4
        if (hy <= wy + 1 && cq <= 1 + (wz >> 2)) {
            vp.off = wrap_idx(j0 - 1 + hy, g.ny) * g.nz + wrap_idx(k0 - 4 + 4 * cq, g.nz);
            vp.dst = hy * TT_PZ + 4 * cq;
        }
    }
    return vp;
}

template <class T, int NS>
__device__ __forceinline__ void stage_plane_vec(TiledSmem<T, NS>& sm, int b, const Fields<T, 2 * NS + 3>& f,
                                                const Geom& g, int pi, const VecPlan& vp)
{
    static_assert(sizeof(T) == 4, "16-byte staging is for FP32 fields");
    if (vp.dst >= 0) {
        const int s = pi * g.syz + vp.off;
        T* th = &sm.th[b][0][0][0] + vp.dst;
        T* ph = &sm.ph[b][0][0][0] + vp.dst;
#pragma unroll
        for (int m = 0; m < 3; ++m) __pipeline_memcpy_async(th + m * TT_HY * TT_PZ, f.now[2 * NS + m] + s, 16);
#pragma unroll
        for (int c = 0; c < 2 * NS; ++c) __pipeline_memcpy_async(ph + c * TT_HY * TT_PZ, f.now[c] + s, 16);
    }
    __pipeline_commit();
}

// Whether the tiled step may stage by 16-byte copies: FP32 fields, periodic z
// with nz a multiple of 4 (rows and chunk starts on 16-byte boundaries) and
// every field pointer 16-byte aligned.
template <class T, int NC>
inline bool tiled_vec_ok(const Geom& g, const Fields<T, NC>& f)
{
    if (sizeof(T) != 4 || g.loz != 0 || g.hiz != g.nz || (g.nz & 3) != 0) return false;
    for (int c = 0; c < NC; ++c)
        if ((reinterpret_cast<uintptr_t>(f.now[c]) & 15) != 0) return false;
    return true;
}

// One tile: columns (bx*TZ.., by*TY..) of the evolved region, x-planes
// [bz*chunk, bz*chunk + chunk).  Called by every thread of the CTA.  With DIAG
// the CTA's energy and |G| sums are written to part[0], part[1].  `vec`
// selects the 16-byte staging (only where tiled_vec_ok holds); both stagings
// fill the same shared-memory positions, so the results are bitwise equal.
template <class T, int NS, bool DIAG>
__device__ __forceinline__ void tiled_tile(TiledSmem<T, NS>& sm, const Geom& g, const Fields<T, 2 * NS + 3>& f,
                                           const StepCoefT<T>& c, const Charges<T>& ch, const DiagOut& d, int bx,
                                           int by, int bz, int chunk, double* part, bool vec)
{
    using TR = Trig<T>;
    using LI = LinkIdx<NS>;
    constexpr int TH0 = 2 * NS;  // first theta component

    const int tz = threadIdx.x, ty = threadIdx.y;
    const int k0 = g.loz + bx * TT_Z;
    const int j0 = g.loy + by * TT_Y;
    const int ib = g.lox + bz * chunk;
    const int ie = min(ib + chunk, g.hix);
    const int k = k0 + tz, j = j0 + ty;
    const bool active = (k < g.hiz) && (j < g.hiy);
    const int kk = wrap_idx(k, g.nz), jj = wrap_idx(j, g.ny);   // in-range copy for loads
    const int hy = ty + 1, hz = tz + 1;                          // own position in the staged plane

    // second link-data position: the low halo row j0-1 (33 sites) and column k0-1 (8 sites)
    const int tid = ty * TT_Z + tz;
    int ly2 = -1, lz2 = -1;
    if (tid < TT_LZ) { ly2 = 0; lz2 = tid; }
    else if (tid < TT_LZ + TT_Y) { ly2 = tid - TT_LZ + 1; lz2 = 0; }

    // ---- prologue: link data and fields of plane ib-1 for the own column
    const int im = wrap_idx(ib - 1, g.nx);
    T cxm[NS], sxm[NS], vm[2 * NS];
    T sPxy_xm, sPxz_xm, txm_prev;
    {
        const int s = (im * g.ny + jj) * g.nz + kk;
        const int sxp = (wrap_idx(ib, g.nx) * g.ny + jj) * g.nz + kk;
        const int syp = (im * g.ny + wrap_idx(jj + 1, g.ny)) * g.nz + kk;
        const int szp = (im * g.ny + jj) * g.nz + wrap_idx(kk + 1, g.nz);
        const T tx = f.now[TH0][s], tyv = f.now[TH0 + 1][s], tzv = f.now[TH0 + 2][s];
        T c1, s1;
        TR::sincos(tx, &s1, &c1);
#pragma unroll
        for (int q = 0; q < NS; ++q) charged<T>(tx, c1, s1, ch, q, cxm[q], sxm[q]);
        sPxy_xm = TR::sin(tx + f.now[TH0 + 1][sxp] - f.now[TH0][syp] - tyv);
        sPxz_xm = TR::sin(tx + f.now[TH0 + 2][sxp] - f.now[TH0][szp] - tzv);
        txm_prev = tx;
#pragma unroll
        for (int cc = 0; cc < 2 * NS; ++cc) vm[cc] = f.now[cc][s];
    }
    // in-range rows and columns of the tile
    const int wy = min(TT_Y, g.hiy - j0), wz = min(TT_Z, g.hiz - k0);
    VecPlan vp{0, -1};
    if (vec) vp = vec_plan(g, j0, k0, wy, wz);
    auto stage = [&](int b, int pi) {
        if (vec) stage_plane_vec<T, NS>(sm, b, f, g, pi, vp);
        else stage_plane<T, NS>(sm, b, f, g, pi, j0, k0, wy, wz);
    };
    int cur = 0;
    stage(0, wrap_idx(ib, g.nx));
    stage(1, wrap_idx(ib + 1, g.nx));

    double e_acc = 0.0, g_acc = 0.0;

    // Two barriers per plane.  The first (after the wait) makes planes i and
    // i+1 visible and ends every read of plane i-1's stage and of the link
    // data of plane i-1, so plane i+2 may then be copied into that stage and
    // the link data rewritten.  The second publishes the link data.
    for (int i = ib; i < ie; ++i) {
        const int nxt = cur == 2 ? 0 : cur + 1;
        const int nn = nxt == 2 ? 0 : nxt + 1;
        __pipeline_wait_prior(0);  // planes i and i+1 have landed
        __syncthreads();
        if (i + 1 < ie) stage(nn, wrap_idx(i + 2, g.nx));
        // the own site's level n-1, loaded now so that the link phase covers
        // the memory latency
        const int s = (i * g.ny + jj) * g.nz + kk;
        T qv[2 * NS], qx = 0, qy = 0, qz = 0;
#pragma unroll
        for (int cc = 0; cc < 2 * NS; ++cc) qv[cc] = 0;
        if (active) {
#pragma unroll
            for (int cc = 0; cc < 2 * NS; ++cc) qv[cc] = f.past[cc][s];
            qx = f.past[TH0][s];
            qy = f.past[TH0 + 1][s];
            qz = f.past[TH0 + 2][s];
        }

        // ---- link data of one staged position (ly, lz) of the current plane
        auto links = [&](int ly, int lz, T* cyq, T* syq, T* czq, T* szq, T& sxy, T& sxz, T& syz, T* cxq, T* sxq,
                         T* cpo) {
            const T tx = sm.th[cur][0][ly][lz + TT_C0], tyv = sm.th[cur][1][ly][lz + TT_C0], tzv = sm.th[cur][2][ly][lz + TT_C0];
            const T tyxp = sm.th[nxt][1][ly][lz + TT_C0], tzxp = sm.th[nxt][2][ly][lz + TT_C0];
            const T txyp = sm.th[cur][0][ly + 1][lz + TT_C0], tzyp = sm.th[cur][2][ly + 1][lz + TT_C0];
            const T txzp = sm.th[cur][0][ly][lz + 1 + TT_C0], tyzp = sm.th[cur][1][ly][lz + 1 + TT_C0];
            T c1, s1;
            TR::sincos(tyv, &s1, &c1);
#pragma unroll
            for (int q = 0; q < NS; ++q) charged<T>(tyv, c1, s1, ch, q, cyq[q], syq[q]);
            TR::sincos(tzv, &s1, &c1);
#pragma unroll
            for (int q = 0; q < NS; ++q) charged<T>(tzv, c1, s1, ch, q, czq[q], szq[q]);
            if (cxq) {
                TR::sincos(tx, &s1, &c1);
#pragma unroll
                for (int q = 0; q < NS; ++q) charged<T>(tx, c1, s1, ch, q, cxq[q], sxq[q]);
            }
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
        };
        T cx[NS], sx[NS], cy[NS], sy[NS], cz[NS], sz[NS], sPxy, sPxz, sPyz, cP[3];
        links(hy, hz, cy, sy, cz, sz, sPxy, sPxz, sPyz, cx, sx, DIAG ? cP : nullptr);
#pragma unroll
        for (int q = 0; q < NS; ++q) {
            sm.L[LI::cy(q)][hy][hz] = cy[q];
            sm.L[LI::sy(q)][hy][hz] = sy[q];
            sm.L[LI::cz(q)][hy][hz] = cz[q];
            sm.L[LI::sz(q)][hy][hz] = sz[q];
        }
        sm.L[LI::pxy][hy][hz] = sPxy;
        sm.L[LI::pxz][hy][hz] = sPxz;
        sm.L[LI::pyz][hy][hz] = sPyz;
        if (ly2 >= 0) {
            T a_cy[NS], a_sy[NS], a_cz[NS], a_sz[NS], a4, a5, a6;
            links(ly2, lz2, a_cy, a_sy, a_cz, a_sz, a4, a5, a6, nullptr, nullptr, nullptr);
#pragma unroll
            for (int q = 0; q < NS; ++q) {
                sm.L[LI::cy(q)][ly2][lz2] = a_cy[q];
                sm.L[LI::sy(q)][ly2][lz2] = a_sy[q];
                sm.L[LI::cz(q)][ly2][lz2] = a_cz[q];
                sm.L[LI::sz(q)][ly2][lz2] = a_sz[q];
            }
            sm.L[LI::pxy][ly2][lz2] = a4;
            sm.L[LI::pxz][ly2][lz2] = a5;
            sm.L[LI::pyz][ly2][lz2] = a6;
        }
        __syncthreads();

        T v[2 * NS];
#pragma unroll
        for (int cc = 0; cc < 2 * NS; ++cc) v[cc] = sm.ph[cur][cc][hy][hz + TT_C0];
        const T tx = sm.th[cur][0][hy][hz + TT_C0], tyv = sm.th[cur][1][hy][hz + TT_C0], tzv = sm.th[cur][2][hy][hz + TT_C0];
        if (active) {
            const T sPxy_ym = sm.L[LI::pxy][hy - 1][hz], sPyz_ym = sm.L[LI::pyz][hy - 1][hz];
            const T sPxz_zm = sm.L[LI::pxz][hy][hz - 1], sPyz_zm = sm.L[LI::pyz][hy][hz - 1];

            T mag[NS];
#pragma unroll
            for (int q = 0; q < NS; ++q) mag[q] = v[2 * q] * v[2 * q] + v[2 * q + 1] * v[2 * q + 1];
            T pot[NS];
            if constexpr (NS == 1) {
                pot[0] = c.halfLambda * (mag[0] - c.etaSq);
            } else {
                pot[0] = c.halfLambda * (mag[0] - c.etaSq) + c.halfLambda12 * (mag[1] - c.eta2Sq);
                pot[1] = c.halfLambda2 * (mag[1] - c.eta2Sq) + c.halfLambda12 * (mag[0] - c.etaSq);
            }
            T acc[2 * NS];
            T curx = 0, cury = 0, curz = 0;
            T pt[2 * NS], pd[NS][3][2], gsum = 0;
#pragma unroll
            for (int q = 0; q < NS; ++q) {
                const T re = v[2 * q], imv = v[2 * q + 1];
                const T rexp = sm.ph[nxt][2 * q][hy][hz + TT_C0], imxp = sm.ph[nxt][2 * q + 1][hy][hz + TT_C0];
                const T reyp = sm.ph[cur][2 * q][hy + 1][hz + TT_C0], imyp = sm.ph[cur][2 * q + 1][hy + 1][hz + TT_C0];
                const T reym = sm.ph[cur][2 * q][hy - 1][hz + TT_C0], imym = sm.ph[cur][2 * q + 1][hy - 1][hz + TT_C0];
                const T rezp = sm.ph[cur][2 * q][hy][hz + 1 + TT_C0], imzp = sm.ph[cur][2 * q + 1][hy][hz + 1 + TT_C0];
                const T rezm = sm.ph[cur][2 * q][hy][hz - 1 + TT_C0], imzm = sm.ph[cur][2 * q + 1][hy][hz - 1 + TT_C0];
                const T rexm = vm[2 * q], imxm = vm[2 * q + 1];
                const T cym = sm.L[LI::cy(q)][hy - 1][hz], sym = sm.L[LI::sy(q)][hy - 1][hz];
                const T czm = sm.L[LI::cz(q)][hy][hz - 1], szm = sm.L[LI::sz(q)][hy][hz - 1];
                // covariant Laplacian: c = +1 for the real part, -1 for the imaginary part
                T a_re = (cx[q] * rexp + sx[q] * imxp - 2 * re + cxm[q] * rexm - sxm[q] * imxm) * c.inv_dx2
                       + (cy[q] * reyp + sy[q] * imyp - 2 * re + cym * reym - sym * imym) * c.inv_dy2
                       + (cz[q] * rezp + sz[q] * imzp - 2 * re + czm * rezm - szm * imzm) * c.inv_dz2 - pot[q] * re;
                T a_im = (cx[q] * imxp - sx[q] * rexp - 2 * imv + cxm[q] * imxm + sxm[q] * rexm) * c.inv_dx2
                       + (cy[q] * imyp - sy[q] * reyp - 2 * imv + cym * imym + sym * reym) * c.inv_dy2
                       + (cz[q] * imzp - sz[q] * rezp - 2 * imv + czm * imzm + szm * rezm) * c.inv_dz2 - pot[q] * imv;
                if (c.fric != 0) {
                    a_re -= c.fric * (re - qv[2 * q]) * c.inv_dt;
                    a_im -= c.fric * (imv - qv[2 * q + 1]) * c.inv_dt;
                }
                acc[2 * q] = a_re;
                acc[2 * q + 1] = a_im;
                // gauge current of this scalar
                T jx = cx[q] * (imv * rexp - re * imxp) + sx[q] * (re * rexp + imv * imxp);
                T jy = cy[q] * (imv * reyp - re * imyp) + sy[q] * (re * reyp + imv * imyp);
                T jz = cz[q] * (imv * rezp - re * imzp) + sz[q] * (re * rezp + imv * imzp);
                if (ch.charge_current) {
                    jx *= ch.q[q];
                    jy *= ch.q[q];
                    jz *= ch.q[q];
                }
                curx += jx;
                cury += jy;
                curz += jz;
                if constexpr (DIAG) {
                    pt[2 * q] = (re - qv[2 * q]) * c.inv_dt;
                    pt[2 * q + 1] = (imv - qv[2 * q + 1]) * c.inv_dt;
                    pd[q][0][0] = (re - cxm[q] * rexm + sxm[q] * imxm) * c.inv_dx;
                    pd[q][0][1] = (imv - cxm[q] * imxm - sxm[q] * rexm) * c.inv_dx;
                    pd[q][1][0] = (re - cym * reym + sym * imym) * c.inv_dy;
                    pd[q][1][1] = (imv - cym * imym - sym * reym) * c.inv_dy;
                    pd[q][2][0] = (re - czm * rezm + szm * imzm) * c.inv_dz;
                    pd[q][2][1] = (imv - czm * imzm - szm * rezm) * c.inv_dz;
                    const T qq = NS == 1 ? (T)1 : ch.q[q];
                    gsum += qq * (imv * pt[2 * q] - re * pt[2 * q + 1]);
                }
            }
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
                const T tym = sm.th[cur][1][hy - 1][hz + TT_C0], tzm = sm.th[cur][2][hy][hz - 1 + TT_C0];
                divNow = (tx - txm_prev) * c.inv_dx2 + (tyv - tym) * c.inv_dy2 + (tzv - tzm) * c.inv_dz2;
            }
            if constexpr (DIAG) {
                T tdc = 0, fc = 0, gauss = 0;
                if (d.energy_form == LAT_ENERGY_MPI) {
                    const T a0 = (tx - qx) * c.inv_dt, a1 = (tyv - qy) * c.inv_dt, a2 = (tzv - qz) * c.inv_dt;
                    tdc = (T)0.5 * (a0 * a0 + a1 * a1 + a2 * a2);
                    fc = (1 - cP[0]) * c.inv_gxy2 + (1 - cP[1]) * c.inv_gxz2 + (1 - cP[2]) * c.inv_gyz2;
                }
                if (c.g != 0) {
                    const T divPast = reinterpret_cast<const T*>(d.divbuf)[s];
                    gauss = (divNow - divPast) * c.inv_dt * c.inv_g - c.twog * gsum;
                    if (d.energy_form != LAT_ENERGY_MPI) {
                        const T a0 = (tx - qx) * c.inv_gdtdx, a1 = (tyv - qy) * c.inv_gdtdy, a2 = (tzv - qz) * c.inv_gdtdz;
                        tdc = (T)0.5 * (a0 * a0 + a1 * a1 + a2 * a2);
                        fc = (1 - cP[0]) * c.inv_gxy2 + (1 - cP[1]) * c.inv_gxz2 + (1 - cP[2]) * c.inv_gyz2;
                    }
                }
                T ed = 0;
#pragma unroll
                for (int q = 0; q < NS; ++q)
                    ed += pt[2 * q] * pt[2 * q] + pt[2 * q + 1] * pt[2 * q + 1] + pd[q][0][0] * pd[q][0][0]
                        + pd[q][0][1] * pd[q][0][1] + pd[q][1][0] * pd[q][1][0] + pd[q][1][1] * pd[q][1][1]
                        + pd[q][2][0] * pd[q][2][0] + pd[q][2][1] * pd[q][2][1];
                const T m1 = mag[0] - c.etaSq;
                ed += tdc + fc + c.quarterLambda * (m1 * m1);
                if constexpr (NS == 2) {
                    const T m2 = mag[1] - c.eta2Sq;
                    ed += c.quarterLambda2 * (m2 * m2) + c.halfLambda12e * m1 * m2;
                }
                e_acc += (double)(d.energy_form == LAT_ENERGY_MPI ? ed * c.dx * c.dy * c.dz : c.dV * ed);
                g_acc += (double)fabs(gauss);
            }
            if (d.store_div) reinterpret_cast<T*>(d.divbuf)[s] = divNow;
            if (d.write) {
#pragma unroll
                for (int cc = 0; cc < 2 * NS; ++cc) f.past[cc][s] = leapfrog<T>(v[cc], qv[cc], c.dt2, acc[cc]);
                f.past[TH0][s] = leapfrog<T>(tx, qx, c.dt2, ttx);
                f.past[TH0 + 1][s] = leapfrog<T>(tyv, qy, c.dt2, tty);
                f.past[TH0 + 2][s] = leapfrog<T>(tzv, qz, c.dt2, ttz);
            }
        }
        // carry the x-backward data of the next plane
#pragma unroll
        for (int q = 0; q < NS; ++q) {
            cxm[q] = cx[q];
            sxm[q] = sx[q];
        }
        sPxy_xm = sPxy;
        sPxz_xm = sPxz;
        txm_prev = tx;
#pragma unroll
        for (int cc = 0; cc < 2 * NS; ++cc) vm[cc] = v[cc];
        cur = nxt;
    }
    __pipeline_wait_prior(0);  // nothing is in flight here; kept for an empty x-range

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
            part[0] = a;
            part[1] = b;
        }
        __syncthreads();  // sm.red is reused by the CTA's next tile
    }
}

template <class T, int NS, bool DIAG>
__global__ void __launch_bounds__(TT_THREADS, NS == 1 ? 4 : 3)
tiled_step_kernel(const Geom g, const Fields<T, 2 * NS + 3> f, const StepCoefT<T> c, const Charges<T> ch,
                  const DiagOut d, const int chunk, const int vec)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TiledSmem<T, NS>& sm = *reinterpret_cast<TiledSmem<T, NS>*>(smem_raw);
    const int blk = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    tiled_tile<T, NS, DIAG>(sm, g, f, c, ch, d, (int)blockIdx.x, (int)blockIdx.y, (int)blockIdx.z, chunk,
                            DIAG ? d.partials + 2 * blk : nullptr, vec != 0);
}

inline dim3 tiled_grid(const Geom& g, int chunk)
{
    return dim3((unsigned)((g.hiz - g.loz + TT_Z - 1) / TT_Z), (unsigned)((g.hiy - g.loy + TT_Y - 1) / TT_Y),
                (unsigned)((g.hix - g.lox + chunk - 1) / chunk));
}

inline int small_int_power(double q)
{
    return (q == (double)(int)q && q != 0 && q >= -4 && q <= 4) ? (int)q : 0;
}

template <class T, int NS>
cudaError_t launch_tiled_t(const Geom& g, const Fields<T, 2 * NS + 3>& f, const StepCoef& c64, const DiagOut& d,
                           bool diag, int chunk, cudaStream_t st, bool allow_vec = true)
{
    const StepCoefT<T> c = coef_as<T>(c64);
    Charges<T> ch;
    if (NS == 1) {
        ch.q[0] = 1;
        ch.q[1] = 0;
        ch.qpow[0] = 1;
        ch.qpow[1] = 0;
    } else {
        ch.q[0] = (T)c64.q1;
        ch.q[1] = (T)c64.q2;
        ch.qpow[0] = small_int_power(c64.q1);
        ch.qpow[1] = small_int_power(c64.q2);
    }
    ch.charge_current = d.charge_current;
    const size_t smem = sizeof(TiledSmem<T, NS>);
    if (smem > 48 * 1024) {  // opt in above the default dynamic shared-memory limit
        cudaFuncSetAttribute(tiled_step_kernel<T, NS, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(tiled_step_kernel<T, NS, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    }
    const dim3 grid = tiled_grid(g, chunk);
    const dim3 block(TT_Z, TT_Y);
    const int vec = allow_vec && tiled_vec_ok(g, f) ? 1 : 0;
    if (diag) tiled_step_kernel<T, NS, true><<<grid, block, smem, st>>>(g, f, c, ch, d, chunk, vec);
    else tiled_step_kernel<T, NS, false><<<grid, block, smem, st>>>(g, f, c, ch, d, chunk, vec);
    return cudaGetLastError();
}

}  // namespace lat
