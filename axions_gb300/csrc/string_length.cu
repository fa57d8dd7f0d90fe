// string_length.cu -- total string length by greedy chaining of crossings.
//
// Reference: ic_w_evolution.cpp:961-1087.  From the current crossing the
// nearest remaining crossing whose squared distance is within the cutoff
// (dx^2+dy^2+dz^2)^2 is next, the last of equally near ones winning; its
// distance goes to L0 (current crossing inside the central quarter box, or no
// split) or L1.  With none in reach the chain closes onto its first crossing
// when that is in reach (adding sqrt(cutoff), as the reference does) and
// restarts at the lowest remaining index.
//
// GPU form, exact on the same crossing list:
//   * Periodic lattice.  Crossings within the cutoff of each other are linked;
//     a chain never leaves a connected component of that graph, and a restart
//     takes the lowest remaining index, which is also its component's lowest
//     remaining index, so components are walked independently.  The links are
//     built once, in parallel, through a cell hash whose cells are at least the
//     cutoff radius wide: per crossing a list of (neighbour, squared distance,
//     the neighbour's own list, the slot of the reverse link).  One warp walks
//     one component over these lists.  A step reads the current crossing's list
//     and the dead marks of its entries in one memory round trip, picks the
//     nearest live neighbour by comparing the squared distances' bit patterns
//     (non-negative doubles order like their bits), and marks dead the reverse
//     links of the crossing it leaves.  No floating point is done in the walk.
//   * The reference visits chains in increasing order of their first index.
//     Each visit is recorded with its chain's first index and its place in the
//     chain; a scan of the chain lengths places every visit in the reference's
//     order, square roots are taken there in parallel, and one warp adds the
//     lengths in that order, so L0 and L1 are the reference's doubles bit for
//     bit.
//   * Any lattice (on a fixed lattice a separation above half the box counts as
//     0 on that axis, which links crossings across the box): a cooperative grid
//     follows the reference's loop directly.  Each CTA owns a slice of the
//     crossings; per step it publishes its slice's nearest live candidate and
//     lowest live index, and after one grid barrier (a bounded wait) every CTA
//     reduces the same winner.
// Compiled with -fmad=false: distances use the reference's unfused products.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>

#include "lattice_internal.cuh"

namespace lat {

namespace {

constexpr int SCAN_T = 1024;            // threads of a scan block
constexpr int SCAN_I = 4;               // items per scan thread
constexpr int SCAN_CHUNK = SCAN_T * SCAN_I;
constexpr int WALK_WARPS = 4;           // warps per walk block
constexpr int EX_T = 512;               // threads per CTA of the cooperative walk
constexpr int UNROLL = 4;
constexpr unsigned FULL = 0xffffffffu;

struct ChainPt {
    double x, y, z;
    int idx;
    int bin;  // hash cell
};

// a link i -> j of the crossing graph
struct AdjEdge {
    unsigned long long d2;  // bits of the squared distance (a non-negative double)
    long long start;        // first link of j
    long long rev;          // slot of the link j -> i
    int j;
    int meta;               // number of links of j | inner(j) << 31
};

// error codes left in counters[2]
constexpr int CHAIN_ERR_UNION = 1;     // union-find retry bound reached
constexpr int CHAIN_ERR_RESTART = 2;   // no remaining member where one must be
constexpr int CHAIN_ERR_LINK = 3;      // the link graph is not symmetric, or a walk outran its component
constexpr int CHAIN_ERR_BARRIER = 4;   // a grid barrier wait gave up
constexpr long long kDefaultWaitPolls = 1LL << 24;

struct ChainDev {
    ChainGeom g;
    const double* xyz;        // [M][3]
    int M;
    int split;
    int nbins;
    // cell hash and links
    int* bin_of;              // [M]
    int* bin_cnt;             // [nbins] counts, then fill cursors
    long long* bin_start;     // [nbins + 1]
    ChainPt* sp;              // [M] crossings sorted by cell
    unsigned char* inner;     // [M] inside the central quarter box
    int* deg;                 // [M] links per crossing
    long long* adj_start;     // [M + 1]
    AdjEdge* adj;             // [E]
    unsigned char* edge_dead; // [E] the link's far end has been left
    // components
    int* parent;              // [M] union-find forest
    int* comp;                // [M] the component's lowest index
    int* csize;               // [M] component sizes (at the component's lowest index)
    int* roots;               // [M]
    unsigned char* alive_o;   // [M]
    // visits
    double* rec_d2;           // [M] squared length added when leaving crossing i
    unsigned char* rec_cls;   // [M] 0: L0, 1: L1, 2: nothing
    int* rec_start;           // [M] first index of i's chain
    int* rec_pos;             // [M] place of i in its chain
    int* chain_len;           // [M] chain lengths at their first index, else 0
    long long* chain_off;     // [M] exclusive scan of chain_len
    double* ord_val;          // [M] visits in the reference's order
    unsigned char* ord_cls;   // [M]
    long long* scan_tot;      // [scan blocks]
    long long* scan_sum;      // [1]
    // cooperative walk
    double* slot_d2;          // [2][grid]
    int* slot_j;              // [2][grid]
    int* slot_min;            // [2][grid]
    unsigned* bar;            // [2] arrivals, generation
    long long wait_polls;     // polls of a barrier wait before it gives up
    unsigned missing;         // arrivals a barrier waits for that never come (0; > 0 only to test the bound)
    int* counters;            // [0] roots, [1] queue head, [2] error
    double* out;              // [2] L0, L1
};

// ---------------------------------------------------------------------------
// the reference's arithmetic (ic_w_evolution.cpp:986-993, 1015-1018, 1035-1042)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double axis_term(double a, double b, double L, double half, int periodic)
{
    const double t = fabs(a - b);
    if (t <= half) {
        const double e = a - b;
        return e * e;
    }
    if (periodic) {
        const double e = L - t;
        return e * e;
    }
    return 0.0;
}

__device__ __forceinline__ double chain_d2(const ChainGeom& g, double ax, double ay, double az, double bx, double by,
                                           double bz)
{
    double d = axis_term(ax, bx, g.L[0], g.half[0], g.periodic[0]);
    d += axis_term(ay, by, g.L[1], g.half[1], g.periodic[1]);
    d += axis_term(az, bz, g.L[2], g.half[2], g.periodic[2]);
    return d;
}

__device__ __forceinline__ bool chain_inner(const ChainGeom& g, double x, double y, double z)
{
    return x >= -g.quarter[0] && x <= g.quarter[0] && y >= -g.quarter[1] && y <= g.quarter[1] &&
           z >= -g.quarter[2] && z <= g.quarter[2];
}

__device__ __forceinline__ int cell1(double v, double lo, double w, int nb)
{
    const double t = floor((v - lo) / w);
    if (!(t >= 0.0)) return 0;
    if (t >= (double)nb) return nb - 1;
    return (int)t;
}

__device__ __forceinline__ int wrap_cell(int i, int nb)
{
    return i < 0 ? i + nb : (i >= nb ? i - nb : i);
}

// lexicographic (smaller squared distance, then larger index)
__device__ __forceinline__ void better(double& best, int& bj, double ob, int oj)
{
    if (ob < best || (ob == best && oj > bj)) {
        best = ob;
        bj = oj;
    }
}

__device__ __forceinline__ void warp_best(double& best, int& bj)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        const double ob = __shfl_xor_sync(FULL, best, o);
        const int oj = __shfl_xor_sync(FULL, bj, o);
        better(best, bj, ob, oj);
    }
}

// ---------------------------------------------------------------------------
// exclusive scan of an int array into long long offsets (two levels)
// ---------------------------------------------------------------------------
__device__ __forceinline__ long long block_scan_ll(long long v, long long* total)
{
    __shared__ long long warp_sums[SCAN_T / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    long long incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long t = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_sums[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        long long ws = warp_sums[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long t = __shfl_up_sync(FULL, ws, o);
            if (lane >= o) ws += t;
        }
        warp_sums[lane] = ws;
    }
    __syncthreads();
    const long long base = wid ? warp_sums[wid - 1] : 0;
    if (total) *total = warp_sums[SCAN_T / 32 - 1];
    const long long r = base + incl - v;
    __syncthreads();
    return r;
}

// pass 1: per-block totals
__global__ void __launch_bounds__(SCAN_T) scan_blocks_kernel(const int* __restrict__ in, long long n,
                                                             long long* __restrict__ tot)
{
    const long long b = (long long)blockIdx.x * SCAN_CHUNK + (long long)threadIdx.x * SCAN_I;
    long long s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_I; ++k)
        if (b + k < n) s += in[b + k];
    long long total;
    block_scan_ll(s, &total);
    if (threadIdx.x == 0) tot[blockIdx.x] = total;
}

// pass 3: local exclusive scan plus the block's offset; out[n] = grand total
__global__ void __launch_bounds__(SCAN_T) scan_apply_kernel(const int* __restrict__ in, long long n,
                                                            const long long* __restrict__ tot,
                                                            const long long* __restrict__ grand,
                                                            long long* __restrict__ out, int write_end)
{
    const long long b = (long long)blockIdx.x * SCAN_CHUNK + (long long)threadIdx.x * SCAN_I;
    int v[SCAN_I];
    long long s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_I; ++k) {
        v[k] = (b + k < n) ? in[b + k] : 0;
        s += v[k];
    }
    long long run = tot[blockIdx.x] + block_scan_ll(s, nullptr);
#pragma unroll
    for (int k = 0; k < SCAN_I; ++k) {
        if (b + k < n) out[b + k] = run;
        run += v[k];
    }
    if (write_end && blockIdx.x == 0 && threadIdx.x == 0) out[n] = *grand;
}

int scan_blocks(long long n) { return (int)((n + SCAN_CHUNK - 1) / SCAN_CHUNK); }

cudaError_t exclusive_scan(const int* in, long long n, long long* out, int write_end, long long* tot,
                           long long* grand, cudaStream_t st, int64_t* launches)
{
    const int nb = scan_blocks(n);
    scan_blocks_kernel<<<nb, SCAN_T, 0, st>>>(in, n, tot);
    cudaError_t e = launch_scan_totals(tot, nb, grand, st);
    if (e != cudaSuccess) return e;
    scan_apply_kernel<<<nb, SCAN_T, 0, st>>>(in, n, tot, grand, out, write_end);
    if (launches) *launches += 3;
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// cell hash
// ---------------------------------------------------------------------------
__global__ void bin_count_kernel(const ChainDev c)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.M) return;
    const double* p = c.xyz + 3 * (size_t)i;
    const int ix = cell1(p[0], c.g.lo[0], c.g.w[0], c.g.nb[0]);
    const int iy = cell1(p[1], c.g.lo[1], c.g.w[1], c.g.nb[1]);
    const int iz = cell1(p[2], c.g.lo[2], c.g.w[2], c.g.nb[2]);
    const int b = (ix * c.g.nb[1] + iy) * c.g.nb[2] + iz;
    c.bin_of[i] = b;
    atomicAdd(&c.bin_cnt[b], 1);
    c.inner[i] = chain_inner(c.g, p[0], p[1], p[2]) ? 1 : 0;
    c.parent[i] = i;
    c.csize[i] = 0;
    c.chain_len[i] = 0;
    c.alive_o[i] = 1;
}

// bin_cnt is zeroed again before this kernel and serves as the fill cursor
__global__ void bin_scatter_kernel(const ChainDev c)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.M) return;
    const int b = c.bin_of[i];
    const long long q = c.bin_start[b] + atomicAdd(&c.bin_cnt[b], 1);
    const double* p = c.xyz + 3 * (size_t)i;
    ChainPt s;
    s.x = p[0];
    s.y = p[1];
    s.z = p[2];
    s.idx = i;
    s.bin = b;
    c.sp[q] = s;
}

// fn(j, d2) for every crossing j != i within the cutoff of crossing i
template <class F>
__device__ __forceinline__ void for_links(const ChainDev& c, int i, F&& fn)
{
    const double* p = c.xyz + 3 * (size_t)i;
    const double x = p[0], y = p[1], z = p[2];
    const int b = c.bin_of[i];
    const int iz = b % c.g.nb[2], t = b / c.g.nb[2];
    const int iy = t % c.g.nb[1], ix = t / c.g.nb[1];
    for (int k = 0; k < c.g.nnb; ++k) {
        const int jx = wrap_cell(ix + c.g.off[k][0], c.g.nb[0]);
        const int jy = wrap_cell(iy + c.g.off[k][1], c.g.nb[1]);
        const int jz = wrap_cell(iz + c.g.off[k][2], c.g.nb[2]);
        const int nb = (jx * c.g.nb[1] + jy) * c.g.nb[2] + jz;
        const long long q1 = c.bin_start[nb + 1];
        for (long long q = c.bin_start[nb]; q < q1; ++q) {
            const ChainPt s = c.sp[q];
            if (s.idx == i) continue;
            const double d = chain_d2(c.g, x, y, z, s.x, s.y, s.z);
            if (d <= c.g.cutoff) fn(s.idx, d);
        }
    }
}

__global__ void adj_count_kernel(const ChainDev c)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.M) return;
    int n = 0;
    for_links(c, i, [&](int, double) { ++n; });
    c.deg[i] = n;
}

// ---------------------------------------------------------------------------
// connected components (union-find; every parent is <= its child, so a root is
// its set's lowest index)
// ---------------------------------------------------------------------------
__device__ __forceinline__ int find_root(int* parent, int x)
{
    volatile int* vp = parent;
    int p = vp[x];
    while (p != x) {
        const int gp = vp[p];
        if (gp != p) vp[x] = gp;  // path halving: gp is still an ancestor of x
        x = p;
        p = gp;
    }
    return x;
}

__device__ void unite(int* parent, int a, int b, int* err)
{
    for (int it = 0; it < (1 << 22); ++it) {
        a = find_root(parent, a);
        b = find_root(parent, b);
        if (a == b) return;
        if (a < b) {
            const int t = a;
            a = b;
            b = t;
        }
        if (atomicCAS(&parent[a], a, b) == a) return;
    }
    atomicExch(err, CHAIN_ERR_UNION);
}

// the links of i, in the order adj_count_kernel counted them; joins the sets
__global__ void adj_fill_kernel(const ChainDev c)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.M) return;
    long long pos = c.adj_start[i];
    for_links(c, i, [&](int j, double d) {
        AdjEdge e;
        e.d2 = (unsigned long long)__double_as_longlong(d);
        e.start = 0;
        e.rev = -1;
        e.j = j;
        e.meta = 0;
        c.adj[pos] = e;
        c.edge_dead[pos] = 0;
        ++pos;
        if (j > i) unite(c.parent, i, j, &c.counters[2]);
    });
}

// where each link's far end keeps its own links, and the reverse link
__global__ void adj_link_kernel(const ChainDev c)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.M) return;
    const long long k1 = c.adj_start[i + 1];
    for (long long k = c.adj_start[i]; k < k1; ++k) {
        const int j = c.adj[k].j;
        const long long s = c.adj_start[j], n = c.deg[j];
        long long rev = -1;
        for (long long q = s; q < s + n; ++q)
            if (c.adj[q].j == i) {
                rev = q;
                break;
            }
        if (rev < 0) atomicExch(&c.counters[2], CHAIN_ERR_LINK);
        c.adj[k].start = s;
        c.adj[k].rev = rev < 0 ? k : rev;
        c.adj[k].meta = (int)((unsigned)n | ((unsigned)c.inner[j] << 31));
    }
}

__global__ void flatten_kernel(const ChainDev c)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.M) return;
    const int r = find_root(c.parent, i);  // no union is pending: r is final
    c.comp[i] = r;
    atomicAdd(&c.csize[r], 1);
    if (r == i) c.roots[atomicAdd(&c.counters[0], 1)] = i;
}

// ---------------------------------------------------------------------------
// one warp walks one component over the links; visits are recorded, not
// summed.  Dead marks are read through L2 (ld.global.cg): the lanes of this
// warp set them, __syncwarp orders the steps.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(32 * WALK_WARPS) walk_kernel(const ChainDev c)
{
    const int lane = threadIdx.x & 31;
    const int nroots = c.counters[0];
    const unsigned long long cut = (unsigned long long)__double_as_longlong(c.g.cutoff);
    for (;;) {
        int qi = 0;
        if (lane == 0) qi = atomicAdd(&c.counters[1], 1);
        qi = __shfl_sync(FULL, qi, 0);
        if (qi >= nroots) return;
        const int r = c.roots[qi];
        const int S = c.csize[r];
        int f = r, start = r, pos = 0;
        long long s0 = c.adj_start[r];
        int n0 = c.deg[r];
        int inner_f = c.inner[r];
        double bx = c.xyz[3 * (size_t)r], by = c.xyz[3 * (size_t)r + 1], bz = c.xyz[3 * (size_t)r + 2];
        bool found = false;
        for (int it = 0; it < S; ++it) {
            unsigned long long best = cut;
            int bj = -1;
            long long wstart = 0;
            int wmeta = 0;
            for (int k = lane; k < n0; k += 32) {
                const AdjEdge e = c.adj[s0 + k];
                const unsigned char dead = __ldcg(c.edge_dead + s0 + k);
                c.edge_dead[e.rev] = 1;  // f is left: the link back to it dies
                if (dead) continue;
                // a live neighbour may be the next crossing: start fetching its links
                asm volatile("prefetch.global.L2 [%0];" ::"l"(c.adj + e.start));
                asm volatile("prefetch.global.L2 [%0];" ::"l"(c.edge_dead + e.start));
                if (e.d2 < best || (e.d2 == best && e.j > bj)) {
                    best = e.d2;
                    bj = e.j;
                    wstart = e.start;
                    wmeta = e.meta;
                }
            }
            const int my_bj = bj;
#pragma unroll
            for (int o = 16; o; o >>= 1) {
                const unsigned long long ob = __shfl_xor_sync(FULL, best, o);
                const int oj = __shfl_xor_sync(FULL, bj, o);
                if (ob < best || (ob == best && oj > bj)) {
                    best = ob;
                    bj = oj;
                }
            }
            found = bj >= 0;
            long long ns0 = 0;
            int nmeta = 0;
            if (found) {
                const int src = __ffs(__ballot_sync(FULL, my_bj == bj)) - 1;
                ns0 = __shfl_sync(FULL, wstart, src);
                nmeta = __shfl_sync(FULL, wmeta, src);
            }
            if (lane == 0) {
                const unsigned char side = (c.split && !inner_f) ? 1 : 0;
                double d2 = 0.0;
                unsigned char cls = 2;
                if (found) {
                    d2 = __longlong_as_double((long long)best);
                    cls = side;
                } else {
                    const double* pf = c.xyz + 3 * (size_t)f;
                    if (chain_d2(c.g, pf[0], pf[1], pf[2], bx, by, bz) <= c.g.cutoff) {
                        d2 = c.g.cutoff;
                        cls = side;
                    }
                }
                c.rec_d2[f] = d2;
                c.rec_cls[f] = cls;
                c.rec_start[f] = start;
                c.rec_pos[f] = pos;
                c.alive_o[f] = 0;
                if (!found) c.chain_len[start] = pos + 1;
            }
            __syncwarp();
            if (found) {
                f = bj;
                s0 = ns0;
                n0 = nmeta & 0x7fffffff;
                inner_f = (int)((unsigned)nmeta >> 31);
                ++pos;
                continue;
            }
            if (it + 1 >= S) break;
            // restart at the component's lowest remaining index (above start)
            int nf = -1;
            for (int cu = start + 1; cu < c.M; cu += 32) {
                const int i = cu + lane;
                const bool ok = i < c.M && c.comp[i] == r && __ldcg(c.alive_o + i);
                const unsigned m = __ballot_sync(FULL, ok);
                if (m) {
                    nf = cu + __ffs(m) - 1;
                    break;
                }
            }
            if (nf < 0) {
                if (lane == 0) atomicExch(&c.counters[2], CHAIN_ERR_RESTART);
                return;
            }
            f = start = nf;
            pos = 0;
            s0 = c.adj_start[f];
            n0 = c.deg[f];
            inner_f = c.inner[f];
            bx = c.xyz[3 * (size_t)f];
            by = c.xyz[3 * (size_t)f + 1];
            bz = c.xyz[3 * (size_t)f + 2];
        }
        if (found && lane == 0) atomicExch(&c.counters[2], CHAIN_ERR_LINK);
    }
}

// every visit's place in the reference's order (chains by first index, then by
// place in the chain) and its length
__global__ void order_kernel(const ChainDev c)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.M) return;
    const long long o = c.chain_off[c.rec_start[i]] + c.rec_pos[i];
    const unsigned char cls = c.rec_cls[i];
    c.ord_val[o] = cls == 2 ? 0.0 : sqrt(c.rec_d2[i]);
    c.ord_cls[o] = cls;
}

// the sums in the reference's order, by one thread.  Every visit adds to both
// sums, 0.0 to the one it does not count to (x + 0.0 == x for the non-negative
// partial sums), so the two dependent chains interleave and the loads of a
// batch are issued together.
__global__ void __launch_bounds__(32) sum_kernel(const ChainDev c)
{
    if (threadIdx.x != 0) return;
    constexpr int B = 16;
    double L0 = 0.0, L1 = 0.0;
    int base = 0;
    for (; base + B <= c.M; base += B) {
        double v[B];
        unsigned char k[B];
#pragma unroll
        for (int u = 0; u < B; ++u) {
            v[u] = c.ord_val[base + u];
            k[u] = c.ord_cls[base + u];
        }
#pragma unroll
        for (int u = 0; u < B; ++u) {
            L0 += k[u] == 0 ? v[u] : 0.0;
            L1 += k[u] == 1 ? v[u] : 0.0;
        }
    }
    for (; base < c.M; ++base) {
        const double v = c.ord_val[base];
        const unsigned char k = c.ord_cls[base];
        L0 += k == 0 ? v : 0.0;
        L1 += k == 1 ? v : 0.0;
    }
    c.out[0] = L0;
    c.out[1] = L1;
}

// ---------------------------------------------------------------------------
// cooperative walk over all crossings (any lattice)
// ---------------------------------------------------------------------------
// Grid barrier for a cooperative launch (all CTAs resident).  The wait is
// bounded: a CTA polls the generation word at most `polls` times (the host's
// default, 2^24 polls, is about a second), then records CHAIN_ERR_BARRIER; a
// CTA that sees the error recorded stops waiting too, and every CTA leaves at
// its barrier.  `missing` arrivals are added to the count the barrier waits
// for: none in normal use; a test sets one, an arrival that never comes, to
// make every wait run out.  Returns false once an error is recorded.
__device__ bool grid_barrier(unsigned* bar, int* err, long long polls, unsigned missing)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* vgen = bar + 1;
        volatile int* verr = err;
        const unsigned gen = *vgen;
        __threadfence();
        if (atomicAdd(bar, 1u) == gridDim.x + missing - 1) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            long long spins = 0;
            while (*vgen == gen) {
                if (*verr != 0) break;
                if (++spins > polls) {
                    atomicExch(err, CHAIN_ERR_BARRIER);
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return *(volatile int*)err == 0;
}

__global__ void __launch_bounds__(EX_T) walk_coop_kernel(const ChainDev c)
{
    __shared__ double s_best[EX_T / 32];
    __shared__ int s_bj[EX_T / 32];
    __shared__ unsigned s_min[EX_T / 32];
    __shared__ int r_bj, r_min;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int G = gridDim.x, b = blockIdx.x;
    const int lo = (int)((long long)c.M * b / G), hi = (int)((long long)c.M * (b + 1) / G);
    for (int i = lo + tid; i < hi; i += EX_T) c.alive_o[i] = 1;
    int f = 0;
    double bx = c.xyz[0], by = c.xyz[1], bz = c.xyz[2];
    double L0 = 0.0, L1 = 0.0;  // kept by thread 0 of CTA 0
    __syncthreads();
    for (int it = 0; it < c.M; ++it) {
        const double fx = c.xyz[3 * (size_t)f], fy = c.xyz[3 * (size_t)f + 1], fz = c.xyz[3 * (size_t)f + 2];
        double best = c.g.cutoff;
        int bj = -1;
        unsigned mn = (unsigned)INT_MAX;  // lowest live index other than f
        for (int j0 = lo + tid; j0 < hi; j0 += EX_T * UNROLL) {
            unsigned char al[UNROLL];
            double px[UNROLL], py[UNROLL], pz[UNROLL];
#pragma unroll
            for (int u = 0; u < UNROLL; ++u) {
                const int j = j0 + u * EX_T;
                al[u] = 0;
                if (j < hi) {
                    al[u] = c.alive_o[j];
                    px[u] = c.xyz[3 * (size_t)j];
                    py[u] = c.xyz[3 * (size_t)j + 1];
                    pz[u] = c.xyz[3 * (size_t)j + 2];
                }
            }
#pragma unroll
            for (int u = 0; u < UNROLL; ++u) {
                const int j = j0 + u * EX_T;
                if (!al[u] || j == f) continue;
                mn = min(mn, (unsigned)j);
                better(best, bj, chain_d2(c.g, fx, fy, fz, px[u], py[u], pz[u]), j);
            }
        }
        warp_best(best, bj);
        mn = __reduce_min_sync(FULL, mn);
        if (lane == 0) {
            s_best[wid] = best;
            s_bj[wid] = bj;
            s_min[wid] = mn;
        }
        __syncthreads();
        if (wid == 0) {
            best = lane < EX_T / 32 ? s_best[lane] : c.g.cutoff;
            bj = lane < EX_T / 32 ? s_bj[lane] : -1;
            mn = lane < EX_T / 32 ? s_min[lane] : (unsigned)INT_MAX;
            warp_best(best, bj);
            mn = __reduce_min_sync(FULL, mn);
            if (lane == 0) {
                const int sl = (it & 1) * G + b;
                c.slot_d2[sl] = best;
                c.slot_j[sl] = bj;
                c.slot_min[sl] = (int)mn;
            }
        }
        if (!grid_barrier(c.bar, &c.counters[2], c.wait_polls, c.missing)) return;
        if (wid == 0) {
            best = c.g.cutoff;
            bj = -1;
            mn = (unsigned)INT_MAX;
            for (int k = lane; k < G; k += 32) {
                const int sl = (it & 1) * G + k;
                better(best, bj, __ldcg(c.slot_d2 + sl), __ldcg(c.slot_j + sl));
                mn = min(mn, (unsigned)__ldcg(c.slot_min + sl));
            }
            warp_best(best, bj);
            mn = __reduce_min_sync(FULL, mn);
            if (lane == 0) {
                r_bj = bj;
                r_min = (int)mn;
                if (f >= lo && f < hi) c.alive_o[f] = 0;  // f's owner retires it
                if (b == 0) {
                    const bool outer = c.split && !chain_inner(c.g, fx, fy, fz);
                    if (bj >= 0) {
                        if (outer) L1 += sqrt(best);
                        else L0 += sqrt(best);
                    } else if (chain_d2(c.g, fx, fy, fz, bx, by, bz) <= c.g.cutoff) {
                        if (outer) L1 += c.g.root_cutoff;
                        else L0 += c.g.root_cutoff;
                    }
                }
            }
        }
        __syncthreads();
        const int nbj = r_bj, nmin = r_min;
        if (nbj >= 0) {
            f = nbj;
            continue;
        }
        if (it + 1 >= c.M) break;
        if (nmin == INT_MAX) {
            if (tid == 0) atomicExch(&c.counters[2], CHAIN_ERR_RESTART);
            return;
        }
        f = nmin;
        bx = c.xyz[3 * (size_t)f];
        by = c.xyz[3 * (size_t)f + 1];
        bz = c.xyz[3 * (size_t)f + 2];
    }
    if (b == 0 && tid == 0) {
        c.out[0] = L0;
        c.out[1] = L1;
    }
}

// ---------------------------------------------------------------------------
// workspace
// ---------------------------------------------------------------------------
struct Carver {
    char* base;
    size_t off = 0;
    template <class T>
    T* take(size_t n)
    {
        off = (off + 255) & ~(size_t)255;
        T* p = base ? (T*)(base + off) : nullptr;
        off += sizeof(T) * (n ? n : 1);
        return p;
    }
};

long long chain_bins(const ChainGeom& g) { return (long long)g.nb[0] * g.nb[1] * g.nb[2]; }

// everything but the links (sized once their number is known)
ChainDev carve(void* ws, const ChainGeom& g, int64_t M, int method, int grid, size_t* bytes)
{
    ChainDev c{};
    Carver k{(char*)ws};
    c.g = g;
    c.counters = k.take<int>(4);
    c.out = k.take<double>(2);
    c.alive_o = k.take<unsigned char>(M);
    if (method == LAT_CHAIN_EXHAUSTIVE) {
        c.slot_d2 = k.take<double>(2 * (size_t)grid);
        c.slot_j = k.take<int>(2 * (size_t)grid);
        c.slot_min = k.take<int>(2 * (size_t)grid);
        c.bar = k.take<unsigned>(2);
    } else {
        const long long nbins = chain_bins(g);
        c.nbins = (int)nbins;
        c.bin_of = k.take<int>(M);
        c.bin_cnt = k.take<int>(nbins);
        c.bin_start = k.take<long long>(nbins + 1);
        c.sp = k.take<ChainPt>(M);
        c.inner = k.take<unsigned char>(M);
        c.deg = k.take<int>(M);
        c.adj_start = k.take<long long>(M + 1);
        c.parent = k.take<int>(M);
        c.comp = k.take<int>(M);
        c.csize = k.take<int>(M);
        c.roots = k.take<int>(M);
        c.rec_d2 = k.take<double>(M);
        c.rec_cls = k.take<unsigned char>(M);
        c.rec_start = k.take<int>(M);
        c.rec_pos = k.take<int>(M);
        c.chain_len = k.take<int>(M);
        c.chain_off = k.take<long long>(M);
        c.ord_val = k.take<double>(M);
        c.ord_cls = k.take<unsigned char>(M);
        c.scan_tot = k.take<long long>(std::max(scan_blocks(nbins), scan_blocks(M + 1)));
        c.scan_sum = k.take<long long>(1);
    }
    *bytes = k.off;
    return c;
}

// grow a device buffer to `need` bytes; `held` tracks the bytes held
int grow(void** p, size_t* have, size_t need, int64_t* held)
{
    if (need <= *have && *p) return LAT_OK;
    if (*p) {
        cudaFree(*p);
        if (held) *held -= (int64_t)*have;
        *p = nullptr;
        *have = 0;
    }
    const size_t want = need ? need : 256;
    const cudaError_t e = cudaMalloc(p, want);
    if (e != cudaSuccess) {
        *p = nullptr;
        set_error(std::string("string length: cudaMalloc: ") + cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? LAT_ERR_NOMEM : LAT_ERR_CUDA;
    }
    *have = want;
    if (held) *held += (int64_t)want;
    return LAT_OK;
}

// Bound of the cooperative walk's barrier waits and the test's missing
// arrivals (lat_set_chain_wait).  Process-wide.
std::atomic<long long> g_wait_polls{kDefaultWaitPolls};
std::atomic<unsigned> g_missing{0};

// CTAs of the cooperative walk: all resident at once (at most one per SM), at
// most one per EX_T crossings
int coop_grid(int64_t M, int* grid)
{
    int dev = 0, sms = 0, coop = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, walk_coop_kernel, EX_T, 0);
    if (e != cudaSuccess || !coop || per_sm < 1) {
        set_error("string length: the device cannot run the cooperative walk");
        return LAT_ERR_CUDA;
    }
    const int64_t want = std::max<int64_t>(1, (M + EX_T - 1) / EX_T);
    *grid = (int)std::min<int64_t>(want, (int64_t)sms);
    return LAT_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
ChainGeom make_chain_geom(const lat_params& p, int64_t M)
{
    ChainGeom g{};
    const int64_t n[3] = {p.nx, p.ny, p.nz};
    const double d[3] = {p.dx, p.dy, p.dz};
    const double c0 = p.dx * p.dx + p.dy * p.dy + p.dz * p.dz;
    g.cutoff = c0 * c0;  // pow(., 2) of ic_w_evolution.cpp:979
    g.root_cutoff = std::sqrt(g.cutoff);
    g.periodic[0] = g.periodic[1] = p.bc == LAT_BC_PERIODIC;
    g.periodic[2] = bc_z_kind(p) == LAT_BC_PERIODIC;
    long long nb[3];
    for (int a = 0; a < 3; ++a) {
        g.L[a] = (double)n[a] * d[a];
        g.half[a] = (0.5 * (double)n[a]) * d[a];
        g.quarter[a] = (0.25 * (double)n[a]) * d[a];
        const int64_t x0 = (int64_t)(0.5 * (double)(n[a] - 1));  // ic_w_evolution.cpp:96-98
        g.lo[a] = (double)(0 - x0) * d[a];
        const double want = g.root_cutoff * (1.0 + 1e-6);
        double q = std::floor(g.L[a] / want);
        if (!(q >= 1.0)) q = 1.0;
        if (q > (double)n[a]) q = (double)n[a];
        nb[a] = (long long)q;
    }
    // at most about two cells per crossing: wider cells only add candidates
    const long long cap = std::max<long long>(64, 2 * std::max<int64_t>(M, 1));
    while (nb[0] * nb[1] * nb[2] > cap) {
        int a = 0;
        if (nb[1] > nb[a]) a = 1;
        if (nb[2] > nb[a]) a = 2;
        nb[a] = std::max<long long>(1, (nb[a] * 3) / 4);
    }
    for (int a = 0; a < 3; ++a) {
        g.nb[a] = (int)nb[a];
        g.w[a] = g.L[a] / (double)nb[a];
    }
    // distinct neighbour offsets per axis: -1, 0, +1 wrap onto each other below 3 cells
    int offs[3][3], no[3];
    for (int a = 0; a < 3; ++a) {
        if (nb[a] >= 3) {
            offs[a][0] = -1;
            offs[a][1] = 0;
            offs[a][2] = 1;
            no[a] = 3;
        } else if (nb[a] == 2) {
            offs[a][0] = 0;
            offs[a][1] = 1;
            no[a] = 2;
        } else {
            offs[a][0] = 0;
            no[a] = 1;
        }
    }
    g.nnb = 0;
    for (int i = 0; i < no[0]; ++i)
        for (int j = 0; j < no[1]; ++j)
            for (int k = 0; k < no[2]; ++k) {
                g.off[g.nnb][0] = (signed char)offs[0][i];
                g.off[g.nnb][1] = (signed char)offs[1][j];
                g.off[g.nnb][2] = (signed char)offs[2][k];
                ++g.nnb;
            }
    return g;
}

bool chain_points_in_box(const ChainGeom& g, const double* xyz, int64_t M)
{
    for (int64_t i = 0; i < M; ++i)
        for (int a = 0; a < 3; ++a) {
            const double v = xyz[3 * i + a];
            const double eps = 1e-9 * g.L[a];
            if (!(v >= g.lo[a] - eps && v <= g.lo[a] + g.L[a] + eps)) return false;
        }
    return true;
}


void chain_buffers_release(ChainBuffers& b, int64_t* held)
{
    cudaFree(b.ws);
    cudaFree(b.edges);
    if (held) *held -= (int64_t)(b.ws_bytes + b.edge_bytes);
    b = ChainBuffers{};
}

#define CH_CK(call)                                                                          \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            set_error(std::string("string length: ") + #call + ": " + cudaGetErrorString(e_)); \
            return LAT_ERR_CUDA;                                                             \
        }                                                                                    \
    } while (0)

int chain_length_run(const ChainGeom& g, const double* d_xyz, int64_t M, int split, int method, ChainBuffers& buf,
                     int64_t* held, cudaStream_t st, double* out, int64_t* launches)
{
    out[0] = out[1] = 0.0;
    if (M <= 0) return LAT_OK;
    if (M >= (int64_t)INT_MAX / 2) {
        set_error("string length: too many crossings");
        return LAT_ERR_INVALID;
    }
    if (method != LAT_CHAIN_HASH && method != LAT_CHAIN_EXHAUSTIVE) {
        set_error("string length: method must be resolved");
        return LAT_ERR_INVALID;
    }
    int grid = 1, rc;
    if (method == LAT_CHAIN_EXHAUSTIVE && (rc = coop_grid(M, &grid))) return rc;
    size_t need = 0;
    carve(nullptr, g, M, method, grid, &need);
    if ((rc = grow(&buf.ws, &buf.ws_bytes, need, held))) return rc;
    ChainDev c = carve(buf.ws, g, M, method, grid, &need);
    c.xyz = d_xyz;
    c.M = (int)M;
    c.split = split ? 1 : 0;
    int64_t nl = 0;
    CH_CK(cudaMemsetAsync(c.counters, 0, 4 * sizeof(int), st));
    if (method == LAT_CHAIN_EXHAUSTIVE) {
        CH_CK(cudaMemsetAsync(c.bar, 0, 2 * sizeof(unsigned), st));
        c.wait_polls = g_wait_polls.load();
        c.missing = g_missing.load();
        void* args[] = {(void*)&c};
        CH_CK(cudaLaunchCooperativeKernel((const void*)walk_coop_kernel, dim3(grid), dim3(EX_T), args, 0, st));
        ++nl;
    } else {
        const int tb = 256;
        const int blocks = (int)((M + tb - 1) / tb);
        const size_t cnt_bytes = sizeof(int) * (size_t)c.nbins;
        CH_CK(cudaMemsetAsync(c.bin_cnt, 0, cnt_bytes, st));
        bin_count_kernel<<<blocks, tb, 0, st>>>(c);
        CH_CK(exclusive_scan(c.bin_cnt, c.nbins, c.bin_start, 1, c.scan_tot, c.scan_sum, st, &nl));
        CH_CK(cudaMemsetAsync(c.bin_cnt, 0, cnt_bytes, st));
        bin_scatter_kernel<<<blocks, tb, 0, st>>>(c);
        adj_count_kernel<<<blocks, tb, 0, st>>>(c);
        CH_CK(exclusive_scan(c.deg, M, c.adj_start, 1, c.scan_tot, c.scan_sum, st, &nl));
        long long E = 0;
        CH_CK(cudaMemcpyAsync(&E, c.adj_start + M, sizeof(E), cudaMemcpyDeviceToHost, st));
        CH_CK(cudaStreamSynchronize(st));
        const size_t ebytes = sizeof(AdjEdge) * (size_t)E + 256 + (size_t)E;
        if ((rc = grow(&buf.edges, &buf.edge_bytes, ebytes, held))) return rc;
        c.adj = (AdjEdge*)buf.edges;
        c.edge_dead = (unsigned char*)buf.edges + ((sizeof(AdjEdge) * (size_t)E + 255) & ~(size_t)255);
        adj_fill_kernel<<<blocks, tb, 0, st>>>(c);
        adj_link_kernel<<<blocks, tb, 0, st>>>(c);
        flatten_kernel<<<blocks, tb, 0, st>>>(c);
        const int wgrid = (int)std::min<int64_t>(152 * 8, (M + WALK_WARPS - 1) / WALK_WARPS);
        walk_kernel<<<wgrid, 32 * WALK_WARPS, 0, st>>>(c);
        CH_CK(exclusive_scan(c.chain_len, M, c.chain_off, 0, c.scan_tot, c.scan_sum, st, &nl));
        order_kernel<<<blocks, tb, 0, st>>>(c);
        sum_kernel<<<1, 32, 0, st>>>(c);
        nl += 10;
    }
    CH_CK(cudaGetLastError());
    int err = 0;
    CH_CK(cudaMemcpyAsync(out, c.out, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
    CH_CK(cudaMemcpyAsync(&err, c.counters + 2, sizeof(int), cudaMemcpyDeviceToHost, st));
    CH_CK(cudaStreamSynchronize(st));
    if (launches) *launches += nl;
    if (err) {
        out[0] = out[1] = 0.0;
        set_error(err == CHAIN_ERR_UNION     ? "string length: union-find retry bound reached"
                  : err == CHAIN_ERR_BARRIER ? "string length: a grid barrier wait timed out"
                                             : "string length: inconsistent component walk");
        return (err == CHAIN_ERR_UNION || err == CHAIN_ERR_BARRIER) ? LAT_ERR_TIMEOUT : LAT_ERR_STATE;
    }
    return LAT_OK;
}

}  // namespace lat

extern "C" int lat_set_chain_wait(int64_t polls, int32_t missing_arrivals)
{
    using namespace lat;
    if (polls < 0 || missing_arrivals < 0 || missing_arrivals > 1024) {
        set_error("lat_set_chain_wait: polls >= 0 and 0 <= missing_arrivals <= 1024");
        return LAT_ERR_INVALID;
    }
    g_wait_polls.store(polls ? (long long)polls : kDefaultWaitPolls);
    g_missing.store((unsigned)missing_arrivals);
    return LAT_OK;
}

extern "C" int lat_string_length_points(const lat_params* p, const double* xyz, int64_t M, int32_t split,
                                        int32_t method, double* L0, double* L1)
{
    using namespace lat;
    if (!p || !L0 || !L1 || M < 0 || (M > 0 && !xyz) || p->nx < 1 || p->ny < 1 || p->nz < 1 ||
        !(p->dx > 0) || !(p->dy > 0) || !(p->dz > 0) || method < LAT_CHAIN_AUTO || method > LAT_CHAIN_EXHAUSTIVE) {
        set_error("lat_string_length_points: invalid argument");
        return LAT_ERR_INVALID;
    }
    *L0 = *L1 = 0.0;
    if (M == 0) return LAT_OK;
    const ChainGeom g = make_chain_geom(*p, M);
    const bool hashable = g.periodic[0] && g.periodic[1] && g.periodic[2] && chain_points_in_box(g, xyz, M);
    if (method == LAT_CHAIN_HASH && !hashable) {
        set_error("lat_string_length_points: the hash needs a periodic lattice and points inside the box");
        return LAT_ERR_INVALID;
    }
    if (method == LAT_CHAIN_AUTO) method = hashable ? LAT_CHAIN_HASH : LAT_CHAIN_EXHAUSTIVE;
    cudaStream_t st = nullptr;
    double* d_xyz = nullptr;
    ChainBuffers buf;
    int rc = LAT_OK;
    double out[2] = {0.0, 0.0};
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&d_xyz, sizeof(double) * 3 * (size_t)M);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_xyz, xyz, sizeof(double) * 3 * (size_t)M, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) {
        set_error(std::string("lat_string_length_points: ") + cudaGetErrorString(e));
        rc = e == cudaErrorMemoryAllocation ? LAT_ERR_NOMEM : LAT_ERR_CUDA;
    } else {
        rc = chain_length_run(g, d_xyz, M, split, method, buf, nullptr, st, out, nullptr);
    }
    if (st) cudaStreamSynchronize(st);
    chain_buffers_release(buf, nullptr);
    cudaFree(d_xyz);
    if (st) cudaStreamDestroy(st);
    if (rc == LAT_OK) {
        *L0 = out[0];
        *L1 = out[1];
    }
    return rc;
}
