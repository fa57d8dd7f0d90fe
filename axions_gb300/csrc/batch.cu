// Batched stepping of many independent lattices ("ensemble" and serving).
//
// The reference runs one lattice per program invocation; an ensemble of small
// lattices (different seeds, couplings and sizes) is a loop of separate runs.
// Here every lattice of a batch advances in the same kernel launch: a
// persistent grid (one or two CTAs per SM) walks a table of work items, one
// item per (lattice, y/z tile, x-chunk) of the FP32 step: the pair tile
// (pair_step.cuh, two z-sites per thread) where the lattice's layout allows
// it, else the tiled step's tile (tiled_step.cuh).  A call advancing K steps is one CUDA graph: a copy of the
// K per-step job tables from pinned host memory, then for each step the step
// kernel and a per-lattice diagnostic reduction.  The graph is reused as long
// as K is; lattices join and leave between calls by rewriting the tables.
//
// Each lattice's arithmetic uses only its own fields and coefficients and the
// same tile decomposition as the single-lattice path, and its diagnostics are
// reduced in a fixed order; so a lattice gives bitwise the same result alone,
// in any mix, and through lat_step on its own handle.
#include <algorithm>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "lattice_handle.hpp"
#include "pair_step.cuh"
#include "tiled_step.cuh"

namespace lat {

constexpr int kBatchMaxJobs = 256;

struct BatchJob {
    Geom g;
    Fields<float, 7> f;     // AH uses the first 5 components
    union {
        StepCoefT<float> c;  // tiled tile
        PairCoef pc;         // pair tile
    };
    Charges<float> ch;
    DiagOut d;
    int ns;                 // scalars: 1 (AH) or 2 (Moore)
    int diag;               // record diagnostics at this step
    int chunk;
    int vec;                // 16-byte staging (tiled_vec_ok)
    int pair;               // the pair tile (pair_ok); else the tiled tile
    int tiles_z, tiles_y;
    int items;              // tiles_z * tiles_y * x-chunks
    int item_begin;         // first work item of this job in the step
    double* diag_out;       // finalized (energy, |G|) of this step
};

struct BatchStep {
    int njobs;
    int total_items;
    int begin[kBatchMaxJobs];  // jobs[q].item_begin, contiguous for the item -> job lookup
    BatchJob jobs[kBatchMaxJobs];
};

// x-planes per work item of a lattice in a batch: long x-ranges (one
// prologue per 64 planes), but at least two x-chunks for x-ranges up to 32
// planes, where a single chunk leaves too few items per lattice.  Chosen from
// a sweep of 4..128 on ensembles of 32^3, 64^3 and 128^3 lattices.
int batch_chunk(const Geom& g)
{
    const int x = g.hix - g.lox;
    return std::min(x, x <= 32 ? 16 : 64);
}

namespace {

template <int NS, bool PAIR, bool DIAG, bool Q12>
__device__ __forceinline__ void run_item(unsigned char* smem_raw, const BatchJob& J, const Fields<float, 5>& f5,
                                         int bx, int by, int bz, double* part)
{
    if constexpr (PAIR) {
        PairSmem<NS>& ps = *reinterpret_cast<PairSmem<NS>*>(smem_raw);
        if constexpr (NS == 1) pair_tile<1, DIAG>(ps, J.g, f5, J.pc, J.ch, J.d, bx, by, bz, J.chunk, part);
        else pair_tile<2, DIAG, false, Q12>(ps, J.g, J.f, J.pc, J.ch, J.d, bx, by, bz, J.chunk, part);
        return;
    }
    TiledSmem<float, NS>& sm = *reinterpret_cast<TiledSmem<float, NS>*>(smem_raw);
    if constexpr (NS == 1) {
        tiled_tile<float, 1, DIAG>(sm, J.g, f5, J.c, J.ch, J.d, bx, by, bz, J.chunk, part, J.vec != 0);
    } else {
        tiled_tile<float, 2, DIAG>(sm, J.g, J.f, J.c, J.ch, J.d, bx, by, bz, J.chunk, part, J.vec != 0);
    }
}

// Persistent step kernel for the lattices with NS scalars that use the pair
// tile (PAIR) or the tiled tile: CTAs stride over the work items of all of
// them.  One kernel per model and tile keeps each kernel's register use to
// that tile's: four 4-warp CTAs per SM for the pair tile, as the pair step,
// four (Abelian-Higgs) or three (Moore) 8-warp CTAs for the tiled tile.  Q12:
// the Moore pair lattices with charges 1 and 2, whose link factors the tile
// forms in closed form (pair_step.cuh).
template <int NS, bool PAIR, bool Q12 = false>
__global__ void __launch_bounds__(PAIR ? PT_THREADS : TT_THREADS, PAIR ? 4 : (NS == 1 ? 4 : 3))
batch_step_kernel(const BatchStep* __restrict__ tab)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ BatchJob sj;
    __shared__ Fields<float, 5> sf5;  // Abelian-Higgs view of sj.f
    __shared__ int s_job;
    const int total = tab->total_items;
    const int nj = tab->njobs;
    const int tid = threadIdx.y * TT_Z + threadIdx.x;
    for (int w = blockIdx.x; w < total; w += gridDim.x) {
        if (tid < 32) {
            // the job of item w: jobs whose first item is <= w, counted by one
            // warp over the contiguous begin[] (all loads independent)
            int cnt = 0;
#pragma unroll
            for (int r = 0; r < kBatchMaxJobs / 32; ++r) {
                const int q = r * 32 + tid;
                const bool le = q < nj && tab->begin[q] <= w;
                cnt += __popc(__ballot_sync(0xffffffffu, le));
            }
            if (tid == 0) s_job = cnt - 1;
        }
        __syncthreads();
        // stage the job descriptor in shared memory (its coefficients are read
        // throughout the tile)
        {
            const int* src = reinterpret_cast<const int*>(&tab->jobs[s_job]);
            int* dst = reinterpret_cast<int*>(&sj);
            const int nthreads = (int)(blockDim.x * blockDim.y);
            for (int q = tid; q < (int)(sizeof(BatchJob) / sizeof(int)); q += nthreads) dst[q] = src[q];
            if (tid < 5) {
                sf5.now[tid] = tab->jobs[s_job].f.now[tid];
                sf5.past[tid] = tab->jobs[s_job].f.past[tid];
            }
        }
        __syncthreads();
        const int local = w - sj.item_begin;
        const int bx = local % sj.tiles_z;
        const int r = local / sj.tiles_z;
        const int by = r % sj.tiles_y;
        const int bz = r / sj.tiles_y;
        double* part = sj.diag ? sj.d.partials + 2 * local : nullptr;
        if (sj.diag) run_item<NS, PAIR, true, Q12>(smem_raw, sj, sf5, bx, by, bz, part);
        else run_item<NS, PAIR, false, Q12>(smem_raw, sj, sf5, bx, by, bz, part);
        __syncthreads();  // sj and the tile's shared memory are reused by the next item
    }
}

// Per-job reduction of the diagnostic partials, in the same fixed order as the
// single-lattice path (misc.cu finalize_kernel).
__global__ void __launch_bounds__(1024) batch_finalize_kernel(const BatchStep* __restrict__ tab)
{
    const int jid = blockIdx.x;
    if (jid >= tab->njobs) return;
    const BatchJob& J = tab->jobs[jid];
    if (!J.diag) return;
    __shared__ double se[1024], sg[1024];
    double e = 0, ce = 0, g = 0, cg = 0;
    for (int b = threadIdx.x; b < J.items; b += 1024) {
        const double x = J.d.partials[2 * b], y = J.d.partials[2 * b + 1];
        double t = e + x;
        ce += (fabs(e) >= fabs(x)) ? (e - t) + x : (x - t) + e;
        e = t;
        t = g + y;
        cg += (fabs(g) >= fabs(y)) ? (g - t) + y : (y - t) + g;
        g = t;
    }
    se[threadIdx.x] = e + ce;
    sg[threadIdx.x] = g + cg;
    __syncthreads();
    for (int w = 512; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            se[threadIdx.x] += se[threadIdx.x + w];
            sg[threadIdx.x] += sg[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        J.diag_out[0] = se[0];
        J.diag_out[1] = sg[0];
    }
}

template <int NS, bool PAIR>
size_t batch_smem_ns()
{
    return PAIR ? sizeof(PairSmem<NS>) : sizeof(TiledSmem<float, NS>);
}

// job tables per step: [tiled AH, tiled Moore, pair AH, pair Moore, pair Moore
// with charges 1 and 2]
constexpr int kTables = 5;

}  // namespace

}  // namespace lat

using namespace lat;

struct lat_batch {
    struct Job {
        lat_handle* h;
        int32_t diag_every;
        int64_t stop_step;          // the job advances until its time step reaches this
        std::vector<lat_diag> diags;  // recorded, not yet taken
    };
    std::vector<Job> jobs;
    int device = 0;
    int max_jobs = 0;
    cudaStream_t stream = nullptr;
    int grid[kTables] = {};          // persistent CTAs of each step kernel (table order)
    int K = 0;                       // steps in the captured graph
    unsigned mask = 0;               // tables whose kernels the graph launches
    int chunk = 0;                   // x-planes per work item; 0: the per-shape rule
    BatchStep* tab_host = nullptr;   // pinned [K][kTables]: per step, the jobs of each kernel
    BatchStep* tab_dev = nullptr;    // [K][kTables]
    double* diag_dev = nullptr;      // [K][max_jobs][2]
    double* diag_host = nullptr;     // pinned copy
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t launches = 0;
};

#define BATCH_CK(call)                                                             \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess) {                                                   \
            set_error(std::string(#call) + ": " + cudaGetErrorString(e_));         \
            return e_ == cudaErrorMemoryAllocation ? LAT_ERR_NOMEM : LAT_ERR_CUDA; \
        }                                                                          \
    } while (0)

static void release_graph(lat_batch* b)
{
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    cudaFreeHost(b->tab_host);
    cudaFree(b->tab_dev);
    cudaFree(b->diag_dev);
    cudaFreeHost(b->diag_host);
    b->exec = nullptr;
    b->graph = nullptr;
    b->tab_host = nullptr;
    b->tab_dev = nullptr;
    b->diag_dev = nullptr;
    b->diag_host = nullptr;
    b->K = 0;
}

// Build (or reuse) the graph of K steps, launching per step the step and
// finalize kernels of the tables in `mask` only (an empty table's launches
// cost more than a 32^3 lattice's step).
static int ensure_graph(lat_batch* b, int K, unsigned mask)
{
    if (b->K == K && b->mask == mask && b->exec) return LAT_OK;
    release_graph(b);
    BATCH_CK(cudaMallocHost((void**)&b->tab_host, sizeof(BatchStep) * kTables * (size_t)K));
    BATCH_CK(cudaMalloc((void**)&b->tab_dev, sizeof(BatchStep) * kTables * (size_t)K));
    BATCH_CK(cudaMalloc((void**)&b->diag_dev, sizeof(double) * 2 * (size_t)K * b->max_jobs));
    BATCH_CK(cudaMallocHost((void**)&b->diag_host, sizeof(double) * 2 * (size_t)K * b->max_jobs));
    BATCH_CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    cudaMemcpyAsync(b->tab_dev, b->tab_host, sizeof(BatchStep) * kTables * (size_t)K, cudaMemcpyHostToDevice,
                    b->stream);
    for (int s = 0; s < K; ++s) {
        BatchStep* t = b->tab_dev + kTables * s;
        const dim3 tt(TT_Z, TT_Y), pt(PT_TZ, PT_Y);
        if (mask & 1u) batch_step_kernel<1, false><<<b->grid[0], tt, batch_smem_ns<1, false>(), b->stream>>>(t);
        if (mask & 2u) batch_step_kernel<2, false><<<b->grid[1], tt, batch_smem_ns<2, false>(), b->stream>>>(t + 1);
        if (mask & 4u) batch_step_kernel<1, true><<<b->grid[2], pt, batch_smem_ns<1, true>(), b->stream>>>(t + 2);
        if (mask & 8u) batch_step_kernel<2, true><<<b->grid[3], pt, batch_smem_ns<2, true>(), b->stream>>>(t + 3);
        if (mask & 16u) batch_step_kernel<2, true, true><<<b->grid[4], pt, batch_smem_ns<2, true>(), b->stream>>>(t + 4);
        for (int q = 0; q < kTables; ++q)
            if (mask & (1u << q)) batch_finalize_kernel<<<b->max_jobs, 1024, 0, b->stream>>>(t + q);
    }
    cudaMemcpyAsync(b->diag_host, b->diag_dev, sizeof(double) * 2 * (size_t)K * b->max_jobs, cudaMemcpyDeviceToHost,
                    b->stream);
    BATCH_CK(cudaStreamEndCapture(b->stream, &b->graph));
    BATCH_CK(cudaGraphInstantiate(&b->exec, b->graph, 0));
    b->K = K;
    b->mask = mask;
    return LAT_OK;
}

// The table (step kernel) of a lattice: the pair tile where its own layout
// allows it, else the tiled tile; its model; for a Moore pair lattice whether
// its charges are 1 and 2.  The choice depends on the lattice alone, never on
// its company.
static int table_of(const lat_handle* h, const Fields<float, 7>& fj)
{
    Fields<float, 5> f5;
    for (int c = 0; c < 5; ++c) {
        f5.now[c] = fj.now[c];
        f5.past[c] = fj.past[c];
    }
    const bool moore = h->p.model == LAT_MODEL_MOORE;
    const bool pair = moore ? pair_ok(h->geom, fj) : pair_ok(h->geom, f5);
    const bool q12 = moore && pair && small_int_power(h->p.q1) == 1 && small_int_power(h->p.q2) == 2;
    return q12 ? 4 : (pair ? 2 : 0) + (moore ? 1 : 0);
}

static Fields<float, 7> level_fields(const lat_handle* h, int64_t n)
{
    const int tNow = (int)((n + 1) % 2), tPast = (int)(n % 2);
    Fields<float, 7> fj{};
    for (int c = 0; c < h->ncomp; ++c) {
        fj.now[c] = (const float*)h->slot(c, tNow);
        fj.past[c] = (float*)h->slot(c, tPast);
    }
    return fj;
}

extern "C" {

int lat_batch_create(int32_t max_jobs, lat_batch** out)
{
    if (!out || max_jobs < 1 || max_jobs > kBatchMaxJobs) {
        set_error("lat_batch_create: max_jobs must be in [1, 256]");
        return LAT_ERR_INVALID;
    }
    *out = nullptr;
    lat_batch* b = new lat_batch();
    b->max_jobs = max_jobs;
    cudaGetDevice(&b->device);
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete b;
        set_error("lat_batch_create: no CUDA device or stream");
        return LAT_ERR_NODEVICE;
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
    auto grid_of = [&](auto kernel, int threads, size_t smem) {
        if (smem > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
        return std::max(1, sms * std::max(1, per_sm));
    };
    b->grid[0] = grid_of(batch_step_kernel<1, false>, TT_THREADS, batch_smem_ns<1, false>());
    b->grid[1] = grid_of(batch_step_kernel<2, false>, TT_THREADS, batch_smem_ns<2, false>());
    b->grid[2] = grid_of(batch_step_kernel<1, true>, PT_THREADS, batch_smem_ns<1, true>());
    b->grid[3] = grid_of(batch_step_kernel<2, true>, PT_THREADS, batch_smem_ns<2, true>());
    b->grid[4] = grid_of(batch_step_kernel<2, true, true>, PT_THREADS, batch_smem_ns<2, true>());
    *out = b;
    return LAT_OK;
}

int lat_batch_destroy(lat_batch* b)
{
    if (!b) return LAT_OK;
    cudaSetDevice(b->device);
    cudaStreamSynchronize(b->stream);
    release_graph(b);
    cudaStreamDestroy(b->stream);
    delete b;
    return LAT_OK;
}

int lat_batch_add(lat_batch* b, lat_handle* h, int32_t diag_every, int64_t stop_step)
{
    if (!b || !h || diag_every < 0) {
        set_error("lat_batch_add: bad argument");
        return LAT_ERR_INVALID;
    }
    if (h->p.precision != LAT_F32 || h->p.kernel_variant != 0) {
        set_error("lat_batch_add: batches step FP32 lattices (LAT_F32, default kernels)");
        return LAT_ERR_INVALID;
    }
    if (h->p.bc > LAT_BC_FIXED || bc_z_kind(h->p) > LAT_BC_FIXED) {
        set_error("lat_batch_add: batches step lattices with periodic or fixed boundaries");
        return LAT_ERR_INVALID;
    }
    if ((int)b->jobs.size() >= b->max_jobs) {
        set_error("lat_batch_add: batch is full");
        return LAT_ERR_CAPACITY;
    }
    for (auto& j : b->jobs)
        if (j.h == h) {
            set_error("lat_batch_add: handle already in the batch");
            return LAT_ERR_STATE;
        }
    b->jobs.push_back({h, diag_every, stop_step, {}});
    return (int)b->jobs.size() - 1;
}

int lat_batch_remove(lat_batch* b, lat_handle* h)
{
    if (!b || !h) {
        set_error("lat_batch_remove: bad argument");
        return LAT_ERR_INVALID;
    }
    for (size_t q = 0; q < b->jobs.size(); ++q)
        if (b->jobs[q].h == h) {
            b->jobs.erase(b->jobs.begin() + (long)q);
            return LAT_OK;
        }
    set_error("lat_batch_remove: handle not in the batch");
    return LAT_ERR_STATE;
}

int lat_batch_size(const lat_batch* b) { return b ? (int)b->jobs.size() : LAT_ERR_INVALID; }

int lat_batch_set_chunk(lat_batch* b, int32_t chunk)
{
    if (!b || chunk < 0 || chunk > 4096) {
        set_error("lat_batch_set_chunk: chunk must be in [0, 4096]");
        return LAT_ERR_INVALID;
    }
    b->chunk = chunk;
    return LAT_OK;
}

int64_t lat_batch_kernel_launches(const lat_batch* b) { return b ? b->launches : LAT_ERR_INVALID; }

int lat_batch_advance(lat_batch* b, int32_t nsteps)
{
    if (!b || nsteps < 1) {
        set_error("lat_batch_advance: bad argument");
        return LAT_ERR_INVALID;
    }
    if (b->jobs.empty()) return 0;
    BATCH_CK(cudaSetDevice(b->device));
    const int K = nsteps;
    // previous work of the handles (uploads, single steps) must be complete
    for (auto& j : b->jobs) BATCH_CK(cudaStreamSynchronize(j.h->stream));
    // host-side schedule of every job over the K steps
    struct Plan {
        int steps;
        int64_t n0;
        int table;
    };
    std::vector<Plan> plan(b->jobs.size());
    unsigned mask = 0;
    for (size_t q = 0; q < b->jobs.size(); ++q) {
        auto& j = b->jobs[q];
        const int64_t left = j.stop_step - j.h->n;
        plan[q] = {(int)std::max<int64_t>(0, std::min<int64_t>(K, left)), j.h->n, table_of(j.h, level_fields(j.h, j.h->n))};
        if (plan[q].steps > 0) mask |= 1u << plan[q].table;
        // a diagnostic on the first step needs the divergence of the past level
        const int64_t n = j.h->n;
        if (plan[q].steps > 0 && j.diag_every > 0 && n % j.diag_every == 0 && j.h->p.g != 0 && !j.h->div_valid) {
            lat_handle* h = j.h;
            const int tPast = (int)(n % 2), th0 = h->ncomp - 3;
            cudaError_t e = launch_divergence_f32(h->geom, (const float*)h->slot(th0, tPast),
                                                  (const float*)h->slot(th0 + 1, tPast),
                                                  (const float*)h->slot(th0 + 2, tPast), make_coef(h->p, n),
                                                  (float*)h->divbuf, b->stream);
            if (e != cudaSuccess) {
                set_error(std::string("lat_batch_advance: ") + cudaGetErrorString(e));
                return LAT_ERR_CUDA;
            }
            ++b->launches;
        }
    }
    int rc = ensure_graph(b, K, mask);
    if (rc) return rc;
    std::vector<std::vector<int>> diag_slots(b->jobs.size());
    for (int s = 0; s < K; ++s) {
        for (int q = 0; q < kTables; ++q) {
            b->tab_host[kTables * s + q].njobs = 0;
            b->tab_host[kTables * s + q].total_items = 0;
        }
        for (size_t q = 0; q < b->jobs.size(); ++q) {
            if (s >= plan[q].steps) continue;
            auto& j = b->jobs[q];
            lat_handle* h = j.h;
            const int64_t n = plan[q].n0 + s;
            const Fields<float, 7> fj = level_fields(h, n);
            const bool pair = plan[q].table >= 2;
            BatchStep& T = b->tab_host[kTables * s + plan[q].table];
            BatchJob& J = T.jobs[T.njobs];
            std::memset(&J, 0, sizeof(J));
            J.g = h->geom;
            J.f = fj;
            const StepCoef c64 = make_coef(h->p, n);
            J.ns = h->p.model == LAT_MODEL_MOORE ? 2 : 1;
            if (J.ns == 1) {
                J.ch.q[0] = 1;
                J.ch.qpow[0] = 1;
            } else {
                J.ch.q[0] = (float)h->p.q1;
                J.ch.q[1] = (float)h->p.q2;
                J.ch.qpow[0] = small_int_power(h->p.q1);
                J.ch.qpow[1] = small_int_power(h->p.q2);
            }
            J.ch.charge_current = h->p.moore_current == LAT_MOORE_CURRENT_CHARGE;
            const bool diag = j.diag_every > 0 && n % j.diag_every == 0;
            const bool next_diag = j.diag_every > 0 && (n + 1) % j.diag_every == 0;
            J.d.partials = h->partials;
            J.d.divbuf = h->divbuf;
            J.d.use_div = 1;
            J.d.store_div = next_diag && h->p.g != 0;  // keep div(theta) for the next step's Gauss term
            J.d.energy_form = h->p.energy_form;
            J.d.charge_current = J.ch.charge_current;
            J.d.write = 1;
            J.diag = diag ? 1 : 0;
            // In a batch the other lattices supply the parallelism, so each
            // lattice marches long x-ranges (batch_chunk).  The value depends
            // on the lattice's own shape only, never on its company, so
            // results do not depend on the mix.
            J.chunk = b->chunk > 0 ? std::min(h->geom.hix - h->geom.lox, b->chunk) : batch_chunk(h->geom);
            J.vec = h->p.kernel_variant != 2 && tiled_vec_ok(h->geom, J.f) ? 1 : 0;
            J.pair = pair ? 1 : 0;
            if (pair) J.pc = pair_coef(c64);
            else J.c = coef_as<float>(c64);
            const dim3 tg = pair ? pair_grid(h->geom, J.chunk) : tiled_grid(h->geom, J.chunk);
            J.tiles_z = (int)tg.x;
            J.tiles_y = (int)tg.y;
            J.items = (int)(tg.x * tg.y * tg.z);
            J.item_begin = T.total_items;
            T.begin[T.njobs] = T.total_items;
            J.diag_out = b->diag_dev + 2 * ((size_t)s * b->max_jobs + (size_t)q);
            T.total_items += J.items;
            ++T.njobs;
            if (diag) diag_slots[q].push_back(s);
        }
    }
    BATCH_CK(cudaGraphLaunch(b->exec, b->stream));
    BATCH_CK(cudaStreamSynchronize(b->stream));
    b->launches += (int64_t)__builtin_popcount(mask) * K;
    int active = 0;
    for (size_t q = 0; q < b->jobs.size(); ++q) {
        auto& j = b->jobs[q];
        lat_handle* h = j.h;
        for (int s : diag_slots[q]) {
            const double* v = b->diag_host + 2 * ((size_t)s * b->max_jobs + q);
            lat_diag dg;
            dg.energy = v[0];
            dg.gauss_abs_sum = v[1];
            const Geom& g = h->geom;
            dg.sites = (int64_t)(g.hix - g.lox) * (g.hiy - g.loy) * (g.hiz - g.loz);
            dg.time_step = plan[q].n0 + s;
            j.diags.push_back(dg);
        }
        if (plan[q].steps > 0) {
            const int64_t nlast = plan[q].n0 + plan[q].steps - 1;
            h->div_valid = j.diag_every > 0 && (nlast + 1) % j.diag_every == 0 && h->p.g != 0;
            h->n = plan[q].n0 + plan[q].steps;
            h->launches += 0;
        }
        if (h->n < j.stop_step) ++active;
    }
    return active;
}

int lat_batch_take_diags(lat_batch* b, lat_handle* h, lat_diag* out, int64_t cap, int64_t* count)
{
    if (!b || !h || !count || (cap > 0 && !out)) {
        set_error("lat_batch_take_diags: bad argument");
        return LAT_ERR_INVALID;
    }
    for (auto& j : b->jobs)
        if (j.h == h) {
            const int64_t n = std::min<int64_t>(cap, (int64_t)j.diags.size());
            for (int64_t q = 0; q < n; ++q) out[q] = j.diags[(size_t)q];
            *count = (int64_t)j.diags.size();
            j.diags.erase(j.diags.begin(), j.diags.begin() + n);
            return LAT_OK;
        }
    set_error("lat_batch_take_diags: handle not in the batch");
    return LAT_ERR_STATE;
}

}  // extern "C"
