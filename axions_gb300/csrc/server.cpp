// Serving loop: a queue of simulation jobs (mixed sizes and models) advanced
// with continuous batching.
//
// The reference runs one job per program invocation (run_mpi_evol.sh,
// submit_job.sh).  Here a worker thread owns one lattice batch (batch.cu):
//   * jobs are admitted from the queue in arrival order while their device
//     footprint fits the HBM budget (a job that does not fit waits, and so do
//     the ones behind it: no job is overtaken);
//   * an admitted job gets a lattice (reused from a pool of idle lattices of
//     the same shape, else allocated), a device-side random-phase IC, and joins
//     the batch; its fields stay on the device until it finishes;
//   * the batch advances `tick_steps` steps at a time (one CUDA graph); jobs
//     that arrive meanwhile join at the next tick, finished ones leave;
//   * a finished job records its diagnostics, the final energy/Gauss values and
//     the total |winding| of its (first) scalar, and its lattice returns to the
//     pool (pooled lattices count against the budget and are freed when a new
//     job needs the room).
// A job's results do not depend on the other jobs in the batch (batch.cu).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "lattice_handle.hpp"

using namespace lat;

namespace lat {
int reconfigure_handle(lat_handle* h, const lat_params* p);
}

namespace {

using Clock = std::chrono::steady_clock;
using ShapeKey = std::tuple<int, int, int, int64_t, int64_t, int64_t>;  // model, precision, bc|bc_z, nx, ny, nz

ShapeKey shape_of(const lat_params& p) { return ShapeKey(p.model, p.precision, p.bc + 16 * p.bc_z, p.nx, p.ny, p.nz); }

struct JobState {
    lat_job_spec spec;
    lat_job_result res;
    std::vector<lat_diag> diags;
    lat_handle* h = nullptr;
    int64_t bytes = 0;
};

}  // namespace

struct lat_server {
    lat_server_config cfg;
    int device = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<int64_t> queue;
    std::map<int64_t, JobState> jobs;
    std::vector<int64_t> running;
    std::multimap<ShapeKey, std::pair<lat_handle*, int64_t>> pool;  // idle lattices and their bytes
    int64_t next_id = 1;
    int64_t running_bytes = 0, pooled_bytes = 0, peak_bytes = 0;
    int64_t done = 0, failed = 0, site_updates = 0, ticks = 0;
    double busy_s = 0;
    bool stop = false;
    Clock::time_point t0;
    lat_batch* batch = nullptr;
    std::thread worker;
    std::string error;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

// Take a lattice for `p`: an idle one of the same shape, else a new one.
int acquire(lat_server* s, const lat_params& p, lat_handle** out, int64_t* bytes)
{
    auto it = s->pool.find(shape_of(p));
    if (it != s->pool.end()) {
        lat_handle* h = it->second.first;
        *bytes = it->second.second;
        s->pooled_bytes -= *bytes;
        s->pool.erase(it);
        int rc = reconfigure_handle(h, &p);
        if (rc == LAT_OK) {
            *out = h;
            return LAT_OK;
        }
        lat_destroy(h);
    }
    int rc = lat_create(&p, out);
    if (rc) return rc;
    *bytes = lat_device_bytes(*out);
    return LAT_OK;
}

// Free idle lattices until `need` more bytes fit the budget.
void make_room(lat_server* s, int64_t need)
{
    while (!s->pool.empty() && s->running_bytes + s->pooled_bytes + need > s->cfg.hbm_budget_bytes) {
        auto it = s->pool.begin();
        s->pooled_bytes -= it->second.second;
        lat_destroy(it->second.first);
        s->pool.erase(it);
    }
}

void finish(lat_server* s, int64_t id, int status)
{
    JobState& j = s->jobs[id];
    if (j.h) {
        int64_t cnt = 0;
        std::vector<lat_diag> d(64);
        for (;;) {
            lat_batch_take_diags(s->batch, j.h, d.data(), (int64_t)d.size(), &cnt);
            const int64_t got = std::min<int64_t>(cnt, (int64_t)d.size());
            j.diags.insert(j.diags.end(), d.begin(), d.begin() + got);
            if (cnt <= (int64_t)d.size()) break;
        }
        lat_batch_remove(s->batch, j.h);
        if (status == 2) {
            // the per-shape chunk of the batch, so that the final diagnostics
            // depend on the job only (not on tuning done elsewhere in the process)
            j.h->chunk = lat::batch_chunk(j.h->geom);
            lat_diag fd;
            if (lat_diagnostics(j.h, &fd) == LAT_OK) {
                j.res.final_energy = fd.energy;
                j.res.final_gauss = fd.gauss_abs_sum;
            }
            if (j.spec.winding_at_end) {
                int64_t w = 0;
                if (lat_winding(j.h, LAT_FIELD_PHI1, nullptr, &w) == LAT_OK) j.res.winding_abs = w;
            }
            j.res.site_updates = (int64_t)j.spec.params.nx * j.spec.params.ny * j.spec.params.nz * j.spec.nsteps;
            s->site_updates += j.res.site_updates;
        }
        s->running_bytes -= j.bytes;
        s->pool.emplace(shape_of(j.spec.params), std::make_pair(j.h, j.bytes));
        s->pooled_bytes += j.bytes;
        j.h = nullptr;
    }
    j.res.status = status;
    j.res.ndiag = (int32_t)j.diags.size();
    j.res.end_s = s->now();
    if (status == 2) ++s->done;
    else ++s->failed;
}

void worker_main(lat_server* s)
{
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lock(s->mu);
    while (true) {
        // admission, in arrival order
        while (!s->queue.empty() && (int)s->running.size() < s->cfg.max_running) {
            const int64_t id = s->queue.front();
            JobState& j = s->jobs[id];
            const int64_t need = lat_footprint_bytes(&j.spec.params);
            if (need > s->cfg.hbm_budget_bytes) {  // can never run
                s->queue.pop_front();
                j.res.status = LAT_ERR_CAPACITY;
                j.res.end_s = s->now();
                ++s->failed;
                continue;
            }
            const bool reuse = s->pool.count(shape_of(j.spec.params)) > 0;
            if (!reuse) make_room(s, need);
            if (!reuse && s->running_bytes + s->pooled_bytes + need > s->cfg.hbm_budget_bytes) break;
            s->queue.pop_front();
            int64_t bytes = 0;
            int rc = acquire(s, j.spec.params, &j.h, &bytes);
            if (rc == LAT_OK) rc = lat_random_phase_ic_device(j.h, j.spec.seed, j.spec.independent);
            if (rc == LAT_OK) rc = lat_batch_add(s->batch, j.h, j.spec.diag_every, j.spec.nsteps) >= 0 ? LAT_OK : rc;
            if (rc != LAT_OK) {
                if (j.h) lat_destroy(j.h);
                j.h = nullptr;
                j.res.status = rc;
                j.res.end_s = s->now();
                ++s->failed;
                continue;
            }
            j.bytes = bytes;
            s->running_bytes += bytes;
            s->peak_bytes = std::max(s->peak_bytes, s->running_bytes + s->pooled_bytes);
            j.res.status = 1;
            j.res.start_s = s->now();
            s->running.push_back(id);
        }
        // jobs refused at admission (too large for the budget, no memory) are
        // finished: wake their waiters before sleeping on new work
        s->cv_done.notify_all();
        if (s->running.empty()) {
            if (s->stop) break;
            s->cv_work.wait(lock);
            continue;
        }
        // one tick of the batch, outside the lock (submissions continue)
        lock.unlock();
        const double t0 = s->now();
        const int active = lat_batch_advance(s->batch, s->cfg.tick_steps);
        const double t1 = s->now();
        lock.lock();
        s->busy_s += t1 - t0;
        ++s->ticks;
        if (active < 0) {
            s->error = lat_last_error();
            for (int64_t id : s->running) finish(s, id, active);
            s->running.clear();
        } else {
            std::vector<int64_t> still;
            for (int64_t id : s->running) {
                JobState& j = s->jobs[id];
                if (lat_time_step(j.h) >= j.spec.nsteps) finish(s, id, 2);
                else still.push_back(id);
            }
            s->running.swap(still);
        }
        s->cv_done.notify_all();
        if (s->stop && s->queue.empty() && s->running.empty()) break;
    }
    s->cv_done.notify_all();
}

}  // namespace

extern "C" {

int lat_server_create(const lat_server_config* cfg, lat_server** out)
{
    if (!cfg || !out || cfg->hbm_budget_bytes <= 0 || cfg->tick_steps < 1 || cfg->max_running < 1 ||
        cfg->max_running > 256) {
        set_error("lat_server_create: bad configuration (budget > 0, tick_steps >= 1, max_running in [1, 256])");
        return LAT_ERR_INVALID;
    }
    *out = nullptr;
    lat_server* s = new lat_server();
    s->cfg = *cfg;
    cudaGetDevice(&s->device);
    int rc = lat_batch_create(cfg->max_running, &s->batch);
    if (rc) {
        delete s;
        return rc;
    }
    s->t0 = Clock::now();
    s->worker = std::thread(worker_main, s);
    *out = s;
    return LAT_OK;
}

int lat_server_submit(lat_server* s, const lat_job_spec* spec, int64_t* job_id)
{
    if (!s || !spec || !job_id || spec->nsteps < 0 || spec->diag_every < 0) {
        set_error("lat_server_submit: bad argument");
        return LAT_ERR_INVALID;
    }
    if (spec->params.precision != LAT_F32) {
        set_error("lat_server_submit: served jobs run the FP32 path (params.precision = LAT_F32)");
        return LAT_ERR_INVALID;
    }
    if (lat_footprint_bytes(&spec->params) < 0) return LAT_ERR_INVALID;
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->stop) {
        set_error("lat_server_submit: server is shutting down");
        return LAT_ERR_STATE;
    }
    const int64_t id = s->next_id++;
    JobState& j = s->jobs[id];
    j.spec = *spec;
    std::memset(&j.res, 0, sizeof(j.res));
    j.res.job_id = id;
    j.res.status = 0;
    j.res.submit_s = s->now();
    s->queue.push_back(id);
    *job_id = id;
    s->cv_work.notify_one();
    return LAT_OK;
}

int lat_server_poll(lat_server* s, int64_t job_id, lat_job_result* out)
{
    if (!s || !out) {
        set_error("lat_server_poll: bad argument");
        return LAT_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->jobs.find(job_id);
    if (it == s->jobs.end()) {
        set_error("lat_server_poll: unknown job");
        return LAT_ERR_INVALID;
    }
    *out = it->second.res;
    return LAT_OK;
}

int lat_server_wait(lat_server* s, int64_t job_id, double timeout_s, lat_job_result* out)
{
    if (!s || !out) {
        set_error("lat_server_wait: bad argument");
        return LAT_ERR_INVALID;
    }
    std::unique_lock<std::mutex> lock(s->mu);
    auto it = s->jobs.find(job_id);
    if (it == s->jobs.end()) {
        set_error("lat_server_wait: unknown job");
        return LAT_ERR_INVALID;
    }
    const auto deadline = Clock::now() + std::chrono::duration<double>(timeout_s);
    while (it->second.res.status == 0 || it->second.res.status == 1) {
        if (s->cv_done.wait_until(lock, deadline) == std::cv_status::timeout) {
            *out = it->second.res;
            set_error("lat_server_wait: timed out");
            return LAT_ERR_TIMEOUT;
        }
    }
    *out = it->second.res;
    return LAT_OK;
}

int lat_server_diags(lat_server* s, int64_t job_id, lat_diag* out, int64_t cap, int64_t* count)
{
    if (!s || !count || (cap > 0 && !out)) {
        set_error("lat_server_diags: bad argument");
        return LAT_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->jobs.find(job_id);
    if (it == s->jobs.end()) {
        set_error("lat_server_diags: unknown job");
        return LAT_ERR_INVALID;
    }
    const auto& d = it->second.diags;
    *count = (int64_t)d.size();
    for (int64_t q = 0; q < std::min<int64_t>(cap, (int64_t)d.size()); ++q) out[q] = d[(size_t)q];
    return LAT_OK;
}

int lat_server_get_stats(lat_server* s, lat_server_stats* out)
{
    if (!s || !out) {
        set_error("lat_server_get_stats: bad argument");
        return LAT_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(s->mu);
    out->submitted = s->next_id - 1;
    out->queued = (int64_t)s->queue.size();
    out->running = (int64_t)s->running.size();
    out->done = s->done;
    out->failed = s->failed;
    out->site_updates = s->site_updates;
    out->ticks = s->ticks;
    out->running_bytes = s->running_bytes;
    out->pooled_bytes = s->pooled_bytes;
    out->peak_bytes = s->peak_bytes;
    out->busy_s = s->busy_s;
    out->wall_s = s->now();
    return LAT_OK;
}

int lat_server_destroy(lat_server* s)
{
    if (!s) return LAT_OK;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stop = true;
        s->queue.clear();  // queued jobs are dropped; running ones finish
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    for (auto& kv : s->pool) lat_destroy(kv.second.first);
    for (auto& kv : s->jobs)
        if (kv.second.h) lat_destroy(kv.second.h);
    lat_batch_destroy(s->batch);
    delete s;
    return LAT_OK;
}

}  // extern "C"
