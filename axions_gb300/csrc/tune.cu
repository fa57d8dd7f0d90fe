// Autotuning of the tiled FP32 step: the number of x-planes each CTA marches
// through ("chunk").  Short chunks give small lattices enough CTAs to fill the
// 152 SMs; long chunks spend less on each CTA's prologue (one extra plane of
// link data and the pipeline fill).  lat_autotune() times every candidate on a
// scratch lattice of the caller's shape (device-generated IC, the caller's
// state is not touched), applies the fastest to the handle and remembers it
// per shape; new handles of a tuned shape start with the remembered value and
// untuned ones with a heuristic that aims at four CTAs per SM.  The cache can
// be saved to and loaded from a small JSON file.
#include <algorithm>
#include <cstdio>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <tuple>
#include <vector>

#include "lattice_handle.hpp"

using namespace lat;

namespace {

using Key = std::tuple<int, int, int, int64_t, int64_t, int64_t>;  // model, precision, bc, nx, ny, nz

struct Entry {
    int chunk;
    double ms;
};

std::mutex g_tune_mu;
std::map<Key, Entry> g_tune;

Key key_of(const lat_params& p) { return Key(p.model, p.precision, p.bc, p.nx, p.ny, p.nz); }

const int kCandidates[] = {4, 8, 16, 32, 64, 128};

}  // namespace

namespace lat {

// Default chunk for a handle: the tuned value of its shape, else the largest
// candidate that still gives about four CTAs per SM.
int default_chunk(const lat_params& p)
{
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        auto it = g_tune.find(key_of(p));
        if (it != g_tune.end()) return it->second.chunk;
    }
    const Geom g = make_geom(p);
    const int64_t cols = (int64_t)((g.hiz - g.loz + 31) / 32) * ((g.hiy - g.loy + 7) / 8);
    const int64_t want = 4 * 152;
    int best = kCandidates[0];
    for (int c : kCandidates)
        if (cols * ((g.hix - g.lox + c - 1) / c) >= want) best = c;
    return best;
}

}  // namespace lat

extern "C" {

int lat_get_tuning(const lat_handle* h, lat_tuning* out)
{
    if (!h || !out) {
        set_error("lat_get_tuning: null argument");
        return LAT_ERR_INVALID;
    }
    out->chunk = h->chunk;
    out->candidates = 0;
    out->ms_per_step = 0;
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune.find(key_of(h->p));
    if (it != g_tune.end() && it->second.chunk == h->chunk) out->ms_per_step = it->second.ms;
    return LAT_OK;
}

int lat_set_tuning(lat_handle* h, const lat_tuning* t)
{
    if (!h || !t || t->chunk < 1) {
        set_error("lat_set_tuning: bad argument");
        return LAT_ERR_INVALID;
    }
    h->chunk = t->chunk;
    return LAT_OK;
}

int lat_autotune(lat_handle* h, int32_t trial_steps, lat_tuning* out)
{
    if (!h || trial_steps < 1) {
        set_error("lat_autotune: bad argument");
        return LAT_ERR_INVALID;
    }
    if (h->elem != 4 || h->p.kernel_variant == 1) {  // only the tiled FP32 step has a chunk
        if (out) {
            out->chunk = h->chunk;
            out->candidates = 0;
            out->ms_per_step = 0;
        }
        return LAT_OK;
    }
    lat_handle* t = nullptr;
    int rc = lat_create(&h->p, &t);
    if (rc) return rc;
    rc = lat_random_phase_ic_device(t, 12345, 1);
    if (rc) {
        lat_destroy(t);
        return rc;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const Geom& g = h->geom;
    double best_ms = 1e300;
    int best = h->chunk, tried = 0;
    for (int c : kCandidates) {
        if (c > 2 * (g.hix - g.lox) && c != kCandidates[0]) continue;  // beyond the lattice: same as a shorter one
        t->chunk = c;
        if ((rc = lat_step(t, 1))) break;  // warm-up
        cudaEventRecord(e0, t->stream);
        if ((rc = lat_step(t, trial_steps))) break;
        cudaEventRecord(e1, t->stream);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        ++tried;
        if (ms / trial_steps < best_ms) {
            best_ms = ms / trial_steps;
            best = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    lat_destroy(t);
    if (rc) return rc;
    h->chunk = best;
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tune[key_of(h->p)] = {best, best_ms};
    }
    if (out) {
        out->chunk = best;
        out->candidates = tried;
        out->ms_per_step = best_ms;
    }
    return LAT_OK;
}

int lat_tune_cache_save(const char* path)
{
    if (!path) {
        set_error("lat_tune_cache_save: null path");
        return LAT_ERR_INVALID;
    }
    std::ofstream o(path);
    if (!o) {
        set_error(std::string("lat_tune_cache_save: cannot write ") + path);
        return LAT_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(g_tune_mu);
    o << "{\"chunk\": [";
    bool first = true;
    for (auto& kv : g_tune) {
        const Key& k = kv.first;
        o << (first ? "" : ",") << "\n  {\"model\": " << std::get<0>(k) << ", \"precision\": " << std::get<1>(k)
          << ", \"bc\": " << std::get<2>(k) << ", \"nx\": " << std::get<3>(k) << ", \"ny\": " << std::get<4>(k)
          << ", \"nz\": " << std::get<5>(k) << ", \"chunk\": " << kv.second.chunk << ", \"ms\": " << kv.second.ms
          << "}";
        first = false;
    }
    o << "\n]}\n";
    return o.good() ? LAT_OK : LAT_ERR_INVALID;
}

// Reads files written by lat_tune_cache_save: one entry per line.
int lat_tune_cache_load(const char* path)
{
    if (!path) {
        set_error("lat_tune_cache_load: null path");
        return LAT_ERR_INVALID;
    }
    std::ifstream in(path);
    if (!in) {
        set_error(std::string("lat_tune_cache_load: cannot read ") + path);
        return LAT_ERR_INVALID;
    }
    std::string line;
    int loaded = 0;
    auto field = [](const std::string& l, const char* name, double& v) {
        const std::string pat = std::string("\"") + name + "\": ";
        const size_t at = l.find(pat);
        if (at == std::string::npos) return false;
        v = std::strtod(l.c_str() + at + pat.size(), nullptr);
        return true;
    };
    while (std::getline(in, line)) {
        double m, pr, bc, nx, ny, nz, ch, ms;
        if (field(line, "model", m) && field(line, "precision", pr) && field(line, "bc", bc) && field(line, "nx", nx) &&
            field(line, "ny", ny) && field(line, "nz", nz) && field(line, "chunk", ch) && field(line, "ms", ms) &&
            ch >= 1) {
            std::lock_guard<std::mutex> lock(g_tune_mu);
            g_tune[Key((int)m, (int)pr, (int)bc, (int64_t)nx, (int64_t)ny, (int64_t)nz)] = {(int)ch, ms};
            ++loaded;
        }
    }
    return loaded;
}

}  // extern "C"
