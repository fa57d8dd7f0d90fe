// Drop-in host programs: see evolve.hpp.
#include "evolve.hpp"

#include <sys/stat.h>
#include <sys/time.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <random>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "ic_io.hpp"
#include "lattice_gpu.h"
#include "sor.hpp"

namespace axh {

namespace {

bool is_moore(Program p) { return p == Program::MooreMpiEvolution || p == Program::MooreEvol; }
bool is_mpi(Program p) { return p == Program::MpiEvolution || p == Program::MooreMpiEvolution; }

std::string trim(const std::string& s)
{
    const size_t a = s.find_first_not_of(" \t\r\n");
    if (a == std::string::npos) return "";
    const size_t b = s.find_last_not_of(" \t\r\n");
    return s.substr(a, b - a + 1);
}

void fail(const std::string& msg)
{
    throw std::runtime_error(msg);
}

void check(int rc, const char* what)
{
    if (rc != LAT_OK) fail(std::string(what) + " failed (" + std::to_string(rc) + "): " + lat_last_error());
}

}  // namespace

// Reference defaults: mpi_evolution.cpp:17-57, evolution.cpp:23-56,
// moore_mpi_evolution.cpp:17-63, mooreEvol.cpp:19-41.
Params::Params(Program prog)
{
    auto& v = vals_;
    v["precision"] = "f64";     // f64 | f32 | f64_fast  (this library)
    v["out_dir"] = ".";         // where Data/ and GifData/ live (reference: next to its source)
    v["digits"] = "6";          // ostream precision of the text output (reference default 6)
    v["countRate"] = "10";
    // initial-condition table under Data/: the reference's text file, or its
    // binary form (ic_io.hpp); MPI programs read it for ic_type = data
    v["ic_file"] = is_moore(prog) ? "moore_ic.txt" : "ic.txt";
    v["scaling"] = "1";
    switch (prog) {
    case Program::MpiEvolution:
        v["nx"] = v["ny"] = v["nz"] = "1001";
        v["nt"] = "2501";
        v["dx"] = v["dy"] = v["dz"] = "0.25";
        v["dt"] = "0.05";
        v["lambda"] = "1";
        v["eta"] = "1";
        v["g"] = "0";
        v["damped_nt"] = "200";
        v["dampFac"] = "0.5";
        v["alpha"] = "3";
        v["makeGif"] = "false";
        v["makeStringPosGif"] = "true";
        v["saveFreq"] = "5";
        v["outTag"] = "global_PRS_dx0p25";
        v["ic_type"] = "random";
        v["seed"] = "42";
        v["stringPos"] = "false";
        v["stringDetect"] = "true";
        v["detectBuffer"] = "true";
        v["splitLength"] = "false";
        v["finalOut"] = "false";
        v["calcEnergy"] = "false";
        break;
    case Program::Evolution:
        v["nx"] = v["ny"] = v["nz"] = "101";
        v["nt"] = "1001";
        v["dx"] = v["dy"] = v["dz"] = "0.5";
        v["dt"] = "0.05";
        v["lambda"] = "1";
        v["eta"] = "1";
        v["g"] = "0";
        v["damped_nt"] = "200";
        v["dampFac"] = "0.5";
        v["alpha"] = "3";
        v["makeGif"] = "false";
        v["makeStringPosGif"] = "true";
        v["saveFreq"] = "5";
        v["xyBC"] = "periodic";
        v["zBC"] = "periodic";
        v["stringPos"] = "false";
        v["stationary_ic"] = "true";
        v["stringDetect"] = "true";
        v["detectBuffer"] = "true";
        v["splitLength"] = "false";
        v["finalOut"] = "false";
        break;
    case Program::MooreMpiEvolution:
        v["nx"] = v["ny"] = v["nz"] = "1001";
        v["nt"] = "2501";
        v["dx"] = v["dy"] = v["dz"] = "0.25";
        v["dt"] = "0.05";
        v["lambda1"] = "1";
        v["lambda2"] = "1";
        v["lambda12"] = "0";
        v["eta1"] = "1";
        v["eta2"] = "1";
        v["q1"] = "2";
        v["q2"] = "";           // default q1 - 1 (moore_mpi_evolution.cpp:34)
        v["g"] = "";            // default from lambda1, eta1, q1, q2 (:35)
        v["damped_nt"] = "200";
        v["dampFac"] = "0.5";
        v["alpha"] = "3";
        v["makeGif"] = "false";
        v["makeStringPosGif"] = "true";
        v["saveFreq"] = "5";
        v["outTag"] = "Moore_PRS_dx0p25";
        v["ic_type"] = "random";
        v["seed"] = "42";
        v["stringPos"] = "false";
        v["stringDetect"] = "true";
        v["detectBuffer"] = "true";
        v["splitLength"] = "false";
        v["finalOut"] = "false";
        v["calcEnergy"] = "false";
        v["moore_ic_phase"] = "equal";   // equal (reference) | independent
        v["detect_phi2"] = "false";      // also write phi2 crossings (extension)
        break;
    case Program::MooreEvol:
        v["nx"] = "201";
        v["ny"] = "201";
        v["nz"] = "51";
        v["nt"] = "6001";
        v["dx"] = v["dy"] = v["dz"] = "0.7";
        v["dt"] = "0.3";
        v["eta1"] = "1";
        v["eta2"] = "1";
        v["lambda1"] = "2";
        v["lambda2"] = "2";
        v["lambda12"] = "0";
        v["q1"] = "2";
        v["q2"] = "";
        v["g"] = "";
        v["makeGif"] = "true";
        v["saveFreq"] = "10";
        v["xyBC"] = "fixed";
        break;
    case Program::IcwEvolution:
        // ic_w_evolution.cpp:23-50 and the ic_func.cpp:25-58 constants it uses
        v["nx"] = v["ny"] = v["nz"] = "201";
        v["nt"] = "2001";
        v["dx"] = v["dy"] = v["dz"] = "0.35";
        v["dt"] = "0.05";
        v["lambda"] = "1";
        v["eta"] = "1";
        v["g"] = "0";
        v["damped_nt"] = "0";
        v["dampFac"] = "0";
        v["makeGif"] = "true";
        v["saveFreq"] = "10";
        v["xyBC"] = "periodic";
        v["zBC"] = "periodic";
        v["stringPos"] = "false";
        v["stringDetect"] = "true";
        v["splitLength"] = "true";
        // ic_func.cpp:25 ships with "loop collision" (its older form,
        // :966-1720); "random" and "boost" are its other in-process types,
        // and "data" reads two levels of Data/<ic_file>
        v["ic_type"] = "loop collision";
        v["seed"] = "1";
        // the profile table: Data/SOR_Fields.txt for "loop collision"
        // (ic_func.cpp:978), SOR_Fields.txt next to the program for "boost" (:692)
        v["sor_file"] = "";
        v["SORnx"] = "30001";
        v["SORa"] = "0.01";
        v["n"] = "1";
        // the strings of "loop collision" (ic_func.cpp:61-72 when empty)
        for (const char* k : {"pos1s", "pos1a", "pos2s", "pos2a", "v1s", "v1a", "v2s", "v2a"}) v[k] = "";
        v["v1x"] = "0.24";                  // ic_func.cpp:62-64
        v["v1y"] = "0.5499090833947008";
        v["v1z"] = "0";
        break;
    case Program::InitialConditions:
        // initialConditions.cpp:22-60 ("random" is the family provided here;
        // ic_type = convert rewrites a table between text and binary)
        v["ic_type"] = "random";
        v["nx"] = v["ny"] = v["nz"] = "401";
        v["dx"] = v["dy"] = v["dz"] = "0.5";
        v["dt"] = "0.05";
        v["g"] = "0";
        v["seed"] = "42";
        v["mean"] = "0";
        v["stdev"] = "0.5";
        v["ic_in"] = "";     // convert: the table to read (under Data/)
        v["cols"] = "5";     // convert: columns of the table
        v["levels"] = "1";   // convert: rows = levels * nx * ny * nz
        // boost and loop collision (initialConditions.cpp:41-44,62-84): the
        // straight-string table (singleSemiAnalytic's output; the reference
        // reads it from its own directory for boost, from Data/ for loop
        // collision; sor_file, relative to out_dir, overrides), the boost
        // velocity 0.6*(0.4, sqrt(1 - 0.4^2), 0), and the loop-collision
        // strings ("a,b" positions, "a,b,c" velocities; empty: the reference's
        // placement for the lattice)
        v["sor_file"] = "";
        v["SORnx"] = "20001";
        v["SORa"] = "0.01";
        v["n"] = "1";
        v["v1x"] = "0.24";
        v["v1y"] = "0.5499090833947008";
        v["v1z"] = "0";
        for (const char* k : {"pos1s", "pos1a", "pos2s", "pos2a", "v1s", "v1a", "v2s", "v2a"}) v[k] = "";
        // NG sine and simple sine (initialConditions.cpp:113-668): the sine
        // amplitude, which the reference reads from standard input
        v["eps"] = "";
        break;
    case Program::SingleSemiAnalytic:
        // singleSemiAnalytic.cpp:19-33; ic_type 0 starts from eta*tanh(r/2),
        // 1 from the current Data/SOR_Fields.txt
        v["nx"] = "30001";
        v["h"] = "0.01";
        v["w"] = "1.5";
        v["maxIter"] = "2000000";
        v["tol"] = "1e-3";
        v["ic_type"] = "0";
        v["n"] = "1";
        v["lambda"] = "1";
        v["eta"] = "1";
        v["g"] = "0";
        break;
    }
}

void Params::set(const std::string& key, const std::string& value)
{
    if (!vals_.count(key)) fail("unknown parameter '" + key + "'");
    vals_[key] = value;
}

void Params::parse_args(int argc, char** argv)
{
    for (int a = 1; a < argc; ++a) {
        const std::string arg = argv[a];
        const size_t eq = arg.find('=');
        if (eq == std::string::npos) fail("arguments are key=value, got '" + arg + "'");
        const std::string key = trim(arg.substr(0, eq)), val = trim(arg.substr(eq + 1));
        if (key == "params") {
            std::ifstream in(val);
            if (!in) fail("cannot read parameter file " + val);
            std::string line;
            while (std::getline(in, line)) {
                const size_t hash = line.find('#');
                if (hash != std::string::npos) line = line.substr(0, hash);
                const size_t e = line.find('=');
                if (trim(line).empty()) continue;
                if (e == std::string::npos) fail("bad line in " + val + ": " + line);
                set(trim(line.substr(0, e)), trim(line.substr(e + 1)));
            }
        }
    }
    for (int a = 1; a < argc; ++a) {  // command-line values win over the file
        const std::string arg = argv[a];
        const size_t eq = arg.find('=');
        const std::string key = trim(arg.substr(0, eq));
        if (key != "params") set(key, trim(arg.substr(eq + 1)));
    }
}

double Params::num(const std::string& k) const
{
    const std::string& s = str(k);
    char* end = nullptr;
    const double v = std::strtod(s.c_str(), &end);
    if (s.empty() || *end) fail("parameter " + k + " is not a number: '" + s + "'");
    return v;
}

long long Params::integer(const std::string& k) const
{
    const double v = num(k);
    if (v != std::floor(v)) fail("parameter " + k + " must be an integer");
    return (long long)v;
}

bool Params::flag(const std::string& k) const
{
    const std::string& s = str(k);
    if (s == "true" || s == "1") return true;
    if (s == "false" || s == "0") return false;
    fail("parameter " + k + " must be true or false");
    return false;
}

const std::string& Params::str(const std::string& k) const
{
    auto it = vals_.find(k);
    if (it == vals_.end()) fail("missing parameter " + k);
    return it->second;
}

namespace {

struct Run {
    Program prog;
    Params prm;
    lat_params p{};
    int ncomp = 5;
    int64_t N = 0;
    std::string dir;
    int digits = 6;
    lat_handle* h = nullptr;

    explicit Run(Program pr) : prog(pr), prm(pr) {}
    ~Run()
    {
        if (h) lat_destroy(h);
    }

    std::string data(const std::string& f) const { return dir + "/Data/" + f; }
    std::string gif(const std::string& f) const { return dir + "/GifData/" + f; }

    std::ofstream open_out(const std::string& path) const
    {
        std::ofstream o(path);
        if (!o) fail("cannot write " + path);
        o.precision(digits);
        return o;
    }

    void build_params()
    {
        check(lat_params_init(&p, is_moore(prog) ? LAT_MODEL_MOORE : LAT_MODEL_AH), "lat_params_init");
        const std::string prec = prm.str("precision");
        if (prec == "f64") p.precision = LAT_F64;
        else if (prec == "f32") p.precision = LAT_F32;
        else if (prec == "f64_fast") p.precision = LAT_F64_FAST;
        else fail("precision must be f64, f32 or f64_fast");
        p.nx = prm.integer("nx");
        p.ny = prm.integer("ny");
        p.nz = prm.integer("nz");
        p.dx = prm.num("dx");
        p.dy = prm.num("dy");
        p.dz = prm.num("dz");
        p.dt = prm.num("dt");
        p.tau0 = 1;  // conformal time starts at 1 (mpi_evolution.cpp:356)
        p.scaling = prm.num("scaling");
        if (is_moore(prog)) {
            p.lambda = prm.num("lambda1");
            p.lambda2 = prm.num("lambda2");
            p.lambda12 = prm.num("lambda12");
            p.eta = prm.num("eta1");
            p.eta2 = prm.num("eta2");
            p.q1 = (double)prm.integer("q1");
            p.q2 = prm.str("q2").empty() ? p.q1 - 1 : (double)prm.integer("q2");
            // moore_mpi_evolution.cpp:35 / mooreEvol.cpp:36
            p.g = prm.str("g").empty() ? std::sqrt(0.5 * p.lambda * std::pow(p.eta, 2) / (p.q1 * p.q1 + p.q2 * p.q2))
                                       : prm.num("g");
        } else {
            p.lambda = prm.num("lambda");
            p.eta = prm.num("eta");
            p.g = prm.num("g");
        }
        if (prog == Program::MooreEvol) {  // no damping or expansion at all (mooreEvol.cpp:270-271)
            p.damped_nt = 0;
            p.dampFac = 0;
            p.alpha = 0;
        } else if (prog == Program::IcwEvolution) {  // damping only, no expansion (ic_w_evolution.cpp:281)
            p.damped_nt = (int32_t)prm.integer("damped_nt");
            p.dampFac = prm.num("dampFac");
            p.alpha = 0;
        } else {
            p.damped_nt = (int32_t)prm.integer("damped_nt");
            p.dampFac = prm.num("dampFac");
            p.alpha = prm.num("alpha");
        }
        p.energy_form = is_mpi(prog) ? LAT_ENERGY_MPI : LAT_ENERGY_EVOLUTION;
        p.moore_current = prog == Program::MooreEvol ? LAT_MOORE_CURRENT_CHARGE : LAT_MOORE_CURRENT_PLAIN;
        p.bc = LAT_BC_PERIODIC;
        if (prog == Program::Evolution || prog == Program::MooreEvol || prog == Program::IcwEvolution) {
            const std::string xy = prm.str("xyBC");
            const std::string z = prog == Program::MooreEvol ? std::string("fixed") : prm.str("zBC");
            // evolution.cpp:44-45: "periodic", "neumann", "absorbing" (x and y), any
            // other string fixed; the library rejects what a model does not provide
            p.bc = xy == "periodic" ? LAT_BC_PERIODIC
                 : xy == "neumann" ? LAT_BC_NEUMANN
                 : xy == "absorbing" ? LAT_BC_ABSORBING
                                     : LAT_BC_FIXED;
            p.bc_z = z == "periodic" ? LAT_BCZ_PERIODIC : z == "neumann" ? LAT_BCZ_NEUMANN : LAT_BCZ_FIXED;
        }
        ncomp = is_moore(prog) ? 7 : 5;
        N = p.nx * p.ny * p.nz;
        dir = prm.str("out_dir");
        digits = (int)prm.integer("digits");
        ::mkdir((dir + "/Data").c_str(), 0755);
        ::mkdir((dir + "/GifData").c_str(), 0755);
    }

    // Whitespace-separated columns, one line per site in linear order.
    // The text file or its binary form (ic_io.hpp), parsed on all host cores.
    void read_ic(const std::string& path, int cols, int levels, std::vector<double>& lv0, std::vector<double>& lv1)
    {
        std::vector<double> tab;
        read_table(path, cols, (int64_t)levels * N, tab);
        const size_t rows = (size_t)levels * (size_t)N;
        lv0.assign((size_t)ncomp * N, 0.0);
        lv1.assign((size_t)ncomp * N, 0.0);
        for (int t = 0; t < levels; ++t) {
            std::vector<double>& dst = t == 0 ? lv0 : lv1;
            for (int c = 0; c < cols; ++c)
                std::copy(tab.begin() + (ptrdiff_t)(c * rows + (size_t)t * N),
                          tab.begin() + (ptrdiff_t)(c * rows + (size_t)(t + 1) * N), dst.begin() + (ptrdiff_t)c * N);
        }
        if (levels == 1) lv1 = lv0;
    }

    // Write the crossing list of one frame (mpi_evolution.cpp:795-888).
    int64_t write_crossings(int field, const std::string& path)
    {
        int64_t n = 0;
        check(lat_detect_crossings(h, field, nullptr, 0, &n), "lat_detect_crossings");
        std::vector<double> xyz((size_t)std::max<int64_t>(n, 1) * 3);
        if (n) check(lat_detect_crossings(h, field, xyz.data(), n, &n), "lat_detect_crossings");
        std::ofstream o = open_out(path);
        for (int64_t q = 0; q < n; ++q) o << xyz[3 * q] << " " << xyz[3 * q + 1] << " " << xyz[3 * q + 2] << std::endl;
        return n;
    }

    // evolution.cpp:1404-1408: x/y and z normalised by their own boundary kind
    double evolution_deviation(double D) const
    {
        const bool pxy = p.bc == LAT_BC_PERIODIC;
        const bool pz = p.bc_z == LAT_BCZ_PERIODIC || (p.bc_z == LAT_BCZ_AS_XY && pxy);
        D = pxy ? D / (double)(p.nx * p.ny) : D / (double)((p.nx - 2) * (p.ny - 2));
        return pz ? D / (double)p.nz : D / (double)(p.nz - 2);
    }

    void write_final_field(const std::string& path)
    {
        std::vector<double> now((size_t)ncomp * N);
        check(lat_get_state(h, now.data(), nullptr), "lat_get_state");
        write_table_text(path, ncomp, N, now.data(), digits);
    }

    // Position of the string along y = z = 0 by a parabolic fit to the
    // minimum of |phi|^2 (evolution.cpp:695-720).
    double string_position()
    {
        std::vector<double> now((size_t)ncomp * N);
        check(lat_get_state(h, now.data(), nullptr), "lat_get_state");
        const int64_t x0 = (int64_t)(0.5 * (p.nx - 1)), y0 = (int64_t)(0.5 * (p.ny - 1)), z0 = (int64_t)(0.5 * (p.nz - 1));
        auto mag = [&](int64_t i) {
            const int64_t s = (i * p.ny + y0) * p.nz + z0;
            return std::pow(now[s], 2) + std::pow(now[N + s], 2);
        };
        double smallest = 1;
        int64_t is = 0;
        for (int64_t i = 0; i < p.nx; ++i)
            if (mag(i) < smallest) {
                smallest = mag(i);
                is = i;
            }
        if (is < 1 || is + 1 >= p.nx) return (is - x0) * p.dx;
        const double l = mag(is - 1), r = mag(is + 1);
        return (is - x0) * p.dx + p.dx * (l - r) / (2 * l - 4 * smallest + 2 * r);
    }
};

// gifData frames written while the run goes on.  A frame is a snapshot of
// |phi|^2 (lat_snapshot_begin) into one of two pinned buffers; its copy is
// waited for only when the next frame starts (saveFreq steps later), and its
// text is formatted and written by a background thread meanwhile.
class AsyncFrames {
public:
    AsyncFrames(lat_handle* h, int cols, int64_t N, int digits) : h_(h), cols_(cols), N_(N), digits_(digits) {}
    ~AsyncFrames()
    {
        try {
            close();
        } catch (...) {
        }
        for (double* b : buf_) lat_host_free(b);
    }

    void begin(const std::string& path)
    {
        hand_over();
        if (!buf_[cur_]) {
            buf_[cur_] = (double*)lat_host_alloc((int64_t)sizeof(double) * cols_ * N_);
            if (!buf_[cur_]) fail(std::string("lat_host_alloc: ") + lat_last_error());
        }
        check(lat_snapshot_begin(h_, LAT_SNAP_MAGNITUDE, buf_[cur_]), "lat_snapshot_begin");
        pending_ = true;
        pending_path_ = path;
        pending_buf_ = cur_;
        cur_ ^= 1;
    }

    void close()
    {
        hand_over();
        join();
    }

private:
    // the pending frame's copy is complete: give it to the writer thread (the
    // previous writer, which used the other buffer, finishes first)
    void hand_over()
    {
        if (!pending_) return;
        check(lat_snapshot_wait(h_), "lat_snapshot_wait");
        pending_ = false;
        join();
        const double* src = buf_[pending_buf_];
        const std::string path = pending_path_;
        writer_ = std::thread([this, src, path] {
            try {
                write_table_text(path, cols_, N_, src, digits_);
            } catch (const std::exception& e) {
                error_ = e.what();
            }
        });
    }

    void join()
    {
        if (writer_.joinable()) writer_.join();
        if (!error_.empty()) fail(error_);
    }

    lat_handle* h_;
    int cols_;
    int64_t N_;
    int digits_;
    double* buf_[2] = {nullptr, nullptr};
    int cur_ = 0;
    bool pending_ = false;
    std::string pending_path_;
    int pending_buf_ = 0;
    std::thread writer_;
    std::string error_;
};

void progress(long long TimeStep, long long& counter, long long countRate)
{
    if (TimeStep > counter) {
        std::cout << "\rTimestep " << TimeStep - 1 << " completed." << std::flush;
        counter += countRate;
    }
}

int run_mpi(Run& r)
{
    // mpi_evolution.cpp:354-995 / moore_mpi_evolution.cpp:378-1063
    Params& q = r.prm;
    const long long nt = q.integer("nt"), saveFreq = q.integer("saveFreq"), countRate = q.integer("countRate");
    const long long seed = q.integer("seed");
    const bool detect = q.flag("stringDetect"), buffer = q.flag("detectBuffer"), posGif = q.flag("makeStringPosGif");
    const bool calcEnergy = q.flag("calcEnergy");
    const bool moore = is_moore(r.prog);
    struct timeval start, end;
    gettimeofday(&start, nullptr);

    std::string tagPart = q.str("outTag") + "_nx" + std::to_string(r.p.nx);
    if (moore) tagPart += "_q1" + std::to_string((long long)r.p.q1);
    tagPart += "_seed" + std::to_string(seed);
    std::ofstream valsPerLoop = r.open_out(r.data("valsPerLoop_" + tagPart + ".txt"));
    { std::ofstream ff = r.open_out(r.data("finalField.txt")); }  // opened, never written (mpi_evolution.cpp:126)

    std::vector<double> now, past;
    const std::string ic_type = q.str("ic_type");
    if (ic_type == "random") {
        now.assign((size_t)r.ncomp * r.N, 0.0);
        const bool indep = moore && q.str("moore_ic_phase") == "independent";
        check(lat_random_phase_ic(&r.p, (uint32_t)seed, indep, now.data()), "lat_random_phase_ic");
        past = now;
    } else if (ic_type == "stationary data") {
        r.read_ic(r.data(q.str("ic_file")), r.ncomp, 1, past, now);
    } else if (ic_type == "data") {
        r.read_ic(r.data(q.str("ic_file")), r.ncomp, 2, past, now);  // block 0 = slot 0 = past
    } else {
        fail("ic_type must be random, data or stationary data");
    }
    check(lat_create(&r.p, &r.h), "lat_create");
    check(lat_set_state(r.h, now.data(), past.data(), 0), "lat_set_state");
    gettimeofday(&end, nullptr);
    std::cout << "Initial data loaded/generated in: " << end.tv_sec - start.tv_sec << "s" << std::endl;

    long long counter = 0, frame = 0;
    bool stringsExist = true;
    const bool phi2 = moore && q.flag("detect_phi2");
    std::vector<lat_diag> diags;
    long long n = 0;
    while (n < nt) {
        progress(n, counter, countRate);
        if (detect && saveFreq > 0 && n % saveFreq == 0 && posGif && stringsExist && (!buffer || n >= r.p.damped_nt)) {
            const std::string name = "gifStringPosData_" + tagPart + "_" + std::to_string(frame) + ".txt";
            const int64_t cnt = r.write_crossings(LAT_FIELD_PHI1, r.gif(name));
            if (phi2) r.write_crossings(LAT_FIELD_PHI2, r.gif("gifStringPosData2_" + tagPart + "_" + std::to_string(frame) + ".txt"));
            ++frame;
            if (cnt == 0) stringsExist = false;
        }
        // advance to the next step that prints progress or may write a frame
        long long stop = std::min(nt, std::max(n + 1, counter + 1));
        if (detect && saveFreq > 0 && posGif && stringsExist) stop = std::min(stop, (n / saveFreq + 1) * saveFreq);
        const int32_t k = (int32_t)std::max(1LL, stop - n);
        if (calcEnergy) {
            diags.resize((size_t)k);
            int64_t got = 0;
            check(lat_advance(r.h, k, 1, diags.data(), k, &got), "lat_advance");
            for (int64_t d = 0; d < got; ++d) valsPerLoop << diags[d].energy << std::endl;
        } else {
            check(lat_step(r.h, k), "lat_step");
        }
        n += k;
    }
    std::cout << "\rTimestep " << nt << " completed." << std::endl;
    gettimeofday(&end, nullptr);
    std::cout << "Time taken: " << end.tv_sec - start.tv_sec << "s" << std::endl;
    return 0;
}

int run_openmp(Run& r)
{
    // evolution.cpp:60-1471 / mooreEvol.cpp:44-746
    Params& q = r.prm;
    const bool moore = r.prog == Program::MooreEvol;
    const long long nt = q.integer("nt"), saveFreq = q.integer("saveFreq"), countRate = q.integer("countRate");
    struct timeval start, end;
    gettimeofday(&start, nullptr);

    std::string tag;
    std::string valsName = "valsPerLoop.txt";
    if (!moore) {
        std::cout << "Enter a tag for output files: " << std::flush;
        std::cin >> tag;
        valsName = "valsPerLoop_" + tag + ".txt";
    }
    std::vector<double> now, past;
    if (moore) r.read_ic(r.data(q.str("ic_file")), 7, 1, past, now);
    else r.read_ic(r.data(q.str("ic_file")), 5, q.flag("stationary_ic") ? 1 : 2, past, now);
    check(lat_create(&r.p, &r.h), "lat_create");
    check(lat_set_state(r.h, now.data(), past.data(), 0), "lat_set_state");
    AsyncFrames frames(r.h, moore ? 2 : 1, r.N, r.digits);
    std::ofstream valsPerLoop = r.open_out(r.data(valsName));

    const bool makeGif = q.flag("makeGif");
    const bool detect = !moore && q.flag("stringDetect");
    const bool buffer = !moore && q.flag("detectBuffer");
    const bool posGif = !moore && q.flag("makeStringPosGif");
    const bool stringPos = !moore && q.flag("stringPos");
    const bool split = !moore && q.flag("splitLength");
    // deviation normalisation: evolution.cpp:1404-1408, mooreEvol.cpp:383,697
    const double interior = (double)(r.p.nx - 2) * (r.p.ny - 2) * (r.p.nz - 2);
    long long counter = 0, gifFrame = 0, posFrame = 0;
    std::vector<lat_diag> diags;
    long long n = 0;
    while (n < nt) {
        progress(n, counter, countRate);
        const double pos = stringPos ? r.string_position() : 0;
        if (detect && (!buffer || n >= r.p.damped_nt) && posGif && saveFreq > 0 && n % saveFreq == 0) {
            r.write_crossings(LAT_FIELD_PHI1, r.gif("gifStringPosData_" + std::to_string(posFrame) + ".txt"));
            ++posFrame;
        }
        long long stop = std::min(nt, std::max(n + 1, counter + 1));
        if (saveFreq > 0 && (makeGif || (detect && posGif))) stop = std::min(stop, (n / saveFreq + 1) * saveFreq);
        if (makeGif && saveFreq > 0 && n % saveFreq == 0) stop = n + 1;  // the frame is the level after this step
        if (stringPos) stop = n + 1;
        const int32_t k = (int32_t)std::max(1LL, stop - n);
        diags.resize((size_t)k);
        int64_t got = 0;
        check(lat_advance(r.h, k, 1, diags.data(), k, &got), "lat_advance");
        for (int64_t d = 0; d < got; ++d) {
            double dev = diags[d].gauss_abs_sum;
            if (moore) {
                dev = dev / interior / interior;
            } else {
                dev = r.evolution_deviation(dev);
            }
            valsPerLoop << diags[d].energy << " " << dev;
            if (stringPos) valsPerLoop << " " << pos;
            // the reference prints an uninitialised stringLength here
            // (evolution.cpp:66,1415); this program prints 0
            if (detect) {
                valsPerLoop << " " << 0.0;
                if (split) valsPerLoop << " " << 0.0;
            }
            valsPerLoop << std::endl;
        }
        if (makeGif && saveFreq > 0 && n % saveFreq == 0) {
            frames.begin(r.gif("gifData_" + std::to_string(gifFrame) + ".txt"));
            ++gifFrame;
        }
        n += k;
    }
    frames.close();
    std::cout << "\rTimestep " << nt << " completed." << std::endl;
    if (moore || q.flag("finalOut")) r.write_final_field(r.data("finalField.txt"));
    gettimeofday(&end, nullptr);
    std::cout << "Time taken: " << end.tv_sec - start.tv_sec << "s" << std::endl;
    return 0;
}

// ic_func.cpp:647-683 "random": per site in linear order phi_re, phi_im (and,
// when g != 0, the three links dmu*u) drawn from minstd_rand(seed) through
// uniform_real_distribution<double>(-1, 1); both levels equal.
void icfunc_random(const Run& r, double seed, std::vector<double>& now)
{
    std::minstd_rand eng;
    eng.seed((std::minstd_rand::result_type)seed);
    std::uniform_real_distribution<double> unif(-1, 1);
    now.assign((size_t)5 * r.N, 0.0);
    const double d[3] = {r.p.dx, r.p.dy, r.p.dz};
    for (int64_t s = 0; s < r.N; ++s) {
        now[s] = unif(eng);
        now[r.N + s] = unif(eng);
        if (r.p.g != 0)
            for (int m = 0; m < 3; ++m) now[(size_t)(2 + m) * r.N + s] = d[m] * unif(eng);
    }
}

enum class StringIc { Boost, LoopCollision, IcfuncLoopCollision };
void string_ic_table(Params& q, const std::string& dir, StringIc kind, int form, std::vector<double>& tab);

int run_icw(Run& r)
{
    // ic_w_evolution.cpp:52-1190
    Params& q = r.prm;
    const long long nt = q.integer("nt"), saveFreq = q.integer("saveFreq"), countRate = q.integer("countRate");
    const bool makeGif = q.flag("makeGif"), stringPos = q.flag("stringPos"), detect = q.flag("stringDetect");
    const bool split = q.flag("splitLength");
    struct timeval start, end;
    gettimeofday(&start, nullptr);
    // ic_func.cpp "random" and "boost" in-process; "data" reads the two levels
    // of Data/<ic_file> (e.g. initialConditions' loop collision)
    const std::string ic_type = q.str("ic_type");
    std::vector<double> now, past;
    if (ic_type == "random") {
        icfunc_random(r, q.num("seed"), now);
        past = now;
    } else if (ic_type == "boost") {
        std::vector<double> tab;
        string_ic_table(q, q.str("out_dir"), StringIc::Boost, LAT_IC_FORM_INPROCESS, tab);
        past.assign((size_t)5 * r.N, 0.0);
        now.assign((size_t)5 * r.N, 0.0);
        for (int c = 0; c < 5; ++c) {
            std::copy(tab.begin() + (size_t)c * 2 * r.N, tab.begin() + (size_t)c * 2 * r.N + r.N, past.begin() + (size_t)c * r.N);
            std::copy(tab.begin() + (size_t)c * 2 * r.N + r.N, tab.begin() + (size_t)(c + 1) * 2 * r.N, now.begin() + (size_t)c * r.N);
        }
    } else if (ic_type == "loop collision") {
        std::vector<double> tab;
        string_ic_table(q, q.str("out_dir"), StringIc::IcfuncLoopCollision, LAT_IC_FORM_INPROCESS, tab);
        past.assign((size_t)5 * r.N, 0.0);
        now.assign((size_t)5 * r.N, 0.0);
        for (int c = 0; c < 5; ++c) {
            std::copy(tab.begin() + (size_t)c * 2 * r.N, tab.begin() + (size_t)c * 2 * r.N + r.N, past.begin() + (size_t)c * r.N);
            std::copy(tab.begin() + (size_t)c * 2 * r.N + r.N, tab.begin() + (size_t)(c + 1) * 2 * r.N, now.begin() + (size_t)c * r.N);
        }
    } else if (ic_type == "data") {
        r.read_ic(r.data(q.str("ic_file")), 5, 2, past, now);
    } else {
        fail("ic_type: this program provides ic_func.cpp's \"loop collision\", \"random\" and \"boost\", and \"data\"");
    }
    check(lat_create(&r.p, &r.h), "lat_create");
    check(lat_set_state(r.h, now.data(), past.data(), 0), "lat_set_state");
    AsyncFrames frames(r.h, 1, r.N, r.digits);
    std::ofstream valsPerLoop = r.open_out(r.data("valsPerLoop_test.txt"));  // input = "test" (:67)
    long long counter = 0, gifFrame = 0;
    for (long long n = 0; n < nt; ++n) {
        progress(n, counter, countRate);
        const double pos = stringPos ? r.string_position() : 0;
        double L0 = 0, L1 = 0;
        if (detect) check(lat_string_length(r.h, LAT_FIELD_PHI1, split ? 1 : 0, LAT_CHAIN_AUTO, &L0, &L1, nullptr),
                          "lat_string_length");
        lat_diag d;
        check(lat_step_diag(r.h, &d), "lat_step_diag");
        const double dev = r.evolution_deviation(d.gauss_abs_sum);  // ic_w_evolution.cpp:1141-1145
        valsPerLoop << d.energy << " " << dev;
        if (stringPos) valsPerLoop << " " << pos;
        if (detect) {
            valsPerLoop << " " << L0;
            if (split) valsPerLoop << " " << L1;
        }
        valsPerLoop << std::endl;
        if (makeGif && saveFreq > 0 && n % saveFreq == 0) {
            frames.begin(r.gif("gifData_" + std::to_string(gifFrame) + ".txt"));
            ++gifFrame;
        }
    }
    frames.close();
    std::cout << "\rTimestep " << nt << " completed." << std::endl;
    r.write_final_field(r.data("finalField.txt"));
    gettimeofday(&end, nullptr);
    std::cout << "Time taken: " << end.tv_sec - start.tv_sec << "s" << std::endl;
    return 0;
}

bool ends_with(const std::string& s, const std::string& suffix)
{
    return s.size() >= suffix.size() && s.compare(s.size() - suffix.size(), suffix.size(), suffix) == 0;
}

// "a,b,c" (commas or spaces) -> exactly n numbers
std::vector<double> numbers(const std::string& key, const std::string& text, size_t n)
{
    std::vector<double> out;
    std::string t = text;
    for (char& ch : t)
        if (ch == ',') ch = ' ';
    std::istringstream in(t);
    std::string tok;
    while (in >> tok) {
        char* end = nullptr;
        const double v = std::strtod(tok.c_str(), &end);
        if (!end || *end) fail("bad number in " + key + ": " + tok);
        out.push_back(v);
    }
    if (out.size() != n) fail(key + " needs " + std::to_string(n) + " numbers");
    return out;
}

// A string-profile IC (both levels) built on the GPU from the straight-string
// table: column-major [5][2N], level 0 (t = 0) rows first.
void string_ic_table(Params& q, const std::string& dir, StringIc kind, int form, std::vector<double>& tab)
{
    const int64_t m = q.integer("SORnx");
    std::vector<double> prof;
    std::string file = q.str("sor_file");
    if (file.empty()) file = kind == StringIc::Boost ? "SOR_Fields.txt" : "Data/SOR_Fields.txt";
    read_table(dir + "/" + file, 2, m, prof);
    lat_params p;
    check(lat_params_init(&p, LAT_MODEL_AH), "lat_params_init");
    p.nx = q.integer("nx");
    p.ny = q.integer("ny");
    p.nz = q.integer("nz");
    p.dx = q.num("dx");
    p.dy = q.num("dy");
    p.dz = q.num("dz");
    p.dt = q.num("dt");
    p.g = q.num("g");
    p.precision = LAT_F64;
    lat_handle* h = nullptr;
    check(lat_create(&p, &h), "lat_create");
    lat_string_profile sp;
    sp.phi = prof.data();
    sp.A = prof.data() + m;
    sp.m = m;
    sp.h = q.num("SORa");
    sp.winding = q.num("n");
    int64_t off = 0;
    int rc;
    if (kind == StringIc::Boost) {
        lat_boost_ic b;
        b.v[0] = q.num("v1x");
        b.v[1] = q.num("v1y");
        b.v[2] = q.num("v1z");
        b.form = form;
        b.reserved = 0;
        rc = lat_boost_ic_device(h, &sp, &b, &off);
    } else {
        const double Ly = (double)(p.ny - 1), Lz = (double)(p.nz - 1), Lx = (double)(p.nx - 1);
        const double a = 0.6 * 0.4, b = 0.6 * std::sqrt(1 - std::pow(0.4, 2));
        const std::vector<std::pair<const char*, std::vector<double>>> def =
            kind == StringIc::LoopCollision
                ? std::vector<std::pair<const char*, std::vector<double>>>{   // initialConditions.cpp:72-84
                      {"pos1s", {0.15 * Ly * p.dy, -0.25 * Lz * p.dz}}, {"pos1a", {-0.15 * Ly * p.dy, 0.25 * Lz * p.dz}},
                      {"pos2s", {0.25 * Lx * p.dx, 0}},                {"pos2a", {-0.25 * Lx * p.dx, 0}},
                      {"v1s", {0, -0.75, 0}}, {"v1a", {0, 0.75, 0}}, {"v2s", {0, 0, 0}}, {"v2a", {0, 0, 0}}}
                : std::vector<std::pair<const char*, std::vector<double>>>{   // ic_func.cpp:61-72
                      {"pos1s", {2, -0.25 * Lz * p.dz}}, {"pos1a", {-2, 0.25 * Lz * p.dz}},
                      {"pos2s", {0.25 * Lx * p.dx, -1}}, {"pos2a", {-0.25 * Lx * p.dx, 1}},
                      {"v1s", {0, -b, -a}}, {"v1a", {0, b, a}}, {"v2s", {a, b, 0}}, {"v2a", {-a, -b, 0}}};
        lat_loop_collision_ic c;
        double* dst[8] = {c.pos1s, c.pos1a, c.pos2s, c.pos2a, c.v1s, c.v1a, c.v2s, c.v2a};
        for (int w = 0; w < 8; ++w) {
            const std::string& txt = q.str(def[w].first);
            const std::vector<double> v = txt.empty() ? def[w].second : numbers(def[w].first, txt, def[w].second.size());
            for (size_t e = 0; e < v.size(); ++e) dst[w][e] = v[e];
        }
        rc = kind == StringIc::LoopCollision ? lat_loop_collision_ic_device(h, &sp, &c, &off)
                                             : lat_icfunc_loop_collision_ic_device(h, &sp, &c, &off);
    }
    if (rc != LAT_OK) {
        lat_destroy(h);
        check(rc, kind == StringIc::Boost           ? "lat_boost_ic_device"
                  : kind == StringIc::LoopCollision ? "lat_loop_collision_ic_device"
                                                    : "lat_icfunc_loop_collision_ic_device");
    }
    const int64_t N = p.nx * p.ny * p.nz;
    std::vector<double> now((size_t)5 * N), past((size_t)5 * N);
    check(lat_get_state(h, now.data(), past.data()), "lat_get_state");
    lat_destroy(h);
    if (off) std::cout << "Off straight string solution grid at " << off << " site evaluations" << std::endl;
    tab.assign((size_t)10 * N, 0.0);
    for (int c = 0; c < 5; ++c) {
        std::copy(past.begin() + c * N, past.begin() + (c + 1) * N, tab.begin() + (size_t)c * 2 * N);
        std::copy(now.begin() + c * N, now.begin() + (c + 1) * N, tab.begin() + (size_t)c * 2 * N + N);
    }
}

// A perturbed straight string (initialConditions.cpp:113-668, "NG sine" or
// "simple sine") built on the GPU from Data/SOR_Fields.txt (sor_file
// overrides): one level, column-major [5][N].
void sine_ic_table(Params& q, const std::string& dir, bool ng, std::vector<double>& tab)
{
    if (q.str("eps").empty()) fail("ic_type = \"" + q.str("ic_type") + "\" needs eps=<amplitude in [0, 1)>");
    const int64_t m = q.integer("SORnx");
    std::vector<double> prof;
    std::string file = q.str("sor_file");
    if (file.empty()) file = "Data/SOR_Fields.txt";
    read_table(dir + "/" + file, 2, m, prof);
    lat_params p;
    check(lat_params_init(&p, LAT_MODEL_AH), "lat_params_init");
    p.nx = q.integer("nx");
    p.ny = q.integer("ny");
    p.nz = q.integer("nz");
    p.dx = q.num("dx");
    p.dy = q.num("dy");
    p.dz = q.num("dz");
    p.dt = q.num("dt");
    p.g = q.num("g");
    p.precision = LAT_F64;
    lat_handle* h = nullptr;
    check(lat_create(&p, &h), "lat_create");
    lat_string_profile sp;
    sp.phi = prof.data();
    sp.A = prof.data() + m;
    sp.m = m;
    sp.h = q.num("SORa");
    sp.winding = q.num("n");
    int64_t off = 0;
    const int rc = ng ? lat_ng_sine_ic_device(h, &sp, q.num("eps"), &off)
                      : lat_simple_sine_ic_device(h, &sp, q.num("eps"), &off);
    if (rc != LAT_OK) {
        lat_destroy(h);
        check(rc, ng ? "lat_ng_sine_ic_device" : "lat_simple_sine_ic_device");
    }
    const int64_t N = p.nx * p.ny * p.nz;
    tab.assign((size_t)5 * N, 0.0);
    check(lat_get_state(h, tab.data(), nullptr), "lat_get_state");
    lat_destroy(h);
    if (off) std::cout << "Off straight string solution grid at " << off << " site evaluations" << std::endl;
}

// initialConditions.cpp:670-708 ("random"): per site in linear order phi_re,
// phi_im from normal_distribution<double>(mean, stdev) over
// default_random_engine(seed); the link columns are dmu*g*A with A = 0.
// Written as Data/<ic_file>: text (the reference's format and precision) or,
// for a name ending in .bin, the binary form.  ic_type = convert reads
// Data/<ic_in> (text or binary) and writes it as Data/<ic_file>.
int run_initial_conditions(Params& q)
{
    struct timeval start, end;
    gettimeofday(&start, nullptr);
    const std::string dir = q.str("out_dir");
    ::mkdir((dir + "/Data").c_str(), 0755);
    const std::string out = dir + "/Data/" + q.str("ic_file");
    const int digits = (int)q.integer("digits");
    const int64_t N = q.integer("nx") * q.integer("ny") * q.integer("nz");
    std::vector<double> tab;
    int cols = 5;
    int64_t rows = N;
    const std::string type = q.str("ic_type");
    if (type == "random") {
        std::default_random_engine generator((std::default_random_engine::result_type)q.num("seed"));
        std::normal_distribution<double> distribution(q.num("mean"), q.num("stdev"));
        tab.assign((size_t)5 * N, 0.0);
        const double A = 0.0, g = q.num("g");
        for (int64_t s = 0; s < N; ++s) {
            tab[s] = distribution(generator);
            tab[N + s] = distribution(generator);
            tab[2 * N + s] = q.num("dx") * g * A;
            tab[3 * N + s] = q.num("dy") * g * A;
            tab[4 * N + s] = q.num("dz") * g * A;
        }
    } else if (type == "boost" || type == "loop collision") {
        string_ic_table(q, dir, type == "boost" ? StringIc::Boost : StringIc::LoopCollision, LAT_IC_FORM_FILE, tab);
        rows = 2 * N;
    } else if (type == "NG sine" || type == "simple sine") {
        sine_ic_table(q, dir, type == "NG sine", tab);
    } else if (type == "convert") {
        cols = (int)q.integer("cols");
        rows = q.integer("levels") * N;
        if (q.str("ic_in").empty()) fail("ic_type = convert needs ic_in");
        read_table(dir + "/Data/" + q.str("ic_in"), cols, rows, tab);
    } else {
        fail("ic_type: this program provides \"random\", \"NG sine\", \"simple sine\", \"boost\", "
             "\"loop collision\" and \"convert\"");
    }
    if (ends_with(out, ".bin")) write_table_bin(out, cols, rows, tab.data());
    else write_table_text(out, cols, rows, tab.data(), digits);
    gettimeofday(&end, nullptr);
    std::cout << "Time taken: " << end.tv_sec - start.tv_sec << "s" << std::endl;
    return 0;
}

int run_single_semi_analytic(Params& q)
{
    struct timeval start, end;
    gettimeofday(&start, nullptr);
    const std::string dir = q.str("out_dir");
    ::mkdir((dir + "/Data").c_str(), 0755);
    const std::string path = dir + "/Data/SOR_Fields.txt";
    SorParams p;
    p.nx = q.integer("nx");
    p.h = q.num("h");
    p.w = q.num("w");
    p.max_iter = q.integer("maxIter");
    p.tol = q.num("tol");
    p.n = q.num("n");
    p.lambda = q.num("lambda");
    p.eta = q.num("eta");
    p.g = q.num("g");
    if (p.nx < 3) fail("nx must be at least 3");
    std::vector<double> phi, A;
    if (q.integer("ic_type") == 1) {
        std::vector<double> tab;
        read_table(path, 2, p.nx, tab);
        phi.assign(tab.begin(), tab.begin() + p.nx);
        A.assign(tab.begin() + p.nx, tab.end());
    } else {
        sor_initial_guess(p, phi, A);
    }
    const SorResult r = solve_sor(p, std::move(phi), std::move(A));
    std::vector<double> tab(r.phi);
    tab.insert(tab.end(), r.A.begin(), r.A.end());
    write_table_text(path, 2, p.nx, tab.data(), (int)q.integer("digits"));
    std::cout << "Number of iterations: " << r.iterations << std::endl;
    gettimeofday(&end, nullptr);
    std::cout << "Time taken: " << end.tv_sec - start.tv_sec << "s" << std::endl;
    return 0;
}

}  // namespace

int run_program(Program prog, int argc, char** argv)
{
    try {
        if (prog == Program::InitialConditions || prog == Program::SingleSemiAnalytic) {
            Params q(prog);
            q.parse_args(argc, argv);
            return prog == Program::InitialConditions ? run_initial_conditions(q) : run_single_semi_analytic(q);
        }
        Run r(prog);
        r.prm.parse_args(argc, argv);
        r.build_params();
        if (prog == Program::IcwEvolution) return run_icw(r);
        return is_mpi(prog) ? run_mpi(r) : run_openmp(r);
    } catch (const std::exception& e) {
        std::cerr << "error: " << e.what() << std::endl;
        return 2;
    }
}

}  // namespace axh
