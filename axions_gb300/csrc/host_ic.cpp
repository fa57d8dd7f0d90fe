// Seeded random-phase initial conditions, generated on the host exactly as
// the reference does (mpi_evolution.cpp:287-312, moore_mpi_evolution.cpp:293-323):
// std::mt19937(seed) and std::uniform_real_distribution<double>(0, 2*pi),
// one draw per site in linear order, phi = eta*(cos, sin), both time levels
// equal, link phases zero.
#include <cmath>
#include <cstring>
#include <random>
#include <string>

#include "../../include/lattice_gpu.h"

namespace lat {
void set_error(const std::string& msg);
}

extern "C" int lat_random_phase_ic(const lat_params* p, uint32_t seed, int32_t independent, double* fields)
{
    if (!p || !fields) {
        lat::set_error("lat_random_phase_ic: null argument");
        return LAT_ERR_INVALID;
    }
    if (p->nx <= 0 || p->ny <= 0 || p->nz <= 0) {
        lat::set_error("lat_random_phase_ic: bad lattice size");
        return LAT_ERR_INVALID;
    }
    const double pi = 4.0 * std::atan(1.0);
    const int64_t N = p->nx * p->ny * p->nz;
    const int nc = p->model == LAT_MODEL_MOORE ? 7 : 5;
    std::memset(fields, 0, sizeof(double) * (size_t)nc * (size_t)N);
    std::mt19937 generator(seed);
    std::uniform_real_distribution<double> distribution(0.0, 2 * pi);
    double* re1 = fields;
    double* im1 = fields + N;
    double* re2 = fields + 2 * N;
    double* im2 = fields + 3 * N;
    for (int64_t s = 0; s < N; ++s) {
        const double phase = distribution(generator);
        re1[s] = p->eta * std::cos(phase);
        im1[s] = p->eta * std::sin(phase);
        if (p->model == LAT_MODEL_MOORE) {
            const double phase2 = independent ? distribution(generator) : phase;
            re2[s] = p->eta2 * std::cos(phase2);
            im2[s] = p->eta2 * std::sin(phase2);
        }
    }
    return LAT_OK;
}
