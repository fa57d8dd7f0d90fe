// Radial profile of a straight, static string of winding n: the scalar
// magnitude f(r) and the gauge profile A(r), relaxed by successive
// over-relaxation (singleSemiAnalytic.cpp).  The string-profile IC families
// (boost, loop collision) interpolate this table.
#pragma once

#include <cstdint>
#include <vector>

namespace axh {

struct SorParams {
    int64_t nx = 30001;       // radial points, r = i*h
    double h = 0.01;
    double w = 1.5;           // over-relaxation factor
    int64_t max_iter = 2000000;
    double tol = 1e-3;        // stop when max |residual| <= tol
    double n = 1;             // winding
    double lambda = 1;
    double eta = 1;
    double g = 0;             // gauge coupling (0: global string)
};

struct SorResult {
    std::vector<double> phi, A;
    int64_t iterations = 0;
};

// Relax from `phi0`, `A0` (both of size nx; phi(0) and A(0) are set to 0).
// Sweeps in increasing r, updating in place (Gauss-Seidel order), as
// singleSemiAnalytic.cpp:85-134 does on one thread.
SorResult solve_sor(const SorParams& p, std::vector<double> phi0, std::vector<double> A0);

// The reference's starting guess (singleSemiAnalytic.cpp:51-58):
// phi = eta*tanh(r/2), A = 0.
void sor_initial_guess(const SorParams& p, std::vector<double>& phi, std::vector<double>& A);

}  // namespace axh
