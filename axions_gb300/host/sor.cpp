// Successive over-relaxation for the straight-string profile
// (singleSemiAnalytic.cpp:67-134).  The sweep is sequential along r: each
// point reads the already-updated value at r - h, so the 30001-point profile
// is a chain of dependent updates with no parallelism to give to a GPU.  It
// runs once per parameter set, on the host.
//
// The residuals and their Newton denominators are the reference's:
//   F_phi = ((n - g A)/r)^2 + lambda/2 (phi^2 - eta^2)) phi
//           - (phi(r+h) - phi(r-h))/(2 r h) - (phi(r+h) - 2 phi + phi(r-h))/h^2
//   dF_phi = ((n - g A)/r)^2 + lambda/2 (3 phi^2 - eta^2) + 2/h^2
//   F_A   = -2 g (n - g A) phi^2 + (A(r+h) - A(r-h))/(2 r h) - (A(r+h) - 2 A + A(r-h))/h^2
//   dF_A  = 2 (g phi)^2 + 2/h^2
// with phi += -w F_phi/dF_phi, A += -w F_A/dF_A, written with the same
// operations and pow() calls so that the table matches the reference's
// single-thread run bit for bit.  The outer boundary is Neumann
// (value copied from r - h before each sweep), the centre is 0.
#include "sor.hpp"

#include <cmath>

namespace axh {

void sor_initial_guess(const SorParams& p, std::vector<double>& phi, std::vector<double>& A)
{
    phi.assign((size_t)p.nx, 0.0);
    A.assign((size_t)p.nx, 0.0);
    for (int64_t i = 0; i < p.nx; ++i) {
        phi[(size_t)i] = p.eta * std::tanh(0.5 * p.h * (double)i);
        A[(size_t)i] = 0;
    }
}

SorResult solve_sor(const SorParams& p, std::vector<double> phi, std::vector<double> A)
{
    const int64_t nx = p.nx;
    const double h = p.h, w = p.w, n = p.n, lambda = p.lambda, eta = p.eta, g = p.g;
    std::vector<double> Fphi((size_t)nx, 0.0), FA((size_t)nx, 0.0);
    phi[0] = 0;
    A[0] = 0;
    double tolTest = 1;
    int64_t iter = 0;
    while (tolTest > p.tol && iter < p.max_iter) {
        tolTest = 0;
        iter += 1;
        phi[(size_t)(nx - 1)] = phi[(size_t)(nx - 2)];
        A[(size_t)(nx - 1)] = A[(size_t)(nx - 2)];
        for (int64_t j = 1; j < nx - 1; ++j) {
            const double jd = (double)j;
            const double f0 = (std::pow((n - g * A[j]) / (jd * h), 2) + 0.5 * lambda * (std::pow(phi[j], 2) - std::pow(eta, 2))) * phi[j]
                            - (phi[j + 1] - phi[j - 1]) / (2 * jd * h * h) - (phi[j + 1] - 2 * phi[j] + phi[j - 1]) / (h * h);
            const double f1 = std::pow((n - g * A[j]) / (jd * h), 2) + 0.5 * lambda * (3 * std::pow(phi[j], 2) - std::pow(eta, 2))
                            + 2 / (h * h);
            const double a0 = -2 * g * (n - g * A[j]) * std::pow(phi[j], 2) + (A[j + 1] - A[j - 1]) / (2 * jd * h * h)
                            - (A[j + 1] - 2 * A[j] + A[j - 1]) / (h * h);
            const double a1 = 2 * std::pow(g * phi[j], 2) + 2 / (h * h);
            Fphi[j] = f0;
            FA[j] = a0;
            phi[j] += -w * f0 / f1;
            A[j] += -w * a0 / a1;
        }
        for (int64_t j = 1; j < nx - 1; ++j) {
            if (std::fabs(Fphi[j]) > tolTest) tolTest = std::fabs(Fphi[j]);
            if (std::fabs(FA[j]) > tolTest) tolTest = std::fabs(FA[j]);
        }
    }
    SorResult r;
    r.phi = std::move(phi);
    r.A = std::move(A);
    r.iterations = iter;
    return r;
}

}  // namespace axh
