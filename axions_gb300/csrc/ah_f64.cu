// Abelian-Higgs step kernels, double instantiation.
#include "ah_step.cuh"
#include "ah_twopass.cuh"

namespace lat {

cudaError_t launch_ah_step_f64(const Geom& g, const Fields<double, 5>& f, const StepCoef& c, const DiagOut& d, bool diag,
                               cudaStream_t st)
{
    return launch_ah_step_t<double>(g, f, c, d, diag, st);
}

int ah_link_slots() { return L_COUNT; }

cudaError_t launch_ah_twopass_strict(const Geom& g, const Fields<double, 5>& f, double* L, const StepCoef& c,
                                     const DiagOut& d, bool diag, bool recip, cudaStream_t st)
{
    return launch_ah_twopass<true>(g, f, L, c, d, diag, recip, st);
}

cudaError_t launch_divergence_f64(const Geom& g, const double* tx, const double* ty, const double* tz, const StepCoef& c,
                                  double* out, cudaStream_t st)
{
    return launch_divergence_t<double>(g, tx, ty, tz, c, out, st);
}

}  // namespace lat
