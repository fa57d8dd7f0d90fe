// Moore-model step kernels, double instantiation.
#include "moore_step.cuh"

namespace lat {

cudaError_t launch_moore_step_f64(const Geom& g, const Fields<double, 7>& f, const StepCoef& c, const DiagOut& d,
                                  bool diag, cudaStream_t st)
{
    return launch_moore_step_t<double>(g, f, c, d, diag, st);
}

}  // namespace lat
