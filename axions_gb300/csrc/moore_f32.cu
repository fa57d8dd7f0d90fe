// Moore-model step kernels, float instantiation.
#include "moore_step.cuh"

namespace lat {

cudaError_t launch_moore_step_f32(const Geom& g, const Fields<float, 7>& f, const StepCoef& c, const DiagOut& d,
                                  bool diag, cudaStream_t st)
{
    return launch_moore_step_t<float>(g, f, c, d, diag, st);
}

}  // namespace lat
