// Moore-model step kernels, float instantiation: the tiled FP32 step
// (tiled_step.cuh, two scalars) and the one-pass kernel kept for cross-checks.
#include "moore_step.cuh"
#include "tiled_step.cuh"

namespace lat {

cudaError_t launch_moore_step_f32(const Geom& g, const Fields<float, 7>& f, const StepCoef& c, const DiagOut& d,
                                  bool diag, cudaStream_t st)
{
    return launch_moore_step_t<float>(g, f, c, d, diag, st);
}

cudaError_t launch_moore_tiled_f32(const Geom& g, const Fields<float, 7>& f, const StepCoef& c, const DiagOut& d,
                                   bool diag, int chunk, cudaStream_t st, bool allow_vec)
{
    return launch_tiled_t<float, 2>(g, f, c, d, diag, chunk, st, allow_vec);
}

}  // namespace lat
