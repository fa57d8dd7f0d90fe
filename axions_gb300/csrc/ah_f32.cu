// Abelian-Higgs step kernels, float instantiation: the tiled FP32 step
// (tiled_step.cuh) and the one-pass kernel kept for cross-checks.
#include "ah_step.cuh"
#include "tiled_step.cuh"

namespace lat {

cudaError_t launch_ah_step_f32(const Geom& g, const Fields<float, 5>& f, const StepCoef& c, const DiagOut& d, bool diag,
                               cudaStream_t st)
{
    return launch_ah_step_t<float>(g, f, c, d, diag, st);
}

cudaError_t launch_ah_tiled_f32(const Geom& g, const Fields<float, 5>& f, const StepCoef& c, const DiagOut& d,
                                bool diag, int chunk, cudaStream_t st, bool allow_vec)
{
    return launch_tiled_t<float, 1>(g, f, c, d, diag, chunk, st, allow_vec);
}

cudaError_t launch_divergence_f32(const Geom& g, const float* tx, const float* ty, const float* tz, const StepCoef& c,
                                  float* out, cudaStream_t st)
{
    return launch_divergence_t<float>(g, tx, ty, tz, c, out, st);
}

}  // namespace lat

namespace lat {

int tiled_blocks(const Geom& g, int chunk)
{
    const dim3 t = tiled_grid(g, chunk);
    return (int)(t.x * t.y * t.z);
}

}  // namespace lat
