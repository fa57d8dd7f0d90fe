// Abelian-Higgs step kernels, float instantiation: the tiled FP32 step
// (tiled_step.cuh) and the one-pass kernel kept for cross-checks.
#include "ah_step.cuh"
#include "pair_step.cuh"
#include "tiled_step.cuh"

namespace lat {

cudaError_t launch_ah_step_f32(const Geom& g, const Fields<float, 5>& f, const StepCoef& c, const DiagOut& d, bool diag,
                               cudaStream_t st)
{
    return launch_ah_step_t<float>(g, f, c, d, diag, st);
}

// variant 0: the pair step where the layout allows it, else the tiled step
// (16-byte staging where allowed); 2: the tiled step staging one element per
// copy; 3: the tiled step with 16-byte staging.  *blocks = the CTAs (and
// diagnostic partials) of the kernel that ran.
cudaError_t launch_ah_tiled_f32(const Geom& g, const Fields<float, 5>& f, const StepCoef& c, const DiagOut& d,
                                  bool diag, int chunk, cudaStream_t st, int variant, int* blocks)
{
    if (variant == 0) {
        const cudaError_t e = launch_pair_t<1>(g, f, c, d, diag, chunk, st);
        if (e != cudaErrorNotSupported) {
            const dim3 t = pair_grid(g, chunk);
            *blocks = (int)(t.x * t.y * t.z);
            return e;
        }
    }
    const dim3 t = tiled_grid(g, chunk);
    *blocks = (int)(t.x * t.y * t.z);
    return launch_tiled_t<float, 1>(g, f, c, d, diag, chunk, st, variant != 2);
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
