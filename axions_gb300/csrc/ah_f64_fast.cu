// Abelian-Higgs two-pass FP64 step, LAT_F64_FAST variant (compiled with
// multiply-add contraction).
#include "ah_twopass.cuh"

namespace lat {

cudaError_t launch_ah_twopass_fast(const Geom& g, const Fields<double, 5>& f, double* L, const StepCoef& c,
                                   const DiagOut& d, bool diag, bool recip, cudaStream_t st)
{
    return launch_ah_twopass<false>(g, f, L, c, d, diag, recip, st);
}

}  // namespace lat
