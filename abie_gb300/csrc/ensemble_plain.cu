// The plain FP64 form of the batched Radau15 kernel, the comparator for the
// ensemble's fast and mixed forms: the reference's own per-component
// operations (its Horner predictor on b, b rebuilt from g after every force,
// the previous step's g kept by the predictor, the division in the
// convergence test, pow in the step control; src/integrator_gauss_radau15.c:
// 56-218, :281-367) and the pair term of its GPU offload gpuforce_v2
// (src/gpuforce.cu:61-84: d2, rsqrt, inv^3), in the same batched kernel as
// the other forms.  This unit alone is compiled with FMA contraction
// (--fmad=true), as a straightforward GPU port of those expressions would be.
#include "ensemble_kernel.cuh"

namespace abie {

const void *ensemble_plain_fn(int w)
{
    return w == 1 ? (const void *)ensemble_kernel<ABIE_FORCE_NAIVE, 1, false>
                  : (w == 2 ? (const void *)ensemble_kernel<ABIE_FORCE_NAIVE, 2, false>
                            : (const void *)ensemble_kernel<ABIE_FORCE_NAIVE, 4, false>);
}

}  // namespace abie
