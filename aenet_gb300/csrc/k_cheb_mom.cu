// FP32 instantiations of the Chebyshev descriptor and adjoint kernels with
// the angular terms in moment form (mixed-precision path).
#include "k_cheb_impl.cuh"

namespace cheb {

int dispatch_moments(const PotDevice& pd, const DescBuffers& b, bool adjoint, cudaStream_t s) {
  int rN, aN;
  if (!uniform_sizes(pd, rN, aN)) return AE_MOM_NA;
  if ((size_t)b.mom_pad < (size_t)(2 * aN * aN)) return AE_MOM_NA;
  if (rN == 11 && aN == 5) return launch_lpa<float, 11, 5, true>(pd, b, adjoint, s);
  if (rN == 13 && aN == 7) return launch_lpa<float, 13, 7, true>(pd, b, adjoint, s);
  if (rN == 17 && aN == 5) return launch_lpa<float, 17, 5, true>(pd, b, adjoint, s);
  return AE_MOM_NA;
}

}  // namespace cheb
