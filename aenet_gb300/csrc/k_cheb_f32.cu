// FP32 instantiations of the Chebyshev descriptor and adjoint kernels
// (mixed-precision path) and the launch entry points of both precisions.
#include "k_cheb_impl.cuh"

int ae_cheb_f64(const PotDevice& pd, const DescBuffers& b, bool adjoint, cudaStream_t s);

int ae_launch_chebyshev_forward(const PotDevice& pd, const DescBuffers& b, int fp64,
                                cudaStream_t s) {
  if (b.natoms <= 0) return 0;
  return fp64 ? ae_cheb_f64(pd, b, false, s) : cheb::dispatch<float>(pd, b, false, s);
}

int ae_launch_chebyshev_adjoint(const PotDevice& pd, const DescBuffers& b, int fp64,
                                cudaStream_t s) {
  if (b.natoms <= 0) return 0;
  return fp64 ? ae_cheb_f64(pd, b, true, s) : cheb::dispatch<float>(pd, b, true, s);
}
