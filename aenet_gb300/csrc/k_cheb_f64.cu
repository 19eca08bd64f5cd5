// FP64 instantiations of the Chebyshev descriptor and adjoint kernels
// (the plain path).
#include "k_cheb_impl.cuh"

int ae_cheb_f64(const PotDevice& pd, const DescBuffers& b, bool adjoint, cudaStream_t s) {
  return cheb::dispatch<double>(pd, b, adjoint, s);
}
