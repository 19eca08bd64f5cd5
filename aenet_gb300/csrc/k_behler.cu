// Behler-Parrinello symmetry functions (placeholder until the kernels land).
#include "common.h"

int ae_launch_behler_forward(const PotDevice&, const DescBuffers&, int, cudaStream_t) {
  return (int)cudaErrorNotSupported;
}
int ae_launch_behler_adjoint(const PotDevice&, const DescBuffers&, int, cudaStream_t) {
  return (int)cudaErrorNotSupported;
}
