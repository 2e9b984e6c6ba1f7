// Adjoint LML kernels (FitzHugh-Nagumo) in float bulk precision.
#include "lml_adj_launch.cuh"

cudaError_t pdq_launch_lml_adj_fhn_f32(const pdq::LmlAdjArgs& aa, int nu, bool backward, cudaStream_t stream) {
  return pdq::launch_lml_adj<float, pdq::FitzHughNagumo>(aa, nu, backward, stream);
}
