// Log-marginal-likelihood kernels (FitzHugh-Nagumo) in float bulk precision.
#include "lml_launch.cuh"

cudaError_t pdq_launch_lml_fhn_f32(const pdq::LmlArgs& a, int nu, cudaStream_t stream) {
  return pdq::launch_lml_precision<float, pdq::FitzHughNagumo>(a, nu, stream);
}
