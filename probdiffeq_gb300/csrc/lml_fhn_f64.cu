// Log-marginal-likelihood kernels (FitzHugh-Nagumo, Lotka-Volterra) in double bulk precision.
#include "lml_launch.cuh"

cudaError_t pdq_launch_lml_fhn_f64(const pdq::LmlArgs& a, int nu, cudaStream_t stream) {
  return pdq::launch_lml_precision<double, pdq::FitzHughNagumo>(a, nu, stream);
}

cudaError_t pdq_launch_lml_lv_f64(const pdq::LmlArgs& a, int nu, cudaStream_t stream) {
  return pdq::launch_lml_precision<double, pdq::LotkaVolterra>(a, nu, stream);
}
