// Adjoint LML kernels (FitzHugh-Nagumo, Lotka-Volterra) in double bulk precision.
#include "lml_adj_launch.cuh"

cudaError_t pdq_launch_lml_adj_fhn_f64(const pdq::LmlAdjArgs& aa, int nu, bool backward, cudaStream_t stream) {
  return pdq::launch_lml_adj<double, pdq::FitzHughNagumo>(aa, nu, backward, stream);
}

cudaError_t pdq_launch_lml_adj_lv_f64(const pdq::LmlAdjArgs& aa, int nu, bool backward, cudaStream_t stream) {
  return pdq::launch_lml_adj<double, pdq::LotkaVolterra>(aa, nu, backward, stream);
}
