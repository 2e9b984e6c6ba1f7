// Block-diagonal cluster kernels (Burgers stencil) in float bulk precision.
#include "bd_launch.cuh"

cudaError_t pdq_launch_bd_burgers_f32(const pdq::BdArgs& a, int nu, cudaStream_t stream) {
  return pdq::launch_bd_precision<float>(a, nu, stream);
}
