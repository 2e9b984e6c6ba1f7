// The sampling entry point (the kernels are in sample_kernels.cuh).
#include <cuda_runtime.h>

#include "pdq_nvtx.h"
#include "pdq.h"
#include "sample_kernels.cuh"

using pdq::kMaxDenseN;
using pdq::kMaxIsoD;
using pdq::kMaxIsoN;
using pdq::sample_dense_kernel;
using pdq::sample_iso_kernel;

extern "C" pdq_status pdq_sample_markov(const pdq_sample_args* args, void* stream_ptr) {
  pdq::NvtxRange nvtx_range("pdq_sample_markov");
  if (args == nullptr) return PDQ_ERROR_INVALID_VALUE;
  const pdq_sample_args& a = *args;
  if (a.num_instances < 0 || a.num_samples < 0 || a.num_points < 1 || a.num_derivatives < 1 || a.ode_dim < 1)
    return PDQ_ERROR_INVALID_VALUE;
  const int n = a.num_derivatives + 1;
  if (a.ssm == PDQ_SSM_ISOTROPIC) {
    if (n > kMaxIsoN || a.ode_dim > kMaxIsoD) return PDQ_ERROR_UNSUPPORTED;
  } else if (a.ssm == PDQ_SSM_DENSE) {
    if (n * a.ode_dim > kMaxDenseN) return PDQ_ERROR_UNSUPPORTED;
  } else {
    return PDQ_ERROR_UNSUPPORTED;
  }
  const int64_t threads = a.num_instances * a.num_samples;
  if (threads == 0) return PDQ_SUCCESS;
  if (!a.marginal_mean || !a.marginal_chol || !a.normals || !a.samples ||
      (a.num_points > 1 && (!a.cond_A || !a.cond_noise_mean || !a.cond_noise_chol || !a.cond_to_latent ||
                            !a.cond_to_observed)))
    return PDQ_ERROR_INVALID_VALUE;
  cudaStream_t stream = static_cast<cudaStream_t>(stream_ptr);
  const int block = 128;
  const unsigned grid = unsigned((threads + block - 1) / block);
  if (a.ssm == PDQ_SSM_ISOTROPIC)
    sample_iso_kernel<<<grid, block, 0, stream>>>(a);
  else
    sample_dense_kernel<<<grid, block, 0, stream>>>(a);
  return cudaGetLastError() == cudaSuccess ? PDQ_SUCCESS : PDQ_ERROR_CUDA;
}
