// Launchers of the off-grid marginal kernels (offgrid_kernels.cuh):
// solver.offgrid_marginals (_probdiffeq/solvers.py:149-203), one thread per
// (instance, query), float64.
#include <cuda_runtime.h>

#include "offgrid_kernels.cuh"
#include "offgrid.h"

namespace {

template <auto KERNEL>
cudaError_t launch(const OffgridArgs& args, cudaStream_t stream) {
  cudaError_t e = pdq::ensure_stack<KERNEL>();
  if (e != cudaSuccess) return e;
  const int64_t threads = args.a.num_instances * args.a.num_queries;
  const int block = 64;
  KERNEL<<<unsigned((threads + block - 1) / block), block, 0, stream>>>(args);
  return cudaGetLastError();
}

}  // namespace

cudaError_t pdq_launch_offgrid(const pdq_offgrid_args& a, const double (&q1)[pdq::kMaxN][pdq::kMaxN],
                               cudaStream_t stream) {
  OffgridArgs args;
  args.a = a;
  for (int i = 0; i < kMaxN; ++i)
    for (int j = 0; j < kMaxN; ++j) args.q1[i][j] = q1[i][j];
  if (a.ssm == PDQ_SSM_ISOTROPIC) {
    switch (a.num_derivatives) {
      case 1: return launch<offgrid_iso_kernel<1>>(args, stream);
      case 2: return launch<offgrid_iso_kernel<2>>(args, stream);
      case 3: return launch<offgrid_iso_kernel<3>>(args, stream);
      case 4: return launch<offgrid_iso_kernel<4>>(args, stream);
      case 5: return launch<offgrid_iso_kernel<5>>(args, stream);
      default: return cudaErrorInvalidValue;
    }
  }
  if (a.ssm == PDQ_SSM_DENSE && a.ode_dim == 2) {
    switch (a.num_derivatives) {
      case 2: return launch<offgrid_dense_kernel<2, 2>>(args, stream);
      case 3: return launch<offgrid_dense_kernel<3, 2>>(args, stream);
      default: return cudaErrorInvalidValue;
    }
  }
  return cudaErrorInvalidValue;
}
