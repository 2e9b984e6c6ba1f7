// Cluster launch of the block-diagonal kernel.
#pragma once

#include "bd_solver.cuh"

namespace pdq {

// Cluster size: aim at ~4 dimensions per thread, d divisible by the cluster.
inline int bd_cluster_size(int d) {
  int cl = 1;
  while (cl < 8 && (d / cl) > kBdThreads * 4) cl *= 2;
  while (cl > 1 && d % cl != 0) cl /= 2;
  return cl;
}

// One cluster of a.cluster CTAs per instance with `smem` bytes of dynamic
// shared memory per CTA; `kernel` is a bd_adaptive_kernel instantiation
// (built in, or compiled at run time for a user stencil).
inline cudaError_t launch_bd_cluster(const void* kernel, BdArgs a, size_t smem, cudaStream_t stream) {
  const int CL = a.cluster;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(unsigned(a.B * CL), 1, 1);
  cfg.blockDim = dim3(kBdThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  void* args[] = {&a};
  cudaError_t e = cudaLaunchKernelExC(&cfg, kernel, args);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

template <typename T, int NU, bool FP>
cudaError_t launch_bd_kernel(BdArgs a, cudaStream_t stream) {
  cudaError_t e = ensure_stack<bd_adaptive_kernel<T, NU, FP>>();
  if (e != cudaSuccess) return e;
  return launch_bd_cluster(reinterpret_cast<const void*>(bd_adaptive_kernel<T, NU, FP>), a,
                           bd_smem_bytes<T, NU>(a.d / a.cluster), stream);
}

template <typename T, int NU>
cudaError_t launch_bd_nu(const BdArgs& a, cudaStream_t stream) {
  return a.fixedpoint ? launch_bd_kernel<T, NU, true>(a, stream) : launch_bd_kernel<T, NU, false>(a, stream);
}

template <typename T>
cudaError_t launch_bd_precision(const BdArgs& a, int nu, cudaStream_t stream) {
  switch (nu) {
    case 2: return launch_bd_nu<T, 2>(a, stream);
    case 3: return launch_bd_nu<T, 3>(a, stream);
    case 4: return launch_bd_nu<T, 4>(a, stream);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace pdq

cudaError_t pdq_launch_bd_burgers_f32(const pdq::BdArgs& a, int nu, cudaStream_t stream);
cudaError_t pdq_launch_bd_burgers_f64(const pdq::BdArgs& a, int nu, cudaStream_t stream);
