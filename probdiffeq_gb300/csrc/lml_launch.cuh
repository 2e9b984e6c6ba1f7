// Dispatch of the log-marginal-likelihood kernel over (precision, nu, field).
#pragma once

#include "lml_solver.cuh"

namespace pdq {

template <typename T, int NU, class F>
cudaError_t launch_lml_nu(const LmlArgs& a, cudaStream_t stream) {
  // the shared covariance plan (skipped on the device when the workspace holds it already)
  cudaError_t e = ensure_stack<lml_plan_kernel<T, NU>>();
  if (e != cudaSuccess) return e;
  lml_plan_kernel<T, NU><<<1, kLmlPlanThreads, 0, stream>>>(a);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = ensure_stack<lml_kernel<T, NU, F>>();
  if (e != cudaSuccess) return e;
  const int block = kLmlThreads;
  const int64_t threads = a.B * a.lanes_per_sample;
  lml_kernel<T, NU, F><<<unsigned((threads + block - 1) / block), block, 0, stream>>>(a);
  return cudaGetLastError();
}

template <typename T, class F>
cudaError_t launch_lml_precision(const LmlArgs& a, int nu, cudaStream_t stream) {
  switch (nu) {
    case 2: return launch_lml_nu<T, 2, F>(a, stream);
    case 3: return launch_lml_nu<T, 3, F>(a, stream);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace pdq

cudaError_t pdq_launch_lml_fhn_f32(const pdq::LmlArgs& a, int nu, cudaStream_t stream);
cudaError_t pdq_launch_lml_fhn_f64(const pdq::LmlArgs& a, int nu, cudaStream_t stream);
cudaError_t pdq_launch_lml_lv_f64(const pdq::LmlArgs& a, int nu, cudaStream_t stream);
