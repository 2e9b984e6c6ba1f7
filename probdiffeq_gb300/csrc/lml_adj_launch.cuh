// Dispatch of the adjoint log-marginal-likelihood kernels over (precision, nu, field).
#pragma once

#include "lml_adjoint.cuh"

namespace pdq {

// Value pass: the shared plan (skipped on the device when the workspace
// holds it already), then one thread per sample.
template <typename T, int NU, class F>
cudaError_t launch_lml_adj_fwd_nu(const LmlAdjArgs& aa, cudaStream_t stream) {
  cudaError_t e = ensure_stack<lml_plan_kernel<T, NU>>();
  if (e != cudaSuccess) return e;
  lml_plan_kernel<T, NU><<<1, kLmlPlanThreads, 0, stream>>>(aa.base);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = ensure_stack<lml_adj_fwd_kernel<T, NU, F>>();
  if (e != cudaSuccess) return e;
  const int64_t blocks = (aa.base.B + kLmlThreads - 1) / kLmlThreads;
  lml_adj_fwd_kernel<T, NU, F><<<unsigned(blocks), kLmlThreads, 0, stream>>>(aa);
  return cudaGetLastError();
}

// Adjoint pass (reads the plan and residuals the value pass left in the workspace).
template <typename T, int NU, class F>
cudaError_t launch_lml_adj_bwd_nu(const LmlAdjArgs& aa, cudaStream_t stream) {
  cudaError_t e = ensure_stack<lml_adj_bwd_kernel<T, NU, F>>();
  if (e != cudaSuccess) return e;
  const int64_t blocks = (aa.base.B + kLmlThreads - 1) / kLmlThreads;
  lml_adj_bwd_kernel<T, NU, F><<<unsigned(blocks), kLmlThreads, 0, stream>>>(aa);
  return cudaGetLastError();
}

template <typename T, class F>
cudaError_t launch_lml_adj(const LmlAdjArgs& aa, int nu, bool backward, cudaStream_t stream) {
  switch (nu) {
    case 2: return backward ? launch_lml_adj_bwd_nu<T, 2, F>(aa, stream) : launch_lml_adj_fwd_nu<T, 2, F>(aa, stream);
    case 3: return backward ? launch_lml_adj_bwd_nu<T, 3, F>(aa, stream) : launch_lml_adj_fwd_nu<T, 3, F>(aa, stream);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace pdq

cudaError_t pdq_launch_lml_adj_fhn_f32(const pdq::LmlAdjArgs& aa, int nu, bool backward, cudaStream_t stream);
cudaError_t pdq_launch_lml_adj_fhn_f64(const pdq::LmlAdjArgs& aa, int nu, bool backward, cudaStream_t stream);
cudaError_t pdq_launch_lml_adj_lv_f64(const pdq::LmlAdjArgs& aa, int nu, bool backward, cudaStream_t stream);
