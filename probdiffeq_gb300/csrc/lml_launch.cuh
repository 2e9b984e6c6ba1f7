// Dispatch of the log-marginal-likelihood kernel over (precision, nu, field).
#pragma once

#include "lml_solver.cuh"

namespace pdq {

template <typename T, int NU, class F>
cudaError_t launch_lml_nu(const LmlArgs& a, cudaStream_t stream) {
  cudaError_t e = ensure_stack<lml_kernel<T, NU, F>>();
  if (e != cudaSuccess) return e;
  const int block = 32;
  lml_kernel<T, NU, F><<<unsigned((a.B + block - 1) / block), block, 0, stream>>>(a);
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

template <int NU, int D, int P>
constexpr size_t lml_cond_floats() {
  return size_t(2 * (NU + 1) * (NU + 1) + (NU + 1) * D) * (P + 1) + 2 * (NU + 1);
}

}  // namespace pdq

cudaError_t pdq_launch_lml_fhn_f32(const pdq::LmlArgs& a, int nu, cudaStream_t stream);
cudaError_t pdq_launch_lml_fhn_f64(const pdq::LmlArgs& a, int nu, cudaStream_t stream);
cudaError_t pdq_launch_lml_lv_f64(const pdq::LmlArgs& a, int nu, cudaStream_t stream);
