// Template dispatch of the dense kernel over (precision, nu, TS0/TS1, filter/fixed-point).
#pragma once

#include "dense_solver.cuh"

namespace pdq {

template <typename T, int NU, class F, bool TS1, bool FP>
cudaError_t launch_dense_variant(const DenseArgs& a, cudaStream_t stream, int block) {
  auto kernel = dense_adaptive_kernel<T, NU, F, TS1, FP>;
  cudaError_t e = ensure_stack<dense_adaptive_kernel<T, NU, F, TS1, FP>>();
  if (e != cudaSuccess) return e;
  const unsigned grid = unsigned((a.B + block - 1) / block);
  kernel<<<grid, block, 0, stream>>>(a);
  return cudaGetLastError();
}

template <typename T, int NU, class F>
cudaError_t launch_dense_nu(const DenseArgs& a, bool ts1, bool fp, cudaStream_t stream, int block) {
  if (ts1) return fp ? launch_dense_variant<T, NU, F, true, true>(a, stream, block)
                     : launch_dense_variant<T, NU, F, true, false>(a, stream, block);
  return fp ? launch_dense_variant<T, NU, F, false, true>(a, stream, block)
            : launch_dense_variant<T, NU, F, false, false>(a, stream, block);
}

template <typename T, class F>
cudaError_t launch_dense_precision(const DenseArgs& a, int nu, bool ts1, bool fp, cudaStream_t stream, int block) {
  switch (nu) {
    case 2: return launch_dense_nu<T, 2, F>(a, ts1, fp, stream, block);
    case 3: return launch_dense_nu<T, 3, F>(a, ts1, fp, stream, block);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace pdq

#define PDQ_DECLARE_DENSE_LAUNCH(NAME) \
  cudaError_t NAME(const pdq::DenseArgs& a, int nu, bool ts1, bool fp, cudaStream_t stream, int block);

PDQ_DECLARE_DENSE_LAUNCH(pdq_launch_dense_lv_f32)
PDQ_DECLARE_DENSE_LAUNCH(pdq_launch_dense_lv_f64)
PDQ_DECLARE_DENSE_LAUNCH(pdq_launch_dense_vdp_f32)
PDQ_DECLARE_DENSE_LAUNCH(pdq_launch_dense_vdp_f64)
PDQ_DECLARE_DENSE_LAUNCH(pdq_launch_dense_fhn_f32)
PDQ_DECLARE_DENSE_LAUNCH(pdq_launch_dense_fhn_f64)

#define PDQ_DEFINE_DENSE_LAUNCH(NAME, T, F)                                                                 \
  cudaError_t NAME(const pdq::DenseArgs& a, int nu, bool ts1, bool fp, cudaStream_t stream, int block) { \
    return pdq::launch_dense_precision<T, F>(a, nu, ts1, fp, stream, block);                              \
  }
