// Template dispatch of the terminal-value adjoint's two kernels over nu.
#pragma once

#include "tv_adjoint.cuh"

namespace pdq {

template <typename T, int NU, class F>
cudaError_t launch_tv_nu(const IsoArgs& a, const TvAdjArgs* t, cudaStream_t stream) {
  constexpr int block = 64;
  const unsigned grid = unsigned((a.B + block - 1) / block);
  if (t == nullptr) {
    cudaError_t e = ensure_stack<iso_adaptive_kernel<T, NU, F, false, false, false, false, true>>();
    if (e != cudaSuccess) return e;
    iso_adaptive_kernel<T, NU, F, false, false, false, false, true><<<grid, block, 0, stream>>>(a);
  } else {
    cudaError_t e = ensure_stack<iso_tv_bwd_kernel<T, NU, F>>();
    if (e != cudaSuccess) return e;
    iso_tv_bwd_kernel<T, NU, F><<<grid, block, 0, stream>>>(a, *t);
  }
  return cudaGetLastError();
}

// t == nullptr: the record pass; otherwise the adjoint pass
template <typename T, class F>
cudaError_t launch_tv(const IsoArgs& a, const TvAdjArgs* t, int nu, cudaStream_t stream) {
  switch (nu) {
    case 1: return launch_tv_nu<T, 1, F>(a, t, stream);
    case 2: return launch_tv_nu<T, 2, F>(a, t, stream);
    case 3: return launch_tv_nu<T, 3, F>(a, t, stream);
    case 4: return launch_tv_nu<T, 4, F>(a, t, stream);
    case 5: return launch_tv_nu<T, 5, F>(a, t, stream);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace pdq

#define PDQ_DECLARE_TV_LAUNCH(NAME) \
  cudaError_t NAME(const pdq::IsoArgs& a, const pdq::TvAdjArgs* t, int nu, cudaStream_t stream);

PDQ_DECLARE_TV_LAUNCH(pdq_launch_tv_lv_f32)
PDQ_DECLARE_TV_LAUNCH(pdq_launch_tv_lv_f64)
PDQ_DECLARE_TV_LAUNCH(pdq_launch_tv_vdp_f32)
PDQ_DECLARE_TV_LAUNCH(pdq_launch_tv_vdp_f64)
PDQ_DECLARE_TV_LAUNCH(pdq_launch_tv_fhn_f32)
PDQ_DECLARE_TV_LAUNCH(pdq_launch_tv_fhn_f64)

#define PDQ_DEFINE_TV_LAUNCH(NAME, T, F)                                                          \
  cudaError_t NAME(const pdq::IsoArgs& a, const pdq::TvAdjArgs* t, int nu, cudaStream_t stream) { \
    return pdq::launch_tv<T, F>(a, t, nu, stream);                                                \
  }
