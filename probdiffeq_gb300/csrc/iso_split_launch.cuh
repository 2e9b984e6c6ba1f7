// Template dispatch of the split isotropic kernel (a covariance warp and a
// mean warp per 32 instances) over nu.
#pragma once

#include "iso_split.cuh"

namespace pdq {

// instances per block of the split kernel (one lane of each warp per instance)
constexpr int kIsoSplitWidth = 32;

template <typename T, int NU, class F>
cudaError_t launch_iso_split_nu(const IsoArgs& a, cudaStream_t stream) {
  constexpr int W = kIsoSplitWidth;
  cudaError_t e = ensure_stack<iso_split_kernel<T, NU, F, W>>();
  if (e != cudaSuccess) return e;
  const unsigned grid = unsigned((a.B + W - 1) / W);
  iso_split_kernel<T, NU, F, W><<<grid, 2 * W, 0, stream>>>(a);
  return cudaGetLastError();
}

template <typename T, class F>
cudaError_t launch_iso_split(const IsoArgs& a, int nu, cudaStream_t stream) {
  switch (nu) {
    case 1: return launch_iso_split_nu<T, 1, F>(a, stream);
    case 2: return launch_iso_split_nu<T, 2, F>(a, stream);
    case 3: return launch_iso_split_nu<T, 3, F>(a, stream);
    case 4: return launch_iso_split_nu<T, 4, F>(a, stream);
    case 5: return launch_iso_split_nu<T, 5, F>(a, stream);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace pdq

#define PDQ_DECLARE_ISO_SPLIT_LAUNCH(NAME) cudaError_t NAME(const pdq::IsoArgs& a, int nu, cudaStream_t stream);

PDQ_DECLARE_ISO_SPLIT_LAUNCH(pdq_launch_iso_split_lv_f32)
PDQ_DECLARE_ISO_SPLIT_LAUNCH(pdq_launch_iso_split_lv_f64)
PDQ_DECLARE_ISO_SPLIT_LAUNCH(pdq_launch_iso_split_vdp_f32)
PDQ_DECLARE_ISO_SPLIT_LAUNCH(pdq_launch_iso_split_vdp_f64)
PDQ_DECLARE_ISO_SPLIT_LAUNCH(pdq_launch_iso_split_fhn_f32)
PDQ_DECLARE_ISO_SPLIT_LAUNCH(pdq_launch_iso_split_fhn_f64)

#define PDQ_DEFINE_ISO_SPLIT_LAUNCH(NAME, T, F)                          \
  cudaError_t NAME(const pdq::IsoArgs& a, int nu, cudaStream_t stream) { \
    return pdq::launch_iso_split<T, F>(a, nu, stream);                   \
  }
