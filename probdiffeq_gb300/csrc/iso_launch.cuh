// Template dispatch of the isotropic kernel over (precision, nu, interpolation).
#pragma once

#include "iso_lean.cuh"
#include "iso_solver.cuh"
#include "iso_warp.cuh"

namespace pdq {

// Lanes per instance of the warp-cooperative kernel.
constexpr int kIsoLanes = 8;

// minb: 2 lets the compiler use up to 128 registers per lane (no spills),
// 3 caps it at 85 (more resident warps, a few spills to L1).
template <typename T, int NU, class F>
cudaError_t launch_iso_warp_nu(const IsoArgs& a, int minb, cudaStream_t stream) {
  const int block = kIsoLanes * (a.instances_per_block > 0 ? a.instances_per_block : 32);
  const int64_t threads = a.B * kIsoLanes;
  const unsigned grid = unsigned((threads + block - 1) / block);
  cudaError_t e;
  if (minb == 3) {
    e = ensure_stack<iso_warp_kernel<T, NU, F, kIsoLanes, 3>>();
    if (e != cudaSuccess) return e;
    iso_warp_kernel<T, NU, F, kIsoLanes, 3><<<grid, block, 0, stream>>>(a);
  } else {
    e = ensure_stack<iso_warp_kernel<T, NU, F, kIsoLanes, 2>>();
    if (e != cudaSuccess) return e;
    iso_warp_kernel<T, NU, F, kIsoLanes, 2><<<grid, block, 0, stream>>>(a);
  }
  return cudaGetLastError();
}

template <typename T, int NU, class F, bool INTERP, bool FP, bool GEN>
cudaError_t launch_iso_kernel(const IsoArgs& a, cudaStream_t stream, int block) {
  cudaError_t e = ensure_stack<iso_adaptive_kernel<T, NU, F, INTERP, FP, GEN>>();
  if (e != cudaSuccess) return e;
  const unsigned grid = unsigned((a.B + block - 1) / block);
  iso_adaptive_kernel<T, NU, F, INTERP, FP, GEN><<<grid, block, 0, stream>>>(a);
  return cudaGetLastError();
}

// Forward-mode sensitivities: P + d threads per instance.
template <typename T, int NU, class F, bool INTERP>
cudaError_t launch_iso_tangents(const IsoArgs& a, cudaStream_t stream, int block) {
  cudaError_t e = ensure_stack<iso_adaptive_kernel<T, NU, F, INTERP, false, false, true>>();
  if (e != cudaSuccess) return e;
  const int64_t threads = a.B * int64_t(F::P + F::D);
  const unsigned grid = unsigned((threads + block - 1) / block);
  iso_adaptive_kernel<T, NU, F, INTERP, false, false, true><<<grid, block, 0, stream>>>(a);
  return cudaGetLastError();
}

// The branch-light lean kernel (iso_lean.cuh): the filter with undamped TS0,
// error_residual_std and exact landings.
template <typename T, int NU, class F>
cudaError_t launch_iso_lean(const IsoArgs& a, cudaStream_t stream, int block) {
  cudaError_t e = ensure_stack<iso_lean_kernel<T, NU, F>>();
  if (e != cudaSuccess) return e;
  const unsigned grid = unsigned((a.B + block - 1) / block);
  iso_lean_kernel<T, NU, F><<<grid, block, 0, stream>>>(a);
  return cudaGetLastError();
}

// The fixed-point smoother, TS1, error_state_std and a damped update take
// the general instantiation; the filter with undamped TS0 and
// error_residual_std the lean one (whose update is the single-QR array form),
// with exact landings the branch-light kernel.
template <typename T, int NU, class F, bool FP>
cudaError_t launch_iso_nu(const IsoArgs& a, bool interp, cudaStream_t stream, int block) {
  if constexpr (!FP) {
    if (a.tangents) return interp ? launch_iso_tangents<T, NU, F, true>(a, stream, block)
                                  : launch_iso_tangents<T, NU, F, false>(a, stream, block);
    if (!interp && !a.ts1 && !a.state_error && a.damp == 0.0) return launch_iso_lean<T, NU, F>(a, stream, block);
  }
  if (FP || a.ts1 || a.state_error || a.damp != 0.0)
    return interp ? launch_iso_kernel<T, NU, F, true, FP, true>(a, stream, block)
                  : launch_iso_kernel<T, NU, F, false, FP, true>(a, stream, block);
  return interp ? launch_iso_kernel<T, NU, F, true, FP, FP>(a, stream, block)
                : launch_iso_kernel<T, NU, F, false, FP, FP>(a, stream, block);
}

template <typename T, class F, bool FP = false>
cudaError_t launch_iso_precision(const IsoArgs& a, int nu, bool interp, cudaStream_t stream, int block) {
  if constexpr (FP) {
    if (block <= 0) return cudaErrorInvalidValue;  // the lane-cooperative kernel is filter-only
  } else if (block <= 0) {  // lane-cooperative variant (clip_dt only); -block = min blocks per SM
    const int minb = -block;
    switch (nu) {
      case 1: return launch_iso_warp_nu<T, 1, F>(a, minb, stream);
      case 2: return launch_iso_warp_nu<T, 2, F>(a, minb, stream);
      case 3: return launch_iso_warp_nu<T, 3, F>(a, minb, stream);
      case 4: return launch_iso_warp_nu<T, 4, F>(a, minb, stream);
      case 5: return launch_iso_warp_nu<T, 5, F>(a, minb, stream);
      default: return cudaErrorInvalidValue;
    }
  }
  switch (nu) {
    case 1: return launch_iso_nu<T, 1, F, FP>(a, interp, stream, block);
    case 2: return launch_iso_nu<T, 2, F, FP>(a, interp, stream, block);
    case 3: return launch_iso_nu<T, 3, F, FP>(a, interp, stream, block);
    case 4: return launch_iso_nu<T, 4, F, FP>(a, interp, stream, block);
    case 5: return launch_iso_nu<T, 5, F, FP>(a, interp, stream, block);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace pdq

// Per-(field, precision) entry points, each defined in its own translation
// unit so the instantiations compile in parallel.
#define PDQ_DECLARE_ISO_LAUNCH(NAME) \
  cudaError_t NAME(const pdq::IsoArgs& a, int nu, bool interp, cudaStream_t stream, int block);

PDQ_DECLARE_ISO_LAUNCH(pdq_launch_iso_lv_f32)
PDQ_DECLARE_ISO_LAUNCH(pdq_launch_iso_lv_f64)
PDQ_DECLARE_ISO_LAUNCH(pdq_launch_iso_vdp_f32)
PDQ_DECLARE_ISO_LAUNCH(pdq_launch_iso_vdp_f64)
PDQ_DECLARE_ISO_LAUNCH(pdq_launch_iso_fhn_f32)
PDQ_DECLARE_ISO_LAUNCH(pdq_launch_iso_fhn_f64)
// the same with the fixed-point smoother
PDQ_DECLARE_ISO_LAUNCH(pdq_launch_iso_fp_lv_f32)
PDQ_DECLARE_ISO_LAUNCH(pdq_launch_iso_fp_lv_f64)
PDQ_DECLARE_ISO_LAUNCH(pdq_launch_iso_fp_vdp_f32)
PDQ_DECLARE_ISO_LAUNCH(pdq_launch_iso_fp_vdp_f64)
PDQ_DECLARE_ISO_LAUNCH(pdq_launch_iso_fp_fhn_f32)
PDQ_DECLARE_ISO_LAUNCH(pdq_launch_iso_fp_fhn_f64)

#define PDQ_DEFINE_ISO_LAUNCH(NAME, T, F)                                                       \
  cudaError_t NAME(const pdq::IsoArgs& a, int nu, bool interp, cudaStream_t stream, int block) { \
    return pdq::launch_iso_precision<T, F>(a, nu, interp, stream, block);                       \
  }

#define PDQ_DEFINE_ISO_FP_LAUNCH(NAME, T, F)                                                    \
  cudaError_t NAME(const pdq::IsoArgs& a, int nu, bool interp, cudaStream_t stream, int block) { \
    return pdq::launch_iso_precision<T, F, true>(a, nu, interp, stream, block);                 \
  }
