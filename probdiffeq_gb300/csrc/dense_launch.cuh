// Template dispatch of the dense kernel over (precision, nu, TS0/TS1, filter/fixed-point).
#pragma once

#include "dense_coop.cuh"
#include "dense_solver.cuh"
#include "dense_struct.cuh"

namespace pdq {

// Lane-cooperative kernel: one instance per warp (lanes 0-7), up to four
// warps per block (instances_per_block), their states in dynamic shared memory.
template <typename T, int NU, class F, bool TS1, bool FP>
cudaError_t launch_dense_coop(const DenseArgs& a, cudaStream_t stream) {
  constexpr int N = (NU + 1) * F::D;
  constexpr int max_groups = 4;
  const int groups = a.instances_per_block > 0 ? a.instances_per_block : max_groups;
  const size_t smem = size_t(groups) * sizeof(CoopState<T, N, F::D>);
  static bool attr_set = false;  // per process; the attribute is per function, device-independent in practice
  cudaError_t e = ensure_stack<dense_coop_kernel<T, NU, F, TS1, FP>>();
  if (e != cudaSuccess) return e;
  if (!attr_set) {
    e = cudaFuncSetAttribute(dense_coop_kernel<T, NU, F, TS1, FP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             int(max_groups * sizeof(CoopState<T, N, F::D>)));
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  const unsigned grid = unsigned((a.B + groups - 1) / groups);
  dense_coop_kernel<T, NU, F, TS1, FP><<<grid, groups * 32, smem, stream>>>(a);
  return cudaGetLastError();
}

// Structure-exploiting kernel: L lanes per instance (four; eight or sixteen
// in their own translation units), 32 / L instances per warp-sized block,
// their states in dynamic shared memory.
constexpr int kDenseStructLanes = 4;

template <typename T, int NU, class F, bool TS1, bool FP, int L = kDenseStructLanes>
cudaError_t launch_dense_struct(const DenseArgs& a, cudaStream_t stream) {
  static_assert(L == 4 || L == 8 || L == 16, "lane groups of four, eight or sixteen");
  constexpr int IPW = 32 / L;
  const size_t smem = dense_struct_smem_bytes<NU, F::D>(sizeof(T), L);
  static bool attr_set = false;
  cudaError_t e = ensure_stack<dense_struct_kernel<T, NU, F, TS1, FP, L>>();
  if (e != cudaSuccess) return e;
  if (!attr_set) {
    e = cudaFuncSetAttribute(dense_struct_kernel<T, NU, F, TS1, FP, L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             int(smem));
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  const unsigned grid = unsigned((a.B + IPW - 1) / IPW);
  dense_struct_kernel<T, NU, F, TS1, FP, L><<<grid, 32, smem, stream>>>(a);
  return cudaGetLastError();
}

// block: 1 one thread per instance, 3 the structure-exploiting lanes, else the 8-lane cooperative kernel
template <typename T, int NU, class F, bool TS1, bool FP>
cudaError_t launch_dense_variant(const DenseArgs& a, cudaStream_t stream, int block) {
  if (block == 3) return launch_dense_struct<T, NU, F, TS1, FP>(a, stream);
  if (block != 1) return launch_dense_coop<T, NU, F, TS1, FP>(a, stream);
  block = a.instances_per_block > 0 ? a.instances_per_block : 32;  // one thread per instance
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

// The structure-exploiting kernel with L lanes per instance, dispatched over
// (nu, TS0/TS1, filter/fixed-point).
template <typename T, class F, int L>
cudaError_t launch_dense_struct_precision(const DenseArgs& a, int nu, bool ts1, bool fp, cudaStream_t stream) {
  switch (nu) {
    case 2:
      return ts1 ? (fp ? launch_dense_struct<T, 2, F, true, true, L>(a, stream)
                       : launch_dense_struct<T, 2, F, true, false, L>(a, stream))
                 : (fp ? launch_dense_struct<T, 2, F, false, true, L>(a, stream)
                       : launch_dense_struct<T, 2, F, false, false, L>(a, stream));
    case 3:
      return ts1 ? (fp ? launch_dense_struct<T, 3, F, true, true, L>(a, stream)
                       : launch_dense_struct<T, 3, F, true, false, L>(a, stream))
                 : (fp ? launch_dense_struct<T, 3, F, false, true, L>(a, stream)
                       : launch_dense_struct<T, 3, F, false, false, L>(a, stream));
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

// the structure-exploiting kernel with eight or sixteen lanes per instance
#define PDQ_DECLARE_DENSE_LANES_LAUNCH(NAME) \
  cudaError_t NAME(const pdq::DenseArgs& a, int nu, bool ts1, bool fp, int lanes, cudaStream_t stream);

PDQ_DECLARE_DENSE_LANES_LAUNCH(pdq_launch_dense_lanes_lv_f32)
PDQ_DECLARE_DENSE_LANES_LAUNCH(pdq_launch_dense_lanes_lv_f64)
PDQ_DECLARE_DENSE_LANES_LAUNCH(pdq_launch_dense_lanes_vdp_f32)
PDQ_DECLARE_DENSE_LANES_LAUNCH(pdq_launch_dense_lanes_vdp_f64)
PDQ_DECLARE_DENSE_LANES_LAUNCH(pdq_launch_dense_lanes_fhn_f32)
PDQ_DECLARE_DENSE_LANES_LAUNCH(pdq_launch_dense_lanes_fhn_f64)

#define PDQ_DEFINE_DENSE_LANES_LAUNCH(NAME, T, F)                                                         \
  cudaError_t NAME(const pdq::DenseArgs& a, int nu, bool ts1, bool fp, int lanes, cudaStream_t stream) { \
    if (lanes == 8) return pdq::launch_dense_struct_precision<T, F, 8>(a, nu, ts1, fp, stream);           \
    if (lanes == 16) return pdq::launch_dense_struct_precision<T, F, 16>(a, nu, ts1, fp, stream);         \
    return cudaErrorInvalidValue;                                                                          \
  }
