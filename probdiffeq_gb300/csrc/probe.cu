// FP32 FMA throughput probe used by the benchmark to state the CUDA-core
// roofline (include/pdq_probe.h).
#include <cuda_runtime.h>

#include "pdq_probe.h"

namespace {

__global__ void fma_probe_kernel(float* out, int64_t iters) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  float a0 = 1.0f + tid * 1e-7f, a1 = a0 + 1e-3f, a2 = a0 + 2e-3f, a3 = a0 + 3e-3f;
  float a4 = a0 + 4e-3f, a5 = a0 + 5e-3f, a6 = a0 + 6e-3f, a7 = a0 + 7e-3f;
  const float m = 0.999999f, c = 1e-7f;
  for (int64_t i = 0; i < iters; ++i) {
    a0 = fmaf(a0, m, c);
    a1 = fmaf(a1, m, c);
    a2 = fmaf(a2, m, c);
    a3 = fmaf(a3, m, c);
    a4 = fmaf(a4, m, c);
    a5 = fmaf(a5, m, c);
    a6 = fmaf(a6, m, c);
    a7 = fmaf(a7, m, c);
  }
  out[tid] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

}  // namespace

extern "C" int pdq_probe_fp32_fma(float* out, int64_t iters, int32_t blocks, int32_t threads, void* stream) {
  fma_probe_kernel<<<blocks, threads, 0, static_cast<cudaStream_t>(stream)>>>(out, iters);
  return cudaGetLastError() == cudaSuccess ? 0 : 3;
}

extern "C" int pdq_probe_sm_count(void) {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  return n;
}
