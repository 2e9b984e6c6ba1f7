// Stand-in for <cuda_runtime.h> that lets the solver headers compile with a
// host C++ compiler, so the float64 instantiations of a kernel body can run
// on the CPU, one "thread" at a time, under AddressSanitizer.  Test
// infrastructure only: the qualifiers become no-ops, the read-only-cache
// load is a plain load, warp primitives act on a single lane, and the CUDA
// runtime calls used by the launch helpers are inert.  Only kernels that
// need no cooperation between threads can run this way.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>

#define __host__
#define __device__
#define __global__
#define __forceinline__ inline
#define __shared__ static
#define __align__(n) __attribute__((aligned(n)))
#define __launch_bounds__(...)
#define __restrict__

struct pdq_host_uint3 {
  unsigned x, y, z;
};
extern thread_local pdq_host_uint3 threadIdx, blockIdx, blockDim;

struct float4 {
  float x, y, z, w;
};
struct double2 {
  double x, y;
};

template <typename T>
inline T __ldg(const T* p) {
  return *p;
}
template <typename T>
inline T __shfl_xor_sync(unsigned, T v, int, int = 32) {
  return v;
}
inline void __syncwarp(unsigned = 0xffffffffu) {}
inline bool __any_sync(unsigned, bool p) { return p; }  // one lane: its own predicate
inline void __syncthreads() {}
inline void __threadfence() {}
inline double __longlong_as_double(long long v) {
  double d;
  std::memcpy(&d, &v, 8);
  return d;
}
inline long long __double_as_longlong(double v) {
  long long d;
  std::memcpy(&d, &v, 8);
  return d;
}
inline float __fdividef(float a, float b) { return a / b; }
inline float __frcp_rn(float a) { return 1.0f / a; }
inline float __powf(float a, float b) { return std::pow(a, b); }
inline float rsqrtf(float a) { return 1.0f / std::sqrt(a); }
inline double rsqrt(double a) { return 1.0 / std::sqrt(a); }
using std::fabs;
using std::fmax;
using std::isfinite;
using std::isinf;
using std::isnan;
using std::max;
using std::min;
using std::pow;
using std::sqrt;

typedef int cudaError_t;
enum { cudaSuccess = 0, cudaErrorInvalidValue = 1, cudaErrorInvalidDevice = 101, cudaLimitStackSize = 0 };
typedef void* cudaStream_t;
struct cudaFuncAttributes {
  size_t localSizeBytes;
};
template <typename K>
inline cudaError_t cudaFuncGetAttributes(cudaFuncAttributes* a, K) {
  a->localSizeBytes = 0;
  return cudaSuccess;
}
inline cudaError_t cudaDeviceGetLimit(size_t* v, int) {
  *v = size_t(1) << 20;
  return cudaSuccess;
}
inline cudaError_t cudaDeviceSetLimit(int, size_t) { return cudaSuccess; }
inline cudaError_t cudaGetDevice(int* d) {
  *d = 0;
  return cudaSuccess;
}
