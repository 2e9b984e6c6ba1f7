// Device building blocks shared by the solver kernels.
//
// Everything here works on small fixed-size matrices held in registers (or in
// per-thread local arrays the compiler keeps in registers when all indices are
// compile-time constants).  Sizes are template parameters so every loop is
// fully unrolled.
#pragma once

#if !defined(__CUDACC_RTC__)
#include <cuda_runtime.h>
#include <stdint.h>
#endif

#include "pdq.h"

#define PDQ_HD __host__ __device__ __forceinline__
#define PDQ_D __device__ __forceinline__

namespace pdq {

#if !defined(__CUDACC_RTC__)
// Raise this context's per-thread stack limit to what `kernel` needs (its
// local frame plus headroom for calls) before its first launch.  Kernels
// whose frame exceeds the default limit (1 KB) otherwise overrun the stack.
// cudaDeviceSetLimit waits for the device, so it is only called when the
// limit actually grows (once per process for each larger kernel).
template <typename K>
inline cudaError_t ensure_stack_for_uncached(K kernel) {
  cudaFuncAttributes attr;
  cudaError_t e = cudaFuncGetAttributes(&attr, kernel);
  if (e != cudaSuccess) return e;
  size_t cur = 0;
  e = cudaDeviceGetLimit(&cur, cudaLimitStackSize);
  if (e != cudaSuccess) return e;
  const size_t need = attr.localSizeBytes + 1024;
  if (need > cur) return cudaDeviceSetLimit(cudaLimitStackSize, need);
  return cudaSuccess;
}

// Cached per kernel (template argument) and device (bit d of a 64-bit
// mask), so steady-state launches do no attribute queries.
template <auto KERNEL>
inline cudaError_t ensure_stack() {
  static unsigned long long ready = 0ull;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = (dev >= 0 && dev < 64) ? (1ull << dev) : 0ull;
  if (bit && (__atomic_load_n(&ready, __ATOMIC_ACQUIRE) & bit)) return cudaSuccess;
  e = ensure_stack_for_uncached(KERNEL);
  if (e == cudaSuccess && bit) __atomic_fetch_or(&ready, bit, __ATOMIC_RELEASE);
  return e;
}
#endif  // !__CUDACC_RTC__

// ---------------------------------------------------------------------------
// Scalar helpers
// ---------------------------------------------------------------------------

PDQ_D float dev_sqrt(float x) { return sqrtf(x); }
PDQ_D double dev_sqrt(double x) { return sqrt(x); }
PDQ_D float dev_rsqrt(float x) { return rsqrtf(x); }
PDQ_D double dev_rsqrt(double x) { return rsqrt(x); }
PDQ_D float dev_abs(float x) { return fabsf(x); }
PDQ_D double dev_abs(double x) { return fabs(x); }
PDQ_D float dev_pow(float x, float y) { return powf(x, y); }
PDQ_D double dev_pow(double x, double y) { return pow(x, y); }
// Fast variants for the float32 bulk path (a few ulp); exact in float64.
PDQ_D float dev_div(float a, float b) { return __fdividef(a, b); }
PDQ_D double dev_div(double a, double b) { return a / b; }
PDQ_D float dev_rcp(float a) { return __frcp_rn(a); }
PDQ_D double dev_rcp(double a) { return 1.0 / a; }
PDQ_D float dev_fpow(float x, float y) { return __powf(x, y); }
PDQ_D double dev_fpow(double x, double y) { return pow(x, y); }

// Sums of squares leave the normal range of T for entries beyond ~1e19
// (float) or below ~1e-19; the QR and rotation kernels then recompute the
// norm with scaling (as LAPACK's geqrf does).  The common case costs one test.
PDQ_D bool norm2_out_of_range(float s) { return !(s < 1e36f) || s < 1e-30f; }
PDQ_D bool norm2_out_of_range(double s) { return !(s < 1e300) || s < 1e-290; }

template <typename T>
PDQ_D T dev_fmax_abs(T a, T b) {
  return fmax(dev_abs(a), dev_abs(b));
}

// Single-instruction approximations (PTX .approx, flush-to-zero) for the
// float32 hot loops, where the IEEE-rounded library sequences would sit on
// the dependency chain of every step attempt.  Callers keep the arguments in
// the normal range (the QR and rotation code checks sums of squares against
// [1e-30, 1e36] before using these).  In float64 they are the exact ops.
PDQ_D float fast_sqrt(float x) {
#if defined(__CUDA_ARCH__)
  float r;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  return sqrtf(x);  // host runs of the kernel bodies (tests)
#endif
}
PDQ_D float fast_rsqrt(float x) {
#if defined(__CUDA_ARCH__)
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  return 1.0f / sqrtf(x);  // host runs of the kernel bodies (tests)
#endif
}
PDQ_D float fast_rcp(float x) {
#if defined(__CUDA_ARCH__)
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  return 1.0f / x;  // host runs of the kernel bodies (tests)
#endif
}
PDQ_D double fast_sqrt(double x) { return sqrt(x); }
PDQ_D double fast_rsqrt(double x) { return rsqrt(x); }
PDQ_D double fast_rcp(double x) { return 1.0 / x; }

// Host runs of the kernel bodies (tests) either run a warp's lanes one at a
// time or as concurrent threads; device code never reads this.
#if defined(PDQ_HOST_SIM)
#define PDQ_HOST_LANES_CONCURRENT (pdq_host_warp != nullptr)
#else
#define PDQ_HOST_LANES_CONCURRENT false
#endif

// Named CTA barriers for a producer / consumer pair of warps: the producer
// arrives (and goes on), the consumer waits until `count` threads (both
// warps) have arrived.  Shared-memory writes before the arrive are visible
// to the consumer after its wait.  The warp reconverges first, since the
// aligned barrier wants every lane of the warp at the same instruction.
PDQ_D void named_arrive(int id, int count) {
#if defined(__CUDA_ARCH__)
  __syncwarp();
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(count) : "memory");
#elif defined(PDQ_HOST_SIM)
  pdq_host_named_arrive(id);  // host runs of the kernel bodies (tests)
#endif
}
PDQ_D void named_sync(int id, int count) {
#if defined(__CUDA_ARCH__)
  __syncwarp();
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
#elif defined(PDQ_HOST_SIM)
  pdq_host_named_sync(id);  // host runs of the kernel bodies (tests)
#endif
}

// ---------------------------------------------------------------------------
// Wide scalars for time and accumulators
// ---------------------------------------------------------------------------
// With T = double they are doubles.  With T = float they are unevaluated
// float pairs hi + lo (|lo| <= ulp(hi) / 2, a 48-bit significand) built from
// error-free transformations -- Knuth's TwoSum, Dekker's Fast2Sum and the
// FMA two-product -- so the time, the error-norm sum and the calibration sum
// keep near-float64 accuracy while running on the FP32 pipes: GB300's FP64
// pipe issues a warp instruction only every 64 cycles, which made the
// handful of float64 operations per attempt a third of a float32 solve.

struct FloatPair {
  float hi, lo;
  FloatPair() = default;
  PDQ_HD constexpr FloatPair(float h, float l) : hi(h), lo(l) {}
  // exact conversions (the vector fields write constants as T(1), T(3))
  PDQ_HD constexpr FloatPair(float x) : hi(x), lo(0.0f) {}
  PDQ_HD constexpr FloatPair(int x) : hi(float(x)), lo(0.0f) {}
};

// The sums and products of the error-free transformations use the _rn
// intrinsics, which the compiler never contracts into an FMA: a product
// fused into the following sum would break the transformation's exactness.
// (Host runs of the kernel bodies compile with FMA contraction off.)
PDQ_HD float add_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
PDQ_HD float sub_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
PDQ_HD float mul_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
// A product rounded on its own and a product-sum rounded once, both fixed by
// the source rather than by the compiler's choice of which product to fuse
// into which sum: kernels that share an update (the one-thread isotropic
// kernel and its split twin) then round it alike.
PDQ_HD float mul_nc(float a, float b) { return mul_rn(a, b); }
PDQ_HD double mul_nc(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
PDQ_HD float fma_nc(float a, float b, float c) { return fmaf(a, b, c); }
PDQ_HD double fma_nc(double a, double b, double c) { return fma(a, b, c); }

// a / b to a few ulp (single-instruction reciprocal and a product)
PDQ_HD float div_approx(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fdividef(a, b);
#else
  return a / b;
#endif
}
PDQ_HD FloatPair two_sum(float a, float b) {
  const float s = add_rn(a, b);
  const float bb = sub_rn(s, a);
  return {s, add_rn(sub_rn(a, sub_rn(s, bb)), sub_rn(b, bb))};
}
PDQ_HD FloatPair fast_two_sum(float a, float b) {  // requires |a| >= |b| or a == 0
  const float s = add_rn(a, b);
  return {s, sub_rn(b, sub_rn(s, a))};
}

// ---------------------------------------------------------------------------
// Float-pair arithmetic (the "double-float" number type of Dekker 1971 with
// the error-free sum of Knuth and the FMA product), ~44 significant bits.
// The float32 isotropic kernels evaluate the TS0 residual u' - f(u) in it:
// the residual is a difference of two numbers of the size of the solution's
// derivative and, at rtol 1e-6, about 1e-5 of them, so formed in float32 its
// rounding (the state's and the field's, ~1e-7 of the terms) puts a noise
// floor under the error estimate that rejects and shortens steps float64
// accepts.  Every field is generic over its scalar type, so the same source
// evaluates in pairs.  Accuracy ~2^-44 relative per operation (the "sloppy"
// sum, which loses it only under cancellation of the low parts).
// ---------------------------------------------------------------------------

PDQ_HD FloatPair operator-(FloatPair a) { return {-a.hi, -a.lo}; }
PDQ_HD FloatPair operator+(FloatPair a, FloatPair b) {
  const FloatPair s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, add_rn(s.lo, add_rn(a.lo, b.lo)));
}
PDQ_HD FloatPair operator+(FloatPair a, float b) {
  const FloatPair s = two_sum(a.hi, b);
  return fast_two_sum(s.hi, add_rn(s.lo, a.lo));
}
PDQ_HD FloatPair operator+(float a, FloatPair b) { return b + a; }
PDQ_HD FloatPair operator-(FloatPair a, FloatPair b) { return a + (-b); }
PDQ_HD FloatPair operator-(FloatPair a, float b) { return a + (-b); }
PDQ_HD FloatPair operator-(float a, FloatPair b) { return (-b) + a; }
PDQ_HD FloatPair operator*(FloatPair a, FloatPair b) {
  const float p = mul_rn(a.hi, b.hi);
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}
PDQ_HD FloatPair operator*(FloatPair a, float b) {
  const float p = mul_rn(a.hi, b);
  float e = fmaf(a.hi, b, -p);
  e = fmaf(a.lo, b, e);
  return fast_two_sum(p, e);
}
PDQ_HD FloatPair operator*(float a, FloatPair b) { return b * a; }
// quotient by one correction step: q = a / b to float accuracy, then the
// float remainder a - q b, formed exactly in pairs, divided once more
PDQ_HD FloatPair operator/(FloatPair a, FloatPair b) {
  const float q = div_approx(a.hi, b.hi);
  const FloatPair r = a - b * q;
  return fast_two_sum(q, div_approx(r.hi, b.hi));
}
PDQ_HD FloatPair& operator+=(FloatPair& a, FloatPair b) { return a = a + b; }
PDQ_HD FloatPair& operator-=(FloatPair& a, FloatPair b) { return a = a - b; }
PDQ_HD FloatPair& operator*=(FloatPair& a, FloatPair b) { return a = a * b; }

template <typename T>
struct WideOf {
  using type = double;
};
template <>
struct WideOf<float> {
  using type = FloatPair;
};
template <typename T>
using Wide = typename WideOf<T>::type;

PDQ_D double wide_from(double x, double) { return x; }
PDQ_D FloatPair wide_from(double x, float) {
  const float hi = float(x);
  return {hi, float(x - double(hi))};
}
PDQ_D double wide_value(double x) { return x; }
PDQ_D double wide_value(FloatPair x) { return double(x.hi) + double(x.lo); }
PDQ_D double wide_hi(double x) { return x; }
PDQ_D float wide_hi(FloatPair x) { return x.hi; }
PDQ_D double wide_lo(double) { return 0.0; }
PDQ_D float wide_lo(FloatPair x) { return x.lo; }

// x + y for a narrow y
PDQ_D double wide_add(double x, double y) { return x + y; }
PDQ_D FloatPair wide_add(FloatPair x, float y) {
  const FloatPair s = two_sum(x.hi, y);
  return fast_two_sum(s.hi, s.lo + x.lo);
}
// x + y^2
PDQ_D double wide_add_sq(double x, double y) { return x + y * y; }
PDQ_D FloatPair wide_add_sq(FloatPair x, float y) {
  const float p = y * y;
  const float pe = fmaf(y, y, -p);
  const FloatPair s = two_sum(x.hi, p);
  return fast_two_sum(s.hi, s.lo + (pe + x.lo));
}
// x + y for two wide values (reductions)
PDQ_D double wide_add_wide(double x, double y) { return x + y; }
PDQ_D FloatPair wide_add_wide(FloatPair x, FloatPair y) {
  const FloatPair s = two_sum(x.hi, y.hi);
  return fast_two_sum(s.hi, s.lo + (x.lo + y.lo));
}
// butterfly exchange of a wide value within a warp
PDQ_D double wide_shfl_xor(double x, int lane_mask) { return __shfl_xor_sync(0xffffffffu, x, lane_mask); }
PDQ_D FloatPair wide_shfl_xor(FloatPair x, int lane_mask) {
  return {__shfl_xor_sync(0xffffffffu, x.hi, lane_mask), __shfl_xor_sync(0xffffffffu, x.lo, lane_mask)};
}
// x - y rounded to the narrow type (the difference of two nearby times)
PDQ_D double wide_diff(double x, double y) { return x - y; }
PDQ_D float wide_diff(FloatPair x, FloatPair y) {
  const FloatPair s = two_sum(x.hi, -y.hi);
  return s.hi + (s.lo + (x.lo - y.lo));
}
// x <= c for a narrow constant c
PDQ_D bool wide_le(double x, double c) { return x <= c; }
PDQ_D bool wide_le(FloatPair x, float c) { return x.hi < c || (x.hi == c && x.lo <= 0.0f); }

// A compile-time boolean as a type (selects an instantiation of a generic lambda).
template <bool B>
struct BoolTag {
  static constexpr bool value = B;
};

template <int K>
struct Factorial {
  static constexpr double value = K * Factorial<K - 1>::value;
};
template <>
struct Factorial<0> {
  static constexpr double value = 1.0;
};

// Small-integer combinatorics as straight loops (no recursion), so that
// with the compile-time arguments of the unrolled kernels they fold to
// immediates instead of becoming float64 calls inside the step loop.
PDQ_HD constexpr double factorial(int k) {
  double r = 1.0;
  for (int i = 2; i <= k; ++i) r *= double(i);
  return r;
}

PDQ_HD constexpr int binom_int(int n, int k) {
  if (k < 0 || k > n) return 0;
  int r = 1;
  for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
  return r;
}

PDQ_HD constexpr double binom(int n, int k) { return double(binom_int(n, k)); }

// IWP transition matrix in preconditioned coordinates (the reference's
// flip(Pascal)): A[i][j] = binom(nu - i, nu - j) for j >= i, else 0.
template <int NU>
PDQ_HD constexpr int iwp_a(int i, int j) {
  return j >= i ? binom_int(NU - i, NU - j) : 0;
}

// ---------------------------------------------------------------------------
// Truncated Taylor series ("jet") with normalised coefficients.
// ---------------------------------------------------------------------------

template <typename T, int K>
struct Jet {
  T c[K];
  PDQ_HD Jet() {
#pragma unroll
    for (int k = 0; k < K; ++k) c[k] = T(0);
  }
  PDQ_HD Jet(T x) {
    c[0] = x;
#pragma unroll
    for (int k = 1; k < K; ++k) c[k] = T(0);
  }
};

template <typename T, int K>
PDQ_HD Jet<T, K> operator+(const Jet<T, K>& a, const Jet<T, K>& b) {
  Jet<T, K> r;
#pragma unroll
  for (int k = 0; k < K; ++k) r.c[k] = a.c[k] + b.c[k];
  return r;
}
template <typename T, int K>
PDQ_HD Jet<T, K> operator-(const Jet<T, K>& a, const Jet<T, K>& b) {
  Jet<T, K> r;
#pragma unroll
  for (int k = 0; k < K; ++k) r.c[k] = a.c[k] - b.c[k];
  return r;
}
template <typename T, int K>
PDQ_HD Jet<T, K> operator-(const Jet<T, K>& a) {
  Jet<T, K> r;
#pragma unroll
  for (int k = 0; k < K; ++k) r.c[k] = -a.c[k];
  return r;
}
template <typename T, int K>
PDQ_HD Jet<T, K> operator*(const Jet<T, K>& a, const Jet<T, K>& b) {
  Jet<T, K> r;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    T acc = T(0);
#pragma unroll
    for (int j = 0; j <= k; ++j) acc += a.c[j] * b.c[k - j];
    r.c[k] = acc;
  }
  return r;
}
template <typename T, int K>
PDQ_HD Jet<T, K> operator*(T s, const Jet<T, K>& a) {
  Jet<T, K> r;
#pragma unroll
  for (int k = 0; k < K; ++k) r.c[k] = s * a.c[k];
  return r;
}
template <typename T, int K>
PDQ_HD Jet<T, K> operator*(const Jet<T, K>& a, T s) {
  return s * a;
}
template <typename T, int K>
PDQ_HD Jet<T, K> operator+(T s, const Jet<T, K>& a) {
  Jet<T, K> r = a;
  r.c[0] += s;
  return r;
}
template <typename T, int K>
PDQ_HD Jet<T, K> operator+(const Jet<T, K>& a, T s) {
  return s + a;
}
template <typename T, int K>
PDQ_HD Jet<T, K> operator-(T s, const Jet<T, K>& a) {
  Jet<T, K> r = -a;
  r.c[0] += s;
  return r;
}
template <typename T, int K>
PDQ_HD Jet<T, K> operator-(const Jet<T, K>& a, T s) {
  Jet<T, K> r = a;
  r.c[0] -= s;
  return r;
}

// ---------------------------------------------------------------------------
// Forward-mode dual numbers with K tangent directions (Jacobians of the
// registered fields: jacobian_materialize, _probdiffeq/jacobians.py:78-113).
// ---------------------------------------------------------------------------

template <typename T, int K>
struct Dual {
  T v;
  T g[K];
  PDQ_HD Dual() : v(T(0)) {
#pragma unroll
    for (int k = 0; k < K; ++k) g[k] = T(0);
  }
  PDQ_HD Dual(T x) : v(x) {
#pragma unroll
    for (int k = 0; k < K; ++k) g[k] = T(0);
  }
  PDQ_HD Dual& operator+=(const Dual& o) {
    v += o.v;
#pragma unroll
    for (int k = 0; k < K; ++k) g[k] += o.g[k];
    return *this;
  }
  PDQ_HD Dual& operator-=(const Dual& o) {
    v -= o.v;
#pragma unroll
    for (int k = 0; k < K; ++k) g[k] -= o.g[k];
    return *this;
  }
};

template <typename T, int K>
PDQ_HD Dual<T, K> operator+(const Dual<T, K>& a, const Dual<T, K>& b) {
  Dual<T, K> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.g[k] = a.g[k] + b.g[k];
  return r;
}
template <typename T, int K>
PDQ_HD Dual<T, K> operator-(const Dual<T, K>& a, const Dual<T, K>& b) {
  Dual<T, K> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.g[k] = a.g[k] - b.g[k];
  return r;
}
template <typename T, int K>
PDQ_HD Dual<T, K> operator-(const Dual<T, K>& a) {
  Dual<T, K> r;
  r.v = -a.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.g[k] = -a.g[k];
  return r;
}
template <typename T, int K>
PDQ_HD Dual<T, K> operator*(const Dual<T, K>& a, const Dual<T, K>& b) {
  Dual<T, K> r;
  r.v = a.v * b.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.g[k] = a.g[k] * b.v + a.v * b.g[k];
  return r;
}
template <typename T, int K>
PDQ_HD Dual<T, K> operator*(T s, const Dual<T, K>& a) {
  Dual<T, K> r;
  r.v = s * a.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.g[k] = s * a.g[k];
  return r;
}
template <typename T, int K>
PDQ_HD Dual<T, K> operator*(const Dual<T, K>& a, T s) {
  return s * a;
}
template <typename T, int K>
PDQ_HD Dual<T, K> operator+(T s, const Dual<T, K>& a) {
  Dual<T, K> r = a;
  r.v += s;
  return r;
}
template <typename T, int K>
PDQ_HD Dual<T, K> operator+(const Dual<T, K>& a, T s) {
  return s + a;
}
template <typename T, int K>
PDQ_HD Dual<T, K> operator-(T s, const Dual<T, K>& a) {
  Dual<T, K> r = -a;
  r.v += s;
  return r;
}
template <typename T, int K>
PDQ_HD Dual<T, K> operator-(const Dual<T, K>& a, T s) {
  Dual<T, K> r = a;
  r.v -= s;
  return r;
}

template <typename T, int K>
PDQ_HD Dual<T, K> operator/(const Dual<T, K>& a, const Dual<T, K>& b) {
  Dual<T, K> r;
  const T inv = T(1) / b.v;
  r.v = a.v * inv;
#pragma unroll
  for (int k = 0; k < K; ++k) r.g[k] = (a.g[k] - r.v * b.g[k]) * inv;
  return r;
}
template <typename T, int K>
PDQ_HD Dual<T, K> operator/(const Dual<T, K>& a, T b) {
  Dual<T, K> r;
  const T inv = T(1) / b;
  r.v = a.v * inv;
#pragma unroll
  for (int k = 0; k < K; ++k) r.g[k] = a.g[k] * inv;
  return r;
}
template <typename T, int K>
PDQ_HD Dual<T, K> operator/(T a, const Dual<T, K>& b) {
  return Dual<T, K>(a) / b;
}
// f(u) and the Jacobian J[i][j] = df_i/du_j of a registered field.
template <class F, typename T>
PDQ_HD void eval_with_jacobian(const T* u, const T* p, T* f, T (&J)[F::D][F::D]) {
  Dual<T, F::D> x[F::D], y[F::D];
#pragma unroll
  for (int j = 0; j < F::D; ++j) {
    x[j] = Dual<T, F::D>(u[j]);
    x[j].g[j] = T(1);
  }
  F::eval(x, p, y);
#pragma unroll
  for (int i = 0; i < F::D; ++i) {
    f[i] = y[i].v;
#pragma unroll
    for (int j = 0; j < F::D; ++j) J[i][j] = y[i].g[j];
  }
}

// ---------------------------------------------------------------------------
// Vector-field registry.  Each field is written once, generic over the
// scalar type S (float, double, Jet<...>, Dual<...>), so one definition gives
// the value, the Taylor-mode initial derivatives and the Jacobian.
//   eval(u, p, out): u[D] state, p[P] parameters (type T), out[D]
// ---------------------------------------------------------------------------

struct LotkaVolterra {
  static constexpr int D = 2;
  static constexpr int P = 4;
  template <typename S, typename T>
  PDQ_HD static void eval(const S* u, const T* p, S* out) {
    S y01 = u[0] * u[1];
    out[0] = p[0] * u[0] - p[1] * y01;
    out[1] = p[3] * y01 - p[2] * u[1];
  }
};

struct VanDerPol {
  static constexpr int D = 2;
  static constexpr int P = 1;
  template <typename S, typename T>
  PDQ_HD static void eval(const S* u, const T* p, S* out) {
    out[0] = u[1];
    out[1] = p[0] * ((T(1) - u[0] * u[0]) * u[1] - u[0]);
  }
};

struct FitzHughNagumo {
  static constexpr int D = 2;
  static constexpr int P = 3;
  template <typename S, typename T>
  PDQ_HD static void eval(const S* u, const T* p, S* out) {
    const T a = p[0], b = p[1], c = p[2];
    out[0] = c * (u[0] - u[0] * u[0] * u[0] * (T(1) / T(3)) + u[1]);
    out[1] = -(T(1) / c) * (u[0] - a - b * u[1]);
  }
};

// Taylor-mode initial derivatives u(t0), u'(t0), ..., u^(NU)(t0) of an
// autonomous ODE u' = f(u): with u(t) = sum a_k (t - t0)^k,
// (k + 1) a_{k+1} = [f(u)]_k.  Returned as derivatives u^(k) = k! a_k.
template <typename F, int NU, typename T>
PDQ_HD void taylor_init(const T* y0, const T* p, T (&out)[NU + 1][F::D]) {
  constexpr int K = NU + 1;
  Jet<T, K> u[F::D];
#pragma unroll
  for (int j = 0; j < F::D; ++j) u[j] = Jet<T, K>(y0[j]);
#pragma unroll
  for (int k = 0; k < NU; ++k) {
    Jet<T, K> f[F::D];
    F::eval(u, p, f);
#pragma unroll
    for (int j = 0; j < F::D; ++j) u[j].c[k + 1] = f[j].c[k] / T(k + 1);
  }
#pragma unroll
  for (int k = 0; k < K; ++k) {
#pragma unroll
    for (int j = 0; j < F::D; ++j) out[k][j] = u[j].c[k] * T(factorial(k));
  }
}

// ---------------------------------------------------------------------------
// Register-resident orthogonal triangularisation
// ---------------------------------------------------------------------------

// Rotate rows a and b of a register matrix (columns c0..NC-1) so that
// M[b][c0] becomes zero; M[a][c0] becomes hypot(M[a][c0], M[b][c0]) >= 0.
template <typename T, int NR, int NC>
PDQ_D void givens_rows(T (&M)[NR][NC], int a, int b, int c0) {
  const T x = M[a][c0], y = M[b][c0];
  T r2 = x * x + y * y;
  T cs, sn;
  if (norm2_out_of_range(r2)) {
    const T s = dev_fmax_abs(x, y);
    if (!(s > T(0))) return;
    const T xs = x / s, ys = y / s;
    const T inv = dev_rsqrt(xs * xs + ys * ys);
    cs = xs * inv;
    sn = ys * inv;
    r2 = T(1);
  } else {
    const T inv = fast_rsqrt(r2);
    cs = x * inv;
    sn = y * inv;
  }
  if (r2 > T(0)) {
#pragma unroll
    for (int j = 0; j < NC; ++j) {
      if (j >= c0) {
        const T ma = M[a][j], mb = M[b][j];
        M[a][j] = cs * ma + sn * mb;
        M[b][j] = cs * mb - sn * ma;
      }
    }
    M[b][c0] = T(0);
  }
}

// Householder R factor of a register matrix M (R x C, R >= C), in place:
// afterwards M[0..C-1][*] holds R (upper triangle), rows below are zero.
// Unstructured; used where the inputs carry no exploitable zero pattern.
template <typename T, int NR, int NC>
PDQ_D void householder_r(T (&M)[NR][NC]) {
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    T nrm2 = T(0);
#pragma unroll
    for (int r = c; r < NR; ++r) nrm2 += M[r][c] * M[r][c];
    T nrm;
    if (norm2_out_of_range(nrm2)) {
      T sc = T(0);
#pragma unroll
      for (int r = c; r < NR; ++r) sc = fmax(sc, dev_abs(M[r][c]));
      T acc = T(0);
      if (sc > T(0)) {
        const T inv = T(1) / sc;
#pragma unroll
        for (int r = c; r < NR; ++r) acc += (M[r][c] * inv) * (M[r][c] * inv);
      }
      nrm = sc * dev_sqrt(acc);
      nrm2 = nrm > T(0) ? T(1) : T(0);
    } else {
      nrm = dev_sqrt(nrm2);
    }
    if (nrm2 > T(0)) {
      const T alpha = M[c][c];
      const T beta = alpha >= T(0) ? -nrm : nrm;
      const T vinv = dev_rcp(alpha - beta);
      const T tau = dev_div(beta - alpha, beta);
#pragma unroll
      for (int r = c + 1; r < NR; ++r) M[r][c] *= vinv;
#pragma unroll
      for (int j = c + 1; j < NC; ++j) {
        T w = M[c][j];
#pragma unroll
        for (int r = c + 1; r < NR; ++r) w += M[r][c] * M[r][j];
        w *= tau;
        M[c][j] -= w;
#pragma unroll
        for (int r = c + 1; r < NR; ++r) M[r][j] -= w * M[r][c];
      }
      M[c][c] = beta;
    }
#pragma unroll
    for (int r = c + 1; r < NR; ++r) M[r][c] = T(0);
  }
}

}  // namespace pdq
