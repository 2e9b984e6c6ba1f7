// Posterior samples of a Markov sequence (MarkovSequence.sample,
// _probdiffeq/estimators_and_losses.py:233-273) from the fixed-point
// smoother's outputs.  One thread per (instance, sample); float64; the
// conditionals of an instance are read by all its samples (L1/L2 hits).
#pragma once

#if !defined(__CUDACC_RTC__)
#include <cuda_runtime.h>
#include <stdint.h>
#endif

#include "pdq.h"

namespace pdq {

constexpr int kMaxIsoN = 8;
constexpr int kMaxIsoD = 64;
constexpr int kMaxDenseN = 64;

__global__ void sample_iso_kernel(pdq_sample_args a) {
  const int64_t tid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int K = a.num_samples;
  if (tid >= a.num_instances * K) return;
  const int64_t b = tid / K;
  const int n = a.num_derivatives + 1, d = a.ode_dim, S = a.num_points;
  const double* z = a.normals + tid * int64_t(S) * n;
  double* out = a.samples + tid * int64_t(S) * n * d;  // the previous point's sample is read back from here
  {
    // last point: mean + (L z)[:, None] (IsotropicNormal.sample_flat, ssm_impl_isotropic.py:255-258)
    const double* m = a.marginal_mean + b * n * d;
    const double* L = a.marginal_chol + b * n * n;
    const double* zs = z + int64_t(S - 1) * n;
    double* xs = out + int64_t(S - 1) * n * d;
    for (int i = 0; i < n; ++i) {
      double lz = 0.0;
      for (int l = 0; l < n; ++l) lz += L[i * n + l] * zs[l];
      for (int j = 0; j < d; ++j) xs[i * d + j] = m[i * d + j] + lz;
    }
  }
  for (int s = S - 2; s >= 0; --s) {
    const int64_t cr = b * (S - 1) + s;
    const double* A = a.cond_A + cr * n * n;
    const double* xi = a.cond_noise_mean + cr * n * d;
    const double* X = a.cond_noise_chol + cr * n * n;
    const double* tl = a.cond_to_latent + cr * n;
    const double* to = a.cond_to_observed + cr * n;
    const double* zs = z + int64_t(s) * n;
    const double* xn = out + int64_t(s + 1) * n * d;
    double* xs = out + int64_t(s) * n * d;
    for (int i = 0; i < n; ++i) {
      double xz = 0.0;
      for (int l = 0; l < n; ++l) xz += X[i * n + l] * zs[l];
      const double noise = fabs(to[i]) * xz;
      for (int j = 0; j < d; ++j) {
        double acc = 0.0;
        for (int k = 0; k < n; ++k) acc += A[i * n + k] * tl[k] * xn[k * d + j];
        xs[i * d + j] = to[i] * acc + xi[i * d + j] + noise;  // apply_flat (ssm_impl_isotropic.py:75-79)
      }
    }
  }
}

__global__ void sample_dense_kernel(pdq_sample_args a) {
  const int64_t tid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int K = a.num_samples;
  if (tid >= a.num_instances * K) return;
  const int64_t b = tid / K;
  const int N = (a.num_derivatives + 1) * a.ode_dim, S = a.num_points;
  const double* z = a.normals + tid * int64_t(S) * N;
  double* out = a.samples + tid * int64_t(S) * N;
  {
    // DenseNormal.sample_flat (ssm_impl_dense.py:192-194)
    const double* m = a.marginal_mean + b * N;
    const double* L = a.marginal_chol + b * N * N;
    const double* zs = z + int64_t(S - 1) * N;
    double* xs = out + int64_t(S - 1) * N;
    for (int i = 0; i < N; ++i) {
      double acc = m[i];
      for (int l = 0; l < N; ++l) acc += L[i * N + l] * zs[l];
      xs[i] = acc;
    }
  }
  for (int s = S - 2; s >= 0; --s) {
    const int64_t cr = b * (S - 1) + s;
    const double* A = a.cond_A + cr * N * N;
    const double* xi = a.cond_noise_mean + cr * N;
    const double* X = a.cond_noise_chol + cr * N * N;
    const double* tl = a.cond_to_latent + cr * N;
    const double* to = a.cond_to_observed + cr * N;
    const double* zs = z + int64_t(s) * N;
    const double* xn = out + int64_t(s + 1) * N;
    double* xs = out + int64_t(s) * N;
    for (int i = 0; i < N; ++i) {
      double acc = 0.0, xz = 0.0;
      for (int k = 0; k < N; ++k) {
        acc += A[i * N + k] * tl[k] * xn[k];
        xz += X[i * N + k] * zs[k];
      }
      xs[i] = to[i] * (acc + xi[i]) + fabs(to[i]) * xz;  // apply_flat: to * (A x + xi) (ssm_impl_dense.py:18-22)
    }
  }
}

}  // namespace pdq
