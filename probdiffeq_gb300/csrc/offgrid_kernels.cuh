// Kernels of the marginals at off-grid times of a solution on a grid
// (solver.offgrid_marginals, _probdiffeq/solvers.py:149-203).
//
// One thread per (instance, query), float64.  The query's interval comes
// from a binary search (searchsorted, side left) in the instance's grid; the
// transitions use output_scale[index] with dt = t - t[index-1] and
// t[index] - t.
//   filter (estimators_and_losses.py:403-414): the grid marginal at
//     index-1 predicted to t;
//   fixed-interval smoother (:674-709): the filtering marginal at index-1
//     reverted to t, that prediction reverted to t[index], and the smoothed
//     marginal at index marginalised through the second backward
//     conditional.
// A query on a grid point returns that point's marginal (the limit of both
// formulas; the reference leaves this case undefined); a query outside
// [t[0], t[S-1]] or NaN returns NaN.
// Included by offgrid.cu (the launchers) and by the host runs of the tests;
// the kernels live in an unnamed namespace of the including translation unit.
#pragma once

#include "dense_solver.cuh"
#include "iso_solver.cuh"
#include "pdq.h"

namespace {

using pdq::kMaxN;

struct OffgridArgs {
  pdq_offgrid_args a;
  double q1[kMaxN][kMaxN];
};

__device__ int64_t search_left(const double* ts, int S, double tq) {
  int lo = 0, hi = S;
  while (lo < hi) {
    const int mid = (lo + hi) / 2;
    if (ts[mid] < tq)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

__device__ double nan_value() { return __longlong_as_double(0x7ff8000000000000ULL); }

// Isotropic: the covariance factors are n x n, the means n x d (d at run time).
template <int NU>
__global__ void offgrid_iso_kernel(OffgridArgs args) {
  constexpr int n = NU + 1;
  const pdq_offgrid_args& a = args.a;
  const int64_t tid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int S = a.num_points, Q = a.num_queries, d = a.ode_dim;
  if (tid >= a.num_instances * Q) return;
  const int64_t b = tid / Q;
  const double* ts = a.t + b * S;
  const double tq = a.t_query[tid];
  double* mo = a.mean_out + tid * (n * d);
  double* Lo = a.chol_out + tid * (n * n);
  const int64_t k = search_left(ts, S, tq);
  if (k < S && ts[k] == tq) {
    const int64_t rec = b * S + k;
    for (int i = 0; i < n * d; ++i) mo[i] = a.u_mean[rec * (n * d) + i];
    for (int i = 0; i < n * n; ++i) Lo[i] = a.u_chol[rec * (n * n) + i];
    return;
  }
  if (k == 0 || k == S || !(tq == tq)) {
    for (int i = 0; i < n * d; ++i) mo[i] = nan_value();
    for (int i = 0; i < n * n; ++i) Lo[i] = nan_value();
    return;
  }
  const bool smoother = a.strategy == PDQ_STRATEGY_FIXEDINTERVAL;
  const int64_t prev = b * S + (k - 1), next = b * S + k;
  const double* m0 = (smoother ? a.filter_mean : a.u_mean) + prev * (n * d);
  const double* c0 = (smoother ? a.filter_chol : a.u_chol) + prev * (n * n);
  const double s = a.output_scale[next];
  const double h0 = tq - ts[k - 1];
  double L0[n][n], p0[n], pinv0[n];
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < n; ++j) L0[i][j] = c0[i * n + j];
  pdq::precon<double, NU>(h0, p0, pinv0);

  if (!smoother) {
    // transition.marginalise(rv): mean p A1 (p^-1 m), factor from the 2n x n QR
    double Lp[n][n];
    pdq::iso_predict_chol<double, NU>(args.q1, L0, p0, pinv0, s * sqrt(fabs(h0)), Lp);
    for (int j = 0; j < d; ++j) {
      double ml[n];
#pragma unroll
      for (int i = 0; i < n; ++i) ml[i] = pinv0[i] * m0[i * d + j];
#pragma unroll
      for (int i = 0; i < n; ++i) {
        double acc = 0.0;
#pragma unroll
        for (int c = i; c < n; ++c) acc += double(pdq::iwp_a<NU>(i, c)) * ml[c];
        mo[i * d + j] = p0[i] * acc;
      }
    }
#pragma unroll
    for (int i = 0; i < n; ++i)
#pragma unroll
      for (int j = 0; j < n; ++j) Lo[i * n + j] = Lp[i][j];
    return;
  }

  // Revert to t: the predicted factor Lt (the conditional is not needed).
  // The means enter only linearly; the factor computations take a zero mean.
  const double zero[n][1] = {};
  double Lt[n][n];
  pdq::IsoBackward<double, NU, 1> cond;
  pdq::iso_prior_revert<double, NU, 1>(args.q1, zero, L0, p0, pinv0, s * sqrt(fabs(h0)), Lt, cond);
  // Revert t -> t[index]: the backward conditional from t[index] to t.
  const double h1 = ts[k] - tq;
  double p1[n], pinv1[n], Lt1[n][n];
  pdq::precon<double, NU>(h1, p1, pinv1);
  pdq::iso_prior_revert<double, NU, 1>(args.q1, zero, Lt, p1, pinv1, s * sqrt(fabs(h1)), Lt1, cond);
  // Marginalise the smoothed marginal at t[index] through it.
  const double* mu = a.u_mean + next * (n * d);
  const double* cu = a.u_chol + next * (n * n);
  double Lu[n][n], Lm[n][n];
  double mdummy[n][1];
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < n; ++j) Lu[i][j] = cu[i * n + j];
  pdq::iso_cond_marginalise<double, NU, 1>(cond, zero, Lu, mdummy, Lm);
  for (int j = 0; j < d; ++j) {
    // the prediction at t, then the conditional's offset xi (iso_prior_revert's mean formulas)
    double ml0[n], mt[n], ml1[n], mobs[n], xi[n];
#pragma unroll
    for (int i = 0; i < n; ++i) ml0[i] = pinv0[i] * m0[i * d + j];
#pragma unroll
    for (int i = 0; i < n; ++i) {
      double acc = 0.0;
#pragma unroll
      for (int c = i; c < n; ++c) acc += double(pdq::iwp_a<NU>(i, c)) * ml0[c];
      mt[i] = p0[i] * acc;
    }
#pragma unroll
    for (int i = 0; i < n; ++i) ml1[i] = pinv1[i] * mt[i];
#pragma unroll
    for (int i = 0; i < n; ++i) {
      double acc = 0.0;
#pragma unroll
      for (int c = i; c < n; ++c) acc += double(pdq::iwp_a<NU>(i, c)) * ml1[c];
      mobs[i] = acc;
    }
#pragma unroll
    for (int i = 0; i < n; ++i) {
      double acc = ml1[i];
#pragma unroll
      for (int c = 0; c < n; ++c) acc -= cond.A[i][c] * mobs[c];
      xi[i] = acc;
    }
#pragma unroll
    for (int i = 0; i < n; ++i) {
      double acc = xi[i];
#pragma unroll
      for (int c = 0; c < n; ++c) acc += cond.A[i][c] * cond.tl[c] * mu[c * d + j];
      mo[i * d + j] = cond.to[i] * acc;
    }
  }
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < n; ++j) Lo[i * n + j] = Lm[i][j];
}

// Dense: N = (nu + 1) d coefficient-major.
template <int NU, int D>
__global__ void offgrid_dense_kernel(OffgridArgs args) {
  constexpr int N = (NU + 1) * D;
  const pdq_offgrid_args& a = args.a;
  const int64_t tid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int S = a.num_points, Q = a.num_queries;
  if (tid >= a.num_instances * Q) return;
  const int64_t b = tid / Q;
  const double* ts = a.t + b * S;
  const double tq = a.t_query[tid];
  double* mo = a.mean_out + tid * N;
  double* Lo = a.chol_out + tid * (N * N);
  const int64_t k = search_left(ts, S, tq);
  if (k < S && ts[k] == tq) {
    const int64_t rec = b * S + k;
    for (int i = 0; i < N; ++i) mo[i] = a.u_mean[rec * N + i];
    for (int i = 0; i < N * N; ++i) Lo[i] = a.u_chol[rec * (N * N) + i];
    return;
  }
  if (k == 0 || k == S || !(tq == tq)) {
    for (int i = 0; i < N; ++i) mo[i] = nan_value();
    for (int i = 0; i < N * N; ++i) Lo[i] = nan_value();
    return;
  }
  const bool smoother = a.strategy == PDQ_STRATEGY_FIXEDINTERVAL;
  const int64_t prev = b * S + (k - 1), next = b * S + k;
  const double* m0 = (smoother ? a.filter_mean : a.u_mean) + prev * N;
  const double* c0 = (smoother ? a.filter_chol : a.u_chol) + prev * (N * N);
  const double s = a.output_scale[next];
  const double h0 = tq - ts[k - 1];
  pdq::DNormal<double, N> rv, out;
  for (int i = 0; i < N; ++i) {
    rv.m[i] = m0[i];
    for (int j = 0; j < N; ++j) rv.L[i][j] = c0[i * N + j];
  }
  if (!smoother) {
    pdq::prior_marginalise<double, NU, D>(args.q1, rv, h0, s, out);
  } else {
    pdq::DNormal<double, N> at_t, at_t1, u1;
    pdq::DCond<double, N> cond;
    pdq::prior_revert<double, NU, D>(args.q1, rv, h0, s, at_t, cond);
    pdq::prior_revert<double, NU, D>(args.q1, at_t, ts[k] - tq, s, at_t1, cond);
    for (int i = 0; i < N; ++i) {
      u1.m[i] = a.u_mean[next * N + i];
      for (int j = 0; j < N; ++j) u1.L[i][j] = a.u_chol[next * (N * N) + i * N + j];
    }
    pdq::cond_marginalise<double, N>(cond, u1, out);
  }
  for (int i = 0; i < N; ++i) {
    mo[i] = out.m[i];
    for (int j = 0; j < N; ++j) Lo[i * N + j] = out.L[i][j];
  }
}

}  // namespace
