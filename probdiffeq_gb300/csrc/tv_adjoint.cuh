// Reverse-mode (adjoint) gradient of adaptive terminal values with sqrt(N)
// step checkpointing: the counterpart of jax.grad through
// solve_adaptive_terminal_values with its stop-gradient on the step size
// (solvers_via_adaptive_steps.py:16-43, 294-301), split into the two halves
// of a custom VJP.
//
//   record pass        iso_adaptive_kernel<..., REC> (iso_solver.cuh): the
//                      isotropic TS0 filter solves as pdq_solve_adaptive does
//                      and records, per instance, the size of every accepted
//                      step and the state (mean, Cholesky factor) before
//                      every C-th accepted step.
//   iso_tv_bwd_kernel  for a cotangent of the terminal mean: the accepted
//                      steps in reverse, one segment of C steps at a time --
//                      the segment's steps are recomputed from its stored
//                      state (the predicted u and the gain of each step into
//                      a scratch), then differentiated last to first -- and
//                      finally the Taylor-mode initialisation on dual
//                      numbers, giving d / d params and d / d y0.
//
// With TS0 (H = e_1), the step sizes held constant and a calibration that
// does not scale the prediction (solver, solver_mle: unit scale during the
// solve, the output scale applied at the end), the Cholesky factors and the
// gains depend on the step sizes only, not on the parameters or y0; only the
// mean recursion is differentiated, per accepted step
//     mp = p . A1 (p^-1 . m)                   (IsotropicLatentCond.marginalise, mean)
//     m' = mp - g (mp[1] - f(mp[0], theta))    (TS0 update, revert_conditional)
// by the transpose of each line; f's Jacobian in u and theta comes from one
// evaluation on dual numbers with d + P directions.  The recomputed gains
// are those of the forward pass (the same step sizes, the same factor at the
// segment's start, the same joint predict-update QR); the recomputed means
// run in the bulk type without the forward pass's float-pair rows, which
// moves the points the Jacobians are taken at by rounding only.
//
// Record (type T), element e of instance b at record[e * B + b]:
//   [0, cap)                                   h_k, the size of accepted step k
//   [cap, cap + S (n d + n n))                 before step s C: m (n x d), L (n x n); S = ceil(cap / C)
// Scratch (type T) after the record, element e of instance b at scratch[e * B + b]:
//   [0, C (d + n))                             per step of the segment being reversed: mp[0] (d), g (n)
#pragma once

#include "iso_solver.cuh"

namespace pdq {

struct TvAdjArgs {
  int32_t capacity, ckpt;
  const int32_t* num_steps;  // (B,)
  const int32_t* status;     // (B,)
  const double* cotangent;   // (B, n, d)
  double* grad_params;       // (B, P) or nullptr
  double* grad_y0;           // (B, d) or nullptr
  void* record;
  void* scratch;
};

PDQ_HD int64_t tv_record_elems(int nu, int d, int capacity, int ckpt) {
  const int64_t n = nu + 1;
  const int64_t S = (int64_t(capacity) + ckpt - 1) / ckpt;
  return int64_t(capacity) + S * (n * d + n * n);
}

PDQ_HD int64_t tv_scratch_elems(int nu, int d, int ckpt) { return int64_t(ckpt) * (d + nu + 1); }

template <typename T, int NU, class F>
__global__ void __launch_bounds__(64) iso_tv_bwd_kernel(IsoArgs a, TvAdjArgs t) {
  constexpr int n = NU + 1, D = F::D, P = F::P, NT = D + P;
  constexpr bool kNarrow = sizeof(T) == sizeof(float);
  const int64_t b = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (b >= a.B) return;
  const int64_t B = a.B;
  if (t.status[b] != PDQ_INSTANCE_OK) {
    const double nan = __longlong_as_double(0x7ff8000000000000ULL);
    if (t.grad_params)
      for (int q = 0; q < P; ++q) t.grad_params[b * P + q] = nan;
    if (t.grad_y0)
      for (int j = 0; j < D; ++j) t.grad_y0[b * D + j] = nan;
    return;
  }
  const T* rec = reinterpret_cast<const T*>(t.record);
  T* scr = reinterpret_cast<T*>(t.scratch);
  const int N = t.num_steps[b];
  const int C = t.ckpt;

  double pd[P];
  T th[P];
#pragma unroll
  for (int q = 0; q < P; ++q) {
    pd[q] = a.params[b * P + q];
    th[q] = T(pd[q]);
  }
  // adjoint of the mean, from the cotangent of the terminal mean
  T mb[n][D];
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) mb[i][j] = T(t.cotangent[(b * n + i) * D + j]);
  double thb[P];
#pragma unroll
  for (int q = 0; q < P; ++q) thb[q] = 0.0;

  const int nseg = (N + C - 1) / C;
  for (int seg = nseg - 1; seg >= 0; --seg) {
    const int k0 = seg * C, k1 = min(k0 + C, N);
    // the segment's start
    T m[n][D], L[n][n];
    {
      int64_t e = int64_t(t.capacity) + int64_t(seg) * (n * D + n * n);
#pragma unroll
      for (int i = 0; i < n; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) m[i][j] = rec[(e++) * B + b];
#pragma unroll
      for (int i = 0; i < n; ++i)
#pragma unroll
        for (int j = 0; j < n; ++j) L[i][j] = rec[(e++) * B + b];
    }
    // recompute the segment: predicted u and gain of each step
    for (int k = k0; k < k1; ++k) {
      const T h = rec[int64_t(k) * B + b];
      T p[n], pinv[n], mp[n][D];
      precon<T, NU>(h, p, pinv);
      iso_predict_mean<T, NU, D>(m, p, pinv, mp);
      const T scale_q = kNarrow ? fast_sqrt(dev_abs(h)) : dev_sqrt(dev_abs(h));
      T gain[n], Lnew[n][n];
      bool ok = true;
      if constexpr (kNarrow) {
        iso_predict_update_fast<T, NU>(a.q1f, L, p, pinv, scale_q, gain, Lnew, ok);
      } else {
        iso_predict_update_fast<T, NU>(a.q1, L, p, pinv, scale_q, gain, Lnew, ok);
      }
      if (!ok) {  // the forward pass reran such a step with the range-checked predict and update
        T Lp[n][n];
        if constexpr (kNarrow) {
          iso_predict_chol<T, NU>(a.q1f, L, p, pinv, scale_q, Lp);
        } else {
          iso_predict_chol<T, NU>(a.q1, L, p, pinv, scale_q, Lp);
        }
        ts0_update<T, NU, 1, false>(Lp, T(0), gain, Lnew, T(0));
      }
      int64_t e = int64_t(k - k0) * (D + n);
#pragma unroll
      for (int j = 0; j < D; ++j) scr[(e++) * B + b] = mp[0][j];
#pragma unroll
      for (int i = 0; i < n; ++i) scr[(e++) * B + b] = gain[i];
      T f[D];
      F::eval(mp[0], th, f);
#pragma unroll
      for (int i = 0; i < n; ++i) {
#pragma unroll
        for (int j = 0; j < D; ++j) m[i][j] = mp[i][j] - gain[i] * (mp[1][j] - f[j]);
#pragma unroll
        for (int j = 0; j < n; ++j) L[i][j] = Lnew[i][j];
      }
    }
    // reverse the segment
    T thp[P];
#pragma unroll
    for (int q = 0; q < P; ++q) thp[q] = T(0);
    for (int k = k1 - 1; k >= k0; --k) {
      const T h = rec[int64_t(k) * B + b];
      T p[n], pinv[n];
      precon<T, NU>(h, p, pinv);
      T u[D], g[n];
      int64_t e = int64_t(k - k0) * (D + n);
#pragma unroll
      for (int j = 0; j < D; ++j) u[j] = scr[(e++) * B + b];
#pragma unroll
      for (int i = 0; i < n; ++i) g[i] = scr[(e++) * B + b];
      // m' = mp - g (mp[1] - f(mp[0]))
      T rbar[D];
#pragma unroll
      for (int j = 0; j < D; ++j) {
        T acc = T(0);
#pragma unroll
        for (int i = 0; i < n; ++i) acc += g[i] * mb[i][j];
        rbar[j] = -acc;  // adjoint of the residual mp[1] - f
      }
      T mpb[n][D];
#pragma unroll
      for (int i = 0; i < n; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) mpb[i][j] = mb[i][j];
#pragma unroll
      for (int j = 0; j < D; ++j) mpb[1][j] += rbar[j];
      {
        Dual<T, NT> ud[D], pt[P], fd[D];
#pragma unroll
        for (int j = 0; j < D; ++j) {
          ud[j] = Dual<T, NT>(u[j]);
          ud[j].g[j] = T(1);
        }
#pragma unroll
        for (int q = 0; q < P; ++q) {
          pt[q] = Dual<T, NT>(th[q]);
          pt[q].g[D + q] = T(1);
        }
        F::eval(ud, pt, fd);
#pragma unroll
        for (int j = 0; j < D; ++j) {
          T acc = T(0);
#pragma unroll
          for (int l = 0; l < D; ++l) acc += fd[l].g[j] * rbar[l];
          mpb[0][j] -= acc;  // f enters the residual with a minus sign
        }
#pragma unroll
        for (int q = 0; q < P; ++q) {
          T acc = T(0);
#pragma unroll
          for (int l = 0; l < D; ++l) acc += fd[l].g[D + q] * rbar[l];
          thp[q] -= acc;
        }
      }
      // mp = p . A1 (p^-1 . m)
#pragma unroll
      for (int k2 = 0; k2 < n; ++k2)
#pragma unroll
        for (int j = 0; j < D; ++j) {
          T acc = T(0);
#pragma unroll
          for (int i = 0; i <= k2; ++i) acc += T(iwp_a<NU>(i, k2)) * (p[i] * mpb[i][j]);
          mb[k2][j] = pinv[k2] * acc;
        }
    }
#pragma unroll
    for (int q = 0; q < P; ++q) thb[q] += double(thp[q]);
  }

  // ---- the Taylor-mode initialisation: d m_0 / d (theta, y0) on dual numbers (float64) ----
  constexpr int NI = P + D;
  Dual<double, NI> pdd[P], ydd[D];
#pragma unroll
  for (int q = 0; q < P; ++q) {
    pdd[q] = Dual<double, NI>(pd[q]);
    pdd[q].g[q] = 1.0;
  }
#pragma unroll
  for (int j = 0; j < D; ++j) {
    ydd[j] = Dual<double, NI>(a.y0[b * D + j]);
    ydd[j].g[P + j] = 1.0;
  }
  Dual<double, NI> tcd[n][D];
  taylor_init<F, NU>(ydd, pdd, tcd);
  double acc[NI];
#pragma unroll
  for (int q = 0; q < NI; ++q) acc[q] = 0.0;
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j)
#pragma unroll
      for (int q = 0; q < NI; ++q) acc[q] += double(mb[i][j]) * tcd[i][j].g[q];
  if (t.grad_params) {
#pragma unroll
    for (int q = 0; q < P; ++q) t.grad_params[b * P + q] = thb[q] + acc[q];
  }
  if (t.grad_y0) {
#pragma unroll
    for (int j = 0; j < D; ++j) t.grad_y0[b * D + j] = acc[P + j];
  }
}

}  // namespace pdq
