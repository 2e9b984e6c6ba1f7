// Isotropic TS0 adaptive filter, split over two warps per W instances: a
// covariance warp and a mean warp.
//
// Same algorithm and reference lines as iso_adaptive_kernel (iso_solver.cuh,
// the lean instantiation: TS0 without damping, error_residual_std, exact
// checkpoint landings, solver none or mle), and the same arithmetic, so the
// two agree bit for bit (up to the rare attempt whose later reflectors leave
// the safe range, below).  An ensemble solve is bound by the slowest
// instance's attempts run back to back, and a lone warp issues one
// instruction at a time; here each instance's attempt runs on two warps,
// lane i of each holding instance i of the block:
//
//   covariance warp  (the Cholesky factor L)     mean warp  (m, t, dt, the controller)
//   wait X: h, flags                              advance to the next attempt, publish h; arrive X
//   commit the accepted L, write its records      predict the mean, the TS0 residual
//   joint_x, joint_u, first reflector: gain, R_Y
//   publish gain, R_Y; arrive Y                   wait Y: gain, R_Y
//   the other reflectors: the candidate L         update the mean, error, accept, controller
//
// per attempt the covariance warp's predict-update QR overlaps the mean's
// predict and residual, and its last reflectors overlap the mean update, the
// error estimate and the controller.  The noise scale of the predict is
// sqrt|h| for solver none and mle (it does not wait for the residual), so
// the dynamic solver is not split.
//
// A fast (branch-free) attempt whose first reflector leaves the safe range
// reruns with the range-checked predict and update, as in the one-thread
// kernel; one whose later reflectors do recomputes only the candidate L with
// the range-checked path (the mean warp has used the first reflector's gain,
// which passed its check).
#pragma once

#include "iso_solver.cuh"

namespace pdq {

// The two named barriers of a block (id 0 is __syncthreads'):
// X: the mean warp's flags and step sizes are ready; Y: the gains are ready.
constexpr int kSplitBarX = 1;
constexpr int kSplitBarY = 2;

// flags of one exchange between the warps, per instance
constexpr int kSplitAttempt = 1;   // attempt with step size h
constexpr int kSplitSafe = 2;      // with the range-checked predict and update
constexpr int kSplitCommit = 4;    // the previous attempt was accepted: L = candidate

template <typename T, int NU, int W>
struct SplitShared {
  T h[W];
  int flags[W];
  int rec_lo[W], rec_cnt[W];  // records [rec_lo, rec_lo + rec_cnt) take the (committed) L
  int go;                     // some instance attempts in this exchange
  T gain[NU + 1][W];
  T ry[W];
  int ok[W];
};

// The mean warp's part of an output record (write_record without the
// factor, which the covariance warp writes): the mean with its wide rows,
// unit output scale (solver none; mle rescales at the end), time and steps.
template <typename T, int NU, int D>
PDQ_D void split_record_mean(const IsoArgs& a, int64_t rec, const T (&m)[NU + 1][D], const T (&lo)[2][D], double t,
                             int steps) {
  constexpr int n = NU + 1;
  double* um = a.u_mean + rec * (n * D);
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) um[i * D + j] = double(m[i][j]);
  if constexpr (sizeof(T) == sizeof(float)) {
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) um[i * D + j] += double(lo[i][j]);
  }
  a.output_scale[rec] = 1.0;
  a.t_out[rec] = t;
  a.num_steps[rec] = steps;
}

template <typename T, int NU, class F, int W>
__global__ void __launch_bounds__(2 * W) iso_split_kernel(IsoArgs a) {
  constexpr int n = NU + 1;
  constexpr int D = F::D;
  constexpr int P = F::P;
  constexpr int kThreads = 2 * W;
  constexpr bool kNarrow = sizeof(T) == sizeof(float);
  using Wd = Wide<T>;
  __shared__ SplitShared<T, NU, W> sh;
  const int lane = int(threadIdx.x) % W;
  const bool cov_warp = int(threadIdx.x) < W;
  const int64_t b = int64_t(blockIdx.x) * W + lane;
  const bool valid = b < a.B;  // every lane takes part in the barriers
  const int S = a.S;
  const int S_out = a.terminal_only ? 1 : S;

  if (cov_warp) {
    // ---------------- covariance warp ----------------
    T L[n][n], Lnew[n][n];
#pragma unroll
    for (int i = 0; i < n; ++i)
#pragma unroll
      for (int j = 0; j < n; ++j) L[i][j] = Lnew[i][j] = T(0);
    if (valid && !a.terminal_only) {
      double* uc = a.u_chol + b * S_out * (n * n);
      for (int k = 0; k < n * n; ++k) uc[k] = 0.0;
    }
    for (;;) {
      named_sync(kSplitBarX, kThreads);
      const T h = sh.h[lane];
      const int flags = sh.flags[lane];
      const int rec_lo = sh.rec_lo[lane], rec_cnt = sh.rec_cnt[lane];
      const int go = sh.go;
      if (flags & kSplitCommit) {
#pragma unroll
        for (int i = 0; i < n; ++i)
#pragma unroll
          for (int j = 0; j < n; ++j) L[i][j] = Lnew[i][j];
      }
      for (int r = 0; r < rec_cnt; ++r) {
        double* uc = a.u_chol + (b * S_out + rec_lo + r) * (n * n);
#pragma unroll
        for (int i = 0; i < n; ++i)
#pragma unroll
          for (int j = 0; j < n; ++j) uc[i * n + j] = double(L[i][j]);
      }
      if (!go) break;
      const bool attempt = flags & kSplitAttempt;
      const bool safe = flags & kSplitSafe;
      T p[n], pinv[n], gain[n], R_Y = T(1);
      T Z[2 * n][n + 1];
      bool ok = true;
#pragma unroll
      for (int i = 0; i < n; ++i) gain[i] = T(0);
      if (attempt) {
        precon<T, NU>(h, p, pinv);
        const T scale_q = kNarrow ? fast_sqrt(dev_abs(h)) : dev_sqrt(dev_abs(h));
        if (safe) {
          T Lp[n][n];
          if constexpr (kNarrow) {
            iso_predict_chol<T, NU>(a.q1f, L, p, pinv, scale_q, Lp);
          } else {
            iso_predict_chol<T, NU>(a.q1, L, p, pinv, scale_q, Lp);
          }
          R_Y = ts0_update<T, NU, 1, false>(Lp, T(0), gain, Lnew);
        } else {
          joint_x<T, NU>(L, pinv, Z);
          if constexpr (kNarrow) {
            joint_u<T, NU>(a.q1f, scale_q, Z);
          } else {
            joint_u<T, NU>(a.q1, scale_q, Z);
          }
          R_Y = joint_first<T, NU>(Z, p, pinv, gain, ok);
        }
      }
#pragma unroll
      for (int i = 0; i < n; ++i) sh.gain[i][lane] = gain[i];
      sh.ry[lane] = R_Y;
      sh.ok[lane] = ok ? 1 : 0;
      named_arrive(kSplitBarY, kThreads);
      if (attempt && !safe && ok) {
        bool ok_rest = true;
        joint_rest<T, NU>(Z, p, Lnew, ok_rest);
        if (!ok_rest) {
          const T scale_q = kNarrow ? fast_sqrt(dev_abs(h)) : dev_sqrt(dev_abs(h));
          T Lp[n][n], g2[n];
          if constexpr (kNarrow) {
            iso_predict_chol<T, NU>(a.q1f, L, p, pinv, scale_q, Lp);
          } else {
            iso_predict_chol<T, NU>(a.q1, L, p, pinv, scale_q, Lp);
          }
          ts0_update<T, NU, 1, false>(Lp, T(0), g2, Lnew);
        }
      }
    }
  } else {
    // ---------------- mean warp ----------------
    const double* save_at = a.save_at + (valid ? b : 0) * S;
    double pd[P];
    Wd pw[P];
#pragma unroll
    for (int k = 0; k < P; ++k) {
      pd[k] = valid ? a.params[b * P + k] : 1.0;
      pw[k] = wide_from(pd[k], T(0));
    }
    double y0[D];
#pragma unroll
    for (int j = 0; j < D; ++j) y0[j] = valid ? a.y0[b * D + j] : 1.0;
    double tc[n][D];
    taylor_init<F, NU>(y0, pd, tc);
    T m[n][D], mlo[2][D];
#pragma unroll
    for (int i = 0; i < n; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) m[i][j] = T(tc[i][j]);
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) mlo[i][j] = T(wide_lo(wide_from(tc[i][j], T(0))));

    Wd t = wide_from(save_at[0], T(0));
    T dt = T(valid ? a.dt0[b] : 1.0);
    T pi_prev = T(1);
    Wd mle_sumsq = wide_from(0.0, T(0));
    int num_data = 0, num_steps = 0, attempts = 0, status = PDQ_INSTANCE_OK;
    const T eps = cst<T>(a.eps, a.eps_f);
    constexpr int OUT = 1;
    T q1_out2 = T(0);
#pragma unroll
    for (int j = 0; j < n; ++j) q1_out2 += cst<T>(a.q1[OUT][j], a.q1f[OUT][j]) * cst<T>(a.q1[OUT][j], a.q1f[OUT][j]);
    const T q1_out_norm = dev_sqrt(q1_out2);
    auto before = [&](const Wd& x, const Wd& y) -> bool {
      if constexpr (kNarrow) {
        return wide_diff(y, x) > eps;
      } else {
        return x + a.eps < y;
      }
    };
    if (valid && !a.terminal_only) split_record_mean<T, NU, D>(a, b * S_out, m, mlo, wide_value(t), 0);

    int s = 1;
    Wd t_next = wide_from(save_at[S > 1 ? 1 : 0], T(0));
    bool live = valid && S > 1;
    bool safe = false, commit = false, clipped = false;
    T h = T(0);
    for (;;) {
      // advance to the next attempt: the checkpoint branches
      // (solvers_via_adaptive_steps.py:242-247) and the attempt's checks
      bool attempt = false;
      int rec_lo = 0, rec_cnt = 0;
      while (live) {
        if (before(t, t_next)) {
          const T remaining = wide_diff(t_next, t);
          clipped = a.clip_dt && !(dt < remaining);
          const T dt_use = clipped ? remaining : dt;
          if (!(dev_abs(dt_use) > T(1e-14) * fmax(T(1), dev_abs(T(wide_hi(t)))))) {
            status = PDQ_INSTANCE_DT_UNDERFLOW;
            live = false;
          } else if (attempts >= a.max_attempts) {
            status = PDQ_INSTANCE_MAX_STEPS;
            live = false;
          } else {
            ++attempts;
            h = dt_use;
            attempt = true;
          }
          break;
        }
        // interp_at_t1: the state itself is the solution (estimators_and_losses.py:416-421)
        if (!a.terminal_only || s == S - 1) {
          const int s_out = a.terminal_only ? 0 : s;
          split_record_mean<T, NU, D>(a, b * S_out + s_out, m, mlo, wide_value(t), num_steps);
          if (rec_cnt == 0) rec_lo = s_out;
          ++rec_cnt;
        }
        if (++s >= S) {
          live = false;
        } else {
          t_next = wide_from(save_at[s], T(0));
        }
      }
      sh.h[lane] = h;
      sh.flags[lane] = (attempt ? kSplitAttempt : 0) | (safe ? kSplitSafe : 0) | (commit ? kSplitCommit : 0);
      sh.rec_lo[lane] = rec_lo;
      sh.rec_cnt[lane] = rec_cnt;
      const bool go = __any_sync(0xffffffffu, attempt);
      if (lane == 0) sh.go = go ? 1 : 0;
      commit = false;
      named_arrive(kSplitBarX, kThreads);
      if (!go) break;

      // ---- the attempt's mean part (solvers_via_adaptive_steps.py:249-328) ----
      T p[n], pinv[n], incr[n][D], mp[n][D], mplo[2][D], mobs[D], rms_mobs = T(0);
      if (attempt) {
        precon<T, NU>(h, p, pinv);
        iso_mean_increment<T, NU, D>(m, p, pinv, incr);
        iso_mean_add<T, NU, D>(m, mlo, incr, mp, mplo);
        iso_residual<F, T, NU>(mp, mplo, pw, mobs);
        T mobs2 = T(0);
#pragma unroll
        for (int j = 0; j < D; ++j) mobs2 += mobs[j] * mobs[j];
        rms_mobs = fast_sqrt(mobs2 * T(1.0 / D));
      }
      named_sync(kSplitBarY, kThreads);
      if (!attempt) continue;
      T gain[n];
#pragma unroll
      for (int i = 0; i < n; ++i) gain[i] = sh.gain[i][lane];
      const T R_Y = sh.ry[lane];
      if (!sh.ok[lane]) {  // rerun with the range-checked predict and update
        safe = true;
        --attempts;
        continue;
      }
      safe = false;
      const T ry_inv = fast_rcp(R_Y);
      T mnew[n][D], mnewlo[2][D];
      {
        T dlt[n][D];
#pragma unroll
        for (int i = 0; i < n; ++i)
#pragma unroll
          for (int j = 0; j < D; ++j) dlt[i][j] = fma_nc(-gain[i], mobs[j], incr[i][j]);
        iso_mean_add<T, NU, D>(m, mlo, dlt, mnew, mnewlo);
      }
      bool accepted, nonfinite;
      T pi_new, dt_new;
      iso_accept_and_control<T, NU, D>(a, rms_mobs * h, m, mnew, h, pi_prev, accepted, nonfinite, pi_new, dt_new);
      if (nonfinite) {
        status = PDQ_INSTANCE_NONFINITE;
        live = false;
        continue;
      }
      dt = dt_new;
      pi_prev = pi_new;
      if (accepted) {
        if constexpr (kNarrow) {
          t = clipped ? t_next : wide_add(t, h);
        } else {
          t = t + h;
        }
        ++num_steps;
#pragma unroll
        for (int i = 0; i < n; ++i)
#pragma unroll
          for (int j = 0; j < D; ++j) m[i][j] = mnew[i][j];
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
          for (int j = 0; j < D; ++j) mlo[i][j] = mnewlo[i][j];
        if (a.solver == PDQ_SOLVER_MLE) {
          mle_sumsq = wide_add_sq(mle_sumsq, rms_mobs * dev_abs(ry_inv));
          ++num_data;
        }
        commit = true;
      }
    }

    // the covariance warp's records are written once both warps pass here
    __syncthreads();
    if (valid) {
      if (status == PDQ_INSTANCE_OK) {
        if (a.solver == PDQ_SOLVER_MLE) {
          // calibrated output scale (solvers.py:439-480)
          double scale = num_data > 0 ? sqrt(wide_value(mle_sumsq) / num_data) : 0.0;
          if (a.correct) scale = scale / sqrt(double(a.num_steps[b * S_out + (S_out - 1)]));
          for (int so = 0; so < S_out; ++so) {
            const int64_t rec = b * S_out + so;
            double* uc = a.u_chol + rec * (n * n);
            for (int k = 0; k < n * n; ++k) uc[k] *= scale;
            a.output_scale[rec] = scale;
          }
        }
      } else {
        const double nan = __longlong_as_double(0x7ff8000000000000ULL);
        for (int so = 0; so < S_out; ++so) {
          const int64_t rec = b * S_out + so;
          for (int k = 0; k < n * D; ++k) a.u_mean[rec * (n * D) + k] = nan;
          for (int k = 0; k < n * n; ++k) a.u_chol[rec * (n * n) + k] = nan;
          a.output_scale[rec] = nan;
          a.t_out[rec] = nan;
          a.num_steps[rec] = num_steps;
        }
      }
      a.num_attempts[b] = attempts;
      a.status[b] = status;
    }
    return;
  }
  __syncthreads();
}

}  // namespace pdq
