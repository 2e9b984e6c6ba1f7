// Isotropic TS0 adaptive filter with exact checkpoint landings: the
// instantiation the library launches for the filter with TS0 without
// damping, error_residual_std and clip_dt, with the attempt loop written
// branch-light.
//
// Same algorithm, arithmetic and reference lines as iso_adaptive_kernel's
// lean instantiation (iso_solver.cuh), so the outputs are the same bit for
// bit; what differs is the shape of the loop.  An ensemble solve is bound by
// the slowest instance's attempts run back to back, each a chain of
// dependent operations (the first reflector of the joint predict-update QR,
// the gain, the mean update, the error norm and the controller) that the
// compiler schedules within one basic block.  In the general kernel the
// attempt is framed by branches -- the step-underflow and attempt-bound
// checks before it, the rerun of a range-failed attempt, the non-finite
// exit and the accepted-state update after it -- and no instruction moves
// across a branch, so every attempt also pays the checks' and the state
// update's latency in series.  Here the checks are computed alongside the
// attempt, the state update is a set of selects in the same block, and one
// rarely taken branch after it handles every exit and the rerun.  The
// checkpoint branches (records, the next save point) run at the head of the
// loop only when a step has landed on a checkpoint.
#pragma once

#include "iso_solver.cuh"

namespace pdq {

template <typename T, int NU, class F>
__global__ void __launch_bounds__(64) iso_lean_kernel(IsoArgs a) {
  constexpr int n = NU + 1;
  constexpr int D = F::D;
  constexpr int P = F::P;
  constexpr int OUT = 1;  // ODE u' = f(u): observe coefficient 1 (problems.py:283-295)
  constexpr bool kNarrow = sizeof(T) == sizeof(float);
  using W = Wide<T>;
  const int64_t b = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (b >= a.B) return;

  const int S = a.S;
  const int S_out = a.terminal_only ? 1 : S;
  const double* save_at = a.save_at + b * S;

  // ---- inputs and Taylor-mode initial derivatives (float64) ----
  double pd[P];
#pragma unroll
  for (int k = 0; k < P; ++k) pd[k] = a.params[b * P + k];
  W pw[P];
#pragma unroll
  for (int k = 0; k < P; ++k) pw[k] = wide_from(pd[k], T(0));
  double y0[D];
#pragma unroll
  for (int j = 0; j < D; ++j) y0[j] = a.y0[b * D + j];
  double tc[n][D];
  taylor_init<F, NU>(y0, pd, tc);
  T m[n][D], mlo[2][D], L[n][n];
#pragma unroll
  for (int i = 0; i < n; ++i) {
#pragma unroll
    for (int j = 0; j < D; ++j) m[i][j] = T(tc[i][j]);
#pragma unroll
    for (int j = 0; j < n; ++j) L[i][j] = T(0);
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) mlo[i][j] = T(wide_lo(wide_from(tc[i][j], T(0))));

  W t = wide_from(save_at[0], T(0));
  T dt = T(a.dt0[b]);
  T pi_prev = T(1);  // PI controller state (controllers.py:41-43)
  W mle_sumsq = wide_from(0.0, T(0));
  int num_data = 0, num_steps = 0, attempts = 0, status = PDQ_INSTANCE_OK;
  T sigma_sf = T(1);  // output scale of step_from (dynamic solver)
  const T eps = cst<T>(a.eps, a.eps_f);
  const bool mle = a.solver == PDQ_SOLVER_MLE;
  const bool dynamic = a.solver == PDQ_SOLVER_DYNAMIC;
  T q1_out2 = T(0);
#pragma unroll
  for (int j = 0; j < n; ++j) q1_out2 += cst<T>(a.q1[OUT][j], a.q1f[OUT][j]) * cst<T>(a.q1[OUT][j], a.q1f[OUT][j]);
  const T q1_out_norm = dev_sqrt(q1_out2);

  if (!a.terminal_only) write_record<T, NU, D>(a, b, 0, S_out, m, mlo, L, 1.0, wide_value(t), 0);

  // t + eps < t_next (float64: exactly the reference's comparison; float
  // pairs: the difference, rounded once, against eps)
  auto before = [&](const W& x, const W& y) -> bool {
    if constexpr (kNarrow) {
      return wide_diff(y, x) > eps;
    } else {
      return x + a.eps < y;
    }
  };

  // One attempt per iteration, as in iso_adaptive_kernel
  // (solvers_via_adaptive_steps.py:196-375); before(t, t_next) and
  // t_next - t are carried from the attempt that set t.
  int s = 1;
  W t_next = wide_from(save_at[1], T(0));
  bool bef = before(t, t_next);
  T rem = wide_diff(t_next, t);
  bool safe_next = false;  // this attempt takes the range-checked predict and update
  for (;;) {
    // ---- checkpoint branches, once a step has landed (solvers_via_adaptive_steps.py:242-247) ----
    if (!bef) {
      do {
        // interp_at_t1: the state itself is the solution (estimators_and_losses.py:416-421)
        if (!a.terminal_only || s == S - 1)
          write_record<T, NU, D>(a, b, a.terminal_only ? 0 : s, S_out, m, mlo, L, double(sigma_sf), wide_value(t),
                                 num_steps);
        if (++s >= S) break;
        t_next = wide_from(save_at[s], T(0));
        bef = before(t, t_next);
        rem = wide_diff(t_next, t);
      } while (!bef);
      if (s >= S) break;
    }

    // ---- one attempt of the rejection loop (solvers_via_adaptive_steps.py:249-328) ----
    const bool clipped = !(dt < rem);  // clip_dt
    const T h = clipped ? rem : dt;
    const bool underflow = !(dev_abs(h) > T(1e-14) * fmax(T(1), dev_abs(T(wide_hi(t)))));
    const bool exhausted = attempts >= a.max_attempts;
    // the time after this attempt if it is accepted: a step clipped to the
    // checkpoint lands on it exactly in float pairs; float64 adds as the
    // reference does
    W t_acc;
    if constexpr (kNarrow) {
      t_acc = clipped ? t_next : wide_add(t, h);
    } else {
      t_acc = t + h;
    }
    const bool bef_acc = before(t_acc, t_next);
    const T rem_acc = wide_diff(t_next, t_acc);

    T mnew[n][D], mnewlo[2][D], Lnew[n][n];
    T rms_mobs, sigma_loc, ry_inv, dt_new, pi_new;
    bool accepted, nonfinite, ok;
    auto attempt = [&](auto safe_tag) {
      constexpr bool SAFE = decltype(safe_tag)::value;
      T p[n], pinv[n];
      precon<T, NU>(h, p, pinv);
      // extrapolated mean in increment form, rows 0 and 1 wide (solvers.py:943-944)
      T incr[n][D], mp[n][D], mplo[2][D];
      iso_mean_increment<T, NU, D>(m, p, pinv, incr);
      iso_mean_add<T, NU, D>(m, mlo, incr, mp, mplo);
      // TS0 residual mp_1 - f(mp_0) in the wide type (ssm_impl_isotropic.py:304-317)
      T mobs[D];
      iso_residual<F, T, NU>(mp, mplo, pw, mobs);
      T mobs2 = T(0);
#pragma unroll
      for (int j = 0; j < D; ++j) mobs2 += mobs[j] * mobs[j];
      rms_mobs = fast_sqrt(mobs2 * T(1.0 / D));
      // residual_whitened_rms with the observed std at unit scale (solvers.py:553-566, 955-957)
      sigma_loc = dev_div(rms_mobs, observed_std(p[OUT], h, q1_out_norm, T(0)));
      // predict (marginalise) and update (revert_conditional, H = e_1)
      const T s_pred = dynamic ? sigma_loc : T(1);
      const T scale_q = s_pred * (kNarrow ? fast_sqrt(dev_abs(h)) : dev_sqrt(dev_abs(h)));
      T gain[n], R_Y;
      ok = true;
      if constexpr (SAFE) {
        T Lp[n][n];
        if constexpr (kNarrow) {
          iso_predict_chol<T, NU>(a.q1f, L, p, pinv, scale_q, Lp);
        } else {
          iso_predict_chol<T, NU>(a.q1, L, p, pinv, scale_q, Lp);
        }
        R_Y = ts0_update<T, NU, OUT, false>(Lp, T(0), gain, Lnew);
      } else if constexpr (kNarrow) {
        R_Y = iso_predict_update_fast<T, NU>(a.q1f, L, p, pinv, scale_q, gain, Lnew, ok);
      } else {
        R_Y = iso_predict_update_fast<T, NU>(a.q1, L, p, pinv, scale_q, gain, Lnew, ok);
      }
      ry_inv = fast_rcp(R_Y);
      // mnew = m + (incr - gain mobs), the wide rows summed wide
      T dlt[n][D];
#pragma unroll
      for (int i = 0; i < n; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) dlt[i][j] = fma_nc(-gain[i], mobs[j], incr[i][j]);
      iso_mean_add<T, NU, D>(m, mlo, dlt, mnew, mnewlo);
      // error_residual_std: error = rms * dt (solvers.py:925-996), norm, controller
      iso_accept_and_control<T, NU, D>(a, rms_mobs * h, m, mnew, h, pi_prev, accepted, nonfinite, pi_new, dt_new);
    };
    if (safe_next) {
      attempt(BoolTag<true>{});
    } else {
      attempt(BoolTag<false>{});
    }

    // ---- the state update as selects; every exit and the rerun in one branch ----
    const bool stop = underflow || exhausted;
    const bool counts = !stop && ok;  // an attempt the reference makes (a range-failed one reruns)
    const bool valid = counts && !nonfinite;
    const bool commit = valid && accepted;
    attempts += counts ? 1 : 0;
    dt = valid ? dt_new : dt;
    pi_prev = valid ? pi_new : pi_prev;
    t = commit ? t_acc : t;
    bef = commit ? bef_acc : bef;
    rem = commit ? rem_acc : rem;
    num_steps += commit ? 1 : 0;
#pragma unroll
    for (int i = 0; i < n; ++i) {
#pragma unroll
      for (int j = 0; j < D; ++j) m[i][j] = commit ? mnew[i][j] : m[i][j];
#pragma unroll
      for (int j = 0; j <= i; ++j) L[i][j] = commit ? Lnew[i][j] : L[i][j];
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) mlo[i][j] = commit ? mnewlo[i][j] : mlo[i][j];
    // running scale via the hypot recurrence == RMS of the new terms (solvers.py:421-424)
    const W sumsq_new = wide_add_sq(mle_sumsq, rms_mobs * dev_abs(ry_inv));
    mle_sumsq = (commit && mle) ? sumsq_new : mle_sumsq;
    num_data += (commit && mle) ? 1 : 0;
    sigma_sf = commit ? (dynamic ? sigma_loc : T(1)) : sigma_sf;
    // Termination: every iteration either counts an attempt (bounded by
    // max_attempts, checked above) or, after a fast attempt that left the
    // safe range, reruns it with the range-checked path, which always counts.
    if (!valid) {
      if (stop) {
        status = underflow ? PDQ_INSTANCE_DT_UNDERFLOW : PDQ_INSTANCE_MAX_STEPS;
        break;
      }
      if (!ok) {  // rerun with the range-checked predict and update
        safe_next = true;
        continue;
      }
      status = PDQ_INSTANCE_NONFINITE;  // a non-finite attempt is never accepted
      break;
    }
    safe_next = false;
  }

  // ---- finalize: calibrated output scale (solvers.py:439-480, 601-633, 735-767) ----
  if (status == PDQ_INSTANCE_OK) {
    if (mle) {
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

}  // namespace pdq
