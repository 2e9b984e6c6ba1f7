// Isotropic TS0 filter, warp-specialised: two warps per 32 instances.
//
// Same algorithm and reference lines as iso_solver.cuh (one thread per
// instance, lean instantiation: TS0 without damping, error_residual_std,
// the filter strategy).  An ensemble solve is bound by the latency of the
// slowest instance's attempts, which run back to back, and one thread per
// instance runs an attempt's three chains -- the covariance (predict and
// update in one QR), the mean and its residual, and the error estimate with
// the step-size controller -- one after the other: the compiler does not
// interleave them.  Here lane l of the covariance warp (warp 0) and lane l
// of the control warp (warp 1) hold the same instance:
//   * the covariance warp keeps the Cholesky factor L (and the interpolation
//     factor), forms the joint predict-update matrix, publishes the gain and
//     R_Y after the first reflector and runs the remaining reflectors while
//   * the control warp, which keeps the mean, the time, the step size and
//     every counter, takes the plan decisions (attempt, checkpoint, accept),
//     forms the mean's increment and the residual, and after the gain the
//     updated mean, the error estimate and the controller.
// Per iteration of the flattened loop the two warps meet at two block
// barriers (three for dynamic calibration, whose output scale enters the
// covariance predict): PLAN (the control warp's decisions for this
// iteration), [SIGMA], GAIN.  Both warps execute every barrier; lanes
// without work idle through them, and the loop ends for both warps at the
// same PLAN barrier, when no lane of the pair has work left.  One iteration
// is either one attempt or one checkpoint of an instance, so the per-instance
// sequence of attempts, accept decisions and records is the one-thread
// kernel's.
#pragma once

#include "iso_solver.cuh"

namespace pdq {

// Per-lane plan (control warp -> covariance warp).
enum : int {
  kPlanCommit = 1,      // the previous iteration's attempt was accepted: L <- Lnew
  kPlanAttempt = 2,     // attempt with step h
  kPlanLanding = 4,     // checkpoint reached exactly: the state is the record
  kPlanInterp = 8,      // checkpoint passed: predict the interpolation state by h_cp
  kPlanRecord = 16,     // the checkpoint writes record s_out
};

template <typename T>
struct PairPlan {
  int flags;
  int s_out;
  T h;         // attempt step
  T h_cp;      // interpolation step (kPlanInterp)
  T scale_cp;  // output scale of the interpolation predict
};

template <typename T, int NU, class F, bool INTERP>
__global__ void __launch_bounds__(64) iso_pair_kernel(IsoArgs a) {
  constexpr int n = NU + 1;
  constexpr int D = F::D;
  constexpr int P = F::P;
  constexpr int OUT = 1;
  using W = Wide<T>;
  constexpr bool kNarrow = sizeof(T) == sizeof(float);

  __shared__ PairPlan<T> plan[32];
  __shared__ T sh_gain[n][32];
  __shared__ T sh_ry[32];
  __shared__ T sh_sigma[32];
  __shared__ double sh_scale[32];
  __shared__ int sh_status[32];
  __shared__ int sh_more;

  const int lane = threadIdx.x & 31;
  const bool cov = threadIdx.x < 32;
  const int64_t b = int64_t(blockIdx.x) * 32 + lane;
  const bool valid = b < a.B;
  const int S = a.S;
  const int S_out = a.terminal_only ? 1 : S;
  const bool dynamic = a.solver == PDQ_SOLVER_DYNAMIC;
  const T damp = cst<T>(a.damp, a.damp_f);

  // ---- covariance warp state ----
  T L[n][n], Li[n][n], Lnew[n][n];
  T Z[2 * n][n + 1];
  T p[n], pinv[n];
  bool ok1 = true;
  // ---- control warp state ----
  T m[n][D], mlo[2][D], mi[n][D], milo[2][D];
  Wide<T> pw[P];
  W t, ti, t_next;
  T dt = T(0), pi_prev = T(1), sigma_sf = T(1);
  W mle_sumsq = wide_from(0.0, T(0));
  int num_data = 0, num_steps = 0, attempts = 0, status = PDQ_INSTANCE_OK, s = 1;
  bool active = valid, commit_pending = false;
  const double* save_at = a.save_at + (valid ? b : 0) * S;
  T incr[n][D], mp[n][D], mplo[2][D], mobs[D];
  T rms_mobs = T(0), sigma_loc = T(0), h_att = T(0);
  bool clipped = false;
  const T eps = cst<T>(a.eps, a.eps_f);
  const T atol = cst<T>(a.atol, a.atol_f), rtol = cst<T>(a.rtol, a.rtol_f);
  const T safety = cst<T>(a.safety, a.safety_f);
  const T factor_min = cst<T>(a.factor_min, a.factor_min_f), factor_max = cst<T>(a.factor_max, a.factor_max_f);
  T q1_out2 = T(0);
#pragma unroll
  for (int j = 0; j < n; ++j) q1_out2 += cst<T>(a.q1[OUT][j], a.q1f[OUT][j]) * cst<T>(a.q1[OUT][j], a.q1f[OUT][j]);
  const T q1_out_norm = dev_sqrt(q1_out2);

  auto before = [&](const W& x, const W& y) -> bool {
    if constexpr (kNarrow) {
      return wide_diff(y, x) > eps;
    } else {
      return x + a.eps < y;
    }
  };

  if (cov) {
#pragma unroll
    for (int i = 0; i < n; ++i)
#pragma unroll
      for (int j = 0; j < n; ++j) L[i][j] = Li[i][j] = Lnew[i][j] = T(0);
    if (valid && !a.terminal_only) {
      double* uc = a.u_chol + (b * S_out) * (n * n);
      for (int k = 0; k < n * n; ++k) uc[k] = 0.0;
    }
  } else {
#pragma unroll
    for (int i = 0; i < n; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) m[i][j] = mi[i][j] = T(0);
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) mlo[i][j] = milo[i][j] = T(0);
#pragma unroll
    for (int k = 0; k < P; ++k) pw[k] = wide_from(0.0, T(0));
    t = ti = t_next = wide_from(0.0, T(0));
    if (valid) {
      double pd[P], y0[D], tc[n][D];
#pragma unroll
      for (int k = 0; k < P; ++k) {
        pd[k] = a.params[b * P + k];
        pw[k] = wide_from(pd[k], T(0));
      }
#pragma unroll
      for (int j = 0; j < D; ++j) y0[j] = a.y0[b * D + j];
      taylor_init<F, NU>(y0, pd, tc);
#pragma unroll
      for (int i = 0; i < n; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) m[i][j] = mi[i][j] = T(tc[i][j]);
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) mlo[i][j] = milo[i][j] = T(wide_lo(wide_from(tc[i][j], T(0))));
      t = ti = wide_from(save_at[0], T(0));
      t_next = wide_from(save_at[1], T(0));
      dt = T(a.dt0[b]);
      if (!a.terminal_only) {
        const int64_t rec = b * S_out;
        double* um = a.u_mean + rec * (n * D);
        for (int i = 0; i < n; ++i)
          for (int j = 0; j < D; ++j) um[i * D + j] = double(m[i][j]) + (i < 2 ? double(mlo[i < 2 ? i : 0][j]) : 0.0);
        a.output_scale[rec] = 1.0;
        a.t_out[rec] = wide_value(t);
        a.num_steps[rec] = 0;
      }
    }
  }

  for (;;) {
    // ---- PLAN: the control warp decides this iteration for each instance ----
    if (!cov) {
      int flags = commit_pending ? kPlanCommit : 0;
      commit_pending = false;
      PairPlan<T> pl;
      pl.s_out = 0;
      pl.h = T(0);
      pl.h_cp = T(0);
      pl.scale_cp = T(1);
      if (active && s >= S) active = false;
      if (active) {
        if (before(t, t_next)) {
          // one attempt of the rejection loop (solvers_via_adaptive_steps.py:249-328)
          const T remaining = wide_diff(t_next, t);
          clipped = a.clip_dt && !(dt < remaining);
          const T dt_use = clipped ? remaining : dt;
          if (!(dev_abs(dt_use) > T(1e-14) * fmax(T(1), dev_abs(T(wide_hi(t)))))) {
            status = PDQ_INSTANCE_DT_UNDERFLOW;
            active = false;
          } else if (attempts >= a.max_attempts) {
            status = PDQ_INSTANCE_MAX_STEPS;
            active = false;
          } else {
            ++attempts;
            h_att = dt_use;
            pl.h = dt_use;
            flags |= kPlanAttempt;
          }
        } else {
          // checkpoint s (solvers_via_adaptive_steps.py:242-247): the mean's
          // part here, the covariance's in the other warp
          const int s_out = a.terminal_only ? 0 : s;
          const bool record = (!a.terminal_only) || (s == S - 1);
          pl.s_out = s_out;
          if (record) flags |= kPlanRecord;
          if (INTERP && before(t_next, t)) {
            // interp_beyond_t1: predict from interp_from to t_next
            // (solvers.py:205-269, estimators_and_losses.py:403-414)
            const T h = T(wide_diff(t_next, ti));
            T pp[n], ppi[n], inc[n][D], mq[n][D], mqlo[2][D];
            precon<T, NU>(h, pp, ppi);
            iso_mean_increment<T, NU, D>(mi, pp, ppi, inc);
            iso_mean_add<T, NU, D>(mi, milo, inc, mq, mqlo);
            flags |= kPlanInterp;
            pl.h_cp = h;
            pl.scale_cp = sigma_sf;
            if (record) {
              const int64_t rec = b * S_out + s_out;
              double* um = a.u_mean + rec * (n * D);
              for (int i = 0; i < n; ++i)
                for (int j = 0; j < D; ++j)
                  um[i * D + j] = double(mq[i][j]) + (i < 2 ? double(mqlo[i < 2 ? i : 0][j]) : 0.0);
              a.output_scale[rec] = double(sigma_sf);
              a.t_out[rec] = wide_value(t_next);
              a.num_steps[rec] = num_steps;
            }
            ti = t_next;
#pragma unroll
            for (int i = 0; i < n; ++i)
#pragma unroll
              for (int j = 0; j < D; ++j) mi[i][j] = mq[i][j];
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
              for (int j = 0; j < D; ++j) milo[i][j] = mqlo[i][j];
          } else {
            // interp_at_t1: the state itself is the solution (estimators_and_losses.py:416-421)
            flags |= kPlanLanding;
            if (record) {
              const int64_t rec = b * S_out + s_out;
              double* um = a.u_mean + rec * (n * D);
              for (int i = 0; i < n; ++i)
                for (int j = 0; j < D; ++j)
                  um[i * D + j] = double(m[i][j]) + (i < 2 ? double(mlo[i < 2 ? i : 0][j]) : 0.0);
              a.output_scale[rec] = double(sigma_sf);
              a.t_out[rec] = wide_value(t);
              a.num_steps[rec] = num_steps;
            }
            if constexpr (INTERP) {
              ti = t;
#pragma unroll
              for (int i = 0; i < n; ++i)
#pragma unroll
                for (int j = 0; j < D; ++j) mi[i][j] = m[i][j];
#pragma unroll
              for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < D; ++j) milo[i][j] = mlo[i][j];
            }
          }
          ++s;
          if (s < S) t_next = wide_from(save_at[s], T(0));
        }
      }
      pl.flags = flags;
      plan[lane] = pl;
      const bool more = __any_sync(0xffffffffu, flags != 0);
      if (lane == 0) sh_more = more ? 1 : 0;
    }
    __syncthreads();  // PLAN
    if (!sh_more) break;

    const PairPlan<T> pl = plan[lane];
    const bool attempt = (pl.flags & kPlanAttempt) != 0;
    if (cov) {
      if (pl.flags & kPlanCommit) {
#pragma unroll
        for (int i = 0; i < n; ++i)
#pragma unroll
          for (int j = 0; j < n; ++j) {
            if constexpr (INTERP) Li[i][j] = L[i][j];
            L[i][j] = Lnew[i][j];
          }
      }
      if (pl.flags & (kPlanLanding | kPlanInterp)) {
        T Lr[n][n];
        if (pl.flags & kPlanInterp) {
          T pp[n], ppi[n];
          precon<T, NU>(pl.h_cp, pp, ppi);
          if constexpr (kNarrow) {
            iso_predict_chol<T, NU>(a.q1f, Li, pp, ppi, pl.scale_cp * dev_sqrt(dev_abs(pl.h_cp)), Lr);
          } else {
            iso_predict_chol<T, NU>(a.q1, Li, pp, ppi, pl.scale_cp * dev_sqrt(dev_abs(pl.h_cp)), Lr);
          }
        } else {
#pragma unroll
          for (int i = 0; i < n; ++i)
#pragma unroll
            for (int j = 0; j < n; ++j) Lr[i][j] = L[i][j];
        }
        if (pl.flags & kPlanRecord) {
          double* uc = a.u_chol + (b * S_out + pl.s_out) * (n * n);
          for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) uc[i * n + j] = double(Lr[i][j]);
        }
        if constexpr (INTERP) {
#pragma unroll
          for (int i = 0; i < n; ++i)
#pragma unroll
            for (int j = 0; j < n; ++j) Li[i][j] = Lr[i][j];
        }
      }
      if (attempt) {
        precon<T, NU>(pl.h, p, pinv);
        joint_x<T, NU>(L, pinv, Z);
      }
    } else if (attempt) {
      // extrapolated mean in increment form (rows 0 and 1 wide) and the
      // TS0 residual mp_1 - f(mp_0) in the wide type
      const T h = h_att;
      T pm[n], pminv[n];
      precon<T, NU>(h, pm, pminv);
      iso_mean_increment<T, NU, D>(m, pm, pminv, incr);
      iso_mean_add<T, NU, D>(m, mlo, incr, mp, mplo);
      iso_residual<F, T, NU>(mp, mplo, pw, mobs);
      T mobs2 = T(0);
#pragma unroll
      for (int j = 0; j < D; ++j) mobs2 += mobs[j] * mobs[j];
      rms_mobs = fast_sqrt(mobs2 * T(1.0 / D));
      sigma_loc = dev_div(rms_mobs, observed_std(pm[OUT], h, q1_out_norm, damp));
      sh_sigma[lane] = sigma_loc;
    }
    if (dynamic) __syncthreads();  // SIGMA: the dynamic output scale enters the predict

    if (cov && attempt) {
      const T s_pred = dynamic ? sh_sigma[lane] : T(1);
      const T scale_q = s_pred * (kNarrow ? fast_sqrt(dev_abs(pl.h)) : dev_sqrt(dev_abs(pl.h)));
      T gain[n];
      ok1 = true;
      if constexpr (kNarrow) {
        joint_u<T, NU>(a.q1f, scale_q, Z);
      } else {
        joint_u<T, NU>(a.q1, scale_q, Z);
      }
      T R_Y = joint_first<T, NU>(Z, p, pinv, gain, ok1);
      if (!ok1) {  // the range-checked predict and update
        T Lp[n][n];
        if constexpr (kNarrow) {
          iso_predict_chol<T, NU>(a.q1f, L, p, pinv, scale_q, Lp);
        } else {
          iso_predict_chol<T, NU>(a.q1, L, p, pinv, scale_q, Lp);
        }
        R_Y = ts0_update<T, NU, OUT, false>(Lp, damp, gain, Lnew);
      }
#pragma unroll
      for (int i = 0; i < n; ++i) sh_gain[i][lane] = gain[i];
      sh_ry[lane] = R_Y;
    }
    __syncthreads();  // GAIN

    if (cov) {
      if (attempt && ok1) {
        bool ok = true;
        joint_rest<T, NU>(Z, p, Lnew, ok);
        if (!ok) {  // the range-checked predict and update (the gain was in range)
          const T s_pred = dynamic ? sh_sigma[lane] : T(1);
          const T scale_q = s_pred * (kNarrow ? fast_sqrt(dev_abs(pl.h)) : dev_sqrt(dev_abs(pl.h)));
          T Lp[n][n], g2[n];
          if constexpr (kNarrow) {
            iso_predict_chol<T, NU>(a.q1f, L, p, pinv, scale_q, Lp);
          } else {
            iso_predict_chol<T, NU>(a.q1, L, p, pinv, scale_q, Lp);
          }
          ts0_update<T, NU, OUT, false>(Lp, damp, g2, Lnew);
        }
      }
    } else if (attempt) {
      const T h = h_att;
      T gain[n];
#pragma unroll
      for (int i = 0; i < n; ++i) gain[i] = sh_gain[i][lane];
      const T ry_inv = fast_rcp(sh_ry[lane]);
      // mnew = m + (incr - gain mobs), the wide rows summed wide
      T mnew[n][D], mnewlo[2][D];
      {
        T dlt[n][D];
#pragma unroll
        for (int i = 0; i < n; ++i)
#pragma unroll
          for (int j = 0; j < D; ++j) dlt[i][j] = incr[i][j] - gain[i] * mobs[j];
        iso_mean_add<T, NU, D>(m, mlo, dlt, mnew, mnewlo);
      }
      // error_residual_std (solvers.py:925-996): error = rms * dt^1/1!
      const T err_abs = rms_mobs * h;
      W sumsq = wide_from(0.0, T(0));
#pragma unroll
      for (int j = 0; j < D; ++j) {
        const T ref = fmax(dev_abs(m[0][j]), dev_abs(mnew[0][j]));
        const T ratio = dev_div(err_abs, atol + rtol * ref);
        sumsq = wide_add_sq(sumsq, ratio);
      }
      const T norm2 = T(wide_hi(sumsq)) * T(1.0 / D);
      const bool nonfinite = !(norm2 == norm2) || isinf(norm2);
      const T ep = dev_fpow(norm2, T(-0.5 / n));
      const bool accepted = wide_le(sumsq, T(D));
      // controller (controllers.py:24-84)
      T factor;
      T pi_new = pi_prev;
      if (a.control == PDQ_CONTROL_INTEGRAL) {
        factor = safety * ep;
      } else {
        const T gi = dev_fpow(ep, cst<T>(a.exp_i, a.exp_i_f));
        const T gp = dev_fpow(dev_div(ep, pi_prev), cst<T>(a.exp_p, a.exp_p_f));
        factor = safety * gi * gp;
        if (accepted) pi_new = ep;
      }
      factor = fmax(factor_min, fmin(factor, factor_max));
      if (nonfinite) {
        status = PDQ_INSTANCE_NONFINITE;
        active = false;
      } else {
        dt = factor * h;
        pi_prev = pi_new;
        if (accepted) {
          if constexpr (INTERP) {
            ti = t;
#pragma unroll
            for (int i = 0; i < n; ++i)
#pragma unroll
              for (int j = 0; j < D; ++j) mi[i][j] = m[i][j];
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
              for (int j = 0; j < D; ++j) milo[i][j] = mlo[i][j];
          }
          // a step clipped to the checkpoint lands on it exactly in float
          // pairs; float64 adds as the reference does
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
            // running scale via hypot recurrence == RMS of new terms (solvers.py:421-424)
            mle_sumsq = wide_add_sq(mle_sumsq, rms_mobs * dev_abs(ry_inv));
            ++num_data;
          }
          sigma_sf = dynamic ? sigma_loc : T(1);
          commit_pending = true;
        }
      }
    }
  }

  // ---- finalize: calibrated output scale (solvers.py:439-480, 601-633, 735-767) ----
  if (!cov) {
    double scale = 1.0;
    if (valid && status == PDQ_INSTANCE_OK && a.solver == PDQ_SOLVER_MLE) {
      scale = num_data > 0 ? sqrt(wide_value(mle_sumsq) / num_data) : 0.0;
      if (a.correct) scale = scale / sqrt(double(a.num_steps[b * S_out + (S_out - 1)]));
      for (int k = 0; k < S_out; ++k) a.output_scale[b * S_out + k] = scale;
    }
    if (valid && status != PDQ_INSTANCE_OK) {
      const double nan = __longlong_as_double(0x7ff8000000000000ULL);
      for (int k = 0; k < S_out; ++k) {
        const int64_t rec = b * S_out + k;
        for (int e = 0; e < n * D; ++e) a.u_mean[rec * (n * D) + e] = nan;
        a.output_scale[rec] = nan;
        a.t_out[rec] = nan;
        a.num_steps[rec] = num_steps;
      }
    }
    if (valid) {
      a.num_attempts[b] = attempts;
      a.status[b] = status;
    }
    sh_scale[lane] = scale;
    sh_status[lane] = status;
  }
  __syncthreads();
  if (cov && valid) {
    const double nan = __longlong_as_double(0x7ff8000000000000ULL);
    const bool ok = sh_status[lane] == PDQ_INSTANCE_OK;
    const bool mle = a.solver == PDQ_SOLVER_MLE;
    for (int k = 0; k < S_out; ++k) {
      double* uc = a.u_chol + (b * S_out + k) * (n * n);
      for (int e = 0; e < n * n; ++e) {
        if (!ok) uc[e] = nan;
        else if (mle) uc[e] *= sh_scale[lane];
      }
    }
  }
}

}  // namespace pdq
