// Dense-factorisation adaptive solver: one thread per IVP instance.
//
// State: mean (N,) coefficient-major [u, u', ...] and Cholesky (N, N), with
// N = (nu + 1) d, as in _probdiffeq/ssm_impl_dense.py.  Per attempt it follows
//   DenseWienerIntegrated.transition        ssm_impl_dense.py:347-363
//   DenseLatentCond.apply_flat / marginalise ssm_impl_dense.py:18-33
//   DenseLatentCond.revert / merge          ssm_impl_dense.py:35-77
//   DenseResidual.linearize (TS1)           ssm_impl_dense.py:290-334 with
//     residual_from_ode (problems.py:518-532), taylor_point_prior
//     (taylor_points.py:150-156) and a materialised Jacobian (jacobians.py:93-98)
//   DenseOdeTs0.linearize (TS0)             ssm_impl_dense.py:243-259
//   strategy_filter / strategy_smoother_fixedpoint
//                                           estimators_and_losses.py:347-591
//   solver / solver_mle / solver_dynamic, error_residual_std, controllers,
//   RejectionLoop with checkpoints          as in iso_solver.cuh
// and the backward pass Smoother.finalize / MarkovSequence.evaluate_marginals
// (estimators_and_losses.py:156-178, 437-470).
//
// The per-instance state does not fit in registers for N = 8; the compiler
// places the rest in thread-local memory, which stays L1/L2 resident (a few
// KB per instance).  The fixed-point smoother's backward conditionals at the
// checkpoints go to the workspace (scratch) and are read back by the same
// thread for the backward pass.
#pragma once

#include "iso_solver.cuh"

namespace pdq {

struct DenseArgs {
  int64_t B;
  int32_t S, terminal_only, solver, control, clip_dt, correct, fixedpoint;
  int32_t state_error;  // 0: error_residual_std; 1: error_state_std (derivative 0)
  int32_t instances_per_block;  // launch shape (read by the launchers only)
  double safety, factor_min, factor_max, exp_i, exp_p;
  double atol, rtol, eps, damp;
  int64_t max_attempts;
  double q1[kMaxN][kMaxN];
  const double* save_at;
  const double* params;
  const double* y0;
  const double* dt0;
  double* u_mean;
  double* u_chol;
  double* output_scale;
  double* t_out;
  int32_t* num_steps;
  int32_t* num_attempts;
  int32_t* status;
  // optional outputs (nullptr: not written)
  double* cond_A;
  double* cond_noise_mean;
  double* cond_noise_chol;
  double* cond_to_latent;
  double* cond_to_observed;
  double* filter_mean;
  double* filter_chol;
  // scratch: (B, S - 1) conditionals in T precision (fixed-point smoother)
  void* workspace;
};

template <typename T, int N>
struct DNormal {
  T m[N];
  T L[N][N];
};

template <typename T, int N>
struct DCond {
  T A[N][N];
  T xi[N];
  T X[N][N];  // lower Cholesky factor of the noise
  T tl[N];
  T to[N];
};

template <typename T, int N>
PDQ_D void cond_identity(DCond<T, N>& c) {
#pragma unroll
  for (int i = 0; i < N; ++i) {
#pragma unroll
    for (int j = 0; j < N; ++j) {
      c.A[i][j] = (i == j) ? T(1) : T(0);
      c.X[i][j] = T(0);
    }
    c.xi[i] = T(0);
    c.tl[i] = T(1);
    c.to[i] = T(1);
  }
}

// cond.marginalise(rv) (ssm_impl_dense.py:24-33)
template <typename T, int N>
PDQ_D void cond_marginalise(const DCond<T, N>& c, const DNormal<T, N>& rv, DNormal<T, N>& out) {
  T M[2 * N][N];
#pragma unroll
  for (int r = 0; r < N; ++r)
#pragma unroll
    for (int col = 0; col < N; ++col) {
      T acc = T(0);
#pragma unroll
      for (int k = 0; k < N; ++k) acc += c.A[col][k] * c.tl[k] * rv.L[k][r];
      M[r][col] = acc;                 // (A (tl * L))^T
      M[N + r][col] = c.X[col][r];     // X^T
    }
  householder_r<T, 2 * N, N>(M);
#pragma unroll
  for (int i = 0; i < N; ++i) {
    T acc = T(0);
#pragma unroll
    for (int k = 0; k < N; ++k) acc += c.A[i][k] * c.tl[k] * rv.m[k];
    out.m[i] = c.to[i] * (acc + c.xi[i]);
#pragma unroll
    for (int j = 0; j < N; ++j) out.L[i][j] = (j <= i) ? dev_abs(c.to[i]) * M[j][i] : T(0);
  }
}

// outer.merge(inner) (ssm_impl_dense.py:35-49)
template <typename T, int N>
PDQ_D void cond_merge(const DCond<T, N>& o, const DCond<T, N>& in, DCond<T, N>& out) {
  T Tv[N];
#pragma unroll
  for (int i = 0; i < N; ++i) Tv[i] = o.tl[i] * in.to[i];
  T M[2 * N][N];
#pragma unroll
  for (int i = 0; i < N; ++i) {
#pragma unroll
    for (int j = 0; j < N; ++j) {
      T g = T(0), r1 = T(0);
#pragma unroll
      for (int k = 0; k < N; ++k) {
        g += o.A[i][k] * Tv[k] * in.A[k][j];
        r1 += o.A[i][k] * dev_abs(Tv[k]) * in.X[k][j];
      }
      out.A[i][j] = g;
      M[j][i] = r1;              // R1 = (o.A (|T| in.X))^T
      M[N + j][i] = o.X[i][j];   // R2 = o.X^T
    }
    T x = o.xi[i];
#pragma unroll
    for (int k = 0; k < N; ++k) x += o.A[i][k] * Tv[k] * in.xi[k];
    out.xi[i] = x;
  }
  householder_r<T, 2 * N, N>(M);
#pragma unroll
  for (int i = 0; i < N; ++i) {
#pragma unroll
    for (int j = 0; j < N; ++j) out.X[i][j] = (j <= i) ? M[j][i] : T(0);
    out.tl[i] = in.tl[i];
    out.to[i] = o.to[i];
  }
}

// Preconditioner of the dense prior: p repeated d times (ssm_impl_dense.py:355-357).
template <typename T, int NU, int D>
PDQ_D void dense_precon(T h, T (&p)[(NU + 1) * D], T (&pinv)[(NU + 1) * D]) {
  T pc[NU + 1], pic[NU + 1];
  precon<T, NU>(h, pc, pic);
#pragma unroll
  for (int i = 0; i <= NU; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      p[i * D + j] = pc[i];
      pinv[i * D + j] = pic[i];
    }
}

// transition(h, s).revert(rv) (ssm_impl_dense.py:51-77 with :347-363):
// the predicted marginal and the backward conditional.
template <typename T, int NU, int D>
PDQ_D void prior_revert(const double (&q1)[kMaxN][kMaxN], const DNormal<T, (NU + 1) * D>& rv, T h, T scale,
                        DNormal<T, (NU + 1) * D>& marg, DCond<T, (NU + 1) * D>& cond) {
  constexpr int N = (NU + 1) * D;
  T p[N], pinv[N];
  dense_precon<T, NU, D>(h, p, pinv);
  const T sq = scale * dev_sqrt(dev_abs(h));
  // M = [[R_YX, 0], [R_X_F, R_X]], R_YX = (sq Q)^T, R_X_F = (A chol)^T, R_X = chol^T
  T M[2 * N][2 * N];
  T cl[N][N];
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int j = 0; j < N; ++j) cl[i][j] = dev_abs(pinv[i]) * rv.L[i][j];
#pragma unroll
  for (int r = 0; r < N; ++r)
#pragma unroll
    for (int c = 0; c < N; ++c) {
      // Q = kron(Q1, I_d): Q[c][r] = Q1[c/D][r/D] if c%D == r%D
      const T qcr = (c % D == r % D) ? T(q1[c / D][r / D]) : T(0);
      M[r][c] = sq * qcr;
      M[r][N + c] = T(0);
      // (A cl)[c][r] with A = kron(A1, I)
      T acc = T(0);
#pragma unroll
      for (int k = 0; k < N; ++k)
        if (k % D == c % D) acc += T(iwp_a<NU>(c / D, k / D)) * cl[k][r];
      M[N + r][c] = acc;
      M[N + r][N + c] = cl[c][r];
    }
  householder_r<T, 2 * N, 2 * N>(M);
  // G = solve_triu(R_Y, R12)^T: G^T = R_Y^{-1} R12, back substitution per column
  T Gt[N][N];
#pragma unroll
  for (int col = 0; col < N; ++col) {
#pragma unroll
    for (int i = N - 1; i >= 0; --i) {
      T acc = M[i][N + col];
#pragma unroll
      for (int k = i + 1; k < N; ++k) acc -= M[i][k] * Gt[k][col];
      Gt[i][col] = dev_div(acc, M[i][i]);
    }
  }
  T mean_l[N], mobs[N];
#pragma unroll
  for (int i = 0; i < N; ++i) mean_l[i] = pinv[i] * rv.m[i];
#pragma unroll
  for (int i = 0; i < N; ++i) {
    T acc = T(0);
#pragma unroll
    for (int k = 0; k < N; ++k)
      if (k % D == i % D) acc += T(iwp_a<NU>(i / D, k / D)) * mean_l[k];
    mobs[i] = acc;
  }
#pragma unroll
  for (int i = 0; i < N; ++i) {
    T acc = mean_l[i];
#pragma unroll
    for (int k = 0; k < N; ++k) acc -= Gt[k][i] * mobs[k];
    cond.xi[i] = acc;  // corrected mean
#pragma unroll
    for (int j = 0; j < N; ++j) {
      cond.A[i][j] = Gt[j][i];
      cond.X[i][j] = (j <= i) ? M[N + j][N + i] : T(0);  // R_XY^T
    }
    cond.tl[i] = dev_rcp(p[i]);
    cond.to[i] = dev_rcp(pinv[i]);
    marg.m[i] = p[i] * mobs[i];
#pragma unroll
    for (int j = 0; j < N; ++j) marg.L[i][j] = (j <= i) ? dev_abs(p[i]) * M[j][i] : T(0);
  }
}

// transition(h, s).marginalise(rv) for the filter (ssm_impl_dense.py:24-33, 347-363)
template <typename T, int NU, int D>
PDQ_D void prior_marginalise(const double (&q1)[kMaxN][kMaxN], const DNormal<T, (NU + 1) * D>& rv, T h, T scale,
                             DNormal<T, (NU + 1) * D>& out) {
  constexpr int N = (NU + 1) * D;
  T p[N], pinv[N];
  dense_precon<T, NU, D>(h, p, pinv);
  const T sq = scale * dev_sqrt(dev_abs(h));
  T M[2 * N][N];
#pragma unroll
  for (int r = 0; r < N; ++r)
#pragma unroll
    for (int c = 0; c < N; ++c) {
      T acc = T(0);
#pragma unroll
      for (int k = 0; k < N; ++k)
        if (k % D == c % D) acc += T(iwp_a<NU>(c / D, k / D)) * pinv[k] * rv.L[k][r];
      M[r][c] = acc;
      M[N + r][c] = (c % D == r % D) ? sq * T(q1[c / D][r / D]) : T(0);
    }
  householder_r<T, 2 * N, N>(M);
#pragma unroll
  for (int i = 0; i < N; ++i) {
    T acc = T(0);
#pragma unroll
    for (int k = 0; k < N; ++k)
      if (k % D == i % D) acc += T(iwp_a<NU>(i / D, k / D)) * pinv[k] * rv.m[k];
    out.m[i] = p[i] * acc;
#pragma unroll
    for (int j = 0; j < N; ++j) out.L[i][j] = (j <= i) ? dev_abs(p[i]) * M[j][i] : T(0);
  }
}

template <typename T, int N, int D>
struct DLin {
  T J[D][N];  // linear operator (d x N)
  T b[D];     // noise mean; noise chol = damp I_d
};

template <typename T, int NU, class F, bool TS1>
PDQ_D void dense_linearize(const T (&m)[(NU + 1) * F::D], const T* pt, DLin<T, (NU + 1) * F::D, F::D>& fx) {
  constexpr int D = F::D, N = (NU + 1) * D;
  T f[D];
  if constexpr (TS1) {
    // r(x) = x[u'] - f(x[u]); J = [-Jf, I, 0, ...]; b = r(xi) - J xi at xi = m
    T Jf[D][D];
    eval_with_jacobian<F>(&m[0], pt, f, Jf);
#pragma unroll
    for (int a = 0; a < D; ++a) {
#pragma unroll
      for (int k = 0; k < N; ++k) fx.J[a][k] = T(0);
#pragma unroll
      for (int k = 0; k < D; ++k) fx.J[a][k] = -Jf[a][k];
      fx.J[a][D + a] = T(1);
      T jx = T(0);
#pragma unroll
      for (int k = 0; k < D; ++k) jx += Jf[a][k] * m[k];
      fx.b[a] = -f[a] + jx;
    }
  } else {
    F::eval(&m[0], pt, f);
#pragma unroll
    for (int a = 0; a < D; ++a) {
#pragma unroll
      for (int k = 0; k < N; ++k) fx.J[a][k] = (k == D + a) ? T(1) : T(0);
      fx.b[a] = -f[a];
    }
  }
}

template <typename T, int N>
PDQ_D void store_cond(T* base, const DCond<T, N>& c) {
  int o = 0;
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int j = 0; j < N; ++j) base[o++] = c.A[i][j];
#pragma unroll
  for (int i = 0; i < N; ++i) base[o++] = c.xi[i];
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int j = 0; j <= i; ++j) base[o++] = c.X[i][j];
#pragma unroll
  for (int i = 0; i < N; ++i) base[o++] = c.tl[i];
#pragma unroll
  for (int i = 0; i < N; ++i) base[o++] = c.to[i];
}

template <typename T, int N>
PDQ_D void load_cond(const T* base, DCond<T, N>& c) {
  int o = 0;
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int j = 0; j < N; ++j) c.A[i][j] = base[o++];
#pragma unroll
  for (int i = 0; i < N; ++i) c.xi[i] = base[o++];
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int j = 0; j < N; ++j) c.X[i][j] = (j <= i) ? base[o++] : T(0);
#pragma unroll
  for (int i = 0; i < N; ++i) c.tl[i] = base[o++];
#pragma unroll
  for (int i = 0; i < N; ++i) c.to[i] = base[o++];
}

template <int N>
PDQ_HD constexpr int cond_floats() {
  return N * N + N + N * (N + 1) / 2 + 2 * N;
}

template <typename T, int N>
PDQ_D void write_normal(double* mean, double* chol, const DNormal<T, N>& x) {
  for (int i = 0; i < N; ++i) mean[i] = double(x.m[i]);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) chol[i * N + j] = double(x.L[i][j]);
}

template <typename T, int NU, class F, bool TS1, bool FP>
__global__ void __launch_bounds__(32) dense_adaptive_kernel(DenseArgs a) {
  constexpr int D = F::D, P = F::P, n = NU + 1, N = n * D;
  const int64_t b = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (b >= a.B) return;
  const int S = a.S;
  const int S_out = a.terminal_only ? 1 : S;
  const double* save_at = a.save_at + b * S;
  T* ws = FP ? reinterpret_cast<T*>(a.workspace) + b * int64_t(S - 1) * cond_floats<N>() : nullptr;

  double pd[P];
  T pt[P];
#pragma unroll
  for (int k = 0; k < P; ++k) {
    pd[k] = a.params[b * P + k];
    pt[k] = T(pd[k]);
  }
  double y0[D];
#pragma unroll
  for (int j = 0; j < D; ++j) y0[j] = a.y0[b * D + j];
  double tc[n][D];
  taylor_init<F, NU>(y0, pd, tc);

  DNormal<T, N> x;  // step_from marginal
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) x.m[i * D + j] = T(tc[i][j]);
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int j = 0; j < N; ++j) x.L[i][j] = T(0);
  DCond<T, N> bw;  // step_from backward conditional (fixed-point smoother)
  if constexpr (FP) cond_identity(bw);
  DNormal<T, N> xi_ = x;  // interp_from
  DCond<T, N> bwi;
  if constexpr (FP) cond_identity(bwi);

  double t = save_at[0], ti = t, dt = a.dt0[b], pi_prev = 1.0, mle_sumsq = 0.0;
  int num_data = 0, num_steps = 0, attempts = 0, status = PDQ_INSTANCE_OK;
  T sigma_sf = T(1);
  const T damp = T(a.damp);

  if (!a.terminal_only) {
    write_normal(a.u_mean + (b * S_out) * N, a.u_chol + (b * S_out) * N * N, x);
    a.output_scale[b * S_out] = 1.0;
    a.t_out[b * S_out] = t;
    a.num_steps[b * S_out] = 0;
  }
  if (a.filter_mean) write_normal(a.filter_mean + (b * S) * N, a.filter_chol + (b * S) * N * N, x);

  // One attempt per iteration (the retry loop flattened into the checkpoint
  // loop): a rejected lane retries in the next iteration without holding the
  // other instances of its warp; per instance the sequence of attempts and
  // checkpoint branches is unchanged (solvers_via_adaptive_steps.py:196-375).
  int s = 1;
  double t_next = save_at[1];
  while (s < S) {
    if (t + a.eps < t_next) {
      bool accepted = false;
      {
        const double dt_use = a.clip_dt ? fmin(dt, t_next - t) : dt;
        if (!(fabs(dt_use) > 1e-14 * fmax(1.0, fabs(t)))) {
          status = PDQ_INSTANCE_DT_UNDERFLOW;
          break;
        }
        if (attempts >= a.max_attempts) {
          status = PDQ_INSTANCE_MAX_STEPS;
          break;
        }
        ++attempts;
        const T h = T(dt_use);
        T p[N], pinv[N];
        dense_precon<T, NU, D>(h, p, pinv);
        // u = transition(h, 1).apply_flat(mean): mean mp, chol |p| sqrt|h| Q
        T mp[N];
#pragma unroll
        for (int i = 0; i < N; ++i) {
          T acc = T(0);
#pragma unroll
          for (int k = 0; k < N; ++k)
            if (k % D == i % D) acc += T(iwp_a<NU>(i / D, k / D)) * pinv[k] * x.m[k];
          mp[i] = p[i] * acc;
        }
        DLin<T, N, D> fx;
        dense_linearize<T, NU, F, TS1>(mp, pt, fx);
        // observed = fx.marginalise(u): mean r = J mp + b, chol from qr of [(J Lu)^T; damp I]
        T r[D];
#pragma unroll
        for (int aa = 0; aa < D; ++aa) {
          T acc = fx.b[aa];
#pragma unroll
          for (int k = 0; k < N; ++k) acc += fx.J[aa][k] * mp[k];
          r[aa] = acc;
        }
        T Mo[N + D][D];
        const T sqh = dev_sqrt(dev_abs(h));
#pragma unroll
        for (int rr = 0; rr < N; ++rr)
#pragma unroll
          for (int aa = 0; aa < D; ++aa) {
            // (J Lu)[aa][rr], Lu = |p| sqrt|h| Q
            T acc = T(0);
#pragma unroll
            for (int k = 0; k < N; ++k)
              if (k % D == rr % D && rr / D <= k / D) acc += fx.J[aa][k] * dev_abs(p[k]) * sqh * T(a.q1[k / D][rr / D]);
            Mo[rr][aa] = acc;
          }
#pragma unroll
        for (int i = 0; i < D; ++i)
#pragma unroll
          for (int j = 0; j < D; ++j) Mo[N + i][j] = (i == j) ? damp : T(0);
        householder_r<T, N + D, D>(Mo);
        // observed chol Lo = R^T (lower); sigma = ||Lo^{-1} r|| / sqrt(d)
        T w[D];
#pragma unroll
        for (int i = 0; i < D; ++i) {
          T acc = r[i];
#pragma unroll
          for (int k = 0; k < i; ++k) acc -= Mo[k][i] * w[k];
          w[i] = dev_div(acc, Mo[i][i]);
        }
        T ww = T(0);
#pragma unroll
        for (int i = 0; i < D; ++i) ww += w[i] * w[i];
        const T sigma_loc = dev_sqrt(ww * T(1.0 / D));

        const T s_pred = (a.solver == PDQ_SOLVER_DYNAMIC) ? sigma_loc : T(1);
        DNormal<T, N> pred;
        DCond<T, N> cnew, merged;
        if constexpr (FP) {
          prior_revert<T, NU, D>(a.q1, x, h, s_pred, pred, cnew);
          cond_merge<T, N>(bw, cnew, merged);
        } else {
          prior_marginalise<T, NU, D>(a.q1, x, h, s_pred, pred);
        }
        // update: fx.revert(pred): M2 = [[damp I, 0], [(J Lp)^T, Lp^T]]
        T M2[D + N][D + N];
#pragma unroll
        for (int i = 0; i < D; ++i)
#pragma unroll
          for (int j = 0; j < D + N; ++j) M2[i][j] = (i == j) ? damp : T(0);
#pragma unroll
        for (int rr = 0; rr < N; ++rr) {
#pragma unroll
          for (int aa = 0; aa < D; ++aa) {
            T acc = T(0);
#pragma unroll
            for (int k = 0; k < N; ++k) acc += fx.J[aa][k] * pred.L[k][rr];
            M2[D + rr][aa] = acc;
          }
#pragma unroll
          for (int c = 0; c < N; ++c) M2[D + rr][D + c] = pred.L[c][rr];
        }
        householder_r<T, D + N, D + N>(M2);
        // G = solve_triu(R_Y, R12)^T (N x d); residual of the predicted mean
        T Gt[D][N];
#pragma unroll
        for (int col = 0; col < N; ++col)
#pragma unroll
          for (int i = D - 1; i >= 0; --i) {
            T acc = M2[i][D + col];
#pragma unroll
            for (int k = i + 1; k < D; ++k) acc -= M2[i][k] * Gt[k][col];
            Gt[i][col] = dev_div(acc, M2[i][i]);
          }
        T ro[D];
#pragma unroll
        for (int aa = 0; aa < D; ++aa) {
          T acc = fx.b[aa];
#pragma unroll
          for (int k = 0; k < N; ++k) acc += fx.J[aa][k] * pred.m[k];
          ro[aa] = acc;
        }
        DNormal<T, N> xnew;
#pragma unroll
        for (int i = 0; i < N; ++i) {
          T acc = pred.m[i];
#pragma unroll
          for (int aa = 0; aa < D; ++aa) acc -= Gt[aa][i] * ro[aa];
          xnew.m[i] = acc;
#pragma unroll
          for (int j = 0; j < N; ++j) xnew.L[i][j] = (j <= i) ? M2[D + j][D + i] : T(0);
        }
        // error_residual_std: std of the rescaled observed = sigma * row norms of Lo, times dt;
        // error_state_std (solvers.py:999-1098): sigma * the posterior std of coefficient 0 of the
        // unit-scale extrapolation conditioned on the linearisation, times dt^0 / 0!
        T std_state[D];
        if (a.state_error) {
          T M3[D + N][D + N];
#pragma unroll
          for (int i = 0; i < D; ++i)
#pragma unroll
            for (int j = 0; j < D + N; ++j) M3[i][j] = (i == j) ? damp : T(0);
#pragma unroll
          for (int rr = 0; rr < N; ++rr) {
#pragma unroll
            for (int aa = 0; aa < D; ++aa) {  // (J Lu)^T
              T acc = T(0);
#pragma unroll
              for (int k = 0; k < N; ++k)
                if (k % D == rr % D && rr / D <= k / D) acc += fx.J[aa][k] * dev_abs(p[k]) * sqh * T(a.q1[k / D][rr / D]);
              M3[D + rr][aa] = acc;
            }
#pragma unroll
            for (int c = 0; c < N; ++c)
              M3[D + rr][D + c] = (c % D == rr % D && rr / D <= c / D)
                                      ? dev_abs(p[c]) * sqh * T(a.q1[c / D][rr / D]) : T(0);  // Lu^T
          }
          householder_r<T, D + N, D + N>(M3);
#pragma unroll
          for (int j = 0; j < D; ++j) {
            T rn = T(0);
#pragma unroll
            for (int k = 0; k <= j; ++k) rn += M3[D + k][D + j] * M3[D + k][D + j];
            std_state[j] = dev_sqrt(rn);
          }
        }
        double sumsq = 0.0;
#pragma unroll
        for (int j = 0; j < D; ++j) {
          T rn = T(0);
#pragma unroll
          for (int k = 0; k <= j; ++k) rn += Mo[k][j] * Mo[k][j];
          const T err_abs = a.state_error ? dev_abs(sigma_loc) * std_state[j] : dev_abs(sigma_loc) * dev_sqrt(rn) * h;
          const T ref = fmax(dev_abs(x.m[j]), dev_abs(xnew.m[j]));
          const T ratio = dev_div(err_abs, T(a.atol) + T(a.rtol) * ref);
          sumsq += double(ratio) * double(ratio);
        }
        const double norm2 = sumsq * (1.0 / D);
        if (!(norm2 == norm2) || isinf(norm2)) {
          status = PDQ_INSTANCE_NONFINITE;
          break;
        }
        const T ep = dev_fpow(T(norm2), T(-0.5 / n));
        double factor;
        if (a.control == PDQ_CONTROL_INTEGRAL) {
          factor = a.safety * double(ep);
        } else {
          factor = a.safety * double(dev_fpow(ep, T(a.exp_i))) * double(dev_fpow(dev_div(ep, T(pi_prev)), T(a.exp_p)));
          if (norm2 <= 1.0) pi_prev = double(ep);
        }
        factor = fmax(a.factor_min, fmin(factor, a.factor_max));
        dt = factor * dt_use;
        accepted = norm2 <= 1.0;
        if (accepted) {
          ti = t;
          xi_ = x;
          if constexpr (FP) bwi = bw;
          t = t + dt_use;
          ++num_steps;
          x = xnew;
          if constexpr (FP) bw = merged;
          if (a.solver == PDQ_SOLVER_MLE) {
            // new term: ||R_Y^{-T}... observed residual whitened by R_Y (d x d)
            T wv[D];
#pragma unroll
            for (int i = 0; i < D; ++i) {
              T acc = ro[i];
#pragma unroll
              for (int k = 0; k < i; ++k) acc -= M2[k][i] * wv[k];
              wv[i] = dev_div(acc, M2[i][i]);
            }
            T q = T(0);
#pragma unroll
            for (int i = 0; i < D; ++i) q += wv[i] * wv[i];
            mle_sumsq += double(q) * (1.0 / D);
            ++num_data;
          }
          sigma_sf = (a.solver == PDQ_SOLVER_DYNAMIC) ? sigma_loc : T(1);
        }
      }
      if (!accepted) continue;  // retry in the next iteration
    }
    const bool record = (!a.terminal_only) || (s == S - 1);
    const int s_out = a.terminal_only ? 0 : s;
    const int64_t rec = b * S_out + s_out;
    if (t + a.eps < t_next) {
      // interp_skip
    } else if (t > t_next + a.eps) {
      // interp_beyond_t1 (solvers.py:205-269)
      const T h0 = T(t_next - ti), h1 = T(t - t_next);
      DNormal<T, N> ext_t;
      if constexpr (FP) {
        // estimators_and_losses.py:549-591
        DCond<T, N> c0, m0, c1, idc, m1;
        DNormal<T, N> ext_t1;
        prior_revert<T, NU, D>(a.q1, xi_, h0, sigma_sf, ext_t, c0);
        cond_merge<T, N>(bwi, c0, m0);  // extrapolated_t.conditional
        prior_revert<T, NU, D>(a.q1, ext_t, h1, sigma_sf, ext_t1, c1);
        cond_identity(idc);
        cond_merge<T, N>(idc, c1, m1);  // extrapolated_t1.conditional
        store_cond(ws + int64_t(s - 1) * cond_floats<N>(), m0);
        bw = m1;          // step_from keeps its marginal, new conditional
        xi_ = ext_t;      // interp_from = previous_new
        cond_identity(bwi);
      } else {
        prior_marginalise<T, NU, D>(a.q1, xi_, h0, sigma_sf, ext_t);
        xi_ = ext_t;
      }
      ti = t_next;
      if (record) {
        write_normal(a.u_mean + rec * N, a.u_chol + rec * N * N, ext_t);
        a.output_scale[rec] = double(sigma_sf);
        a.t_out[rec] = t_next;
        a.num_steps[rec] = num_steps;
      }
      if (a.filter_mean) write_normal(a.filter_mean + (b * S + s) * N, a.filter_chol + (b * S + s) * N * N, ext_t);
    } else {
      // interp_at_t1 (solvers.py:271-315)
      if constexpr (FP) {
        store_cond(ws + int64_t(s - 1) * cond_floats<N>(), bw);
        cond_identity(bw);
        cond_identity(bwi);
      }
      xi_ = x;
      ti = t;
      if (record) {
        write_normal(a.u_mean + rec * N, a.u_chol + rec * N * N, x);
        a.output_scale[rec] = double(sigma_sf);
        a.t_out[rec] = t;
        a.num_steps[rec] = num_steps;
      }
      if (a.filter_mean) write_normal(a.filter_mean + (b * S + s) * N, a.filter_chol + (b * S + s) * N * N, x);
    }
    if (!(t + a.eps < t_next)) {  // checkpoint s done
      ++s;
      if (s < S) t_next = save_at[s];
    }
  }

  // ---- finalize (solvers.py:439-480, 601-633, 735-767) ----
  double scale = 1.0;
  if (status == PDQ_INSTANCE_OK && a.solver == PDQ_SOLVER_MLE) {
    scale = num_data > 0 ? sqrt(mle_sumsq / num_data) : 0.0;
    if (a.correct) scale /= sqrt(double(a.num_steps[b * S_out + (S_out - 1)]));
  }
  if (status == PDQ_INSTANCE_OK && FP) {
    // Smoother.finalize: rv_at_t1 = posterior1.conditional.marginalise(marginal),
    // then the reverse scan of marginalise over the checkpoint conditionals
    DNormal<T, N> rv;
    cond_marginalise<T, N>(bw, x, rv);
    const T sc = T(scale);
    for (int s = S - 1; s >= 1; --s) {
      // marginal at checkpoint s
      if (!a.terminal_only || s == S - 1) {
        const int64_t rec = b * S_out + (a.terminal_only ? 0 : s);
        write_normal(a.u_mean + rec * N, a.u_chol + rec * N * N, rv);
      }
      if (a.terminal_only) break;
      DCond<T, N> c;
      load_cond(ws + int64_t(s - 1) * cond_floats<N>(), c);
      if (a.cond_A) {
        const int64_t cr = b * (S - 1) + (s - 1);
        for (int i = 0; i < N; ++i) {
          for (int j = 0; j < N; ++j) {
            a.cond_A[cr * N * N + i * N + j] = double(c.A[i][j]);
            a.cond_noise_chol[cr * N * N + i * N + j] = double(c.X[i][j]) * scale;
          }
          a.cond_noise_mean[cr * N + i] = double(c.xi[i]);
          a.cond_to_latent[cr * N + i] = double(c.tl[i]);
          a.cond_to_observed[cr * N + i] = double(c.to[i]);
        }
      }
      DNormal<T, N> prev;
      cond_marginalise<T, N>(c, rv, prev);
      rv = prev;
      if (s == 1) {
        const int64_t rec = b * S_out;
        write_normal(a.u_mean + rec * N, a.u_chol + rec * N * N, rv);
      }
      (void)sc;
    }
  }
  if (status == PDQ_INSTANCE_OK) {
    if (a.solver == PDQ_SOLVER_MLE) {
      for (int s = 0; s < S_out; ++s) {
        const int64_t rec = b * S_out + s;
        for (int k = 0; k < N * N; ++k) a.u_chol[rec * N * N + k] *= scale;
        a.output_scale[rec] = scale;
      }
      if (a.filter_chol)
        for (int k = 0; k < S * N * N; ++k) a.filter_chol[b * S * N * N + k] *= scale;
    }
  } else {
    const double nan = __longlong_as_double(0x7ff8000000000000ULL);
    for (int s = 0; s < S_out; ++s) {
      const int64_t rec = b * S_out + s;
      for (int k = 0; k < N; ++k) a.u_mean[rec * N + k] = nan;
      for (int k = 0; k < N * N; ++k) a.u_chol[rec * N * N + k] = nan;
      a.output_scale[rec] = nan;
      a.t_out[rec] = nan;
      a.num_steps[rec] = num_steps;
    }
  }
  a.num_attempts[b] = attempts;
  a.status[b] = status;
}

}  // namespace pdq
