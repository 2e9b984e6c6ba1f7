// Isotropic TS0 adaptive solver: one thread per IVP instance.
//
// Follows, per attempt, the reference's isotropic path:
//   IsotropicWienerIntegrated.transition   (_probdiffeq/ssm_impl_isotropic.py:367-378)
//   IsotropicLatentCond.marginalise        (ssm_impl_isotropic.py:81-89)
//   IsotropicOdeTs0.linearize              (ssm_impl_isotropic.py:304-317)
//   IsotropicLatentCond.revert             (ssm_impl_isotropic.py:107-133)
//   revert_conditional / sum_of_sqrtm      (util/cholesky_util.py:27-95)
//   solver / solver_mle / solver_dynamic   (_probdiffeq/solvers.py:395-437, 549-599, 702-733)
//   error_residual_std                     (solvers.py:925-996)
//   control_integral / PI                  (_ivpsolve/controllers.py:24-84)
//   RejectionLoop + save_at checkpoints    (_ivpsolve/solvers_via_adaptive_steps.py:46-375)
// with the filter strategy (_probdiffeq/estimators_and_losses.py:347-421).
//
// Layout: the whole per-instance state (mean (n, d), lower Cholesky (n, n),
// time, step, controller and calibration accumulators) lives in registers for
// the entire solve; global memory is touched only to read the instance's
// inputs once and to write one record per checkpoint.
//
// Precision: T (float or double) for the bulk arithmetic and the step-size
// controller; the time, the MLE sum of squares and the error-norm sum are
// Wide<T> (double, or a float pair with a 48-bit significand for float).
#pragma once

#include "pdq_device.cuh"

namespace pdq {

constexpr int kMaxN = 8;

struct IsoArgs {
  int64_t B;
  int32_t S, terminal_only, solver, control, clip_dt, correct;
  int32_t ts1;  // 0: TS0 (H = e_1); 1: TS1 with the Jacobian trace along d (H = [-tr J_f / d, 1, 0, ...])
  int32_t state_error;  // 0: error_residual_std; 1: error_state_std (derivative 0)
  int32_t instances_per_block;  // launch shape (read by the launchers only)
  int32_t tangents;  // 1: d u_mean / d (params, y0) by forward mode (P + d threads per instance)
  double safety, factor_min, factor_max, exp_i, exp_p;
  double atol, rtol, eps, damp;
  int64_t max_attempts;
  double q1[kMaxN][kMaxN];  // lower square root of flip(Hilbert) (utilities.py:57-71)
  // float copies of the constants, so the float32 kernels read them without
  // conversions on the FP64 pipe
  float q1f[kMaxN][kMaxN];
  float safety_f, factor_min_f, factor_max_f, exp_i_f, exp_p_f;
  float atol_f, rtol_f, eps_f, damp_f;
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
  void* workspace;  // fixed-point smoother: (B, S - 1) backward conditionals in T
  // optional fixed-point outputs (nullptr: not written): the posterior's
  // backward conditionals between consecutive checkpoints and the filtering
  // marginals at the checkpoints
  double* cond_A;            // (B, S - 1, n, n)
  double* cond_noise_mean;   // (B, S - 1, n, d)
  double* cond_noise_chol;   // (B, S - 1, n, n), calibrated
  double* cond_to_latent;    // (B, S - 1, n)
  double* cond_to_observed;  // (B, S - 1, n)
  double* filter_mean;       // (B, S, n, d)
  double* filter_chol;
  // forward-mode sensitivities of the mean records (optional): d u_mean / d params
  // (B, S_out, n, d, P) and d u_mean / d y0 (B, S_out, n, d, d)
  double* tan_params;
  double* tan_y0;       // (B, S, n, n), calibrated
  // record of the accepted steps for the terminal-value adjoint (REC only;
  // layout in tv_adjoint.cuh): step sizes, and the state before every
  // rec_ckpt-th accepted step, for at most rec_capacity accepted steps
  void* record;
  int32_t rec_capacity, rec_ckpt;
};

// A constant in the kernel's precision: the float copy for float, else the double.
template <typename T>
PDQ_D T cst(double d, float f) {
  if constexpr (sizeof(T) == sizeof(float)) {
    return f;
  } else {
    return d;
  }
}

// Preconditioner p_i = h^(NU-i)/(NU-i)!, p_inv_i = 1/p_i (utilities.py:74-84).
template <typename T, int NU>
PDQ_D void precon(T h, T (&p)[NU + 1], T (&pinv)[NU + 1]) {
  const T hinv = fast_rcp(h);
  p[NU] = T(1);
  pinv[NU] = T(1);
#pragma unroll
  for (int i = NU - 1; i >= 0; --i) {
    p[i] = p[i + 1] * h * T(1.0 / (NU - i));
    pinv[i] = pinv[i + 1] * hinv * T(NU - i);
  }
}

// Observed std of the linearised TS0 residual at unit output scale,
//   l = sqrt(p_OUT^2 |h| ||Q1[OUT]||^2 + damp^2),
// formed as |p_OUT| sqrt|h| ||Q1[OUT]|| without squaring p_OUT: the square
// leaves the float32 range for steps below ~1e-5 (nu = 4), while l itself
// stays representable down to the step-underflow bound.
template <typename T>
PDQ_D T observed_std(T p_out, T h, T q1_out_norm, T damp) {
  const T a = dev_abs(p_out) * fast_sqrt(dev_abs(h)) * q1_out_norm;
  return damp == T(0) ? a : fast_sqrt(a * a + damp * damp);
}

// The same for the TS1 operator H = h0 e_0 + e_1 (observed coefficient 1):
// H L_unit = sqrt|h| (h0 |p_0| Q1[0] + |p_1| Q1[1]), and with p_0 = p_1 h / nu
// its norm is |p_1| sqrt|h| ||(h0 (h / nu) q00 + q10, q11)||.
template <typename T, int NU>
PDQ_D T observed_std_ts1(T p1, T h, T h0, T q00, T q10, T q11, T damp) {
  const T c0 = h0 * (dev_abs(h) * T(1.0 / NU)) * q00 + q10;
  const T a = dev_abs(p1) * fast_sqrt(dev_abs(h)) * fast_sqrt(c0 * c0 + q11 * q11);
  return damp == T(0) ? a : fast_sqrt(a * a + damp * damp);
}

// IWP predict of the isotropic mean (marginalise, ssm_impl_isotropic.py:81-89):
//   mp = p * A (pinv * m)
template <typename T, int NU, int D>
PDQ_D void iso_predict_mean(const T (&m)[NU + 1][D], const T (&p)[NU + 1], const T (&pinv)[NU + 1],
                            T (&mp)[NU + 1][D]) {
  constexpr int n = NU + 1;
  T x[n][D];
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) x[i][j] = pinv[i] * m[i][j];
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      T acc = T(0);
#pragma unroll
      for (int k = i; k < n; ++k) acc += T(iwp_a<NU>(i, k)) * x[k][j];
      mp[i][j] = p[i] * acc;
    }
}

// The same predict in increment form, mp_i = m_i + incr_i with
//   incr_i = p_i sum_{k>i} A_ik pinv_k m_k
// (A_ii = 1, so p_i pinv_i m_i = m_i in exact arithmetic).  For the step
// sizes of an adaptive solve the increment is small against m_i, so formed
// in the bulk type and added to a wide m_i it leaves the sum accurate to the
// wide type; the product form rounds m_i itself at every step.
template <typename T, int NU, int D>
PDQ_D void iso_mean_increment(const T (&m)[NU + 1][D], const T (&p)[NU + 1], const T (&pinv)[NU + 1],
                              T (&incr)[NU + 1][D]) {
  constexpr int n = NU + 1;
  T x[n][D];
#pragma unroll
  for (int i = 1; i < n; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) x[i][j] = pinv[i] * m[i][j];
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      T acc = T(0);
#pragma unroll
      for (int k = i + 1; k < n; ++k) acc += T(iwp_a<NU>(i, k)) * x[k][j];
      incr[i][j] = mul_nc(p[i], acc);  // rounded here, whatever consumes it
    }
}

// The isotropic mean is carried with its solution and first-derivative rows
// wide: the bulk-type rows m (all n) and, for float, the low parts lo of rows
// 0 and 1 (a float pair per entry).  The TS0 residual u' - f(u) reads exactly
// these two rows, so they carry the accuracy the error estimate needs; for
// double the low parts stay zero and cost nothing.
template <typename T>
PDQ_D Wide<T> wide_pair(T hi, T lo) {
  if constexpr (sizeof(T) == sizeof(float)) {
    return FloatPair(hi, lo);
  } else {
    return hi;  // the low parts of double means are zero
  }
}

// out = m + d with the wide rows (0, 1) summed in the wide type, rows >= 2 in T
// (out may alias m).
template <typename T, int NU, int D>
PDQ_D void iso_mean_add(const T (&m)[NU + 1][D], const T (&lo)[2][D], const T (&d)[NU + 1][D],
                        T (&out)[NU + 1][D], T (&out_lo)[2][D]) {
  constexpr int n = NU + 1;
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      if constexpr (sizeof(T) == sizeof(float)) {
        const FloatPair s = FloatPair(m[i][j], lo[i][j]) + d[i][j];
        out[i][j] = s.hi;
        out_lo[i][j] = s.lo;
      } else {
        out[i][j] = m[i][j] + d[i][j];
        out_lo[i][j] = T(0);
      }
    }
#pragma unroll
  for (int i = 2; i < n; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) out[i][j] = m[i][j] + d[i][j];
}

// TS0 residual mobs_j = mp_1j - f_j(mp_0) of the extrapolated mean (mp, lo),
// with the field evaluated in the wide type at the wide solution row and the
// wide parameters, rounded once to T.
template <class F, typename T, int NU>
PDQ_D void iso_residual(const T (&mp)[NU + 1][F::D], const T (&lo)[2][F::D], const Wide<T> (&pw)[F::P],
                        T (&mobs)[F::D]) {
  constexpr int D = F::D;
  Wide<T> u[D], f[D];
#pragma unroll
  for (int j = 0; j < D; ++j) u[j] = wide_pair(mp[0][j], lo[0][j]);
  F::eval(u, pw, f);
#pragma unroll
  for (int j = 0; j < D; ++j) mobs[j] = T(wide_hi(wide_pair(mp[1][j], lo[1][j]) - f[j]));
}

// IWP predict of the isotropic Cholesky factor (marginalise, ssm_impl_isotropic.py:81-89):
//   Lp = |p| * qr_r([ (A (pinv * L))^T ; (s sqrt|h| Q1)^T ])^T
// The stacked matrix is 2n x n with an upper-triangular bottom block, so the
// Householder reflector of column c only touches rows c..n-1 of the top block
// and rows 0..c of the bottom block (n + 1 entries).
//
// Reflector of column c with alpha = X[c][c], nrm = ||column||:
//   beta = -sign(alpha) nrm,  v = [alpha - beta, rest],  H = I - g v v^T,
//   g = 2 / (v^T v) = 1 / (nrm (nrm + |alpha|)),
// applied unnormalised so the dot products with the other columns start
// before the square root is known; the dependency chain per column is one
// sum of squares, one square root and one reciprocal.  Sums of squares
// outside [1e-30, 1e36] (where g would leave the float range) take the
// LAPACK-style scaled path with a normalised reflector instead.
template <typename T, int NU, typename Q>
PDQ_D void iso_predict_chol(const Q (&q1)[kMaxN][kMaxN], const T (&L)[NU + 1][NU + 1], const T (&p)[NU + 1],
                            const T (&pinv)[NU + 1], T scale_q, T (&Lp)[NU + 1][NU + 1]) {
  constexpr int n = NU + 1;
  // top block X = (A pinv L)^T: X[r][c] = sum_k A[c][k] pinv[k] L[k][r]
  T X[n][n];
  T U[n][n];  // bottom block (s sqrt|h| Q1)^T, upper triangular
  T PL[n][n];
#pragma unroll
  for (int k = 0; k < n; ++k)
#pragma unroll
    for (int r = 0; r < n; ++r) PL[k][r] = pinv[k] * L[k][r];
#pragma unroll
  for (int c = 0; c < n; ++c)
#pragma unroll
    for (int r = 0; r < n; ++r) {
      T acc = T(0);
#pragma unroll
      for (int k = (c > r ? c : r); k < n; ++k) acc += T(iwp_a<NU>(c, k)) * PL[k][r];
      X[r][c] = acc;
      U[r][c] = (r <= c) ? scale_q * T(q1[c][r]) : T(0);
    }
  // structured Householder QR
#pragma unroll
  for (int c = 0; c < n; ++c) {
    // below-diagonal part of the column, two interleaved partial sums
    T e0 = T(0), e1 = T(0);
#pragma unroll
    for (int r = c + 1; r < n; ++r) {
      if ((r & 1) == 0) e0 += X[r][c] * X[r][c];
      else e1 += X[r][c] * X[r][c];
    }
#pragma unroll
    for (int i = 0; i <= c; ++i) {
      if ((i & 1) == 0) e0 += U[i][c] * U[i][c];
      else e1 += U[i][c] * U[i][c];
    }
    const T alpha = X[c][c];
    const T nrm2 = alpha * alpha + (e0 + e1);
    if (!norm2_out_of_range(nrm2)) {
      const T nrm = fast_sqrt(nrm2);
      const T s = dev_abs(alpha) + nrm;
      const T v0 = alpha >= T(0) ? s : -s;
      const T g = fast_rcp(nrm * s);
#pragma unroll
      for (int j = c + 1; j < n; ++j) {
        T d0 = T(0), d1 = T(0);
#pragma unroll
        for (int r = c + 1; r < n; ++r) {
          if ((r & 1) == 0) d0 += X[r][c] * X[r][j];
          else d1 += X[r][c] * X[r][j];
        }
#pragma unroll
        for (int i = 0; i <= c; ++i) {
          if ((i & 1) == 0) d0 += U[i][c] * U[i][j];
          else d1 += U[i][c] * U[i][j];
        }
        const T w = (v0 * X[c][j] + (d0 + d1)) * g;
        X[c][j] -= w * v0;
#pragma unroll
        for (int r = c + 1; r < n; ++r) X[r][j] -= w * X[r][c];
#pragma unroll
        for (int i = 0; i <= c; ++i) U[i][j] -= w * U[i][c];
      }
      X[c][c] = alpha >= T(0) ? -nrm : nrm;
    } else {
      // scaled norm and normalised reflector v = [1, rest / v0], tau = (beta - alpha) / beta
      T sc = dev_abs(alpha);
#pragma unroll
      for (int r = c + 1; r < n; ++r) sc = fmax(sc, dev_abs(X[r][c]));
#pragma unroll
      for (int i = 0; i <= c; ++i) sc = fmax(sc, dev_abs(U[i][c]));
      if (sc > T(0)) {
        const T inv = T(1) / sc;
        T acc = T(0);
#pragma unroll
        for (int r = c; r < n; ++r) acc += (X[r][c] * inv) * (X[r][c] * inv);
#pragma unroll
        for (int i = 0; i <= c; ++i) acc += (U[i][c] * inv) * (U[i][c] * inv);
        const T nrm = sc * dev_sqrt(acc);
        const T beta = alpha >= T(0) ? -nrm : nrm;
        const T v0 = alpha - beta;
        const T tau = (beta - alpha) / beta;
        const T vinv = T(1) / v0;
#pragma unroll
        for (int r = c + 1; r < n; ++r) X[r][c] *= vinv;
#pragma unroll
        for (int i = 0; i <= c; ++i) U[i][c] *= vinv;
#pragma unroll
        for (int j = c + 1; j < n; ++j) {
          T w = X[c][j];
#pragma unroll
          for (int r = c + 1; r < n; ++r) w += X[r][c] * X[r][j];
#pragma unroll
          for (int i = 0; i <= c; ++i) w += U[i][c] * U[i][j];
          w *= tau;
          X[c][j] -= w;
#pragma unroll
          for (int r = c + 1; r < n; ++r) X[r][j] -= w * X[r][c];
#pragma unroll
          for (int i = 0; i <= c; ++i) U[i][j] -= w * U[i][c];
        }
        X[c][c] = beta;
      }
    }
  }
  // Lp = |p| * R^T (lower triangular)
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < n; ++j) Lp[i][j] = (j <= i) ? dev_abs(p[i]) * X[j][i] : T(0);
}

// Branch-free twin of iso_predict_chol: the same unnormalised reflectors
// without the per-column range test, so the predict is straight-line code the
// compiler interleaves with the rest of the attempt.  Returns false when some
// column's sum of squares left [1e-30, 1e36]; the results are then unusable
// and the caller reruns the attempt with iso_predict_chol.
template <typename T, int NU, typename Q>
PDQ_D bool iso_predict_chol_fast(const Q (&q1)[kMaxN][kMaxN], const T (&L)[NU + 1][NU + 1], const T (&p)[NU + 1],
                                 const T (&pinv)[NU + 1], T scale_q, T (&Lp)[NU + 1][NU + 1]) {
  constexpr int n = NU + 1;
  T X[n][n];
  T U[n][n];
  T PL[n][n];
#pragma unroll
  for (int k = 0; k < n; ++k)
#pragma unroll
    for (int r = 0; r < n; ++r) PL[k][r] = pinv[k] * L[k][r];
#pragma unroll
  for (int c = 0; c < n; ++c)
#pragma unroll
    for (int r = 0; r < n; ++r) {
      T acc = T(0);
#pragma unroll
      for (int k = (c > r ? c : r); k < n; ++k) acc += T(iwp_a<NU>(c, k)) * PL[k][r];
      X[r][c] = acc;
      U[r][c] = (r <= c) ? scale_q * T(q1[c][r]) : T(0);
    }
  bool ok = true;
#pragma unroll
  for (int c = 0; c < n; ++c) {
    T e0 = T(0), e1 = T(0);
#pragma unroll
    for (int r = c + 1; r < n; ++r) {
      if ((r & 1) == 0) e0 += X[r][c] * X[r][c];
      else e1 += X[r][c] * X[r][c];
    }
#pragma unroll
    for (int i = 0; i <= c; ++i) {
      if ((i & 1) == 0) e0 += U[i][c] * U[i][c];
      else e1 += U[i][c] * U[i][c];
    }
    const T alpha = X[c][c];
    const T nrm2 = alpha * alpha + (e0 + e1);
    ok = ok && !norm2_out_of_range(nrm2);
    const T nrm = fast_sqrt(nrm2);
    const T s = dev_abs(alpha) + nrm;
    const T v0 = alpha >= T(0) ? s : -s;
    const T g = fast_rcp(nrm * s);
#pragma unroll
    for (int j = c + 1; j < n; ++j) {
      T d0 = T(0), d1 = T(0);
#pragma unroll
      for (int r = c + 1; r < n; ++r) {
        if ((r & 1) == 0) d0 += X[r][c] * X[r][j];
        else d1 += X[r][c] * X[r][j];
      }
#pragma unroll
      for (int i = 0; i <= c; ++i) {
        if ((i & 1) == 0) d0 += U[i][c] * U[i][j];
        else d1 += U[i][c] * U[i][j];
      }
      const T w = (v0 * X[c][j] + (d0 + d1)) * g;
      X[c][j] -= w * v0;
#pragma unroll
      for (int r = c + 1; r < n; ++r) X[r][j] -= w * X[r][c];
#pragma unroll
      for (int i = 0; i <= c; ++i) U[i][j] -= w * U[i][c];
    }
    X[c][c] = alpha >= T(0) ? -nrm : nrm;
  }
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < n; ++j) Lp[i][j] = (j <= i) ? dev_abs(p[i]) * X[j][i] : T(0);
  return ok;
}

// One unnormalised Householder reflector of a register matrix with a
// compile-time sparsity pattern: column COL, pivot row PIV, the column's
// other nonzero rows in the bit mask BELOW, applied to the columns in the
// bit mask COLS (rows outside PIV and BELOW are not touched).  Branch-free;
// clears ok when the column's sum of squares leaves [1e-30, 1e36].
template <typename T, int R, int C, int COL, int PIV, unsigned BELOW, unsigned COLS>
PDQ_D void hh_step(T (&Z)[R][C], bool& ok) {
  T e0 = T(0), e1 = T(0);
#pragma unroll
  for (int r = 0; r < R; ++r) {
    if ((BELOW >> r) & 1u) {
      if (r & 1) e1 += Z[r][COL] * Z[r][COL];
      else e0 += Z[r][COL] * Z[r][COL];
    }
  }
  const T alpha = Z[PIV][COL];
  const T nrm2 = alpha * alpha + (e0 + e1);
  ok = ok && !norm2_out_of_range(nrm2);
  const T nrm = fast_sqrt(nrm2);
  const T s = dev_abs(alpha) + nrm;
  const T v0 = alpha >= T(0) ? s : -s;
  const T g = fast_rcp(nrm * s);
#pragma unroll
  for (int j = 0; j < C; ++j) {
    if ((COLS >> j) & 1u) {
      T d0 = T(0), d1 = T(0);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        if ((BELOW >> r) & 1u) {
          if (r & 1) d1 += Z[r][COL] * Z[r][j];
          else d0 += Z[r][COL] * Z[r][j];
        }
      }
      const T w = (v0 * Z[PIV][j] + (d0 + d1)) * g;
      Z[PIV][j] -= w * v0;
#pragma unroll
      for (int r = 0; r < R; ++r)
        if ((BELOW >> r) & 1u) Z[r][j] -= w * Z[r][COL];
    }
  }
  Z[PIV][COL] = alpha >= T(0) ? -nrm : nrm;
}

// Reflectors of the columns c = 3..n of the joint predict-update matrix
// (below): pivot row c (X row c, or U row 0 for c = n), the nonzeros below
// it X rows c+1..n-1 and U rows 0..c-1, applied to columns c+1..n.
template <typename T, int n, int c>
PDQ_D void joint_tail(T (&Z)[2 * n][n + 1], bool& ok) {
  if constexpr (c <= n) {
    constexpr unsigned x_below = ((1u << n) - 1u) & ~((1u << (c + 1)) - 1u);
    constexpr unsigned u_rows = ((1u << c) - 1u) << n;
    constexpr unsigned below = (c < n) ? (x_below | u_rows) : (u_rows & ~(1u << n));
    constexpr unsigned cols = ((1u << (n + 1)) - 1u) & ~((1u << (c + 1)) - 1u);
    hh_step<T, 2 * n, n + 1, c, c, below, cols>(Z, ok);
    joint_tail<T, n, c + 1>(Z, ok);
  }
}

// IWP predict and TS0 update (H = e_1, damp = 0) in one orthogonal
// triangularisation -- the array form of the square-root Kalman filter.
// With the preconditioned stacked factor Z = [X; U] (2n x n, X = (A pinv L)^T,
// U = s sqrt|h| Q1^T upper triangular, as in iso_predict_chol), the
// reference's two QRs (marginalise, then revert_conditional on
// [(H Lp)^T, Lp^T] = Q^T [Z e_1, Z] diag(|p_1|, |p|)) equal one QR of [Z e_1, Z]:
//   R' = qr_r([Z e_1, Z]) = [[r_y, r12], [0, R22]],
//   R_Y = |p_1| r_y,  gain_j = r12_j |p_j| / R_Y,  Lnew = diag(|p|) R22^T.
// Column 0 and column 2 are the same vector, so after the first reflector
// column 2 is r_y e_0 (gain_1 = 1: the observed coefficient becomes f) and
// R22 has a zero in its second diagonal entry (the observed coefficient's
// posterior variance is zero); the other n reflectors are structured
// (U is triangular).  Row 0 of R' -- R_Y and the gain -- is final after
// the first reflector, so the error estimate overlaps the rest.  Clears ok
// when a sum of squares left the safe range (the caller then reruns the
// attempt with iso_predict_chol and ts0_update).
// The pieces of the joint predict-update, used in this order: the X rows of
// Z from L (independent of the noise scale) ...
template <typename T, int NU>
PDQ_D void joint_x(const T (&L)[NU + 1][NU + 1], const T (&pinv)[NU + 1], T (&Z)[2 * (NU + 1)][NU + 2]) {
  constexpr int n = NU + 1;
  T PL[n][n];
#pragma unroll
  for (int k = 0; k < n; ++k)
#pragma unroll
    for (int r = 0; r < n; ++r) PL[k][r] = pinv[k] * L[k][r];
  // column c + 1 of Z is column c of [X; U]; column 0 is column 1 of [X; U]
#pragma unroll
  for (int c = 0; c < n; ++c)
#pragma unroll
    for (int r = 0; r < n; ++r) {
      T acc = T(0);
#pragma unroll
      for (int k = (c > r ? c : r); k < n; ++k) acc += T(iwp_a<NU>(c, k)) * PL[k][r];
      Z[r][c + 1] = acc;
    }
#pragma unroll
  for (int r = 0; r < n; ++r) Z[r][0] = Z[r][2];
}

// ... the U rows (the scaled process-noise factor) ...
template <typename T, int NU, typename Q>
PDQ_D void joint_u(const Q (&q1)[kMaxN][kMaxN], T scale_q, T (&Z)[2 * (NU + 1)][NU + 2]) {
  constexpr int n = NU + 1;
#pragma unroll
  for (int c = 0; c < n; ++c)
#pragma unroll
    for (int r = 0; r < n; ++r) Z[n + r][c + 1] = (r <= c) ? scale_q * T(q1[c][r]) : T(0);
#pragma unroll
  for (int r = 0; r < n; ++r) Z[n + r][0] = Z[n + r][2];
}

// ... the first reflector, which finalises row 0 of R': returns R_Y, writes the gain ...
template <typename T, int NU>
PDQ_D T joint_first(T (&Z)[2 * (NU + 1)][NU + 2], const T (&p)[NU + 1], const T (&pinv)[NU + 1], T (&gain)[NU + 1],
                    bool& ok) {
  constexpr int n = NU + 1;
  static_assert(n >= 2, "the joint update needs the observed coefficient 1");
  constexpr unsigned x_rows = (1u << n) - 1u;
  constexpr unsigned u01 = 3u << n;
  constexpr unsigned all_cols = (1u << (n + 1)) - 1u;
  // column 0 (pivot X row 0; X rows 1.., U rows 0, 1), applied to columns 1, 3..n
  hh_step<T, 2 * n, n + 1, 0, 0, (x_rows & ~1u) | u01, all_cols & ~5u>(Z, ok);
#pragma unroll
  for (int r = 0; r < 2 * n; ++r) Z[r][2] = (r == 0) ? Z[0][0] : T(0);
  const T r_inv = fast_rcp(Z[0][0]) * dev_abs(pinv[1]);
#pragma unroll
  for (int i = 0; i < n; ++i) gain[i] = (i == 1) ? T(1) : Z[0][i + 1] * r_inv * dev_abs(p[i]);
  return dev_abs(p[1]) * Z[0][0];
}

// ... and the other reflectors, which give the updated factor.
template <typename T, int NU>
PDQ_D void joint_rest(T (&Z)[2 * (NU + 1)][NU + 2], const T (&p)[NU + 1], T (&Lnew)[NU + 1][NU + 1], bool& ok) {
  constexpr int n = NU + 1;
  constexpr unsigned x_rows = (1u << n) - 1u;
  constexpr unsigned u01 = 3u << n;
  constexpr unsigned all_cols = (1u << (n + 1)) - 1u;
  // column 1 (pivot X row 1; X rows 2.., U rows 0, 1), applied to columns 3..n
  hh_step<T, 2 * n, n + 1, 1, 1, (x_rows & ~3u) | u01, all_cols & ~7u>(Z, ok);
  joint_tail<T, n, 3>(Z, ok);
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < n; ++j) Lnew[i][j] = (j <= i) ? dev_abs(p[i]) * Z[j + 1][i + 1] : T(0);
}

template <typename T, int NU, typename Q>
PDQ_D T iso_predict_update_fast(const Q (&q1)[kMaxN][kMaxN], const T (&L)[NU + 1][NU + 1], const T (&p)[NU + 1],
                                const T (&pinv)[NU + 1], T scale_q, T (&gain)[NU + 1], T (&Lnew)[NU + 1][NU + 1],
                                bool& ok) {
  constexpr int n = NU + 1;
  T Z[2 * n][n + 1];
  joint_x<T, NU>(L, pinv, Z);
  joint_u<T, NU>(q1, scale_q, Z);
  const T R_Y = joint_first<T, NU>(Z, p, pinv, gain, ok);
  joint_rest<T, NU>(Z, p, Lnew, ok);
  return R_Y;
}

template <typename T, int NU, int D, typename Q>
PDQ_D void iso_predict(const Q (&q1)[kMaxN][kMaxN], const T (&m)[NU + 1][D], const T (&L)[NU + 1][NU + 1],
                       const T (&p)[NU + 1], const T (&pinv)[NU + 1], T scale_q, T (&mp)[NU + 1][D],
                       T (&Lp)[NU + 1][NU + 1]) {
  iso_predict_mean<T, NU, D>(m, p, pinv, mp);
  iso_predict_chol<T, NU>(q1, L, p, pinv, scale_q, Lp);
}

// revert_conditional for a TS0 observation of coefficient OUT
// (util/cholesky_util.py:27-82, H = e_OUT, noise chol damp), or a TS1 one
// with H = h0 e_0 + e_OUT (same sparsity of (H Lp)^T): a Givens chain
// on [[damp, 0], [(H Lp)^T, Lp^T]].  Column 0 has nonzeros in rows 0..OUT+1;
// eliminating it bottom-up fills one subdiagonal entry per row, which one
// rotation per column 1..OUT removes.  Returns R_Y; gain = R12^T / R_Y and
// Lnew = R22^T.
template <typename T, int NU, int OUT, bool H0 = true>
PDQ_D T ts0_update(const T (&Lp)[NU + 1][NU + 1], T damp, T (&gain)[NU + 1], T (&Lnew)[NU + 1][NU + 1],
                   T h0 = T(0)) {
  constexpr int n = NU + 1;
  T M[n + 1][n + 1];
#pragma unroll
  for (int c = 0; c <= n; ++c) M[0][c] = (c == 0) ? damp : T(0);
#pragma unroll
  for (int r = 1; r <= n; ++r) {
    // (H Lp)^T with H = h0 e_0 + e_OUT (TS1) or e_OUT (h0 = 0, TS0); Lp is
    // lower triangular, so the h0 term only reaches row 1
    if constexpr (H0) {
      M[r][0] = (r == 1) ? Lp[OUT][0] + h0 * Lp[0][0] : Lp[OUT][r - 1];
    } else {
      M[r][0] = Lp[OUT][r - 1];
    }
#pragma unroll
    for (int c = 1; c <= n; ++c) M[r][c] = (c >= r) ? Lp[c - 1][r - 1] : T(0);
  }
#pragma unroll
  for (int r = OUT + 1; r >= 1; --r) givens_rows<T, n + 1, n + 1>(M, r - 1, r, 0);
#pragma unroll
  for (int c = 1; c <= OUT; ++c) givens_rows<T, n + 1, n + 1>(M, c, c + 1, c);
  const T R_Y = M[0][0];
  const T ry_inv = fast_rcp(R_Y);
#pragma unroll
  for (int i = 0; i < n; ++i) {
    gain[i] = M[0][i + 1] * ry_inv;
#pragma unroll
    for (int j = 0; j < n; ++j) Lnew[i][j] = (j <= i) ? M[j + 1][i + 1] : T(0);
  }
  return R_Y;
}

// Branch-free twin of ts0_update (rotations by the single-instruction
// reciprocal square root, a zero pair rotated by the identity).  Clears ok
// when a rotation's sum of squares left [1e-30, 1e36]; the caller then
// reruns the attempt with ts0_update.
template <typename T, int NR, int NC>
PDQ_D void givens_rows_fast(T (&M)[NR][NC], int a, int b, int c0, bool& ok) {
  const T x = M[a][c0], y = M[b][c0];
  const T r2 = x * x + y * y;
  ok = ok && (r2 == T(0) || !norm2_out_of_range(r2));
  const T inv = fast_rsqrt(r2);
  const bool zero = r2 == T(0);
  const T cs = zero ? T(1) : x * inv;
  const T sn = zero ? T(0) : y * inv;
#pragma unroll
  for (int j = 0; j < NC; ++j) {
    if (j > c0) {
      const T ma = M[a][j], mb = M[b][j];
      M[a][j] = cs * ma + sn * mb;
      M[b][j] = cs * mb - sn * ma;
    }
  }
  M[a][c0] = zero ? x : r2 * inv;
  M[b][c0] = T(0);
}

template <typename T, int NU, int OUT, bool H0 = true>
PDQ_D T ts0_update_fast(const T (&Lp)[NU + 1][NU + 1], T damp, T (&gain)[NU + 1], T (&Lnew)[NU + 1][NU + 1], bool& ok,
                        T h0 = T(0)) {
  constexpr int n = NU + 1;
  T M[n + 1][n + 1];
#pragma unroll
  for (int c = 0; c <= n; ++c) M[0][c] = (c == 0) ? damp : T(0);
#pragma unroll
  for (int r = 1; r <= n; ++r) {
    if constexpr (H0) {
      M[r][0] = (r == 1) ? Lp[OUT][0] + h0 * Lp[0][0] : Lp[OUT][r - 1];
    } else {
      M[r][0] = Lp[OUT][r - 1];
    }
#pragma unroll
    for (int c = 1; c <= n; ++c) M[r][c] = (c >= r) ? Lp[c - 1][r - 1] : T(0);
  }
#pragma unroll
  for (int r = OUT + 1; r >= 1; --r) givens_rows_fast<T, n + 1, n + 1>(M, r - 1, r, 0, ok);
#pragma unroll
  for (int c = 1; c <= OUT; ++c) givens_rows_fast<T, n + 1, n + 1>(M, c, c + 1, c, ok);
  const T R_Y = M[0][0];
  const T ry_inv = fast_rcp(R_Y);
#pragma unroll
  for (int i = 0; i < n; ++i) {
    gain[i] = M[0][i + 1] * ry_inv;
#pragma unroll
    for (int j = 0; j < n; ++j) Lnew[i][j] = (j <= i) ? M[j + 1][i + 1] : T(0);
  }
  return R_Y;
}

// error_state_std: posterior std of coefficient 0 after conditioning the
// unit-scale extrapolation N(., (|p| sqrt|h| Q1)(...)^T) on the linearised
// residual (the Givens update of ts0_update applied to that factor; its row 0
// is (L00, 0, ...), so the std is |L00|).
template <typename T, int NU, int OUT, typename A>
PDQ_D T state_std0(const A& a, const T (&p)[NU + 1], T h, T damp, T h0) {
  constexpr int n = NU + 1;
  constexpr bool kNarrow = sizeof(T) == sizeof(float);
  const T sq = fast_sqrt(dev_abs(h));
  T Lu[n][n];
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < n; ++j) {
      const T q = kNarrow ? T(a.q1f[i][j]) : T(a.q1[i][j]);
      Lu[i][j] = (j <= i) ? dev_abs(p[i]) * sq * q : T(0);
    }
  T g[n], Lc[n][n];
  ts0_update<T, NU, OUT>(Lu, damp, g, Lc, h0);
  return dev_abs(Lc[0][0]);
}

// Error norm, acceptance and step-size controller of one attempt, from the
// absolute error err_abs (error_residual_std or error_state_std): the
// per-dimension ratios err_abs / (atol + rtol max(|m_0j|, |mnew_0j|)) summed
// wide (solvers.py:925-996, the RMS norm), accepted iff the error power
// norm^(-1/n) >= 1, i.e. iff the sum is <= D, and the I or PI controller's
// next step (controllers.py:24-84).
template <typename T, int NU, int D>
PDQ_D void iso_accept_and_control(const IsoArgs& a, T err_abs, const T (&m)[NU + 1][D], const T (&mnew)[NU + 1][D],
                                  T dt_use, T pi_prev, bool& accepted, bool& nonfinite, T& pi_new, T& dt_new) {
  constexpr int n = NU + 1;
  const T atol = cst<T>(a.atol, a.atol_f), rtol = cst<T>(a.rtol, a.rtol_f);
  const T safety = cst<T>(a.safety, a.safety_f);
  const T factor_min = cst<T>(a.factor_min, a.factor_min_f), factor_max = cst<T>(a.factor_max, a.factor_max_f);
  Wide<T> sumsq = wide_from(0.0, T(0));
#pragma unroll
  for (int j = 0; j < D; ++j) {
    const T ref = fmax(dev_abs(m[0][j]), dev_abs(mnew[0][j]));
    const T ratio = dev_div(err_abs, atol + rtol * ref);
    sumsq = wide_add_sq(sumsq, ratio);
  }
  // error_norm^2 = sumsq / D; accepted iff error_power = error_norm^(-1/n)
  // >= 1, i.e. iff sumsq <= D (decided on the wide sum)
  const T norm2 = T(wide_hi(sumsq)) * T(1.0 / D);
  nonfinite = !(norm2 == norm2) || isinf(norm2);
  const T ep = dev_fpow(norm2, T(-0.5 / n));
  accepted = wide_le(sumsq, T(D));
  T factor;
  pi_new = pi_prev;
  if (a.control == PDQ_CONTROL_INTEGRAL) {
    factor = safety * ep;
  } else {
    const T gi = dev_fpow(ep, cst<T>(a.exp_i, a.exp_i_f));
    const T gp = dev_fpow(dev_div(ep, pi_prev), cst<T>(a.exp_p, a.exp_p_f));
    factor = safety * gi * gp;
    if (accepted) pi_new = ep;
  }
  factor = fmax(factor_min, fmin(factor, factor_max));
  dt_new = factor * dt_use;
}

template <typename T, int NU, int D>
PDQ_D void write_record(const IsoArgs& a, int64_t b, int s_out, int S_out, const T (&m)[NU + 1][D],
                        const T (&lo)[2][D], const T (&L)[NU + 1][NU + 1], double scale, double t, int steps) {
  constexpr int n = NU + 1;
  const int64_t rec = b * S_out + s_out;
  double* um = a.u_mean + rec * (n * D);
  double* uc = a.u_chol + rec * (n * n);
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
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < n; ++j) uc[i * n + j] = double(L[i][j]);
  a.output_scale[rec] = scale;
  a.t_out[rec] = t;
  a.num_steps[rec] = steps;
}

// A record of a mean without wide rows.
template <typename T, int NU, int D>
PDQ_D void write_record(const IsoArgs& a, int64_t b, int s_out, int S_out, const T (&m)[NU + 1][D],
                        const T (&L)[NU + 1][NU + 1], double scale, double t, int steps) {
  T lo[2][D];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) lo[i][j] = T(0);
  write_record<T, NU, D>(a, b, s_out, S_out, m, lo, L, scale, t, steps);
}

// ---------------------------------------------------------------------------
// Fixed-point smoother pieces in the isotropic factorisation
// (IsotropicLatentCond, ssm_impl_isotropic.py:72-140): a backward conditional
// x_prev | x = N(to * (A (tl * x) + xi), (|to| X)(|to| X)^T) with A, X (n, n)
// shared by all d dimensions and xi (n, d).
// ---------------------------------------------------------------------------

template <typename T, int NU, int D>
struct IsoBackward {
  T A[NU + 1][NU + 1];
  T xi[NU + 1][D];
  T X[NU + 1][NU + 1];  // lower triangular
  T tl[NU + 1];
  T to[NU + 1];
};

template <int NU, int D>
PDQ_HD constexpr int iso_cond_floats() {
  return (NU + 1) * (NU + 1) + (NU + 1) * D + (NU + 1) * (NU + 2) / 2 + 2 * (NU + 1);
}

template <typename T, int NU, int D>
PDQ_D void iso_cond_identity(IsoBackward<T, NU, D>& c) {
  constexpr int n = NU + 1;
#pragma unroll
  for (int i = 0; i < n; ++i) {
#pragma unroll
    for (int j = 0; j < n; ++j) {
      c.A[i][j] = (i == j) ? T(1) : T(0);
      c.X[i][j] = T(0);
    }
#pragma unroll
    for (int j = 0; j < D; ++j) c.xi[i][j] = T(0);
    c.tl[i] = T(1);
    c.to[i] = T(1);
  }
}

template <typename T, int NU, int D>
PDQ_D void iso_cond_store(T* base, const IsoBackward<T, NU, D>& c) {
  constexpr int n = NU + 1;
  int o = 0;
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < n; ++j) base[o++] = c.A[i][j];
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) base[o++] = c.xi[i][j];
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j <= i; ++j) base[o++] = c.X[i][j];
#pragma unroll
  for (int i = 0; i < n; ++i) base[o++] = c.tl[i];
#pragma unroll
  for (int i = 0; i < n; ++i) base[o++] = c.to[i];
}

template <typename T, int NU, int D>
PDQ_D void iso_cond_load(const T* base, IsoBackward<T, NU, D>& c) {
  constexpr int n = NU + 1;
  int o = 0;
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < n; ++j) c.A[i][j] = base[o++];
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) c.xi[i][j] = base[o++];
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < n; ++j) c.X[i][j] = (j <= i) ? base[o++] : T(0);
#pragma unroll
  for (int i = 0; i < n; ++i) c.tl[i] = base[o++];
#pragma unroll
  for (int i = 0; i < n; ++i) c.to[i] = base[o++];
}

// transition(h, s).revert(rv) (ssm_impl_isotropic.py:107-133 with the IWP
// transition :367-378): the predicted Cholesky factor and the backward
// conditional.  M = [[R_YX, 0], [R_X_F, R_X]] with R_YX = (s sqrt|h| Q1)^T,
// R_X_F = (A cl)^T, R_X = cl^T, cl = |p_inv| L; R = qr_r(M); the predicted
// factor is |p| R_Y^T, G^T = R_Y^{-1} R12, the conditional's noise factor R22^T.
template <typename T, int NU, int D, typename Q>
PDQ_D void iso_prior_revert(const Q (&q1)[kMaxN][kMaxN], const T (&m)[NU + 1][D], const T (&L)[NU + 1][NU + 1],
                            const T (&p)[NU + 1], const T (&pinv)[NU + 1], T scale_q, T (&Lp)[NU + 1][NU + 1],
                            IsoBackward<T, NU, D>& cond) {
  constexpr int n = NU + 1;
  T M[2 * n][2 * n];
  T cl[n][n];
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < n; ++j) cl[i][j] = (j <= i) ? dev_abs(pinv[i]) * L[i][j] : T(0);
#pragma unroll
  for (int r = 0; r < n; ++r)
#pragma unroll
    for (int c = 0; c < n; ++c) {
      M[r][c] = (r <= c) ? scale_q * T(q1[c][r]) : T(0);
      M[r][n + c] = T(0);
      T acc = T(0);
#pragma unroll
      for (int k = c; k < n; ++k) acc += T(iwp_a<NU>(c, k)) * cl[k][r];
      M[n + r][c] = acc;
      M[n + r][n + c] = cl[c][r];
    }
  householder_r<T, 2 * n, 2 * n>(M);
  T Gt[n][n];
#pragma unroll
  for (int col = 0; col < n; ++col)
#pragma unroll
    for (int i = n - 1; i >= 0; --i) {
      T acc = M[i][n + col];
#pragma unroll
      for (int k = i + 1; k < n; ++k) acc -= M[i][k] * Gt[k][col];
      Gt[i][col] = acc / M[i][i];
    }
  T mean_l[n][D], mobs[n][D];
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) mean_l[i][j] = pinv[i] * m[i][j];
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      T acc = T(0);
#pragma unroll
      for (int k = i; k < n; ++k) acc += T(iwp_a<NU>(i, k)) * mean_l[k][j];
      mobs[i][j] = acc;
    }
#pragma unroll
  for (int i = 0; i < n; ++i) {
#pragma unroll
    for (int j = 0; j < D; ++j) {
      T acc = mean_l[i][j];
#pragma unroll
      for (int k = 0; k < n; ++k) acc -= Gt[k][i] * mobs[k][j];
      cond.xi[i][j] = acc;
    }
#pragma unroll
    for (int j = 0; j < n; ++j) {
      cond.A[i][j] = Gt[j][i];
      cond.X[i][j] = (j <= i) ? M[n + j][n + i] : T(0);
      Lp[i][j] = (j <= i) ? dev_abs(p[i]) * M[j][i] : T(0);
    }
    cond.tl[i] = T(1) / p[i];
    cond.to[i] = T(1) / pinv[i];
  }
}

// outer.merge(inner) (ssm_impl_isotropic.py:91-105)
template <typename T, int NU, int D>
PDQ_D void iso_cond_merge(const IsoBackward<T, NU, D>& o, const IsoBackward<T, NU, D>& in,
                          IsoBackward<T, NU, D>& out) {
  constexpr int n = NU + 1;
  T Tv[n];
#pragma unroll
  for (int i = 0; i < n; ++i) Tv[i] = o.tl[i] * in.to[i];
  T M[2 * n][n];
#pragma unroll
  for (int i = 0; i < n; ++i) {
#pragma unroll
    for (int j = 0; j < n; ++j) {
      T g = T(0), r1 = T(0);
#pragma unroll
      for (int k = 0; k < n; ++k) {
        g += o.A[i][k] * Tv[k] * in.A[k][j];
        r1 += o.A[i][k] * dev_abs(Tv[k]) * in.X[k][j];
      }
      out.A[i][j] = g;
      M[j][i] = r1;
      M[n + j][i] = o.X[i][j];
    }
#pragma unroll
    for (int d = 0; d < D; ++d) {
      T x = o.xi[i][d];
#pragma unroll
      for (int k = 0; k < n; ++k) x += o.A[i][k] * Tv[k] * in.xi[k][d];
      out.xi[i][d] = x;
    }
  }
  householder_r<T, 2 * n, n>(M);
#pragma unroll
  for (int i = 0; i < n; ++i) {
#pragma unroll
    for (int j = 0; j < n; ++j) out.X[i][j] = (j <= i) ? M[j][i] : T(0);
    out.tl[i] = in.tl[i];
    out.to[i] = o.to[i];
  }
}

// cond.marginalise(rv) (ssm_impl_isotropic.py:81-89)
template <typename T, int NU, int D>
PDQ_D void iso_cond_marginalise(const IsoBackward<T, NU, D>& c, const T (&m)[NU + 1][D],
                                const T (&L)[NU + 1][NU + 1], T (&mo)[NU + 1][D], T (&Lo)[NU + 1][NU + 1]) {
  constexpr int n = NU + 1;
  T M[2 * n][n];
#pragma unroll
  for (int r = 0; r < n; ++r)
#pragma unroll
    for (int col = 0; col < n; ++col) {
      T acc = T(0);
#pragma unroll
      for (int k = 0; k < n; ++k) acc += c.A[col][k] * c.tl[k] * L[k][r];
      M[r][col] = acc;
      M[n + r][col] = c.X[col][r];
    }
  householder_r<T, 2 * n, n>(M);
#pragma unroll
  for (int i = 0; i < n; ++i) {
#pragma unroll
    for (int d = 0; d < D; ++d) {
      T acc = c.xi[i][d];
#pragma unroll
      for (int k = 0; k < n; ++k) acc += c.A[i][k] * c.tl[k] * m[k][d];
      mo[i][d] = c.to[i] * acc;
    }
#pragma unroll
    for (int j = 0; j < n; ++j) Lo[i][j] = (j <= i) ? dev_abs(c.to[i]) * M[j][i] : T(0);
  }
}

template <typename T, int NU, int D>
PDQ_D void write_filter(const IsoArgs& a, int64_t rec, const T (&m)[NU + 1][D], const T (&L)[NU + 1][NU + 1]) {
  constexpr int n = NU + 1;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < D; ++j) a.filter_mean[rec * (n * D) + i * D + j] = double(m[i][j]);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) a.filter_chol[rec * (n * n) + i * n + j] = double(L[i][j]);
}

template <typename T, int NU, int D>
PDQ_D void write_cond_iso(const IsoArgs& a, int64_t cr, const IsoBackward<T, NU, D>& c, double cal) {
  constexpr int n = NU + 1;
  for (int i = 0; i < n; ++i) {
    for (int j = 0; j < n; ++j) {
      a.cond_A[cr * n * n + i * n + j] = double(c.A[i][j]);
      a.cond_noise_chol[cr * n * n + i * n + j] = double(c.X[i][j]) * cal;
    }
    for (int j = 0; j < D; ++j) a.cond_noise_mean[cr * n * D + i * D + j] = double(c.xi[i][j]);
    a.cond_to_latent[cr * n + i] = double(c.tl[i]);
    a.cond_to_observed[cr * n + i] = double(c.to[i]);
  }
}

template <typename T, int NU, int D>
PDQ_D void write_normal_iso(const IsoArgs& a, int64_t rec, const T (&m)[NU + 1][D], const T (&L)[NU + 1][NU + 1]) {
  constexpr int n = NU + 1;
  double* um = a.u_mean + rec * (n * D);
  double* uc = a.u_chol + rec * (n * n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < D; ++j) um[i * D + j] = double(m[i][j]);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) uc[i * n + j] = double(L[i][j]);
}

// Sensitivity record: direction k < P is d / d params[k], k >= P is d / d y0[k - P].
template <typename T, int NU, int D, int P>
PDQ_D void write_tangent(const IsoArgs& a, int64_t rec, int k, const T (&dm)[NU + 1][D]) {
  constexpr int n = NU + 1;
  double* out = k < P ? a.tan_params : a.tan_y0;
  const int dirs = k < P ? P : D, kk = k < P ? k : k - P;
  if (out == nullptr) return;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < D; ++j) out[((rec * n + i) * D + j) * dirs + kk] = double(dm[i][j]);
}

// One adaptive solve per thread.  INTERP: keep the interpolation state
// (needed unless clip_dt makes every checkpoint an exact landing).  FP: the
// fixed-point smoother (estimators_and_losses.py:473-591): every step also
// forms the prior's backward conditional and merges it into the running one;
// at each checkpoint the running conditional goes to the workspace and
// resets to the identity; after the last step the backward pass
// (Smoother.finalize, MarkovSequence.evaluate_marginals, :156-178, 437-470)
// marginalises from the terminal state through the stored conditionals.
// GEN: TS1 and error_state_std are available (run-time switches); the
// instantiation without them serves TS0 with error_residual_std, whose
// attempt is then free of their branches and of the TS1 term in the update.
// TAN (TS0 filter): forward-mode sensitivities of the mean, P + d threads per
// instance, thread k carrying d / d params[k] (k < P) or d / d y0[k - P].
// Every thread recomputes the same value path (same steps, same records);
// thread 0 writes the values.  The step size carries no tangent (the
// reference stops gradients through dt), and with H = e_1 the covariance
// recursion does not depend on the parameters, so the tangent of an update
// is dm' = dmp - gain (dmp_1 - df), dmp = p A p^-1 dm, df = J_f dmp_0 + df/dtheta.
// REC (lean TS0 filter, exact landings): records each accepted step's size
// and the state before every rec_ckpt-th accepted step for the
// terminal-value adjoint (tv_adjoint.cuh); an instance with more accepted
// steps than rec_capacity finishes its solve and reports
// PDQ_INSTANCE_RECORD_FULL.
template <typename T, int NU, class F, bool INTERP, bool FP = false, bool GEN = true, bool TAN = false, bool REC = false>
__global__ void __launch_bounds__(64) iso_adaptive_kernel(IsoArgs a) {
  constexpr int n = NU + 1;
  constexpr int D = F::D;
  constexpr int P = F::P;
  constexpr int OUT = 1;  // ODE u' = f(u): observe coefficient 1 (problems.py:283-295)
  static_assert(!(TAN && (FP || GEN)), "sensitivities: TS0 filter only");
  static_assert(!(REC && (FP || GEN || TAN || INTERP)), "record: the lean TS0 filter with exact landings only");
  bool rec_full = false;
  const int64_t gtid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t b = TAN ? gtid / (P + D) : gtid;
  const int kdir = TAN ? int(gtid % (P + D)) : 0;
  const bool primary = kdir == 0;  // writes the values
  if (b >= a.B) return;

  const int S = a.S;
  const int S_out = a.terminal_only ? 1 : S;
  const double* save_at = a.save_at + b * S;

  // ---- inputs and Taylor-mode initial derivatives (float64) ----
  double pd[P];
#pragma unroll
  for (int k = 0; k < P; ++k) pd[k] = a.params[b * P + k];
  T pt[P];
  Wide<T> pw[P];  // the parameters in the wide type (the residual's field evaluation)
#pragma unroll
  for (int k = 0; k < P; ++k) {
    pt[k] = T(pd[k]);
    pw[k] = wide_from(pd[k], T(0));
  }
  double y0[D];
#pragma unroll
  for (int j = 0; j < D; ++j) y0[j] = a.y0[b * D + j];
  double tc[n][D];
  taylor_init<F, NU>(y0, pd, tc);

  // mean (rows 0 and 1 wide: m plus the low parts mlo) and Cholesky factor
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
  // tangents of m and of the interpolation state (TAN only): the Taylor
  // coefficients' derivative along this thread's direction
  T dm[n][D], dmi[n][D];
  if constexpr (TAN) {
    Dual<double, 1> yd[D], prd[P], tcd[n][D];
#pragma unroll
    for (int j = 0; j < D; ++j) {
      yd[j] = Dual<double, 1>(y0[j]);
      yd[j].g[0] = (kdir == P + j) ? 1.0 : 0.0;
    }
#pragma unroll
    for (int k = 0; k < P; ++k) {
      prd[k] = Dual<double, 1>(pd[k]);
      prd[k].g[0] = (kdir == k) ? 1.0 : 0.0;
    }
    taylor_init<F, NU>(yd, prd, tcd);
#pragma unroll
    for (int i = 0; i < n; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) dm[i][j] = dmi[i][j] = T(tcd[i][j].g[0]);
  }
  // interpolation state (interp_from); dead code when INTERP is false
  T mi[n][D], milo[2][D], Li[n][n];
  using W = Wide<T>;
  constexpr bool kNarrow = sizeof(T) == sizeof(float);
  W ti = wide_from(save_at[0], T(0));
  if constexpr (INTERP) {
#pragma unroll
    for (int i = 0; i < n; ++i) {
#pragma unroll
      for (int j = 0; j < D; ++j) mi[i][j] = m[i][j];
#pragma unroll
      for (int j = 0; j < n; ++j) Li[i][j] = T(0);
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) milo[i][j] = mlo[i][j];
  }

  // fixed-point smoother: running backward conditional of step_from (bw) and
  // of interp_from (bwi); dead code without FP
  IsoBackward<T, NU, D> bw, bwi;
  T* const ws = FP ? reinterpret_cast<T*>(a.workspace) + b * int64_t(S - 1) * iso_cond_floats<NU, D>() : nullptr;
  if constexpr (FP) {
    iso_cond_identity(bw);
    if constexpr (INTERP) iso_cond_identity(bwi);
  }

  W t = wide_from(save_at[0], T(0));
  T dt = T(a.dt0[b]);
  T pi_prev = T(1);  // PI controller state (controllers.py:41-43)
  W mle_sumsq = wide_from(0.0, T(0));
  int num_data = 0, num_steps = 0, attempts = 0, status = PDQ_INSTANCE_OK;
  T sigma_sf = T(1);  // output scale of step_from (dynamic solver)
  const T damp = cst<T>(a.damp, a.damp_f);
  const T eps = cst<T>(a.eps, a.eps_f);

  // ||Q1 row OUT||^2 enters the observed std of the linearised residual
  T q1_out2 = T(0);
#pragma unroll
  for (int j = 0; j < n; ++j) q1_out2 += cst<T>(a.q1[OUT][j], a.q1f[OUT][j]) * cst<T>(a.q1[OUT][j], a.q1f[OUT][j]);
  const T q1_out_norm = dev_sqrt(q1_out2);
  const T q00 = cst<T>(a.q1[0][0], a.q1f[0][0]), q10 = cst<T>(a.q1[1][0], a.q1f[1][0]),
          q11 = cst<T>(a.q1[1][1], a.q1f[1][1]);

  if (!a.terminal_only) {
    if (primary) write_record<T, NU, D>(a, b, 0, S_out, m, mlo, L, 1.0, wide_value(t), 0);
    if constexpr (TAN) write_tangent<T, NU, D, P>(a, b * S_out, kdir, dm);
  }
  if (FP && a.filter_mean) write_filter<T, NU, D>(a, b * S, m, L);

  // t + eps < t_next (float64: exactly the reference's comparison; float
  // pairs: the difference, rounded once, against eps)
  auto before = [&](const W& x, const W& y) -> bool {
    if constexpr (kNarrow) {
      return wide_diff(y, x) > eps;
    } else {
      return x + a.eps < y;
    }
  };

  // One attempt per iteration: the rejection loop and the loop over
  // checkpoints are flattened into one, so a lane whose attempt is rejected
  // retries in the next iteration while the other lanes of its warp go on
  // (a nested retry loop would hold them at its exit, making every accepted
  // step of a warp cost as many attempts as its slowest lane needs).  Per
  // instance the sequence of attempts, checkpoint branches and records is the
  // nested loop's (solvers_via_adaptive_steps.py:196-375).
  int s = 1;
  W t_next = wide_from(save_at[1], T(0));
  bool safe_next = false;  // the next attempt takes the range-checked predict and update
  // before(t, t_next) and t_next - t, carried across iterations: an attempt
  // forms them for its candidate time alongside its arithmetic, so an
  // accepted step does not recompute them at the head of the next one
  bool bef = before(t, t_next);
  T rem = wide_diff(t_next, t);
  while (s < S) {
    if (bef) {
      // ---- one attempt of the rejection loop (solvers_via_adaptive_steps.py:249-328) ----
      const T remaining = rem;
      const bool clipped = a.clip_dt && !(dt < remaining);
      const T dt_use = clipped ? remaining : dt;
      if (!(dev_abs(dt_use) > T(1e-14) * fmax(T(1), dev_abs(T(wide_hi(t)))))) {
        status = PDQ_INSTANCE_DT_UNDERFLOW;
        break;
      }
      if (attempts >= a.max_attempts) {
        status = PDQ_INSTANCE_MAX_STEPS;
        break;
      }
      ++attempts;
      const T h = dt_use;
      // the time after this attempt if it is accepted: a step clipped to the
      // checkpoint lands on it exactly in float pairs; float64 adds as the
      // reference does
      W t_acc;
      if constexpr (kNarrow) {
        t_acc = clipped ? t_next : wide_add(t, dt_use);
      } else {
        t_acc = t + dt_use;
      }
      const bool bef_acc = before(t_acc, t_next);
      const T rem_acc = wide_diff(t_next, t_acc);
      // The attempt's arithmetic, a generic lambda instantiated twice: with
      // the branch-free predict and update (SAFE false), and with the
      // range-checked ones (SAFE true), which rerun an attempt whose sums of
      // squares left the safe range.  Each instantiation is one block of
      // straight-line code, so the compiler interleaves the mean, the
      // residual, the QR and the error estimate.
      T mnew[n][D], mnewlo[2][D], dmnew[n][D], Lnew[n][n];
      T rms_mobs, sigma_loc, ry_inv, dt_new, pi_new;
      bool accepted, nonfinite, ok;
      IsoBackward<T, NU, D> cnew;  // fixed-point: the prior's backward conditional of this step
      auto attempt = [&](auto safe_tag) {
        constexpr bool SAFE = decltype(safe_tag)::value;
        T p[n], pinv[n];
        precon<T, NU>(h, p, pinv);

        // extrapolated mean: the same for every calibration mode, and the
        // error estimate's apply_flat(previous mean) (solvers.py:943-944),
        // in increment form with rows 0 and 1 wide
        T incr[n][D], mp[n][D], mplo[2][D];
        iso_mean_increment<T, NU, D>(m, p, pinv, incr);
        iso_mean_add<T, NU, D>(m, mlo, incr, mp, mplo);
        // TS0 linearisation at the extrapolated mean (ssm_impl_isotropic.py:304-317):
        // the residual mp_1 - f(mp_0), the field evaluated in the wide type;
        // TS1: H = [-tr J_f(mp_0) / d, 1, 0, ...] (ssm_impl_isotropic.py:320-355,
        // jacobians.py:100-106), same residual mean
        T h0 = T(0);
        if (GEN && a.ts1) {
          T f[D], Jf[D][D];
          eval_with_jacobian<F>(mp[0], pt, f, Jf);
          T tr = T(0);
#pragma unroll
          for (int j = 0; j < D; ++j) tr += Jf[j][j];
          h0 = -tr * T(1.0 / D);
        }
        static_assert(OUT == 1, "the residual observes coefficient 1");
        T mobs[D];
        iso_residual<F, T, NU>(mp, mplo, pw, mobs);
        T mobs2 = T(0);
#pragma unroll
        for (int j = 0; j < D; ++j) mobs2 += mobs[j] * mobs[j];
        rms_mobs = fast_sqrt(mobs2 * T(1.0 / D));
        // fx.marginalise(apply_flat(m)) with unit scale: observed std
        // l = sqrt(|p_OUT|^2 |h| ||Q1[OUT]||^2 + damp^2), and the local scale
        // residual_whitened_rms = rms(mobs) / l (solvers.py:553-566, 955-957)
        const T ell = (GEN && a.ts1) ? observed_std_ts1<T, NU>(p[OUT], h, h0, q00, q10, q11, damp)
                                     : observed_std(p[OUT], h, q1_out_norm, damp);
        sigma_loc = dev_div(rms_mobs, ell);

        // ---- predict (marginalise) and update (revert_conditional, H = e_OUT) ----
        const T s_pred = (a.solver == PDQ_SOLVER_DYNAMIC) ? sigma_loc : T(1);
        const T scale_q = s_pred * (kNarrow ? fast_sqrt(dev_abs(h)) : dev_sqrt(dev_abs(h)));
        T Lp[n][n], gain[n], R_Y;
        ok = true;
        if constexpr (FP) {
          if constexpr (kNarrow) {
            iso_prior_revert<T, NU, D>(a.q1f, m, L, p, pinv, scale_q, Lp, cnew);
          } else {
            iso_prior_revert<T, NU, D>(a.q1, m, L, p, pinv, scale_q, Lp, cnew);
          }
          R_Y = ts0_update<T, NU, OUT, GEN>(Lp, damp, gain, Lnew, h0);
        } else if constexpr (SAFE) {
          if constexpr (kNarrow) {
            iso_predict_chol<T, NU>(a.q1f, L, p, pinv, scale_q, Lp);
          } else {
            iso_predict_chol<T, NU>(a.q1, L, p, pinv, scale_q, Lp);
          }
          R_Y = ts0_update<T, NU, OUT, GEN>(Lp, damp, gain, Lnew, h0);
        } else if ((!GEN && !TAN) || (damp == T(0) && !(GEN && a.ts1))) {
          // TS0 without damping (always so in the lean instantiation, by the
          // launchers' dispatch): the predict and the update in one QR
          if constexpr (kNarrow) {
            R_Y = iso_predict_update_fast<T, NU>(a.q1f, L, p, pinv, scale_q, gain, Lnew, ok);
          } else {
            R_Y = iso_predict_update_fast<T, NU>(a.q1, L, p, pinv, scale_q, gain, Lnew, ok);
          }
        } else {
          if constexpr (kNarrow) {
            ok = iso_predict_chol_fast<T, NU>(a.q1f, L, p, pinv, scale_q, Lp);
          } else {
            ok = iso_predict_chol_fast<T, NU>(a.q1, L, p, pinv, scale_q, Lp);
          }
          R_Y = ts0_update_fast<T, NU, OUT, GEN>(Lp, damp, gain, Lnew, ok, h0);
        }
        ry_inv = fast_rcp(R_Y);
        // mnew = mp - gain mobs = m + (incr - gain mobs), the wide rows summed wide
        {
          T dlt[n][D];
#pragma unroll
          for (int i = 0; i < n; ++i)
#pragma unroll
            for (int j = 0; j < D; ++j) dlt[i][j] = fma_nc(-gain[i], mobs[j], incr[i][j]);
          iso_mean_add<T, NU, D>(m, mlo, dlt, mnew, mnewlo);
        }
        if constexpr (TAN) {
          T dmp[n][D];
          iso_predict_mean<T, NU, D>(dm, p, pinv, dmp);
          Dual<T, 1> ud[D], prd[P], fd[D];
#pragma unroll
          for (int j = 0; j < D; ++j) {
            ud[j] = Dual<T, 1>(mp[0][j]);
            ud[j].g[0] = dmp[0][j];
          }
#pragma unroll
          for (int k = 0; k < P; ++k) {
            prd[k] = Dual<T, 1>(pt[k]);
            prd[k].g[0] = (kdir == k) ? T(1) : T(0);
          }
          F::eval(ud, prd, fd);
#pragma unroll
          for (int i = 0; i < n; ++i)
#pragma unroll
            for (int j = 0; j < D; ++j) dmnew[i][j] = dmp[i][j] - gain[i] * (dmp[OUT][j] - fd[j].g[0]);
        }

        // ---- error estimate (error_residual_std, solvers.py:925-996) ----
        // error_residual_std: the std of the observed residual rescaled by
        // sigma_loc = rms / l is rms, error = rms * dt^1/1! (no division by a
        // possibly tiny l).  error_state_std (solvers.py:1037-1098): condition the
        // unit-scale extrapolation (chol |p| sqrt|h| Q1) on the same
        // linearisation; error = sigma_loc * (posterior std of u), dt^0/0! = 1
        T err_abs;
        if (GEN && a.state_error) {
          err_abs = sigma_loc * state_std0<T, NU, OUT>(a, p, h, damp, h0);
        } else {
          err_abs = rms_mobs * h;
        }
        iso_accept_and_control<T, NU, D>(a, err_abs, m, mnew, dt_use, pi_prev, accepted, nonfinite, pi_new, dt_new);
      };
      if constexpr (FP) {
        attempt(BoolTag<true>{});
      } else if (safe_next) {
        attempt(BoolTag<true>{});
        safe_next = false;
      } else {
        attempt(BoolTag<false>{});
        if (!ok) {  // rerun with the range-checked predict and update
          safe_next = true;
          --attempts;
          continue;
        }
      }
      // (tested after the controller so the attempt stays straight-line code;
      // a non-finite attempt is never accepted)
      if (nonfinite) {
        status = PDQ_INSTANCE_NONFINITE;
        break;
      }
      dt = dt_new;
      pi_prev = pi_new;
      if (accepted) {
        if constexpr (REC) {
          // element e of instance b at record[e * B + b]: the step size, then
          // every rec_ckpt steps the state the step starts from
          if (num_steps < a.rec_capacity) {
            T* rec = reinterpret_cast<T*>(a.record);
            rec[int64_t(num_steps) * a.B + b] = h;
            if (num_steps % a.rec_ckpt == 0) {
              int64_t e = int64_t(a.rec_capacity) + int64_t(num_steps / a.rec_ckpt) * (n * D + n * n);
#pragma unroll
              for (int i = 0; i < n; ++i)
#pragma unroll
                for (int j = 0; j < D; ++j) rec[(e++) * a.B + b] = m[i][j];
#pragma unroll
              for (int i = 0; i < n; ++i)
#pragma unroll
                for (int j = 0; j < n; ++j) rec[(e++) * a.B + b] = L[i][j];
            }
          } else {
            rec_full = true;
          }
        }
        if constexpr (INTERP) {
          ti = t;
#pragma unroll
          for (int i = 0; i < n; ++i) {
#pragma unroll
            for (int j = 0; j < D; ++j) mi[i][j] = m[i][j];
#pragma unroll
            for (int j = 0; j < n; ++j) Li[i][j] = L[i][j];
          }
#pragma unroll
          for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < D; ++j) milo[i][j] = mlo[i][j];
          if constexpr (FP) bwi = bw;
          if constexpr (TAN) {
#pragma unroll
            for (int i = 0; i < n; ++i)
#pragma unroll
              for (int j = 0; j < D; ++j) dmi[i][j] = dm[i][j];
          }
        }
        if constexpr (TAN) {
#pragma unroll
          for (int i = 0; i < n; ++i)
#pragma unroll
            for (int j = 0; j < D; ++j) dm[i][j] = dmnew[i][j];
        }
        if constexpr (FP) {
          IsoBackward<T, NU, D> merged;
          iso_cond_merge(bw, cnew, merged);
          bw = merged;
        }
        t = t_acc;
        bef = bef_acc;
        rem = rem_acc;
        ++num_steps;
#pragma unroll
        for (int i = 0; i < n; ++i) {
#pragma unroll
          for (int j = 0; j < D; ++j) m[i][j] = mnew[i][j];
#pragma unroll
          for (int j = 0; j < n; ++j) L[i][j] = Lnew[i][j];
        }
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
          for (int j = 0; j < D; ++j) mlo[i][j] = mnewlo[i][j];
        if (a.solver == PDQ_SOLVER_MLE) {
          // running scale via hypot recurrence == RMS of new terms (solvers.py:421-424)
          const T new_term = rms_mobs * dev_abs(ry_inv);
          mle_sumsq = wide_add_sq(mle_sumsq, new_term);
          ++num_data;
        }
        sigma_sf = (a.solver == PDQ_SOLVER_DYNAMIC) ? sigma_loc : T(1);
      }
      if (!accepted) continue;  // retry in the next iteration
    }
    // ---- checkpoint branch (solvers_via_adaptive_steps.py:242-247) ----
    const int s_out = a.terminal_only ? 0 : s;
    const bool record = (!a.terminal_only) || (s == S - 1);
    if (bef) {
      // interp_skip: keep stepping towards the checkpoint
    } else if (INTERP && before(t_next, t)) {
      if constexpr (INTERP) {
        // interp_beyond_t1: predict from interp_from to t_next
        // (solvers.py:205-269, estimators_and_losses.py:403-414)
        const T h = T(wide_diff(t_next, ti));
        T p[n], pinv[n], mp[n][D], mplo[2][D], Lp[n][n];
        precon<T, NU>(h, p, pinv);
        {
          T incr[n][D];
          iso_mean_increment<T, NU, D>(mi, p, pinv, incr);
          iso_mean_add<T, NU, D>(mi, milo, incr, mp, mplo);
        }
        if constexpr (FP) {
          // estimators_and_losses.py:549-591: the extrapolation to t_next
          // closes the checkpoint's conditional (bwi merged with it); the
          // step_from state keeps its marginal with the conditional from
          // t_next to t, merged into the identity
          IsoBackward<T, NU, D> c0, m0, c1, idc, m1;
          if constexpr (kNarrow) {
            iso_prior_revert<T, NU, D>(a.q1f, mi, Li, p, pinv, sigma_sf * dev_sqrt(dev_abs(h)), Lp, c0);
          } else {
            iso_prior_revert<T, NU, D>(a.q1, mi, Li, p, pinv, sigma_sf * dev_sqrt(dev_abs(h)), Lp, c0);
          }
          iso_cond_merge(bwi, c0, m0);
          iso_cond_store(ws + int64_t(s - 1) * iso_cond_floats<NU, D>(), m0);
          const T h1 = T(wide_diff(t, t_next));
          T p1[n], pinv1[n], mp1[n][D], Lp1[n][n];
          precon<T, NU>(h1, p1, pinv1);
          if constexpr (kNarrow) {
            iso_prior_revert<T, NU, D>(a.q1f, mp, Lp, p1, pinv1, sigma_sf * dev_sqrt(dev_abs(h1)), Lp1, c1);
          } else {
            iso_prior_revert<T, NU, D>(a.q1, mp, Lp, p1, pinv1, sigma_sf * dev_sqrt(dev_abs(h1)), Lp1, c1);
          }
          (void)mp1;
          iso_cond_identity(idc);
          iso_cond_merge(idc, c1, m1);
          bw = m1;
          iso_cond_identity(bwi);
        } else if constexpr (kNarrow) {
          iso_predict_chol<T, NU>(a.q1f, Li, p, pinv, sigma_sf * dev_sqrt(dev_abs(h)), Lp);
        } else {
          iso_predict_chol<T, NU>(a.q1, Li, p, pinv, sigma_sf * dev_sqrt(dev_abs(h)), Lp);
        }
        if (record && primary) write_record<T, NU, D>(a, b, s_out, S_out, mp, mplo, Lp, double(sigma_sf), wide_value(t_next), num_steps);
        if (FP && a.filter_mean) write_filter<T, NU, D>(a, b * S + s, mp, Lp);
        if constexpr (TAN) {
          T dmp[n][D];
          iso_predict_mean<T, NU, D>(dmi, p, pinv, dmp);
          if (record) write_tangent<T, NU, D, P>(a, b * S_out + s_out, kdir, dmp);
#pragma unroll
          for (int i = 0; i < n; ++i)
#pragma unroll
            for (int j = 0; j < D; ++j) dmi[i][j] = dmp[i][j];
        }
        ti = t_next;
#pragma unroll
        for (int i = 0; i < n; ++i) {
#pragma unroll
          for (int j = 0; j < D; ++j) mi[i][j] = mp[i][j];
#pragma unroll
          for (int j = 0; j < n; ++j) Li[i][j] = Lp[i][j];
        }
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
          for (int j = 0; j < D; ++j) milo[i][j] = mplo[i][j];
      }
    } else {
      // interp_at_t1: the state itself is the solution (estimators_and_losses.py:416-421)
      if (record && primary) write_record<T, NU, D>(a, b, s_out, S_out, m, mlo, L, double(sigma_sf), wide_value(t), num_steps);
      if constexpr (TAN) {
        if (record) write_tangent<T, NU, D, P>(a, b * S_out + s_out, kdir, dm);
        if constexpr (INTERP) {
#pragma unroll
          for (int i = 0; i < n; ++i)
#pragma unroll
            for (int j = 0; j < D; ++j) dmi[i][j] = dm[i][j];
        }
      }
      if (FP && a.filter_mean) write_filter<T, NU, D>(a, b * S + s, m, L);
      if constexpr (FP) {
        // estimators_and_losses.py:534-547: close the checkpoint's conditional, reset
        iso_cond_store(ws + int64_t(s - 1) * iso_cond_floats<NU, D>(), bw);
        iso_cond_identity(bw);
        if constexpr (INTERP) iso_cond_identity(bwi);
      }
      if constexpr (INTERP) {
        ti = t;
#pragma unroll
        for (int i = 0; i < n; ++i) {
#pragma unroll
          for (int j = 0; j < D; ++j) mi[i][j] = m[i][j];
#pragma unroll
          for (int j = 0; j < n; ++j) Li[i][j] = L[i][j];
        }
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
          for (int j = 0; j < D; ++j) milo[i][j] = mlo[i][j];
      }
    }
    if (!bef) {  // checkpoint s done
      ++s;
      if (s < S) {
        t_next = wide_from(save_at[s], T(0));
        bef = before(t, t_next);
        rem = wide_diff(t_next, t);
      }
    }
  }

  // ---- fixed-point backward pass: marginals at the checkpoints ----
  if constexpr (FP) {
    if (status == PDQ_INSTANCE_OK) {
      // the calibrated scale multiplies every Cholesky factor (finalize below);
      // the optional conditional outputs take it here
      double cal = 1.0;
      if (a.solver == PDQ_SOLVER_MLE) {
        cal = num_data > 0 ? sqrt(wide_value(mle_sumsq) / num_data) : 0.0;
        if (a.correct) cal /= sqrt(double(num_steps));
      }
      T rm[n][D], rL[n][n];
      iso_cond_marginalise(bw, m, L, rm, rL);
      for (int s = S - 1; s >= 1; --s) {
        if (!a.terminal_only || s == S - 1) write_normal_iso<T, NU, D>(a, b * S_out + (a.terminal_only ? 0 : s), rm, rL);
        IsoBackward<T, NU, D> c;
        iso_cond_load(ws + int64_t(s - 1) * iso_cond_floats<NU, D>(), c);
        if (a.cond_A) write_cond_iso<T, NU, D>(a, b * (S - 1) + (s - 1), c, cal);
        if (a.terminal_only) continue;
        T pm[n][D], pL[n][n];
        iso_cond_marginalise(c, rm, rL, pm, pL);
#pragma unroll
        for (int i = 0; i < n; ++i) {
#pragma unroll
          for (int j = 0; j < D; ++j) rm[i][j] = pm[i][j];
#pragma unroll
          for (int j = 0; j < n; ++j) rL[i][j] = pL[i][j];
        }
        if (s == 1) write_normal_iso<T, NU, D>(a, b * S_out, rm, rL);
      }
    }
  }

  if constexpr (TAN) {
    if (status != PDQ_INSTANCE_OK) {
      T nan_dm[n][D];
#pragma unroll
      for (int i = 0; i < n; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) nan_dm[i][j] = T(__longlong_as_double(0x7ff8000000000000ULL));
      for (int s = 0; s < S_out; ++s) write_tangent<T, NU, D, P>(a, b * S_out + s, kdir, nan_dm);
    }
    if (!primary) return;
  }
  // ---- finalize: calibrated output scale (solvers.py:439-480, 601-633, 735-767) ----
  if (status == PDQ_INSTANCE_OK) {
    if (a.solver == PDQ_SOLVER_MLE) {
      double scale = num_data > 0 ? sqrt(wide_value(mle_sumsq) / num_data) : 0.0;
      if (a.correct) {
        const int last = a.num_steps[b * S_out + (S_out - 1)];
        scale = scale / sqrt(double(last));
      }
      for (int s = 0; s < S_out; ++s) {
        const int64_t rec = b * S_out + s;
        double* uc = a.u_chol + rec * (n * n);
        for (int k = 0; k < n * n; ++k) uc[k] *= scale;
        a.output_scale[rec] = scale;
      }
      if (FP && a.filter_chol)
        for (int k = 0; k < S * n * n; ++k) a.filter_chol[b * S * n * n + k] *= scale;
    }
  } else {
    const double nan = __longlong_as_double(0x7ff8000000000000ULL);
    for (int s = 0; s < S_out; ++s) {
      const int64_t rec = b * S_out + s;
      for (int k = 0; k < n * D; ++k) a.u_mean[rec * (n * D) + k] = nan;
      for (int k = 0; k < n * n; ++k) a.u_chol[rec * (n * n) + k] = nan;
      a.output_scale[rec] = nan;
      a.t_out[rec] = nan;
      a.num_steps[rec] = num_steps;
    }
  }
  a.num_attempts[b] = attempts;
  a.status[b] = (REC && rec_full && status == PDQ_INSTANCE_OK) ? int(PDQ_INSTANCE_RECORD_FULL) : status;
}

}  // namespace pdq
