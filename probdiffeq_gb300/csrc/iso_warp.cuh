// Isotropic TS0 adaptive solver, warp-cooperative: LPI lanes per instance.
//
// Same algorithm and reference lines as iso_solver.cuh (one thread per
// instance); this variant shortens the per-attempt critical path, which is
// what bounds an ensemble solve (the slowest instance's attempts run back to
// back):
//   * lane c owns column c of the stacked predict matrix [X; U] (2n x n) and
//     runs the Householder step of its column; the reflector is broadcast to
//     the other lanes of the instance with sub-warp shuffles, and each lane
//     updates its own column (right-looking, column-parallel);
//   * the update's Givens chain runs on the (n+1)-column matrix with one
//     column per lane (rotation parameters broadcast from the owning lane);
//   * lane i produces row i of the new mean and Cholesky factor, which are
//     re-broadcast so every lane holds the (small) state and takes the same
//     accept / step decision from bitwise-identical data.
// Only the clip_dt (exact checkpoint landing) loop is implemented here; the
// dispatcher uses the one-thread kernel otherwise.
#pragma once

#include "iso_solver.cuh"

namespace pdq {

template <typename T>
PDQ_D T shfl(unsigned mask, T v, int src, int width) {
  return __shfl_sync(mask, v, src, width);
}

// Rotation (cs, sn) taking (x, y) to (r, 0); identity for x = y = 0; the
// squares are rescaled when they leave the normal range.
template <typename T>
PDQ_D void givens_params(T x, T y, T& cs, T& sn) {
  T r2 = x * x + y * y;
  if (norm2_out_of_range(r2)) {
    const T sc = dev_fmax_abs(x, y);
    if (!(sc > T(0))) return;
    x = x / sc;
    y = y / sc;
    r2 = x * x + y * y;
  }
  const T inv = dev_rsqrt(r2);
  cs = x * inv;
  sn = y * inv;
}

template <typename T, int NU, class F, int LPI, int MINB>
__global__ void __launch_bounds__(256, MINB) iso_warp_kernel(IsoArgs a) {
  constexpr int n = NU + 1;
  constexpr int D = F::D;
  constexpr int P = F::P;
  constexpr int OUT = 1;
  static_assert(n + 1 <= LPI, "one lane per column of the (n+1)-column update matrix");
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const int l = lane % LPI;                       // lane within the instance
  const unsigned mask = ((1u << LPI) - 1u) << (lane - l);
  const int64_t b = gtid / LPI;
  if (b >= a.B) return;  // whole groups exit together (B groups of LPI lanes)

  const int S = a.S;
  const int S_out = a.terminal_only ? 1 : S;
  const double* save_at = a.save_at + b * S;

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

  // replicated state
  T m[n][D], L[n][n];
#pragma unroll
  for (int i = 0; i < n; ++i) {
#pragma unroll
    for (int j = 0; j < D; ++j) m[i][j] = T(tc[i][j]);
#pragma unroll
    for (int j = 0; j < n; ++j) L[i][j] = T(0);
  }
  double t = save_at[0], dt = a.dt0[b], pi_prev = 1.0, mle_sumsq = 0.0;
  int num_data = 0, num_steps = 0, attempts = 0, status = PDQ_INSTANCE_OK;
  T sigma_sf = T(1);
  const T damp = T(a.damp);
  T q1_out2 = T(0);
#pragma unroll
  for (int j = 0; j < n; ++j) q1_out2 += T(a.q1[OUT][j]) * T(a.q1[OUT][j]);
  const T q1_out_norm = dev_sqrt(q1_out2);
  // this lane's column of Q1^T (bottom block of the predict matrix), unscaled,
  // and row l of the IWP transition A (zero for lanes l >= n)
  T q1col[n], arow[n];
#pragma unroll
  for (int r = 0; r < n; ++r) {
    q1col[r] = T(0);
    arow[r] = T(0);
  }
#pragma unroll
  for (int c = 0; c < n; ++c)
    if (c == l) {
#pragma unroll
      for (int r = 0; r < n; ++r) {
        q1col[r] = (r <= c) ? T(a.q1[c][r]) : T(0);
        arow[r] = T(iwp_a<NU>(c, r));
      }
    }

  if (!a.terminal_only && l == 0) write_record<T, NU, D>(a, b, 0, S_out, m, L, 1.0, t, 0);

  for (int s = 1; s < S && status == PDQ_INSTANCE_OK; ++s) {
    const double t_next = save_at[s];
    while (t + a.eps < t_next && status == PDQ_INSTANCE_OK) {
      const double dt_use = fmin(dt, t_next - t);
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
      T p[n], pinv[n];
      precon<T, NU>(h, p, pinv);
      // extrapolated mean (redundant in every lane) and the linearisation
      T mp[n][D];
      iso_predict_mean<T, NU, D>(m, p, pinv, mp);
      T f[D];
      F::eval(mp[0], pt, f);
      T mobs[D];
      T mobs2 = T(0);
#pragma unroll
      for (int j = 0; j < D; ++j) {
        mobs[j] = mp[OUT][j] - f[j];
        mobs2 += mobs[j] * mobs[j];
      }
      const T rms_mobs = dev_sqrt(mobs2 * T(1.0 / D));
      const T ell = observed_std(p[OUT], h, q1_out_norm, damp);
      const T sigma_loc = dev_div(rms_mobs, ell);
      const T s_pred = (a.solver == PDQ_SOLVER_DYNAMIC) ? sigma_loc : T(1);
      const T sq = s_pred * dev_sqrt(dev_abs(h));

      // ---- predict QR, column l: X[:, l] = row l of A diag(pinv) L; U[:, l] = sq Q1[l, :]^T ----
      T cx[n], cu[n];
#pragma unroll
      for (int r = 0; r < n; ++r) {
        T acc = T(0);
#pragma unroll
        for (int k = r; k < n; ++k) acc += arow[k] * pinv[k] * L[k][r];
        cx[r] = acc;
        cu[r] = sq * q1col[r];
      }
#pragma unroll
      for (int c = 0; c < n; ++c) {
        // reflector of column c, computed by lane c
        T tau = T(0), v0inv = T(0), beta = T(0);
        bool active = false;
        if (l == c) {
          T nrm2 = T(0);
#pragma unroll
          for (int r = c; r < n; ++r) nrm2 += cx[r] * cx[r];
#pragma unroll
          for (int i = 0; i <= c; ++i) nrm2 += cu[i] * cu[i];
          T nrm;
          if (norm2_out_of_range(nrm2)) {
            T sc = T(0);
#pragma unroll
            for (int r = c; r < n; ++r) sc = fmax(sc, dev_abs(cx[r]));
#pragma unroll
            for (int i = 0; i <= c; ++i) sc = fmax(sc, dev_abs(cu[i]));
            T acc = T(0);
            if (sc > T(0)) {
              const T inv = T(1) / sc;
#pragma unroll
              for (int r = c; r < n; ++r) acc += (cx[r] * inv) * (cx[r] * inv);
#pragma unroll
              for (int i = 0; i <= c; ++i) acc += (cu[i] * inv) * (cu[i] * inv);
            }
            nrm = sc * dev_sqrt(acc);
            nrm2 = nrm > T(0) ? T(1) : T(0);
          } else {
            nrm = dev_sqrt(nrm2);
          }
          if (nrm2 > T(0)) {
            const T alpha = cx[c];
            beta = alpha >= T(0) ? -nrm : nrm;
            v0inv = dev_rcp(alpha - beta);
            tau = (beta - alpha) / beta;
            active = true;
          }
        }
        const T tau_b = shfl(mask, tau, c, LPI);
        T vx[n], vu[n];
#pragma unroll
        for (int r = c + 1; r < n; ++r) vx[r] = shfl(mask, cx[r] * v0inv, c, LPI);
#pragma unroll
        for (int i = 0; i <= c; ++i) vu[i] = shfl(mask, cu[i] * v0inv, c, LPI);
        if (l > c && l < n && tau_b != T(0)) {
          T w = cx[c];
#pragma unroll
          for (int r = c + 1; r < n; ++r) w += vx[r] * cx[r];
#pragma unroll
          for (int i = 0; i <= c; ++i) w += vu[i] * cu[i];
          w *= tau_b;
          cx[c] -= w;
#pragma unroll
          for (int r = c + 1; r < n; ++r) cx[r] -= w * vx[r];
#pragma unroll
          for (int i = 0; i <= c; ++i) cu[i] -= w * vu[i];
        }
        if (l == c && active) {
          cx[c] = beta;
#pragma unroll
          for (int r = c + 1; r < n; ++r) cx[r] = T(0);
        }
      }
      // lane l < n now holds column l of R: R[j][l] = cx[j], j <= l.
      // Lp row l = |p_l| R[:, l]^T; update matrix: lane k < n holds column
      // k+1 = Lp row k (rows 1..n), lane n holds column 0.
      T pl = T(0);
#pragma unroll
      for (int c = 0; c < n; ++c)
        if (c == l) pl = dev_abs(p[c]);
      T mc[n + 1];
      mc[0] = T(0);
#pragma unroll
      for (int r = 1; r <= n; ++r) mc[r] = (l < n && r - 1 <= l) ? pl * cx[r - 1] : T(0);
      // column 0: [damp, Lp[OUT][0..]] from lane OUT
#pragma unroll
      for (int r = 1; r <= n; ++r) {
        const T v = shfl(mask, mc[r], OUT, LPI);
        if (l == n) mc[r] = (r - 1 <= OUT) ? v : T(0);
      }
      if (l == n) mc[0] = damp;
      // Givens chain: column 0 (lane n) bottom-up, then columns 1..OUT
#pragma unroll
      for (int r = OUT + 1; r >= 1; --r) {
        T cs = T(1), sn = T(0);
        if (l == n) {
          givens_params(mc[r - 1], mc[r], cs, sn);
        }
        cs = shfl(mask, cs, n, LPI);
        sn = shfl(mask, sn, n, LPI);
        const T ma = mc[r - 1], mb = mc[r];
        mc[r - 1] = cs * ma + sn * mb;
        mc[r] = cs * mb - sn * ma;
        if (l == n) mc[r] = T(0);
      }
#pragma unroll
      for (int c = 1; c <= OUT; ++c) {
        T cs = T(1), sn = T(0);
        if (l == c - 1) {
          givens_params(mc[c], mc[c + 1], cs, sn);
        }
        cs = shfl(mask, cs, c - 1, LPI);
        sn = shfl(mask, sn, c - 1, LPI);
        const T ma = mc[c], mb = mc[c + 1];
        mc[c] = cs * ma + sn * mb;
        mc[c + 1] = cs * mb - sn * ma;
        if (l == c - 1) mc[c + 1] = T(0);
      }
      const T R_Y = shfl(mask, mc[0], n, LPI);
      const T ry_inv = dev_rcp(R_Y);
      // lane i < n: gain_i = M[0][i+1] / R_Y; new mean row i; new Cholesky row i = M[1..i+1][i+1]
      const T gain = mc[0] * ry_inv;
      T mrow[D];
#pragma unroll
      for (int j = 0; j < D; ++j) {
        T v = T(0);
#pragma unroll
        for (int c = 0; c < n; ++c)
          if (c == l) v = mp[c][j] - gain * mobs[j];
        mrow[j] = v;
      }
      // the new u row (row 0) decides acceptance; the rest is broadcast only on accept
      T mnew0[D];
#pragma unroll
      for (int j = 0; j < D; ++j) mnew0[j] = shfl(mask, mrow[j], 0, LPI);
      // ---- error estimate, control, acceptance (identical in every lane) ----
      const T err_abs = rms_mobs * h;  // |sigma_loc| l = rms
      double sumsq = 0.0;
#pragma unroll
      for (int j = 0; j < D; ++j) {
        const T ref = fmax(dev_abs(m[0][j]), dev_abs(mnew0[j]));
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
      if (norm2 <= 1.0) {
        t = t + dt_use;
        ++num_steps;
        // lane i holds row i of the new mean and of the new Cholesky factor
        // (L+[i][j] = M[j+1][i+1], its column's rows 1..i+1)
#pragma unroll
        for (int i = 0; i < n; ++i) {
#pragma unroll
          for (int j = 0; j < D; ++j) m[i][j] = shfl(mask, mrow[j], i, LPI);
#pragma unroll
          for (int j = 0; j <= i; ++j) L[i][j] = shfl(mask, mc[j + 1], i, LPI);
        }
        if (a.solver == PDQ_SOLVER_MLE) {
          const T new_term = rms_mobs * dev_abs(ry_inv);
          mle_sumsq += double(new_term) * double(new_term);
          ++num_data;
        }
        sigma_sf = (a.solver == PDQ_SOLVER_DYNAMIC) ? sigma_loc : T(1);
      }
    }
    if (status != PDQ_INSTANCE_OK) break;
    // clip_dt: checkpoints are exact landings (interp_at_t1)
    if ((!a.terminal_only || s == S - 1) && l == 0)
      write_record<T, NU, D>(a, b, a.terminal_only ? 0 : s, S_out, m, L, double(sigma_sf), t, num_steps);
  }

  if (l != 0) return;
  if (status == PDQ_INSTANCE_OK) {
    if (a.solver == PDQ_SOLVER_MLE) {
      double scale = num_data > 0 ? sqrt(mle_sumsq / num_data) : 0.0;
      if (a.correct) scale /= sqrt(double(num_steps));
      for (int s = 0; s < S_out; ++s) {
        const int64_t rec = b * S_out + s;
        double* uc = a.u_chol + rec * (n * n);
        for (int k = 0; k < n * n; ++k) uc[k] *= scale;
        a.output_scale[rec] = scale;
      }
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
  a.status[b] = status;
}

}  // namespace pdq
