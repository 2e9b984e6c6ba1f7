// Dense-factorisation adaptive solver with the structure of the IWP prior and
// of the ODE linearisation exploited: L lanes per IVP instance, the
// instance's state in shared memory as a structure of arrays.
//
// Same algorithm, branches and references as dense_adaptive_kernel
// (dense_solver.cuh): IWP transition / revert / merge / marginalise
// (ssm_impl_dense.py:15-84, 347-363), TS1 / TS0 (ssm_impl_dense.py:237-334),
// filter / fixed-point smoother (estimators_and_losses.py:347-591), solver /
// solver_mle / solver_dynamic, error_residual_std, I / PI control and the
// RejectionLoop with checkpoints (solvers_via_adaptive_steps.py:196-375).
// What differs is how each QR is formed and who does the work:
//
// * predict / revert: the input [[s sqrt|h| Q^T, 0], [(A cl)^T, cl^T]]
//   (Q = kron(Q1, I_d) lower triangular, cl = p^-1 L) has an upper-triangular
//   top-left block, so reflector c touches row c and the N bottom rows only;
//   the bottom-right block is then reduced by a dense N x N QR.
// * merge and marginalise: [full N x N; upper-triangular N x N] -- reflector c
//   acts on the contiguous rows c .. c + N.
// * update: the linearisation J = [-J_f, I, 0, ...] (TS1) or [0, I, 0, ...]
//   (TS0) reads only coefficients 0 and 1, so of the (d + N)^2 QR only the d
//   observation rows and the first 2d rows of L^T take part (3d x (d + N),
//   registers); the other rows of the factor carry over unchanged.  The
//   observed covariance of the error estimate likewise reduces to a 3d x d QR.
// * the L lanes of an instance deal the columns of every QR cyclically (a
//   reflector is formed redundantly by all L lanes from shared memory, then
//   each lane applies it to its own columns; no shuffles), and the rows of
//   the matrix products; two __syncwarp per reflector order the shared-memory
//   traffic.  Scalars (time, step, calibration, control, status) are computed
//   identically in all lanes, so the control flow of a group is uniform.
// * element e of instance slot s lives at smem[e * IPW + s] (IPW = 32 / L
//   instances per warp): the lanes of a warp hit distinct banks.
// * the three running normals (step_from, interp_from, proposal) and the
//   three running conditionals (running, interp, merged) rotate through slots
//   by index on acceptance instead of being copied.
//
// * the mean's rows 0 and 1 (the coefficients the residual u' - f(u) reads)
//   carry float-pair low parts in the float32 kernel, the residual is formed
//   with the field in float-pair arithmetic and the update m' = m + (incr -
//   G r) adds wide, as in the isotropic kernel: float32 then matches
//   float64's error against the exact solution.
//
// R factors may differ from a LAPACK QR in the signs of their rows; every
// quantity formed from them (L L^T, R11^-1 R12, R22^T R22) is invariant.
#pragma once

#include "dense_solver.cuh"

// The kernel's dynamic shared memory (a host run of the kernel body supplies a buffer instead).
#ifndef PDQ_DENSE_STRUCT_SMEM
#define PDQ_DENSE_STRUCT_SMEM extern __shared__ __align__(16) unsigned char dense_struct_smem[]
#endif

namespace pdq {

template <int L>
struct LaneGroup {
  unsigned mask;
  int lane;  // 0 .. L - 1
  PDQ_D void sync() const {
    if constexpr (L > 1) __syncwarp(mask);
  }
  // the first index >= j0 dealt to this lane (index j goes to lane j mod L)
  PDQ_D int first(int j0) const { return j0 + ((lane - j0) & (L - 1)); }
  PDQ_D bool owns(int j) const { return (j & (L - 1)) == lane; }
};

template <typename T, int IPW>
struct Soa {
  T* p;  // element 0 of this instance
  PDQ_D T& operator[](int e) const { return p[e * IPW]; }
};

// Matrices are row-major with padded row strides (N + 1, 2N + 1): the lanes
// of a group that own different rows of a matrix then hit different banks
// (with a stride that is a multiple of 32 / IPW they would share one).
template <int NU, int D>
struct DenseLayout {
  static constexpr int n = NU + 1, N = n * D, NN = N * N;
  static constexpr int LD = N + 1;                // row stride of the N x N matrices
  static constexpr int WS = 2 * N + 1;            // row stride of the predict workspace
  static constexpr int WMS = N + 1;               // row stride of the merge workspace
  static constexpr int kNormal = N + N * LD + 2 * D;  // m, L (lower), low parts of m's rows 0 and 1
  static constexpr int kCond = 2 * N * LD + 3 * N;  // A, xi, X (lower), tl, to
  static constexpr int kNormals = 4;            // step_from, interp_from, proposal, prediction (rotating)
  static constexpr int kConds = 4;              // running, interp, merged, scratch (rotating)
  static constexpr int m = 0, L = N, mlo = N + N * LD;
  static constexpr int A = 0, xi = N * LD, X = N * LD + N, tl = 2 * N * LD + N, to = 2 * N * LD + 2 * N;
  static constexpr int normal0 = 0;
  static constexpr int cond0 = kNormals * kNormal;
  static constexpr int cnA = cond0 + kConds * kCond;  // this step's conditional: A (N x N), xi (N)
  static constexpr int cnXi = cnA + N * LD;
  static constexpr int W = cnXi + N;        // predict workspace, 2N x 2N
  static constexpr int WM = W + 2 * N * WS;  // merge / marginalise workspace, 2N x N
  // this step's constants for the lanes' column loops: p (n), p^-1 (n), A1 (n x n), s sqrt|h| Q1 (n x n)
  static constexpr int PT = WM + 2 * N * WMS;
  static constexpr int size = PT + 2 * n + 2 * n * n;
  PDQ_HD static constexpr int normal(int k) { return normal0 + k * kNormal; }
  PDQ_HD static constexpr int cond(int k) { return cond0 + k * kCond; }
};

// ||x|| with a rescaled sum of squares when the plain one leaves
// [1e-30, 1e36] (float) / [1e-290, 1e300] (double), as householder_r.
template <typename T, int K>
PDQ_D void dstruct_norm(const T (&x)[K], T& nrm, T& nrm2) {
  T s0 = T(0), s1 = T(0);
#pragma unroll
  for (int t = 0; t < K; t += 2) s0 += x[t] * x[t];
#pragma unroll
  for (int t = 1; t < K; t += 2) s1 += x[t] * x[t];
  nrm2 = s0 + s1;
  if (norm2_out_of_range(nrm2)) {
    T sc = T(0);
#pragma unroll
    for (int t = 0; t < K; ++t) sc = fmax(sc, dev_abs(x[t]));
    T acc = T(0);
    if (sc > T(0)) {
      const T inv = T(1) / sc;
#pragma unroll
      for (int t = 0; t < K; ++t) acc += (x[t] * inv) * (x[t] * inv);
    }
    nrm = sc * dev_sqrt(acc);
    nrm2 = nrm > T(0) ? T(1) : T(0);
  } else {
    nrm = dev_sqrt(nrm2);
  }
}

// Householder reflector of x (x[0] the diagonal), the convention of
// householder_r: beta = -sign(x0) ||x||, v = [1, x[1:] / (x0 - beta)],
// tau = (beta - x0) / beta.  Returns false for a zero column.
template <typename T, int K>
PDQ_D bool dstruct_reflector(T (&x)[K], T& beta, T& tau) {
  T nrm, nrm2;
  dstruct_norm(x, nrm, nrm2);
  if (!(nrm2 > T(0))) return false;
  const T alpha = x[0];
  beta = alpha >= T(0) ? -nrm : nrm;
  const T vinv = dev_rcp(alpha - beta);
  tau = dev_div(beta - alpha, beta);
#pragma unroll
  for (int t = 1; t < K; ++t) x[t] *= vinv;
  return true;
}

// QR of the 2N x N workspace WM = [full N x N; upper-triangular N x N]
// (rows c .. c + N take part in reflector c); R in rows 0 .. N - 1.
template <typename T, int N, int L, int IPW, int LDM = N + 1>
PDQ_D void dstruct_qr_stacked(Soa<T, IPW> S, const LaneGroup<L>& g, int WM) {
#pragma unroll 1
  for (int c = 0; c < N; ++c) {
    T x[N + 1];
#pragma unroll
    for (int t = 0; t <= N; ++t) x[t] = S[WM + (c + t) * LDM + c];
    g.sync();  // every lane has read column c
    T beta, tau;
    if (dstruct_reflector(x, beta, tau)) {
#pragma unroll(L >= 8 ? 1 : 2)
      for (int j = g.first(c + 1); j < N; j += L) {
        T w0 = S[WM + c * LDM + j], w1 = T(0);
#pragma unroll
        for (int t = 1; t <= N; t += 2) w0 += x[t] * S[WM + (c + t) * LDM + j];
#pragma unroll
        for (int t = 2; t <= N; t += 2) w1 += x[t] * S[WM + (c + t) * LDM + j];
        const T w = tau * (w0 + w1);
        S[WM + c * LDM + j] -= w;
#pragma unroll
        for (int t = 1; t <= N; ++t) S[WM + (c + t) * LDM + j] -= w * x[t];
      }
      if (g.owns(c)) S[WM + c * LDM + c] = beta;
    }
    g.sync();
  }
}

// transition(h, scale).revert(rv) (REVERT: the predicted marginal into `pred`
// and this step's backward conditional: A, xi into cnA / cnXi, its noise
// factor left in W's bottom-right block as R22 (X = R22^T), to = 1 / p^-1,
// tl = 1 / p) or .marginalise(rv) (the predicted marginal only)
// (ssm_impl_dense.py:24-77 with :347-363).
template <typename T, int NU, int D, bool REVERT, int L, int IPW>
PDQ_D void dstruct_predict(Soa<T, IPW> S, const LaneGroup<L>& g, const double (&q1)[kMaxN][kMaxN], int from, T h,
                           T scale, int pred) {
  using Lay = DenseLayout<NU, D>;
  constexpr int n = NU + 1, N = Lay::N, C = REVERT ? 2 * N : N, WS = Lay::WS, LD = Lay::LD;
  constexpr int W = Lay::W;
  T pc[n], pic[n];
  precon<T, NU>(h, pc, pic);
  const T sq = scale * dev_sqrt(dev_abs(h));
  // mean (all lanes): mean_l = p^-1 m, mobs = A mean_l
  T mean_l[N], mobs[N];
#pragma unroll
  for (int i = 0; i < N; ++i) mean_l[i] = pic[i / D] * S[from + Lay::m + i];
#pragma unroll
  for (int i = 0; i < N; ++i) {
    T acc = T(0);
#pragma unroll
    for (int kk = i / D; kk < n; ++kk) acc += T(iwp_a<NU>(i / D, kk)) * mean_l[kk * D + i % D];
    mobs[i] = acc;
  }
  // the preconditioner and A1 for the lanes' column loops (runtime indices read shared memory)
  if (g.lane == 0) {
#pragma unroll
    for (int i = 0; i < n; ++i) {
      S[Lay::PT + i] = pc[i];
      S[Lay::PT + n + i] = pic[i];
#pragma unroll
      for (int k = 0; k < n; ++k) {
        S[Lay::PT + 2 * n + i * n + k] = T(iwp_a<NU>(i, k));
        S[Lay::PT + 2 * n + n * n + i * n + k] = sq * T(q1[i][k]);
      }
    }
  }
  g.sync();
  // fill, column-parallel
#pragma unroll 1
  for (int c = g.lane; c < C; c += L) {
    if (c < N) {
      const int ci = c / D, cd = c - ci * D;
#pragma unroll
      for (int r = 0; r < N; ++r)
        S[W + r * WS + c] = (r % D == cd && r / D <= ci) ? S[Lay::PT + 2 * n + n * n + ci * n + r / D] : T(0);
      // (A cl)[c][r] = sum_k A1[ci][k / D] p^-1_k L[k][r] over k = kk d + cd, kk >= ci, k >= r
      T coef[n];
#pragma unroll
      for (int kk = 0; kk < n; ++kk) coef[kk] = S[Lay::PT + 2 * n + ci * n + kk] * pic[kk];
#pragma unroll
      for (int r = 0; r < N; ++r) {
        T acc = T(0);
#pragma unroll
        for (int kk = 0; kk < n; ++kk) {
          const int k = kk * D + cd;
          if (kk >= ci && k >= r) acc += coef[kk] * S[from + Lay::L + k * LD + r];
        }
        S[W + (N + r) * WS + c] = acc;
      }
    } else {
      const int cc = c - N;
      const T pk = S[Lay::PT + n + cc / D];
#pragma unroll
      for (int r = 0; r < N; ++r) S[W + r * WS + c] = T(0);
#pragma unroll
      for (int r = 0; r < N; ++r) S[W + (N + r) * WS + c] = r <= cc ? pk * S[from + Lay::L + cc * LD + r] : T(0);
    }
  }
  g.sync();
  // reflectors 0 .. N - 1: row c and the N bottom rows
#pragma unroll 1
  for (int c = 0; c < N; ++c) {
    T x[N + 1];
    x[0] = S[W + c * WS + c];
#pragma unroll
    for (int r = 0; r < N; ++r) x[1 + r] = S[W + (N + r) * WS + c];
    g.sync();
    T beta, tau;
    if (dstruct_reflector(x, beta, tau)) {
#pragma unroll(L >= 8 ? 1 : 2)
      for (int j = g.first(c + 1); j < C; j += L) {
        T w0 = S[W + c * WS + j], w1 = T(0);
#pragma unroll
        for (int r = 0; r < N; r += 2) w0 += x[1 + r] * S[W + (N + r) * WS + j];
#pragma unroll
        for (int r = 1; r < N; r += 2) w1 += x[1 + r] * S[W + (N + r) * WS + j];
        const T w = tau * (w0 + w1);
        S[W + c * WS + j] -= w;
#pragma unroll
        for (int r = 0; r < N; ++r) S[W + (N + r) * WS + j] -= w * x[1 + r];
      }
      if (g.owns(c)) S[W + c * WS + c] = beta;
    }
    g.sync();
  }
  if constexpr (REVERT) {
    // the bottom-right N x N block, dense: column N + cc over rows N + cc .. 2N - 1
#pragma unroll 1
    for (int cc = 0; cc < N - 1; ++cc) {
      const int c = N + cc;
      T x[N];
#pragma unroll
      for (int t = 0; t < N; ++t) x[t] = (t < N - cc) ? S[W + (c + t) * WS + c] : T(0);
      g.sync();
      T beta, tau;
      if (dstruct_reflector(x, beta, tau)) {
#pragma unroll(L >= 8 ? 1 : 2)
        for (int j = g.first(c + 1); j < 2 * N; j += L) {
          T w0 = S[W + c * WS + j], w1 = T(0);
#pragma unroll
          for (int t = 1; t < N; t += 2)
            if (t < N - cc) w0 += x[t] * S[W + (c + t) * WS + j];
#pragma unroll
          for (int t = 2; t < N; t += 2)
            if (t < N - cc) w1 += x[t] * S[W + (c + t) * WS + j];
          const T w = tau * (w0 + w1);
          S[W + c * WS + j] -= w;
#pragma unroll
          for (int t = 1; t < N; ++t)
            if (t < N - cc) S[W + (c + t) * WS + j] -= w * x[t];
        }
        if (g.owns(c)) S[W + c * WS + c] = beta;
      }
      g.sync();
    }
  }
  // the predicted marginal: m = p mobs (no low parts), L = |p| R11^T
#pragma unroll
  for (int i = 0; i < N; ++i)
    if (g.owns(i)) {
      S[pred + Lay::m + i] = pc[i / D] * mobs[i];
      if (i < 2 * D) S[pred + Lay::mlo + i] = T(0);
    }
#pragma unroll 1
  for (int i = g.lane; i < N; i += L) {
    const T pa = dev_abs(S[Lay::PT + i / D]);
#pragma unroll
    for (int j = 0; j < N; ++j) S[pred + Lay::L + i * LD + j] = (j <= i) ? pa * S[W + j * WS + i] : T(0);
  }
  if constexpr (REVERT) {
    // G^T = R11^-1 R12 column by column; cond.A[jj][i] = G^T[i][jj], cond.xi = mean_l - G mobs
#pragma unroll 1
    for (int jj = g.lane; jj < N; jj += L) {
      T gc[N];
#pragma unroll
      for (int i = N - 1; i >= 0; --i) {
        T acc = S[W + i * WS + N + jj];
#pragma unroll
        for (int k = i + 1; k < N; ++k) acc -= S[W + i * WS + k] * gc[k];
        gc[i] = dev_div(acc, S[W + i * WS + i]);
      }
      T xi = S[Lay::PT + n + jj / D] * S[from + Lay::m + jj];  // mean_l[jj]
#pragma unroll
      for (int k = 0; k < N; ++k) {
        S[Lay::cnA + jj * LD + k] = gc[k];
        xi -= gc[k] * mobs[k];
      }
      S[Lay::cnXi + jj] = xi;
    }
  }
  g.sync();
}

// outer.merge(inner) (ssm_impl_dense.py:35-49) with the inner conditional
// the one dstruct_predict<REVERT> left (A, xi in cnA / cnXi, X = R22^T in W,
// tl = 1 / p, to = 1 / p^-1 for step h); result into the conditional `out`.
template <typename T, int NU, int D, int L, int IPW>
PDQ_D void dstruct_merge(Soa<T, IPW> S, const LaneGroup<L>& g, int o, T h, int out) {
  using Lay = DenseLayout<NU, D>;
  constexpr int n = NU + 1, N = Lay::N, WS = Lay::WS, LD = Lay::LD, WMS = Lay::WMS;
  constexpr int W = Lay::W, WM = Lay::WM;
  T pc[n], pic[n];
  precon<T, NU>(h, pc, pic);
  T Tv[N];
#pragma unroll
  for (int k = 0; k < N; ++k) Tv[k] = S[o + Lay::tl + k] * dev_rcp(pic[k / D]);
  // out.A = o.A T in.A and R1 = (o.A |T| in.X)^T by columns j of in.A / in.X
#pragma unroll 1
  for (int j = g.lane; j < N; j += L) {
    {
      T u[N], u2[N];
#pragma unroll
      for (int k = 0; k < N; ++k) {
        u[k] = Tv[k] * S[Lay::cnA + k * LD + j];
        u2[k] = k >= j ? dev_abs(Tv[k]) * S[W + (N + j) * WS + N + k] : T(0);
      }
#pragma unroll
      for (int i = 0; i < N; ++i) {
        T ga = T(0), r1 = T(0);
#pragma unroll
        for (int k = 0; k < N; ++k) {
          const T oa = S[o + Lay::A + i * LD + k];
          ga += oa * u[k];
          if (k >= j) r1 += oa * u2[k];
        }
        S[out + Lay::A + i * LD + j] = ga;
        S[WM + j * WMS + i] = r1;
      }
      // R2 row j = (o.X^T) row j
#pragma unroll
      for (int i = 0; i < N; ++i) S[WM + (N + j) * WMS + i] = i >= j ? S[o + Lay::X + i * LD + j] : T(0);
      // out.xi[j] = o.xi[j] + (o.A T in.xi)[j]
      T x = S[o + Lay::xi + j];
#pragma unroll
      for (int k = 0; k < N; ++k) x += S[o + Lay::A + j * LD + k] * Tv[k] * S[Lay::cnXi + k];
      S[out + Lay::xi + j] = x;
      S[out + Lay::tl + j] = dev_rcp(S[Lay::PT + j / D]);
      S[out + Lay::to + j] = S[o + Lay::to + j];
    }
  }
  g.sync();
  dstruct_qr_stacked<T, N, L, IPW, WMS>(S, g, WM);
#pragma unroll 1
  for (int i = g.lane; i < N; i += L) {
#pragma unroll
    for (int j = 0; j < N; ++j) S[out + Lay::X + i * LD + j] = (j <= i) ? S[WM + j * WMS + i] : T(0);
  }
  g.sync();
}

// cond.marginalise(rv) (ssm_impl_dense.py:24-33): the conditional `c`
// applied to the normal `rv`, result into the normal `out`.
template <typename T, int NU, int D, int L, int IPW>
PDQ_D void dstruct_cond_marginalise(Soa<T, IPW> S, const LaneGroup<L>& g, int c, int rv, int out) {
  using Lay = DenseLayout<NU, D>;
  constexpr int N = Lay::N, WM = Lay::WM, LD = Lay::LD, WMS = Lay::WMS;
  // rows r of (A (tl L))^T and of X^T, by rows
#pragma unroll 1
  for (int r = g.lane; r < N; r += L) {
    {
      T u[N];
#pragma unroll
      for (int k = 0; k < N; ++k) u[k] = k >= r ? S[c + Lay::tl + k] * S[rv + Lay::L + k * LD + r] : T(0);
#pragma unroll
      for (int col = 0; col < N; ++col) {
        T acc = T(0);
#pragma unroll
        for (int k = r; k < N; ++k) acc += S[c + Lay::A + col * LD + k] * u[k];
        S[WM + r * WMS + col] = acc;
        S[WM + (N + r) * WMS + col] = col >= r ? S[c + Lay::X + col * LD + r] : T(0);
      }
    }
  }
  // the mean (all lanes read rv before anyone writes out; rv != out)
  T mo[N];
#pragma unroll
  for (int i = 0; i < N; ++i) {
    T acc = T(0);
#pragma unroll
    for (int k = 0; k < N; ++k) acc += S[c + Lay::A + i * LD + k] * S[c + Lay::tl + k] * S[rv + Lay::m + k];
    mo[i] = S[c + Lay::to + i] * (acc + S[c + Lay::xi + i]);
  }
  g.sync();
  dstruct_qr_stacked<T, N, L, IPW, WMS>(S, g, WM);
#pragma unroll
  for (int i = 0; i < N; ++i)
    if (g.owns(i)) S[out + Lay::m + i] = mo[i];
#pragma unroll 1
  for (int i = g.lane; i < N; i += L) {
    const T to = dev_abs(S[c + Lay::to + i]);
#pragma unroll
    for (int j = 0; j < N; ++j) S[out + Lay::L + i * LD + j] = (j <= i) ? to * S[WM + j * WMS + i] : T(0);
  }
  g.sync();
}

template <typename T, int NU, int D, int L, int IPW>
PDQ_D void dstruct_cond_identity(Soa<T, IPW> S, const LaneGroup<L>& g, int c) {
  using Lay = DenseLayout<NU, D>;
  constexpr int N = Lay::N, LD = Lay::LD;
#pragma unroll 1
  for (int i = g.lane; i < N; i += L) {
#pragma unroll
    for (int j = 0; j < N; ++j) {
      S[c + Lay::A + i * LD + j] = (i == j) ? T(1) : T(0);
      S[c + Lay::X + i * LD + j] = T(0);
    }
    S[c + Lay::xi + i] = T(0);
    S[c + Lay::tl + i] = T(1);
    S[c + Lay::to + i] = T(1);
  }
  g.sync();
}

template <typename T, int K, int L, int IPW>
PDQ_D void dstruct_copy(Soa<T, IPW> S, const LaneGroup<L>& g, int dst, int src) {
#pragma unroll 4
  for (int e = g.lane; e < K; e += L) S[dst + e] = S[src + e];
  g.sync();
}

// store_cond / load_cond (dense_solver.cuh: A, xi, the packed lower X, tl,
// to) from / to shared memory: one lane writes the workspace record (rare:
// once per checkpoint).
template <typename T, int NU, int D, int L, int IPW>
PDQ_D void dstruct_store_cond(Soa<T, IPW> S, const LaneGroup<L>& g, int c, T* base) {
  using Lay = DenseLayout<NU, D>;
  constexpr int N = Lay::N, LD = Lay::LD;
  if (g.lane == 0) {
    int o = 0;
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j) base[o++] = S[c + Lay::A + i * LD + j];
    for (int i = 0; i < N; ++i) base[o++] = S[c + Lay::xi + i];
    for (int i = 0; i < N; ++i)
      for (int j = 0; j <= i; ++j) base[o++] = S[c + Lay::X + i * LD + j];
    for (int i = 0; i < N; ++i) base[o++] = S[c + Lay::tl + i];
    for (int i = 0; i < N; ++i) base[o++] = S[c + Lay::to + i];
  }
  g.sync();
}

template <typename T, int NU, int D, int L, int IPW>
PDQ_D void dstruct_load_cond(Soa<T, IPW> S, const LaneGroup<L>& g, int c, const T* base) {
  using Lay = DenseLayout<NU, D>;
  constexpr int N = Lay::N, LD = Lay::LD;
  if (g.lane == 0) {
    int o = 0;
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j) S[c + Lay::A + i * LD + j] = base[o++];
    for (int i = 0; i < N; ++i) S[c + Lay::xi + i] = base[o++];
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j) S[c + Lay::X + i * LD + j] = (j <= i) ? base[o++] : T(0);
    for (int i = 0; i < N; ++i) S[c + Lay::tl + i] = base[o++];
    for (int i = 0; i < N; ++i) S[c + Lay::to + i] = base[o++];
  }
  g.sync();
}

// A normal (mean, Cholesky factor) from shared memory to the float64 outputs (row stride N).
template <typename T, int NU, int D, int L, int IPW>
PDQ_D void dstruct_write_normal(Soa<T, IPW> S, const LaneGroup<L>& g, int x, double* mean, double* chol) {
  using Lay = DenseLayout<NU, D>;
  constexpr int N = Lay::N, LD = Lay::LD;
  for (int e = g.lane; e < N; e += L)
    mean[e] = double(S[x + Lay::m + e]) + (e < 2 * D ? double(S[x + Lay::mlo + e]) : 0.0);
  for (int e = g.lane; e < N * N; e += L) chol[e] = double(S[x + Lay::L + (e / N) * LD + e % N]);
}

template <typename T, int NU, class F, bool TS1, bool FP, int L>
__global__ void __launch_bounds__(32) dense_struct_kernel(DenseArgs a) {
  constexpr int D = F::D, P = F::P, n = NU + 1;
  using Lay = DenseLayout<NU, D>;
  constexpr int N = Lay::N, IPW = 32 / L;
  PDQ_DENSE_STRUCT_SMEM;
  const int slot = int(threadIdx.x) / L;
  const LaneGroup<L> g{((1u << L) - 1u) << (slot * L), int(threadIdx.x) % L};
  // a slot past the batch shadows the last instance (reads only) so that
  // every lane of the warp takes part in the warp-uniform attempt loop
  const bool valid = int64_t(blockIdx.x) * IPW + slot < a.B;
  const int64_t b = valid ? int64_t(blockIdx.x) * IPW + slot : a.B - 1;
  const Soa<T, IPW> S{reinterpret_cast<T*>(dense_struct_smem) + slot};
  const int Sn = a.S;
  const int S_out = a.terminal_only ? 1 : Sn;
  const double* save_at = a.save_at + b * Sn;
  T* ws = FP ? reinterpret_cast<T*>(a.workspace) + b * int64_t(Sn - 1) * cond_floats<N>() : nullptr;

  double pd[P];
  T pt[P];
  Wide<T> pw[P];  // the parameters in the wide type (the residual's field evaluation)
#pragma unroll
  for (int k = 0; k < P; ++k) {
    pd[k] = a.params[b * P + k];
    pt[k] = T(pd[k]);
    pw[k] = wide_from(pd[k], T(0));
  }
  // slots (offsets into the instance's shared-memory record)
  int ix = Lay::normal(0), ii = Lay::normal(1), inew = Lay::normal(2), ipred = Lay::normal(3);
  int ibw = Lay::cond(0), ibwi = Lay::cond(1), img = Lay::cond(2), itmp = Lay::cond(3);
  {
    double y0[D];
#pragma unroll
    for (int j = 0; j < D; ++j) y0[j] = a.y0[b * D + j];
    double tc[n][D];
    taylor_init<F, NU>(y0, pd, tc);
    if (g.lane == 0) {
#pragma unroll
      for (int i = 0; i < n; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) S[ix + Lay::m + i * D + j] = T(tc[i][j]);
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) S[ix + Lay::mlo + i * D + j] = T(wide_lo(wide_from(tc[i][j], T(0))));
      for (int e = 0; e < N * Lay::LD; ++e) S[ix + Lay::L + e] = T(0);
    }
    g.sync();
  }
  dstruct_copy<T, Lay::kNormal, L, IPW>(S, g, ii, ix);
  if constexpr (FP) {
    dstruct_cond_identity<T, NU, D, L, IPW>(S, g, ibw);
    dstruct_cond_identity<T, NU, D, L, IPW>(S, g, ibwi);
  }

  double t = save_at[0], ti = t, dt = a.dt0[b], pi_prev = 1.0, mle_sumsq = 0.0;
  int num_data = 0, num_steps = 0, attempts = 0, status = PDQ_INSTANCE_OK;
  T sigma_sf = T(1);
  const T damp = T(a.damp);

  if (valid && !a.terminal_only) {
    dstruct_write_normal<T, NU, D, L, IPW>(S, g, ix, a.u_mean + (b * S_out) * N, a.u_chol + (b * S_out) * N * N);
    if (g.lane == 0) {
      a.output_scale[b * S_out] = 1.0;
      a.t_out[b * S_out] = t;
      a.num_steps[b * S_out] = 0;
    }
  }
  if (valid && a.filter_mean)
    dstruct_write_normal<T, NU, D, L, IPW>(S, g, ix, a.filter_mean + (b * Sn) * N, a.filter_chol + (b * Sn) * N * N);

  // One attempt per iteration (the retry loop flattened into the checkpoint
  // loop), warp-uniform: every group of the warp runs the attempt's
  // arithmetic in every iteration while any group still solves, so the
  // groups stay converged through the QRs (a group that is not stepping --
  // done, failed, or at a checkpoint -- computes on a dummy step into its
  // scratch slots and discards the result; only the rare checkpoint branches
  // diverge).  Per instance the sequence of attempts and checkpoint branches
  // is the nested loop's (solvers_via_adaptive_steps.py:196-375).
  int s = 1;
  double t_next = save_at[1];
  bool active = valid;
  while (__any_sync(0xffffffffu, active)) {
    bool stepping = active && t + a.eps < t_next;
    bool accepted = false;
    double dt_use = dt;
    if (stepping) {
      dt_use = a.clip_dt ? fmin(dt, t_next - t) : dt;
      if (!(fabs(dt_use) > 1e-14 * fmax(1.0, fabs(t)))) {
        status = PDQ_INSTANCE_DT_UNDERFLOW;
        active = stepping = false;
      } else if (attempts >= a.max_attempts) {
        status = PDQ_INSTANCE_MAX_STEPS;
        active = stepping = false;
      } else {
        ++attempts;
      }
    }
    {
      {
        // a group that is not stepping computes on a finite dummy step
        const T h = stepping ? T(dt_use) : T(1);
        T pc[n], pic[n];
        precon<T, NU>(h, pc, pic);
        // u = transition(h, 1).apply_flat(mean): mean mp, chol |p| sqrt|h| Q
        // extrapolated mean of coefficients 0 and 1 (all the linearisation
        // reads), wide as in the isotropic kernel: mp = m + incr with
        // incr_i = p_i sum_{k > i} A1[i][k] p^-1_k m_k (A1[i][i] p_i p^-1_i = 1)
        T mp[2 * D], mplo[2 * D], incr[2 * D];
#pragma unroll
        for (int i = 0; i < 2 * D; ++i) {
          T acc = T(0);
#pragma unroll
          for (int kk = i / D + 1; kk < n; ++kk) acc += T(iwp_a<NU>(i / D, kk)) * pic[kk] * S[ix + Lay::m + kk * D + i % D];
          incr[i] = pc[i / D] * acc;
          const Wide<T> w = wide_pair(S[ix + Lay::m + i], S[ix + Lay::mlo + i]) + incr[i];
          mp[i] = T(wide_hi(w));
          mplo[i] = T(wide_lo(w));
        }
        // linearisation at mp: J (d x 2d; zero beyond), b; residual r = J mp + b
        T J[D][2 * D], bl[D];
        {
          T f[D];
          if constexpr (TS1) {
            T Jf[D][D];
            eval_with_jacobian<F>(&mp[0], pt, f, Jf);
#pragma unroll
            for (int aa = 0; aa < D; ++aa) {
#pragma unroll
              for (int k = 0; k < D; ++k) {
                J[aa][k] = -Jf[aa][k];
                J[aa][D + k] = (k == aa) ? T(1) : T(0);
              }
              T jx = T(0);
#pragma unroll
              for (int k = 0; k < D; ++k) jx += Jf[aa][k] * mp[k];
              bl[aa] = -f[aa] + jx;
            }
          } else {
            F::eval(&mp[0], pt, f);
#pragma unroll
            for (int aa = 0; aa < D; ++aa) {
#pragma unroll
              for (int k = 0; k < 2 * D; ++k) J[aa][k] = (k == D + aa) ? T(1) : T(0);
              bl[aa] = -f[aa];
            }
          }
        }
        // the residual r = J mp + b = mp_1 - f(mp_0) (the linearisation point is mp), with
        // the field evaluated in the wide type at the wide rows, rounded once
        T r[D];
        {
          Wide<T> u[D], fw[D];
#pragma unroll
          for (int j = 0; j < D; ++j) u[j] = wide_pair(mp[j], mplo[j]);
          F::eval(u, pw, fw);
#pragma unroll
          for (int aa = 0; aa < D; ++aa) r[aa] = T(wide_hi(wide_pair(mp[D + aa], mplo[D + aa]) - fw[aa]));
        }
        (void)bl;
        // observed = fx.marginalise(u): R of [(J Lu)^T (rows < 2d; zero beyond); damp I]
        const T sqh = dev_sqrt(dev_abs(h));
        T Mo[3 * D][D];
#pragma unroll
        for (int rr = 0; rr < 2 * D; ++rr)
#pragma unroll
          for (int aa = 0; aa < D; ++aa) {
            T acc = T(0);
#pragma unroll
            for (int k = 0; k < 2 * D; ++k)
              if (k % D == rr % D && rr / D <= k / D) acc += J[aa][k] * dev_abs(pc[k / D]) * sqh * T(a.q1[k / D][rr / D]);
            Mo[rr][aa] = acc;
          }
#pragma unroll
        for (int i = 0; i < D; ++i)
#pragma unroll
          for (int j = 0; j < D; ++j) Mo[2 * D + i][j] = (i == j) ? damp : T(0);
        householder_r<T, 3 * D, D>(Mo);
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

        // prediction (and this step's backward conditional, merged into the running one)
        dstruct_predict<T, NU, D, FP, L, IPW>(S, g, a.q1, ix, h, s_pred, ipred);
        if constexpr (FP) dstruct_merge<T, NU, D, L, IPW>(S, g, ibw, h, img);

        // update: fx.revert(pred), the 3d rows of [[damp I, 0], [(J Lp)^T, Lp^T]] that take part
        T Wu[3 * D][D + N];
#pragma unroll
        for (int i = 0; i < D; ++i)
#pragma unroll
          for (int j = 0; j < D + N; ++j) Wu[i][j] = (i == j) ? damp : T(0);
#pragma unroll
        for (int rr = 0; rr < 2 * D; ++rr) {
#pragma unroll
          for (int aa = 0; aa < D; ++aa) {
            T acc = T(0);
#pragma unroll
            for (int k = rr; k < 2 * D; ++k) acc += J[aa][k] * S[ipred + Lay::L + k * Lay::LD + rr];
            Wu[D + rr][aa] = acc;
          }
#pragma unroll
          for (int c = 0; c < N; ++c) Wu[D + rr][D + c] = c >= rr ? S[ipred + Lay::L + c * Lay::LD + rr] : T(0);
        }
        householder_r<T, 3 * D, D + N>(Wu);
        // G^T = R_Y^-1 R12 (d x N); the proposal's mean mp - G ro, ro = r (the linearisation point is mp)
        T Gt[D][N];
#pragma unroll
        for (int col = 0; col < N; ++col)
#pragma unroll
          for (int i = D - 1; i >= 0; --i) {
            T acc = Wu[i][D + col];
#pragma unroll
            for (int k = i + 1; k < D; ++k) acc -= Wu[i][k] * Gt[k][col];
            Gt[i][col] = dev_div(acc, Wu[i][i]);
          }
        // the proposal's mean and factor: rows 0 .. 2d - 1 of L^T from Wu, the others from Lp
        T m0new[D];
#pragma unroll
        for (int i = 0; i < N; ++i) {
          T acc;
          if (i < 2 * D) {  // m' = m + (incr - G r), summed wide
            T dl = incr[i];
#pragma unroll
            for (int aa = 0; aa < D; ++aa) dl -= Gt[aa][i] * r[aa];
            const Wide<T> w = wide_pair(S[ix + Lay::m + i], S[ix + Lay::mlo + i]) + dl;
            acc = T(wide_hi(w));
            if (g.owns(i)) S[inew + Lay::mlo + i] = T(wide_lo(w));
          } else {
            acc = S[ipred + Lay::m + i];
#pragma unroll
            for (int aa = 0; aa < D; ++aa) acc -= Gt[aa][i] * r[aa];
          }
          if (i < D) m0new[i] = acc;
          if (g.owns(i)) {
            S[inew + Lay::m + i] = acc;
#pragma unroll
            for (int j = 0; j < N; ++j) {
              T v;
              if (j > i) v = T(0);
              else if (j < 2 * D) v = Wu[D + j][D + i];
              else v = S[ipred + Lay::L + i * Lay::LD + j];
              S[inew + Lay::L + i * Lay::LD + j] = v;
            }
          }
        }
        g.sync();
        // error_residual_std: sigma * row norms of the observed factor * dt
        double sumsq = 0.0;
#pragma unroll
        for (int j = 0; j < D; ++j) {
          T rn = T(0);
#pragma unroll
          for (int k = 0; k <= j; ++k) rn += Mo[k][j] * Mo[k][j];
          const T err_abs = dev_abs(sigma_loc) * dev_sqrt(rn) * h;
          const T ref = fmax(dev_abs(S[ix + Lay::m + j]), dev_abs(m0new[j]));
          const T ratio = dev_div(err_abs, T(a.atol) + T(a.rtol) * ref);
          sumsq += double(ratio) * double(ratio);
        }
        const double norm2 = sumsq * (1.0 / D);
        if (stepping && (!(norm2 == norm2) || isinf(norm2))) {
          status = PDQ_INSTANCE_NONFINITE;
          active = stepping = false;
        }
        const T ep = dev_fpow(T(norm2), T(-0.5 / n));
        double factor;
        if (a.control == PDQ_CONTROL_INTEGRAL) {
          factor = a.safety * double(ep);
        } else {
          factor = a.safety * double(dev_fpow(ep, T(a.exp_i))) * double(dev_fpow(dev_div(ep, T(pi_prev)), T(a.exp_p)));
          if (stepping && norm2 <= 1.0) pi_prev = double(ep);
        }
        factor = fmax(a.factor_min, fmin(factor, a.factor_max));
        if (stepping) dt = factor * dt_use;
        accepted = stepping && norm2 <= 1.0;
        if (accepted) {
          ti = t;
          t = t + dt_use;
          ++num_steps;
          {  // interp_from <- step_from <- proposal
            const int o = ii;
            ii = ix;
            ix = inew;
            inew = o;
          }
          if constexpr (FP) {  // interp conditional <- running <- merged
            const int o = ibwi;
            ibwi = ibw;
            ibw = img;
            img = o;
          }
          if (a.solver == PDQ_SOLVER_MLE) {
            T wv[D];
#pragma unroll
            for (int i = 0; i < D; ++i) {
              T acc = r[i];
#pragma unroll
              for (int k = 0; k < i; ++k) acc -= Wu[k][i] * wv[k];
              wv[i] = dev_div(acc, Wu[i][i]);
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
    }
    // a rejected attempt retries in the next iteration; the checkpoint
    // branches below run when the step reached or passed t_next
    if (!active || t + a.eps < t_next) continue;
    const bool record = (!a.terminal_only) || (s == Sn - 1);
    const int s_out = a.terminal_only ? 0 : s;
    const int64_t rec = b * S_out + s_out;
    if (t > t_next + a.eps) {
      // interp_beyond_t1 (solvers.py:205-269)
      const T h0 = T(t_next - ti), h1 = T(t - t_next);
      if constexpr (FP) {
        // estimators_and_losses.py:549-591
        dstruct_predict<T, NU, D, true, L, IPW>(S, g, a.q1, ii, h0, sigma_sf, ipred);  // extrapolated_t, c0
        dstruct_merge<T, NU, D, L, IPW>(S, g, ibwi, h0, itmp);                         // its conditional
        dstruct_store_cond<T, NU, D, L, IPW>(S, g, itmp, ws + int64_t(s - 1) * cond_floats<N>());
        {  // keep extrapolated_t in the proposal slot
          const int o = inew;
          inew = ipred;
          ipred = o;
        }
        dstruct_predict<T, NU, D, true, L, IPW>(S, g, a.q1, inew, h1, sigma_sf, ipred);  // c1
        dstruct_cond_identity<T, NU, D, L, IPW>(S, g, ibwi);
        dstruct_merge<T, NU, D, L, IPW>(S, g, ibwi, h1, ibw);  // extrapolated_t1.conditional -> step_from's
        {  // interp_from = extrapolated_t
          const int o = ii;
          ii = inew;
          inew = o;
        }
        // the interp conditional stays the identity
      } else {
        dstruct_predict<T, NU, D, false, L, IPW>(S, g, a.q1, ii, h0, sigma_sf, ipred);
        const int o = ii;
        ii = ipred;
        ipred = o;
      }
      ti = t_next;
      if (record) {
        dstruct_write_normal<T, NU, D, L, IPW>(S, g, ii, a.u_mean + rec * N, a.u_chol + rec * N * N);
        if (g.lane == 0) {
          a.output_scale[rec] = double(sigma_sf);
          a.t_out[rec] = t_next;
          a.num_steps[rec] = num_steps;
        }
      }
      if (a.filter_mean)
        dstruct_write_normal<T, NU, D, L, IPW>(S, g, ii, a.filter_mean + (b * Sn + s) * N, a.filter_chol + (b * Sn + s) * N * N);
    } else {
      // interp_at_t1 (solvers.py:271-315)
      if constexpr (FP) {
        dstruct_store_cond<T, NU, D, L, IPW>(S, g, ibw, ws + int64_t(s - 1) * cond_floats<N>());
        dstruct_cond_identity<T, NU, D, L, IPW>(S, g, ibw);
        dstruct_cond_identity<T, NU, D, L, IPW>(S, g, ibwi);
      }
      dstruct_copy<T, Lay::kNormal, L, IPW>(S, g, ii, ix);
      ti = t;
      if (record) {
        dstruct_write_normal<T, NU, D, L, IPW>(S, g, ix, a.u_mean + rec * N, a.u_chol + rec * N * N);
        if (g.lane == 0) {
          a.output_scale[rec] = double(sigma_sf);
          a.t_out[rec] = t;
          a.num_steps[rec] = num_steps;
        }
      }
      if (a.filter_mean)
        dstruct_write_normal<T, NU, D, L, IPW>(S, g, ix, a.filter_mean + (b * Sn + s) * N, a.filter_chol + (b * Sn + s) * N * N);
    }
    // checkpoint s done
    ++s;
    if (s < Sn) {
      t_next = save_at[s];
    } else {
      active = false;
    }
  }

  if (!valid) return;
  // ---- finalize (solvers.py:439-480, 601-633, 735-767) ----
  double scale = 1.0;
  if (status == PDQ_INSTANCE_OK && a.solver == PDQ_SOLVER_MLE) {
    scale = num_data > 0 ? sqrt(mle_sumsq / num_data) : 0.0;
    if (a.correct) scale /= sqrt(double(a.num_steps[b * S_out + (S_out - 1)]));
  }
  if (status == PDQ_INSTANCE_OK && FP) {
    // Smoother.finalize: rv_at_t1 = posterior1.conditional.marginalise(marginal),
    // then the reverse scan of marginalise over the checkpoint conditionals
    int irv = inew, iprev = ipred;
    dstruct_cond_marginalise<T, NU, D, L, IPW>(S, g, ibw, ix, irv);
    for (int s2 = Sn - 1; s2 >= 1; --s2) {
      if (!a.terminal_only || s2 == Sn - 1) {
        const int64_t rec = b * S_out + (a.terminal_only ? 0 : s2);
        dstruct_write_normal<T, NU, D, L, IPW>(S, g, irv, a.u_mean + rec * N, a.u_chol + rec * N * N);
      }
      if (a.terminal_only) break;
      dstruct_load_cond<T, NU, D, L, IPW>(S, g, itmp, ws + int64_t(s2 - 1) * cond_floats<N>());
      if (a.cond_A) {
        const int64_t cr = b * (Sn - 1) + (s2 - 1);
        constexpr int NN = N * N;
        for (int e = g.lane; e < NN; e += L) {
          a.cond_A[cr * NN + e] = double(S[itmp + Lay::A + (e / N) * Lay::LD + e % N]);
          a.cond_noise_chol[cr * NN + e] = double(S[itmp + Lay::X + (e / N) * Lay::LD + e % N]) * scale;
        }
        for (int e = g.lane; e < N; e += L) {
          a.cond_noise_mean[cr * N + e] = double(S[itmp + Lay::xi + e]);
          a.cond_to_latent[cr * N + e] = double(S[itmp + Lay::tl + e]);
          a.cond_to_observed[cr * N + e] = double(S[itmp + Lay::to + e]);
        }
      }
      dstruct_cond_marginalise<T, NU, D, L, IPW>(S, g, itmp, irv, iprev);
      {
        const int o = irv;
        irv = iprev;
        iprev = o;
      }
      if (s2 == 1) {
        const int64_t rec = b * S_out;
        dstruct_write_normal<T, NU, D, L, IPW>(S, g, irv, a.u_mean + rec * N, a.u_chol + rec * N * N);
      }
    }
  }
  __syncwarp(g.mask);  // the group's output writes are ordered before the rescaling below
  if (status == PDQ_INSTANCE_OK) {
    if (a.solver == PDQ_SOLVER_MLE) {
      for (int s2 = 0; s2 < S_out; ++s2) {
        const int64_t rec = b * S_out + s2;
        for (int k = g.lane; k < N * N; k += L) a.u_chol[rec * N * N + k] *= scale;
        if (g.lane == 0) a.output_scale[rec] = scale;
      }
      if (a.filter_chol)
        for (int k = g.lane; k < Sn * N * N; k += L) a.filter_chol[b * Sn * N * N + k] *= scale;
    }
  } else {
    const double nan = __longlong_as_double(0x7ff8000000000000ULL);
    for (int s2 = 0; s2 < S_out; ++s2) {
      const int64_t rec = b * S_out + s2;
      for (int k = g.lane; k < N; k += L) a.u_mean[rec * N + k] = nan;
      for (int k = g.lane; k < N * N; k += L) a.u_chol[rec * N * N + k] = nan;
      if (g.lane == 0) {
        a.output_scale[rec] = nan;
        a.t_out[rec] = nan;
        a.num_steps[rec] = num_steps;
      }
    }
  }
  if (g.lane == 0) {
    a.num_attempts[b] = attempts;
    a.status[b] = status;
  }
}

template <int NU, int D>
constexpr size_t dense_struct_smem_bytes(size_t elem, int L) {
  return size_t(32 / L) * size_t(DenseLayout<NU, D>::size) * elem;
}

}  // namespace pdq
