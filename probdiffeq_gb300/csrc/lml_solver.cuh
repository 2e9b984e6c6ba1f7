// Log-marginal likelihood of time-series data under the fixed-point-smoother
// posterior of an isotropic TS0 solve on a fixed grid, and its gradient with
// respect to the vector-field parameters.  One thread per parameter sample.
//
// Forward (value) path, following the reference:
//   solver (uncalibrated) step              _probdiffeq/solvers.py:702-733
//   strategy_smoother_fixedpoint.predict     _probdiffeq/estimators_and_losses.py:526-532
//     IsotropicLatentCond.revert / merge     _probdiffeq/ssm_impl_isotropic.py:91-133
//   checkpoint reset to the identity         estimators_and_losses.py:534-547
//     (the save_at mechanics on a grid whose steps land on the observations)
//   Smoother.finalize (rv at t1)             estimators_and_losses.py:437-470
//   loss_lml_timeseries / evaluate_lml       estimators_and_losses.py:53-105, 180-218
//     with to_derivative(0, std), bayes_rule_and_logpdf_tree and
//     IsotropicNormal.logpdf_flat            ssm_impl_api.py:118-124, ssm_impl_isotropic.py:217-278
//   Taylor-mode initial derivatives          _probdiffeq/jet_expansion_algorithms.py:49-103
//
// Derivative: forward mode, one tangent direction per thread.  A parameter
// sample is handled by P threads, thread k carrying d/d theta_k, and each of
// them recomputes the value path: redundant arithmetic, but the state of one
// thread is a value and one tangent (registers instead of local-memory
// spills for P tangents) and the threads never communicate.  The rules are
// the reference's: qr_r has the custom JVP R_dot = Q^T M_dot with Q held
// constant (backend/linalg.py:13-37), so the reflectors / rotations computed
// from the values are applied to the tangent matrices and the tangent of a
// triangular factor is a full matrix; triangular solves differentiate
// through the triangle only (back substitution on dual numbers); the time
// step carries no tangent (the reference stops gradients through dt).  For
// the 3 parameters of the configurations this needs no checkpointed
// re-computation; the backward conditionals at the observations are stored.
// The log-likelihood sum and its tangents are float64.
//
// Shared covariance plan.  With TS0 (H = e_1), the uncalibrated solver, a
// fixed step and exact initial coefficients, every covariance-side quantity
// of the forward pass -- predicted factors, reverts, gains, merged backward
// conditionals -- is the same for every parameter sample and carries no
// tangent.  lml_plan_kernel computes them once, with the same arithmetic the
// per-sample pass used (dual numbers with zero tangents, qr_qconst /
// givens_qconst), into a plan in the workspace: per step the update gain and
// the matrix K that maps the mean before the step to the increment of the
// merged backward conditional's offset (xi <- xi + K m, K = bw.A diag(Tv)
// (I - G^T A1) diag(p_inv), formed in double);
// per observation interval the merged conditional's A, noise factor,
// to_latent and to_observed; the terminal factor; the backward pass's
// covariance side (it depends on the observation noise std but not on the
// parameters): per observation the observed std ry and the gain column.
// lml_kernel then runs only the mean recursion (matrix-vector products with
// the plan's tables, staged through shared memory a chunk of steps at a time
// by the warp, the vector field on dual numbers) per sample and tangent.  The
// plan starts with a key (dt, damp, steps, observation
// spacing, nu, precision, and a copy of std) and is rebuilt only when the
// key in the workspace differs.
#pragma once

#include "iso_solver.cuh"

namespace pdq {

template <typename T, int K>
PDQ_HD Dual<T, K> dual_abs_scale(T s, const Dual<T, K>& a) {  // |s| * a for a constant s
  return (s < T(0) ? -s : s) * a;
}

// One warp per block: a batch of 1024 samples x 3 tangent lanes is 96
// warps, fewer than the SMs, so each warp gets an SM to itself.
constexpr int kLmlThreads = 32;

struct LmlArgs {
  int64_t B;
  int32_t num_steps, save_every, average_pdfs, with_gradient;
  int32_t lanes_per_sample;  // P with the gradient (one tangent direction per thread), else 1
  double t0, dt, damp;
  double q1[kMaxN][kMaxN];
  const double* params;  // (B, P)
  const double* y0;      // (B, d)
  const double* data;    // (num_obs, d)
  const double* std;     // (num_obs,)
  double* lml;           // (B,)
  double* grad;          // (B, P) or nullptr
  int32_t* status;       // (B,)
  void* plan;            // the shared covariance plan (lml_plan_elems<T, NU> after a 256-byte key)
  void* workspace;       // (B * lanes, num_obs - 1) backward-conditional offsets xi with tangents, T
};

// Plan layout (in T, after the 256-byte key): per step g[n] and K[n][n]; per
// observation interval
// A[n][n], X[n][n], tl[n], to[n]; the terminal factor rL[n][n]; per
// observation ry and ginv[n]; then (8-byte aligned) the std the plan was
// built for and log|ry| per observation, in double.
constexpr int kLmlPlanKeyBytes = 256;

template <int NU>
PDQ_HD constexpr int lml_plan_step() {
  return (NU + 1) * (NU + 1) + (NU + 1);
}
template <int NU>
PDQ_HD constexpr int lml_plan_obs() {
  return 2 * (NU + 1) * (NU + 1) + 2 * (NU + 1);
}
PDQ_HD int64_t lml_plan_elems(int nu, int num_steps, int save_every) {
  const int64_t n = nu + 1;
  const int64_t step = n * n + n, per = 2 * n * n + 2 * n;
  const int64_t num_obs = num_steps / save_every + 1;
  return int64_t(num_steps) * step + (num_obs - 1) * per + n * n + num_obs * (n + 1);
}
// Offset in bytes (from the plan's start, key included) of the std copy.
PDQ_HD int64_t lml_plan_std_offset(int nu, int num_steps, int save_every, int elem) {
  const int64_t raw = kLmlPlanKeyBytes + lml_plan_elems(nu, num_steps, save_every) * elem;
  return (raw + 7) / 8 * 8;
}
// Plan bytes in total (key, tables, std copy, log|ry|), a multiple of 256.
PDQ_HD int64_t lml_plan_total_bytes(int nu, int num_steps, int save_every, int elem) {
  const int64_t num_obs = num_steps / save_every + 1;
  const int64_t raw = lml_plan_std_offset(nu, num_steps, save_every, elem) + 2 * num_obs * 8;
  return (raw + 255) / 256 * 256;
}
// Steps of plan tables staged in shared memory at a time.
constexpr int kLmlChunk = 32;


// Householder QR (R x C, R >= C) of a dual matrix with the Q-constant tangent
// rule: reflectors from the values; the values become R (zeros below), the
// tangents become the first rows of Q^T M_dot (full, not triangular).
template <typename T, int P, int R, int C>
PDQ_D void qr_qconst(Dual<T, P> (&M)[R][C]) {
#pragma unroll
  for (int c = 0; c < C; ++c) {
    T nrm2 = T(0);
#pragma unroll
    for (int r = c; r < R; ++r) nrm2 += M[r][c].v * M[r][c].v;
    if (nrm2 > T(0)) {
      const T alpha = M[c][c].v;
      const T nrm = dev_sqrt(nrm2);
      const T beta = alpha >= T(0) ? -nrm : nrm;
      const T v0inv = T(1) / (alpha - beta);
      const T tau = (beta - alpha) / beta;
      T v[R];
#pragma unroll
      for (int r = 0; r < R; ++r) v[r] = (r < c) ? T(0) : (r == c ? T(1) : M[r][c].v * v0inv);
      // values: columns > c
#pragma unroll
      for (int j = c + 1; j < C; ++j) {
        T w = T(0);
#pragma unroll
        for (int r = c; r < R; ++r) w += v[r] * M[r][j].v;
        w *= tau;
#pragma unroll
        for (int r = c; r < R; ++r) M[r][j].v -= w * v[r];
      }
      // tangents: every column
#pragma unroll
      for (int k = 0; k < P; ++k)
#pragma unroll
        for (int j = 0; j < C; ++j) {
          T w = T(0);
#pragma unroll
          for (int r = c; r < R; ++r) w += v[r] * M[r][j].g[k];
          w *= tau;
#pragma unroll
          for (int r = c; r < R; ++r) M[r][j].g[k] -= w * v[r];
        }
      M[c][c].v = beta;
#pragma unroll
      for (int r = c + 1; r < R; ++r) M[r][c].v = T(0);
    }
  }
}

// Givens rotation of rows a, b zeroing M[b][c0] in the values; the same
// rotation is applied to all value columns and all tangents (Q constant).
template <typename T, int P, int NR, int NC>
PDQ_D void givens_qconst(Dual<T, P> (&M)[NR][NC], int a, int b, int c0) {
  const T x = M[a][c0].v, y = M[b][c0].v;
  const T r2 = x * x + y * y;
  if (r2 > T(0)) {
    const T inv = dev_rsqrt(r2);
    const T cs = x * inv, sn = y * inv;
#pragma unroll
    for (int j = 0; j < NC; ++j) {
      const Dual<T, P> ma = M[a][j], mb = M[b][j];
      M[a][j] = cs * ma + sn * mb;
      M[b][j] = cs * mb - sn * ma;
    }
    M[b][c0].v = T(0);
  }
}

template <typename T, int P, int NU, int D>
struct LmlCond {
  Dual<T, P> A[NU + 1][NU + 1];
  Dual<T, P> xi[NU + 1][D];
  Dual<T, P> X[NU + 1][NU + 1];
  T tl[NU + 1];
  T to[NU + 1];
};

template <typename T, int P, int NU, int D>
PDQ_D void lml_cond_identity(LmlCond<T, P, NU, D>& c) {
  constexpr int n = NU + 1;
#pragma unroll
  for (int i = 0; i < n; ++i) {
#pragma unroll
    for (int j = 0; j < n; ++j) {
      c.A[i][j] = Dual<T, P>(i == j ? T(1) : T(0));
      c.X[i][j] = Dual<T, P>(T(0));
    }
#pragma unroll
    for (int j = 0; j < D; ++j) c.xi[i][j] = Dual<T, P>(T(0));
    c.tl[i] = T(1);
    c.to[i] = T(1);
  }
}

// cond.marginalise(rv) (ssm_impl_isotropic.py:81-89)
template <typename T, int P, int NU, int D>
PDQ_D void lml_marginalise(const LmlCond<T, P, NU, D>& c, const Dual<T, P> (&m)[NU + 1][D],
                           const Dual<T, P> (&L)[NU + 1][NU + 1], Dual<T, P> (&mo)[NU + 1][D],
                           Dual<T, P> (&Lo)[NU + 1][NU + 1]) {
  constexpr int n = NU + 1;
  using DT = Dual<T, P>;
  DT M[2 * n][n];
#pragma unroll
  for (int r = 0; r < n; ++r)
#pragma unroll
    for (int col = 0; col < n; ++col) {
      DT acc(T(0));
#pragma unroll
      for (int k = 0; k < n; ++k) acc = acc + c.A[col][k] * (c.tl[k] * L[k][r]);
      M[r][col] = acc;
      M[n + r][col] = c.X[col][r];
    }
  qr_qconst<T, P, 2 * n, n>(M);
#pragma unroll
  for (int i = 0; i < n; ++i) {
#pragma unroll
    for (int j = 0; j < D; ++j) {
      DT acc = c.xi[i][j];
#pragma unroll
      for (int k = 0; k < n; ++k) acc = acc + c.A[i][k] * (c.tl[k] * m[k][j]);
      mo[i][j] = c.to[i] * acc;
    }
#pragma unroll
    for (int j = 0; j < n; ++j) Lo[i][j] = dual_abs_scale(c.to[i], M[j][i]);
  }
}

// Threads of the plan kernel's one block.
constexpr int kLmlPlanThreads = 256;

// The covariance side of the forward pass, once for all samples.  Thread 0
// runs the recursion over the steps (it is sequential): the prior revert,
// the merge into the running backward conditional and the update, in the
// bulk type with the isotropic kernel's functions; for every step it leaves
// the revert's A in the step's K slot.  Then the block forms K for all steps
// in parallel, one observation interval per thread, in double: the running
// conditional's A before the step is the product of the interval's
// diag(Tv) A factors, recomputed by the interval's thread.
template <typename T, int NU>
__global__ void __launch_bounds__(kLmlPlanThreads) lml_plan_kernel(LmlArgs a) {
  if (blockIdx.x != 0) return;
  constexpr int n = NU + 1;
  const int tid = threadIdx.x;
  double* key = reinterpret_cast<double*>(a.plan);
  const double want[7] = {1.2345678901234567e89, a.dt, a.damp, double(a.num_steps), double(a.save_every), double(NU),
                          double(sizeof(T))};
  const int num_obs = a.num_steps / a.save_every + 1;
  double* const std_copy = reinterpret_cast<double*>(reinterpret_cast<unsigned char*>(a.plan) +
                                                     lml_plan_std_offset(NU, a.num_steps, a.save_every, int(sizeof(T))));
  __shared__ int s_same;
  if (tid == 0) {
    bool same = key[7] == 1.0;
    for (int i = 0; i < 7; ++i) same = same && __double_as_longlong(key[i]) == __double_as_longlong(want[i]);
    for (int k = 0; same && k < num_obs; ++k) same = __double_as_longlong(std_copy[k]) == __double_as_longlong(a.std[k]);
    s_same = same ? 1 : 0;
    if (!same) key[7] = 0.0;
  }
  __syncthreads();
  if (s_same) return;
  T* const plan = reinterpret_cast<T*>(reinterpret_cast<unsigned char*>(a.plan) + kLmlPlanKeyBytes);
  T* const obs_tbl = plan + int64_t(a.num_steps) * lml_plan_step<NU>();
  const T h = T(a.dt);
  T p[n], pinv[n];
  precon<T, NU>(h, p, pinv);

  if (tid == 0) {
    T q1t[kMaxN][kMaxN];
#pragma unroll
    for (int i = 0; i < kMaxN; ++i)
#pragma unroll
      for (int j = 0; j < kMaxN; ++j) q1t[i][j] = T(a.q1[i][j]);
    T L[n][n], m0[n][1];
#pragma unroll
    for (int i = 0; i < n; ++i) {
      m0[i][0] = T(0);
#pragma unroll
      for (int j = 0; j < n; ++j) L[i][j] = T(0);
    }
    IsoBackward<T, NU, 1> bw;  // xi unused (means are per sample)
    iso_cond_identity(bw);
    const T sq = dev_sqrt(dev_abs(h));
    const T damp = T(a.damp);
    for (int step = 1; step <= a.num_steps; ++step) {
      T* const tbl = plan + int64_t(step - 1) * lml_plan_step<NU>();
      // revert (transition.revert(marginal)), then merge (ssm_impl_isotropic.py:91-105)
      IsoBackward<T, NU, 1> cn, merged;
      T Lp[n][n];
      iso_prior_revert<T, NU, 1>(q1t, m0, L, p, pinv, sq, Lp, cn);
      iso_cond_merge(bw, cn, merged);
      bw = merged;
      // update (Givens, H = e_1): the gain and the corrected factor
      T gain[n], Lnew[n][n];
      ts0_update<T, NU, 1, false>(Lp, damp, gain, Lnew);
#pragma unroll
      for (int i = 0; i < n; ++i) {
        tbl[i] = gain[i];
#pragma unroll
        for (int j = 0; j < n; ++j) {
          tbl[n + i * n + j] = cn.A[i][j];  // replaced by K below
          L[i][j] = Lnew[i][j];
        }
      }
      // observation: the merged conditional goes to the table, reset
      if (step % a.save_every == 0) {
        T* o = obs_tbl + int64_t(step / a.save_every - 1) * lml_plan_obs<NU>();
        for (int i = 0; i < n; ++i)
          for (int j = 0; j < n; ++j) {
            o[i * n + j] = bw.A[i][j];
            o[n * n + i * n + j] = bw.X[i][j];
          }
        for (int i = 0; i < n; ++i) {
          o[2 * n * n + i] = bw.tl[i];
          o[2 * n * n + n + i] = bw.to[i];
        }
        iso_cond_identity(bw);
      }
    }
    // rv_at_t1: the terminal marginal through the (identity) conditional -- its factor
    T rm[n][1], rL[n][n];
    iso_cond_marginalise(bw, m0, L, rm, rL);
    T* const term = obs_tbl + int64_t(num_obs - 1) * lml_plan_obs<NU>();
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) term[i * n + j] = rL[i][j];
    // the backward pass's covariance side: marginalise through each stored
    // conditional, then bayes_rule with to_derivative(0, std_k) (one Givens
    // rotation: the update of coefficient 0 with noise std_k)
    T* const bay = term + n * n;
    for (int k = num_obs - 1; k >= 0; --k) {
      if (k < num_obs - 1) {
        IsoBackward<T, NU, 1> c;
        const T* o = obs_tbl + int64_t(k) * lml_plan_obs<NU>();
        for (int i = 0; i < n; ++i) {
          for (int j = 0; j < n; ++j) {
            c.A[i][j] = o[i * n + j];
            c.X[i][j] = o[n * n + i * n + j];
          }
          c.xi[i][0] = T(0);
          c.tl[i] = o[2 * n * n + i];
          c.to[i] = o[2 * n * n + n + i];
        }
        T pm[n][1], pL[n][n];
        iso_cond_marginalise(c, m0, rL, pm, pL);
        for (int i = 0; i < n; ++i)
          for (int j = 0; j < n; ++j) rL[i][j] = pL[i][j];
      }
      T g[n], Lc[n][n];
      const T ry = ts0_update<T, NU, 0, false>(rL, T(a.std[k]), g, Lc);
      bay[k * (n + 1)] = ry;
      std_copy[num_obs + k] = log(double(ry < T(0) ? -ry : ry));  // log|ry| in double
      for (int i = 0; i < n; ++i) bay[k * (n + 1) + 1 + i] = g[i];
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) rL[i][j] = Lc[i][j];
    }
  }
  __syncthreads();

  // K per step, one observation interval per thread: the offsets are linear
  // in the mean m before the step -- the revert's xi = (I - G^T A1) diag(p_inv) m,
  // merged as xi += bw.A diag(Tv) xi_revert -- so xi += K m with
  // K = bw.A diag(Tv) (I - G^T A1) diag(p_inv), bw.A the running
  // conditional's A before the step (identity after an observation) and
  // Tv = bw.tl * cn.to (bw.tl = 1 after an observation, else the previous
  // step's to_latent 1 / p).
  const int num_seg = (a.num_steps + a.save_every - 1) / a.save_every;
  for (int q = tid; q < num_seg; q += blockDim.x) {
    double bA[n][n];
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) bA[i][j] = (i == j) ? 1.0 : 0.0;
    const int s0 = q * a.save_every + 1;
    const int s1 = min(a.num_steps, (q + 1) * a.save_every);
    for (int step = s0; step <= s1; ++step) {
      T* const k_t = plan + int64_t(step - 1) * lml_plan_step<NU>() + n;
      double G[n][n];  // the revert's A (= G^T)
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) G[i][j] = double(k_t[i * n + j]);
      double Tv[n];
      for (int i = 0; i < n; ++i) {
        const T tl = (step == s0) ? T(1) : T(1) / p[i];
        Tv[i] = double(tl * (T(1) / pinv[i]));
      }
      double C[n][n];  // (I - G^T A1) diag(p_inv)
      for (int k = 0; k < n; ++k)
        for (int j = 0; j < n; ++j) {
          double acc = (k == j) ? 1.0 : 0.0;
          for (int l = 0; l <= j; ++l) acc -= G[k][l] * double(iwp_a<NU>(l, j));
          C[k][j] = acc * double(pinv[j]);
        }
      double nA[n][n];
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
          double acc = 0.0, accA = 0.0;
          for (int k = 0; k < n; ++k) {
            acc += bA[i][k] * Tv[k] * C[k][j];
            accA += bA[i][k] * Tv[k] * G[k][j];
          }
          k_t[i * n + j] = T(acc);
          nA[i][j] = accA;
        }
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) bA[i][j] = nA[i][j];
    }
  }
  __syncthreads();
  if (tid == 0) {
    for (int k = 0; k < num_obs; ++k) std_copy[k] = a.std[k];
    __threadfence();
    for (int i = 0; i < 7; ++i) key[i] = want[i];
    __threadfence();
    key[7] = 1.0;
  }
}

template <typename T, int NU, class F>
__global__ void __launch_bounds__(kLmlThreads) lml_kernel(LmlArgs a) {
  constexpr int n = NU + 1;
  constexpr int D = F::D;
  constexpr int P = F::P;   // parameters
  constexpr int TG = 1;     // tangent directions carried by one thread
  constexpr int OUT = 1;
  using DT = Dual<T, TG>;
  using DD = Dual<double, TG>;
  // lanes_per_sample threads per parameter sample, each carrying the tangent
  // of one parameter (the mean recursion is computed by each)
  const int lanes = a.lanes_per_sample;
  const int64_t gtid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  // threads past the batch stay for the warp's cooperative staging of the plan
  const bool valid = gtid < a.B * lanes;
  const int64_t b = valid ? gtid / lanes : 0;
  const int dir = int(gtid % lanes);
  const int lane = threadIdx.x & 31;
  const int num_obs = a.num_steps / a.save_every + 1;
  constexpr int XF = n * D * (TG + 1);  // numbers per stored offset xi (values and tangents)
  T* ws = reinterpret_cast<T*>(a.workspace) + (valid ? gtid : 0) * int64_t(num_obs - 1) * XF;
  const T* const plan = reinterpret_cast<const T*>(reinterpret_cast<const unsigned char*>(a.plan) + kLmlPlanKeyBytes);
  const T* const obs_tbl = plan + int64_t(a.num_steps) * lml_plan_step<NU>();
  constexpr int kStep = lml_plan_step<NU>();
  __shared__ __align__(16) T stage[kLmlChunk * kStep];  // one warp per block

  // ---- parameters with unit tangents; Taylor-mode initial derivatives ----
  DD pd[P];
  DT pt[P];
#pragma unroll
  for (int k = 0; k < P; ++k) {
    pd[k] = DD(a.params[b * P + k]);
    pd[k].g[0] = (k == dir) ? 1.0 : 0.0;
    pt[k] = DT(T(pd[k].v));
    pt[k].g[0] = (k == dir) ? T(1) : T(0);
  }
  DD y0[D];
#pragma unroll
  for (int j = 0; j < D; ++j) y0[j] = DD(a.y0[b * D + j]);
  DD tc[n][D];
  taylor_init<F, NU>(y0, pd, tc);

  DT m[n][D], bxi[n][D];
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      m[i][j].v = T(tc[i][j].v);
#pragma unroll
      for (int k = 0; k < TG; ++k) m[i][j].g[k] = T(tc[i][j].g[k]);
      bxi[i][j] = DT(T(0));
    }

  const T h = T(a.dt);
  T p[n], pinv[n];
  precon<T, NU>(h, p, pinv);

  int status = PDQ_INSTANCE_OK;
  int to_obs = a.save_every;  // steps to the next observation (a counter, not a division per step)
  T* obs_dst = ws;            // stored offset of the next observation interval
  for (int step = 1; step <= a.num_steps; ++step) {
    const int within = (step - 1) % kLmlChunk;
    if (within == 0) {
      // stage the next chunk of step tables (coalesced, the whole warp)
      const int count = min(kLmlChunk, a.num_steps - (step - 1)) * kStep;
      const T* src = plan + int64_t(step - 1) * kStep;
#if defined(__CUDA_ARCH__)
      __syncwarp();
      for (int e = lane; e < count; e += 32) stage[e] = src[e];
      __syncwarp();
#else
      if (PDQ_HOST_LANES_CONCURRENT) {  // host runs with the warp's lanes as threads
        __syncwarp();
        for (int e = lane; e < count; e += 32) stage[e] = src[e];
        __syncwarp();
      } else {
        // host runs of the kernel body execute one lane at a time: it stages the whole chunk
        for (int e = 0; e < count; ++e) stage[e] = src[e];
      }
#endif
    }
    if (!valid || status != PDQ_INSTANCE_OK) continue;
    // this step's tables into registers in one batch of 16-byte loads, so
    // their latency overlaps instead of preceding each use
    T tb[kStep];
    {
      const T* tbl = stage + within * kStep;
      if constexpr (sizeof(T) == 4 && kStep % 4 == 0) {
        const float4* v = reinterpret_cast<const float4*>(tbl);
#pragma unroll
        for (int e = 0; e < kStep / 4; ++e) {
          const float4 x = v[e];
          tb[4 * e] = x.x;
          tb[4 * e + 1] = x.y;
          tb[4 * e + 2] = x.z;
          tb[4 * e + 3] = x.w;
        }
      } else if constexpr (sizeof(T) == 8 && kStep % 2 == 0) {
        const double2* v = reinterpret_cast<const double2*>(tbl);
#pragma unroll
        for (int e = 0; e < kStep / 2; ++e) {
          const double2 x = v[e];
          tb[2 * e] = x.x;
          tb[2 * e + 1] = x.y;
        }
      } else {
#pragma unroll
        for (int e = 0; e < kStep; ++e) tb[e] = tbl[e];
      }
    }
    const T* g_t = tb;
    const T* k_t = tb + n;
    // ---- predicted mean ----
    DT mean_l[n][D], mobs[n][D], mp[n][D];
#pragma unroll
    for (int i = 0; i < n; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) mean_l[i][j] = pinv[i] * m[i][j];
#pragma unroll
    for (int i = 0; i < n; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) {
        DT acc(T(0));
#pragma unroll
        for (int k = i; k < n; ++k) acc = acc + T(iwp_a<NU>(i, k)) * mean_l[k][j];
        mobs[i][j] = acc;
        mp[i][j] = p[i] * acc;
      }
    // ---- the merged backward conditional's offset: xi + K m (revert and merge) ----
    DT nxi[n][D];
#pragma unroll
    for (int i = 0; i < n; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) {
        DT x = bxi[i][j];
#pragma unroll
        for (int k = 0; k < n; ++k) x = x + k_t[i * n + k] * m[k][j];
        nxi[i][j] = x;
      }
    // ---- TS0 linearisation at the predicted mean; update with the plan's gain ----
    DT f[D];
    F::eval(mp[0], pt, f);
    DT res[D];
#pragma unroll
    for (int j = 0; j < D; ++j) res[j] = mp[OUT][j] - f[j];
#pragma unroll
    for (int i = 0; i < n; ++i) {
      const T g = g_t[i];
#pragma unroll
      for (int j = 0; j < D; ++j) {
        m[i][j] = mp[i][j] - g * res[j];
        bxi[i][j] = nxi[i][j];
      }
    }
    if (!(m[0][0].v == m[0][0].v)) {
      status = PDQ_INSTANCE_NONFINITE;  // stays in the loop for the staging
      continue;
    }
    // ---- checkpoint at an observation: store the offset, reset ----
    if (--to_obs == 0) {
      to_obs = a.save_every;
      T* dst = obs_dst;
      obs_dst += XF;
      int o = 0;
#pragma unroll
      for (int i = 0; i < n; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) {
          dst[o++] = bxi[i][j].v;
#pragma unroll
          for (int k = 0; k < TG; ++k) dst[o++] = bxi[i][j].g[k];
          bxi[i][j] = DT(T(0));
        }
    }
  }

  if (!valid) return;
  // ---- LML: reverse Kalman filter over the data (evaluate_lml) ----
  DD pdf(0.0);
  if (status == PDQ_INSTANCE_OK) {
    // rv_at_t1: the last step lands on the last observation, so the
    // conditional is the identity and the mean is m; the covariance side
    // (marginalise, bayes_rule) comes from the plan
    DT rm[n][D];
#pragma unroll
    for (int i = 0; i < n; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) rm[i][j] = m[i][j];
    const T* const bay = obs_tbl + int64_t(num_obs - 1) * lml_plan_obs<NU>() + n * n;
    const double* const logry = reinterpret_cast<const double*>(
                                    reinterpret_cast<const unsigned char*>(a.plan) +
                                    lml_plan_std_offset(NU, a.num_steps, a.save_every, int(sizeof(T)))) + num_obs;
    const double LOG2PI = 1.8378770664093453;
    int num = 0;
    for (int k = num_obs - 1; k >= 0; --k) {
      if (k < num_obs - 1) {
        // cond.marginalise (ssm_impl_isotropic.py:81-89), mean part
        const T* o = obs_tbl + int64_t(k) * lml_plan_obs<NU>();
        const T* src = ws + int64_t(k) * XF;
        DT pm[n][D];
#pragma unroll
        for (int i = 0; i < n; ++i)
#pragma unroll
          for (int j = 0; j < D; ++j) {
            DT acc;
            acc.v = src[(i * D + j) * (TG + 1)];
#pragma unroll
            for (int t = 0; t < TG; ++t) acc.g[t] = src[(i * D + j) * (TG + 1) + 1 + t];
#pragma unroll
            for (int q = 0; q < n; ++q) acc = acc + o[i * n + q] * (o[2 * n * n + q] * rm[q][j]);
            pm[i][j] = o[2 * n * n + n + i] * acc;
          }
#pragma unroll
        for (int i = 0; i < n; ++i)
#pragma unroll
          for (int j = 0; j < D; ++j) rm[i][j] = pm[i][j];
      }
      // model_k = to_derivative(0, std_k); bayes_rule_and_logpdf_tree
      const T ry = bay[k * (n + 1)];
      const double lr = logry[k];
      // the whitened residual's squared norm (and its tangent) in the bulk
      // type; the log-pdf and the sum over observations in double (few
      // float64 operations: the FP64 pipe issues at 1/64 of the FP32 rate)
      T ww = T(0), wg[TG];
#pragma unroll
      for (int q = 0; q < TG; ++q) wg[q] = T(0);
#pragma unroll
      for (int j = 0; j < D; ++j) {
        const DT dx = DT(T(a.data[int64_t(k) * D + j])) - rm[0][j];
        const DT w = dx / ry;
        ww += w.v * w.v;
#pragma unroll
        for (int q = 0; q < TG; ++q) wg[q] += w.v * w.g[q];
#pragma unroll
        for (int i = 0; i < n; ++i) rm[i][j] = rm[i][j] + bay[k * (n + 1) + 1 + i] * dx;
      }
      DD pdf_n;
      pdf_n.v = -0.5 * (double(D) * (2.0 * lr + LOG2PI) + double(ww));
#pragma unroll
      for (int q = 0; q < TG; ++q) pdf_n.g[q] = -double(wg[q]);
      if (a.average_pdfs && num > 0) {
        pdf.v = (pdf.v * num + pdf_n.v) / (num + 1);
#pragma unroll
        for (int q = 0; q < TG; ++q) pdf.g[q] = (pdf.g[q] * num + pdf_n.g[q]) / (num + 1);
      } else {
        pdf.v += pdf_n.v;
#pragma unroll
        for (int q = 0; q < TG; ++q) pdf.g[q] += pdf_n.g[q];
      }
      ++num;
    }
    if (!(pdf.v == pdf.v)) status = PDQ_INSTANCE_NONFINITE;
  }
  const double nan = __longlong_as_double(0x7ff8000000000000ULL);
  if (dir == 0) {
    a.lml[b] = status == PDQ_INSTANCE_OK ? pdf.v : nan;
    a.status[b] = status;
  }
  if (a.grad && dir < P) a.grad[b * P + dir] = status == PDQ_INSTANCE_OK ? pdf.g[0] : nan;
}

}  // namespace pdq
