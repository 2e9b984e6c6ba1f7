// Reverse-mode (adjoint) gradient of the log-marginal likelihood, with
// sqrt(N) step checkpointing: the counterpart of jax.grad through
// solve_fixed_grid + loss_lml_timeseries, split into the two halves of a
// custom VJP.
//
//   lml_adj_fwd_kernel  value pass: the mean recursion of the fixed-point
//                       smoother on the fixed grid, the LML over the data;
//                       stores the residuals the backward pass needs -- the
//                       state every C steps, the backward conditionals'
//                       offsets xi at the observations and the innovations
//                       y_k - E[u(t_k)] of the LML recursion.
//   lml_adj_bwd_kernel  adjoint pass for a cotangent of the LML: the LML
//                       recursion in reverse (giving the adjoint of each xi
//                       and of the terminal mean), then the solver steps in
//                       reverse, one segment of C steps at a time: the
//                       segment's predicted states are recomputed from its
//                       checkpoint, then its steps are differentiated last
//                       to first.  Finally the Taylor-mode initialisation is
//                       differentiated (dual numbers), giving d lml / d params
//                       and d lml / d y0.
//
// As in the forward-mode kernel (lml_solver.cuh), every covariance-side
// quantity -- gains, the xi increment matrices K, the backward conditionals
// and the LML pass's observed stds and gains -- is parameter-free with TS0,
// the uncalibrated solver and a fixed step, and comes from the shared plan
// (lml_plan_kernel); the adjoint differentiates only the mean recursion:
//   step s (m = mean before the step, tables g_s, K_s of the plan)
//     xi   <- xi + K_s m                        (revert + merge, offset part)
//     mp    = p . A1 (p^-1 . m)                 (IsotropicLatentCond.marginalise, mean)
//     m'    = mp - g_s (mp[1] - f(mp[0]))       (TS0 update, revert_conditional)
//   LML, observations k = K-1 .. 0 (evaluate_lml, estimators_and_losses.py:180-218)
//     r     = to . (xi_k + A_k (tl . r))        (cond.marginalise, mean; not at k = K-1)
//     dx    = y_k - r[0];  pdf_k = -0.5 (2 log ry_k + (dx / ry_k)^2 + log 2 pi)
//     r    <- r + gain_k dx
// The adjoint of each line is its transpose; the vector field's Jacobian at
// the predicted state comes from one evaluation on dual numbers with d + P
// tangent directions (the same field definition).  The cost is independent
// of the number of parameters: one thread per sample runs the value pass,
// one recomputation and one reverse pass.
//
// Residual layout (type T, after the plan): element e of sample b at
// res[e * B + b], so the 32 samples of a warp, which run in lock step on the
// fixed grid, touch consecutive addresses.  The plan's step tables reach the
// warp through shared memory, a chunk of kLmlChunk steps at a time (one
// memory latency per chunk), in either direction; what a step or an
// observation reads from the residuals is loaded one step or observation
// ahead.  Per sample:
//   [0, S n d)              the state at steps 0, C, 2C, ... (S = ceil(N / C))
//   [OX, OX + (K-1) n d)    xi_k (forward pass); the adjoint of xi_k (backward pass)
//   [ODX, ODX + K d)        dx_k, the innovations of the LML recursion
//   [OSB, OSB + C d)        the predicted u of each step of the segment being reversed
#pragma once

#include "lml_solver.cuh"

namespace pdq {

struct LmlAdjArgs {
  LmlArgs base;             // plan, inputs, lml, status, grad (B, P) or nullptr
  int32_t ckpt;             // C, steps between stored states
  int32_t num_ckpt;         // S = ceil(num_steps / C)
  const double* cotangent;  // (B,) or nullptr (ones)
  double* grad_y0;          // (B, d) or nullptr
  void* res;                // residuals (layout above)
};

// Offsets (in elements of T) of the residual arrays of one sample.
struct LmlAdjLayout {
  int64_t ox, odx, osb, total;
  PDQ_HD LmlAdjLayout(int nu, int d, int num_steps, int save_every, int ckpt) {
    const int64_t n = nu + 1;
    const int64_t num_obs = num_steps / save_every + 1;
    const int64_t S = (int64_t(num_steps) + ckpt - 1) / ckpt;
    ox = S * n * d;
    odx = ox + (num_obs - 1) * n * d;
    osb = odx + num_obs * d;
    total = osb + int64_t(ckpt) * d;
  }
};

// The warp copies the step tables of chunk c (steps c * kLmlChunk + 1 ...,
// at most kLmlChunk of them) into shared memory with coalesced loads: one
// memory latency per chunk instead of one per step.  Every lane of the warp
// must call it at the same point (the fixed grid keeps the lanes in lock
// step; lanes without a sample stay in the loops for this).
template <typename T, int KS>
PDQ_D void lml_stage_chunk(T* stage, const T* plan, int chunk, int num_steps, int lane) {
  const int first = chunk * kLmlChunk;
  const int count = min(kLmlChunk, num_steps - first) * KS;
  const T* src = plan + int64_t(first) * KS;
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
    // host runs of the kernel bodies execute one lane at a time: it stages the whole chunk
    for (int e = 0; e < count; ++e) stage[e] = src[e];
  }
#endif
}

// One step's tables (g[n], K[n][n]) from the shared-memory stage into
// registers with 16-byte loads.
template <typename T, int KS>
PDQ_D void lml_read_step_table(const T* tbl, T (&dst)[KS]) {
  if constexpr (sizeof(T) == 4 && KS % 4 == 0) {
    const float4* v = reinterpret_cast<const float4*>(tbl);
#pragma unroll
    for (int e = 0; e < KS / 4; ++e) {
      const float4 x = v[e];
      dst[4 * e] = x.x;
      dst[4 * e + 1] = x.y;
      dst[4 * e + 2] = x.z;
      dst[4 * e + 3] = x.w;
    }
  } else if constexpr (sizeof(T) == 8 && KS % 2 == 0) {
    const double2* v = reinterpret_cast<const double2*>(tbl);
#pragma unroll
    for (int e = 0; e < KS / 2; ++e) {
      const double2 x = v[e];
      dst[2 * e] = x.x;
      dst[2 * e + 1] = x.y;
    }
  } else {
#pragma unroll
    for (int e = 0; e < KS; ++e) dst[e] = tbl[e];
  }
}

// What the LML recursion reads at observation k: the marginalisation's
// tables and offset (k < K-1), the observed std and gain, log|ry| and the
// data.  Loaded one observation ahead so the loads overlap the arithmetic.
template <typename T, int n, int D>
struct LmlObs {
  T xi[n][D];  // offset xi_k (value pass) or innovation dx_k in xi[0] (adjoint pass)
  T A[n][n], tl[n], to[n];
  T ry, gain[n];
  double lr, y[D];
};

template <typename T, int NU, int D>
PDQ_D void lml_load_obs(LmlObs<T, NU + 1, D>& o, int k, int num_obs, const T* obs_tbl, const T* bay,
                        const double* logry, const double* data, const T* res, int64_t ox, int64_t odx, int64_t B,
                        bool adjoint) {
  constexpr int n = NU + 1;
  if (k < num_obs - 1) {
    const T* t = obs_tbl + int64_t(k) * lml_plan_obs<NU>();
#pragma unroll
    for (int i = 0; i < n; ++i) {
#pragma unroll
      for (int q = 0; q < n; ++q) o.A[i][q] = t[i * n + q];
      o.tl[i] = t[2 * n * n + i];
      o.to[i] = t[2 * n * n + n + i];
    }
  }
  if (adjoint) {
#pragma unroll
    for (int j = 0; j < D; ++j) o.xi[0][j] = res[(odx + int64_t(k) * D + j) * B];
  } else {
    if (k < num_obs - 1) {
      const T* x = res + (ox + int64_t(k) * n * D) * B;
#pragma unroll
      for (int i = 0; i < n; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) o.xi[i][j] = x[int64_t(i * D + j) * B];
    }
    o.lr = logry[k];
#pragma unroll
    for (int j = 0; j < D; ++j) o.y[j] = data[int64_t(k) * D + j];
  }
  o.ry = bay[k * (n + 1)];
#pragma unroll
  for (int i = 0; i < n; ++i) o.gain[i] = bay[k * (n + 1) + 1 + i];
}

// One step of the mean recursion on values: predict, TS0 update with the
// plan's gain.  Shared by the value pass and the backward pass's
// recomputation so both produce the same predicted states.  mp0 returns the
// predicted u (the point where the vector field was evaluated).
template <typename T, int NU, class F>
PDQ_D void lml_value_step(T (&m)[NU + 1][F::D], const T* tb, const T (&p)[NU + 1], const T (&pinv)[NU + 1],
                          const T (&th)[F::P], T (&mp0)[F::D]) {
  constexpr int n = NU + 1;
  constexpr int D = F::D;
  constexpr int OUT = 1;
  T mp[n][D];
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      T acc = T(0);
#pragma unroll
      for (int k = i; k < n; ++k) acc += T(iwp_a<NU>(i, k)) * (pinv[k] * m[k][j]);
      mp[i][j] = p[i] * acc;
    }
  T f[D];
  F::eval(mp[0], th, f);
#pragma unroll
  for (int j = 0; j < D; ++j) mp0[j] = mp[0][j];
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) m[i][j] = mp[i][j] - tb[i] * (mp[OUT][j] - f[j]);
}

template <typename T, int NU, class F>
__global__ void __launch_bounds__(kLmlThreads) lml_adj_fwd_kernel(LmlAdjArgs aa) {
  const LmlArgs& a = aa.base;
  constexpr int n = NU + 1;
  constexpr int D = F::D;
  constexpr int P = F::P;
  constexpr int kStep = lml_plan_step<NU>();
  const int64_t B = a.B;
  const int64_t gb = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  // lanes past the batch stay for the warp's staging of the plan
  const bool valid = gb < B;
  const int64_t b = valid ? gb : 0;
  const int lane = threadIdx.x & 31;
  const int N = a.num_steps;
  const int C = aa.ckpt;
  const int num_obs = N / a.save_every + 1;
  const LmlAdjLayout L(NU, D, N, a.save_every, C);
  T* const res = reinterpret_cast<T*>(aa.res) + b;  // element e at res[e * B]
  const T* const plan = reinterpret_cast<const T*>(reinterpret_cast<const unsigned char*>(a.plan) + kLmlPlanKeyBytes);
  const T* const obs_tbl = plan + int64_t(N) * kStep;
  __shared__ __align__(16) T stage[kLmlChunk * kStep];  // one warp per block

  // ---- parameters; Taylor-mode initial derivatives in double ----
  double pd[P];
  T th[P];
#pragma unroll
  for (int k = 0; k < P; ++k) {
    pd[k] = a.params[b * P + k];
    th[k] = T(pd[k]);
  }
  double y0[D];
#pragma unroll
  for (int j = 0; j < D; ++j) y0[j] = a.y0[b * D + j];
  double tc[n][D];
  taylor_init<F, NU>(y0, pd, tc);
  T m[n][D], bxi[n][D];
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      m[i][j] = T(tc[i][j]);
      bxi[i][j] = T(0);
      if (valid) res[int64_t(i * D + j) * B] = m[i][j];  // checkpoint 0
    }
  const T h = T(a.dt);
  T p[n], pinv[n];
  precon<T, NU>(h, p, pinv);

  int status = PDQ_INSTANCE_OK;
  // counters and running pointers instead of run-time divisions per step
  int to_obs = a.save_every, to_ckpt = C;
  T* xi_dst = res + L.ox * B;          // offset of the next observation interval
  T* ck_dst = res + int64_t(n) * D * B;  // checkpoint 1
  for (int s = 1; s <= N; ++s) {
    const int within = (s - 1) & (kLmlChunk - 1);
    if (within == 0) lml_stage_chunk<T, kStep>(stage, plan, (s - 1) / kLmlChunk, N, lane);
    if (!valid || status != PDQ_INSTANCE_OK) continue;
    T tb[kStep];
    lml_read_step_table<T, kStep>(stage + within * kStep, tb);
    // the merged backward conditional's offset: xi + K m (m before the step)
#pragma unroll
    for (int i = 0; i < n; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) {
        T x = bxi[i][j];
#pragma unroll
        for (int k = 0; k < n; ++k) x = x + tb[n + i * n + k] * m[k][j];
        bxi[i][j] = x;
      }
    T mp0[D];
    lml_value_step<T, NU, F>(m, tb, p, pinv, th, mp0);
    if (!(m[0][0] == m[0][0])) {
      status = PDQ_INSTANCE_NONFINITE;  // stays in the loop for the staging
      continue;
    }
    if (--to_obs == 0) {
      to_obs = a.save_every;
#pragma unroll
      for (int i = 0; i < n; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) {
          xi_dst[int64_t(i * D + j) * B] = bxi[i][j];
          bxi[i][j] = T(0);
        }
      xi_dst += int64_t(n) * D * B;
    }
    if (--to_ckpt == 0) {
      to_ckpt = C;
      if (s < N) {
#pragma unroll
        for (int i = 0; i < n; ++i)
#pragma unroll
          for (int j = 0; j < D; ++j) ck_dst[int64_t(i * D + j) * B] = m[i][j];
        ck_dst += int64_t(n) * D * B;
      }
    }
  }
  if (!valid) return;

  // ---- LML: reverse Kalman filter over the data (evaluate_lml), storing the innovations ----
  double pdf = 0.0;
  if (status == PDQ_INSTANCE_OK) {
    T rm[n][D];
#pragma unroll
    for (int i = 0; i < n; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) rm[i][j] = m[i][j];
    const T* const bay = obs_tbl + int64_t(num_obs - 1) * lml_plan_obs<NU>() + n * n;
    const double* const logry = reinterpret_cast<const double*>(
                                    reinterpret_cast<const unsigned char*>(a.plan) +
                                    lml_plan_std_offset(NU, N, a.save_every, int(sizeof(T)))) + num_obs;
    const double LOG2PI = 1.8378770664093453;
    LmlObs<T, n, D> cur, nxt;
    lml_load_obs<T, NU, D>(cur, num_obs - 1, num_obs, obs_tbl, bay, logry, a.data, res, L.ox, L.odx, B, false);
    int num = 0;
    for (int k = num_obs - 1; k >= 0; --k) {
      if (k > 0) lml_load_obs<T, NU, D>(nxt, k - 1, num_obs, obs_tbl, bay, logry, a.data, res, L.ox, L.odx, B, false);
      if (k < num_obs - 1) {
        T pm[n][D];
#pragma unroll
        for (int i = 0; i < n; ++i)
#pragma unroll
          for (int j = 0; j < D; ++j) {
            T acc = cur.xi[i][j];
#pragma unroll
            for (int q = 0; q < n; ++q) acc = acc + cur.A[i][q] * (cur.tl[q] * rm[q][j]);
            pm[i][j] = cur.to[i] * acc;
          }
#pragma unroll
        for (int i = 0; i < n; ++i)
#pragma unroll
          for (int j = 0; j < D; ++j) rm[i][j] = pm[i][j];
      }
      // the whitened residual's squared norm in the bulk type; the log-pdf
      // and the sum over observations in double
      T ww = T(0);
#pragma unroll
      for (int j = 0; j < D; ++j) {
        const T dx = T(cur.y[j]) - rm[0][j];
        res[(L.odx + int64_t(k) * D + j) * B] = dx;
        const T w = dx / cur.ry;
        ww += w * w;
#pragma unroll
        for (int i = 0; i < n; ++i) rm[i][j] = rm[i][j] + cur.gain[i] * dx;
      }
      const double pdf_n = -0.5 * (double(D) * (2.0 * cur.lr + LOG2PI) + double(ww));
      if (a.average_pdfs && num > 0)
        pdf = (pdf * num + pdf_n) / (num + 1);
      else
        pdf += pdf_n;
      ++num;
      if (k > 0) cur = nxt;
    }
    if (!(pdf == pdf)) status = PDQ_INSTANCE_NONFINITE;
  }
  const double nan = __longlong_as_double(0x7ff8000000000000ULL);
  a.lml[b] = status == PDQ_INSTANCE_OK ? pdf : nan;
  a.status[b] = status;
}

template <typename T, int NU, class F>
__global__ void __launch_bounds__(kLmlThreads) lml_adj_bwd_kernel(LmlAdjArgs aa) {
  const LmlArgs& a = aa.base;
  constexpr int n = NU + 1;
  constexpr int D = F::D;
  constexpr int P = F::P;
  constexpr int NT = D + P;  // tangent directions of the Jacobian evaluation
  constexpr int kStep = lml_plan_step<NU>();
  const int64_t B = a.B;
  const int64_t gb = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const bool in_batch = gb < B;
  const int64_t b = in_batch ? gb : 0;
  const int lane = threadIdx.x & 31;
  const double nan = __longlong_as_double(0x7ff8000000000000ULL);
  // samples whose value pass failed get NaN gradients; their lanes (and
  // lanes past the batch) stay for the warp's staging of the plan
  const bool valid = in_batch && a.status[b] == PDQ_INSTANCE_OK;
  if (in_batch && !valid) {
    if (a.grad) {
#pragma unroll
      for (int q = 0; q < P; ++q) a.grad[b * P + q] = nan;
    }
    if (aa.grad_y0) {
#pragma unroll
      for (int j = 0; j < D; ++j) aa.grad_y0[b * D + j] = nan;
    }
  }
  const int N = a.num_steps;
  const int C = aa.ckpt;
  const int num_obs = N / a.save_every + 1;
  const LmlAdjLayout L(NU, D, N, a.save_every, C);
  T* const res = reinterpret_cast<T*>(aa.res) + b;
  const T* const plan = reinterpret_cast<const T*>(reinterpret_cast<const unsigned char*>(a.plan) + kLmlPlanKeyBytes);
  const T* const obs_tbl = plan + int64_t(N) * kStep;
  const T* const bay = obs_tbl + int64_t(num_obs - 1) * lml_plan_obs<NU>() + n * n;
  __shared__ __align__(16) T stage[kLmlChunk * kStep];  // one warp per block
  // d loss / d pdf_k: the cotangent, divided by the number of terms for averaged pdfs
  const double scale =
      valid ? (aa.cotangent ? aa.cotangent[b] : 1.0) / (a.average_pdfs ? double(num_obs) : 1.0) : 0.0;
  const T tscale = T(scale);

  // ---- the LML recursion in reverse: adjoints of xi_k and of the terminal mean ----
  T rb[n][D];
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) rb[i][j] = T(0);
  if (valid) {
    LmlObs<T, n, D> cur, nxt;
    lml_load_obs<T, NU, D>(cur, 0, num_obs, obs_tbl, bay, nullptr, nullptr, res, L.ox, L.odx, B, true);
    for (int k = 0; k < num_obs; ++k) {
      if (k + 1 < num_obs)
        lml_load_obs<T, NU, D>(nxt, k + 1, num_obs, obs_tbl, bay, nullptr, nullptr, res, L.ox, L.odx, B, true);
#pragma unroll
      for (int j = 0; j < D; ++j) {
        // r <- r + gain dx, dx = y - r[0], pdf = -0.5 (dx / ry)^2 + ...: d pdf / d dx = -dx / ry^2
        T t = T(0);
#pragma unroll
        for (int i = 0; i < n; ++i) t += cur.gain[i] * rb[i][j];
        const T w = cur.xi[0][j] / cur.ry;
        rb[0][j] -= t - tscale * (w / cur.ry);
      }
      if (k < num_obs - 1) {
        // r = to . (xi_k + A_k (tl . r))
        T* xib = res + (L.ox + int64_t(k) * n * D) * B;
        T x[n][D];
#pragma unroll
        for (int i = 0; i < n; ++i)
#pragma unroll
          for (int j = 0; j < D; ++j) {
            x[i][j] = cur.to[i] * rb[i][j];
            xib[int64_t(i * D + j) * B] = x[i][j];
          }
#pragma unroll
        for (int q = 0; q < n; ++q)
#pragma unroll
          for (int j = 0; j < D; ++j) {
            T acc = T(0);
#pragma unroll
            for (int i = 0; i < n; ++i) acc += cur.A[i][q] * x[i][j];
            rb[q][j] = cur.tl[q] * acc;
          }
      }
      if (k + 1 < num_obs) cur = nxt;
    }
  }

  // ---- the solver steps in reverse, one checkpointed segment at a time ----
  double pd[P];
  T th[P];
#pragma unroll
  for (int k = 0; k < P; ++k) {
    pd[k] = a.params[b * P + k];
    th[k] = T(pd[k]);
  }
  const T h = T(a.dt);
  T p[n], pinv[n];
  precon<T, NU>(h, p, pinv);
  // d lml / d theta: partial sums over an observation interval in the bulk
  // type (thp), added to the double total (thb) once per interval
  double thb[P];
  T thp[P];
#pragma unroll
  for (int q = 0; q < P; ++q) {
    thb[q] = 0.0;
    thp[q] = T(0);
  }
  T mb[n][D];  // adjoint of the mean after the current step
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) mb[i][j] = rb[i][j];

  int staged = -1;            // chunk of step tables in `stage`
  int kobs = -1, knext = -1;  // observation intervals of xib and of the prefetched xin
  T xib[n][D], xin[n][D];
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) xib[i][j] = xin[i][j] = T(0);
  for (int seg = aa.num_ckpt - 1; seg >= 0; --seg) {
    const int s0 = seg * C;
    const int s1 = min(N, s0 + C);
    // recompute the segment's predicted states from its checkpoint
    {
      T m[n][D];
      const T* src = res + int64_t(seg) * n * D * B;
#pragma unroll
      for (int i = 0; i < n; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) m[i][j] = valid ? src[int64_t(i * D + j) * B] : T(0);
      T* sb = res + L.osb * B;  // predicted u of step s0 + 1, then onwards
      for (int s = s0 + 1; s <= s1; ++s) {
        const int c = (s - 1) / kLmlChunk;
        if (c != staged) {
          lml_stage_chunk<T, kStep>(stage, plan, c, N, lane);
          staged = c;
        }
        if (!valid) continue;
        T tb[kStep];
        lml_read_step_table<T, kStep>(stage + (s - 1 - c * kLmlChunk) * kStep, tb);
        T mp0[D];
        lml_value_step<T, NU, F>(m, tb, p, pinv, th, mp0);
#pragma unroll
        for (int j = 0; j < D; ++j) sb[int64_t(j) * B] = mp0[j];
        sb += int64_t(D) * B;
      }
    }
    // differentiate the segment's steps, last to first
    const T* sb = res + (L.osb + int64_t(s1 - s0 - 1) * D) * B;  // predicted u of step s1, then backwards
    T u1[D];  // the predicted u of the next step to differentiate (loaded one step ahead)
#pragma unroll
    for (int j = 0; j < D; ++j) u1[j] = valid ? sb[int64_t(j) * B] : T(0);
    // observation interval k of step s and its position r within it: s - 1 = k save_every + r
    int k = (s1 - 1) / a.save_every;
    int r = (s1 - 1) - k * a.save_every;
    for (int s = s1; s > s0; --s) {
      const int c = (s - 1) / kLmlChunk;
      if (c != staged) {
        lml_stage_chunk<T, kStep>(stage, plan, c, N, lane);
        staged = c;
      }
      if (!valid) continue;
      T u[D];
#pragma unroll
      for (int j = 0; j < D; ++j) u[j] = u1[j];
      if (s - 1 > s0) {
        sb -= int64_t(D) * B;
#pragma unroll
        for (int j = 0; j < D; ++j) u1[j] = sb[int64_t(j) * B];
      }
      if (k != kobs) {
        if (k == knext) {
#pragma unroll
          for (int i = 0; i < n; ++i)
#pragma unroll
            for (int j = 0; j < D; ++j) xib[i][j] = xin[i][j];
        } else {
          const T* x = res + (L.ox + int64_t(k) * n * D) * B;
#pragma unroll
          for (int i = 0; i < n; ++i)
#pragma unroll
            for (int j = 0; j < D; ++j) xib[i][j] = x[int64_t(i * D + j) * B];
        }
        kobs = k;
        knext = k - 1;
        if (knext >= 0) {
          const T* x = res + (L.ox + int64_t(knext) * n * D) * B;
#pragma unroll
          for (int i = 0; i < n; ++i)
#pragma unroll
            for (int j = 0; j < D; ++j) xin[i][j] = x[int64_t(i * D + j) * B];
        }
      }
      T tb[kStep];
      lml_read_step_table<T, kStep>(stage + (s - 1 - c * kLmlChunk) * kStep, tb);
      // m' = mp - g (mp[1] - f(mp[0]))
      T rbar[D];
#pragma unroll
      for (int j = 0; j < D; ++j) {
        T acc = T(0);
#pragma unroll
        for (int i = 0; i < n; ++i) acc += tb[i] * mb[i][j];
        rbar[j] = -acc;  // adjoint of the residual mp[1] - f
      }
      T mpb[n][D];
#pragma unroll
      for (int i = 0; i < n; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) mpb[i][j] = mb[i][j];
#pragma unroll
      for (int j = 0; j < D; ++j) mpb[1][j] += rbar[j];
      // f(mp[0], theta): Jacobian on dual numbers (directions: u, then theta)
      {
        Dual<T, NT> ud[D], pt[P], f[D];
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
        F::eval(ud, pt, f);
#pragma unroll
        for (int j = 0; j < D; ++j) {
          T acc = T(0);
#pragma unroll
          for (int l = 0; l < D; ++l) acc += f[l].g[j] * rbar[l];
          mpb[0][j] -= acc;  // f enters the residual with a minus sign
        }
#pragma unroll
        for (int q = 0; q < P; ++q) {
          T acc = T(0);
#pragma unroll
          for (int l = 0; l < D; ++l) acc += f[l].g[D + q] * rbar[l];
          thp[q] -= acc;
        }
      }
      // mp = p . A1 (p^-1 . m), and xi_k += K m
#pragma unroll
      for (int k2 = 0; k2 < n; ++k2)
#pragma unroll
        for (int j = 0; j < D; ++j) {
          T acc = T(0);
#pragma unroll
          for (int i = 0; i <= k2; ++i) acc += T(iwp_a<NU>(i, k2)) * (p[i] * mpb[i][j]);
          T x = pinv[k2] * acc;
#pragma unroll
          for (int i = 0; i < n; ++i) x += tb[n + i * n + k2] * xib[i][j];
          mb[k2][j] = x;
        }
      if (--r < 0) {
        r = a.save_every - 1;
        --k;
#pragma unroll
        for (int q = 0; q < P; ++q) {
          thb[q] += double(thp[q]);
          thp[q] = T(0);
        }
      }
    }
  }
  if (!valid) return;
#pragma unroll
  for (int q = 0; q < P; ++q) thb[q] += double(thp[q]);

  // ---- the Taylor-mode initialisation: d m_0 / d (theta, y0) on dual numbers (bulk type) ----
  constexpr int NI = P + D;
  Dual<T, NI> pdd[P], ydd[D];
#pragma unroll
  for (int q = 0; q < P; ++q) {
    pdd[q] = Dual<T, NI>(th[q]);
    pdd[q].g[q] = T(1);
  }
#pragma unroll
  for (int j = 0; j < D; ++j) {
    ydd[j] = Dual<T, NI>(T(a.y0[b * D + j]));
    ydd[j].g[P + j] = T(1);
  }
  Dual<T, NI> tcd[n][D];
  taylor_init<F, NU>(ydd, pdd, tcd);
  T acc[NI];
#pragma unroll
  for (int q = 0; q < NI; ++q) acc[q] = T(0);
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j)
#pragma unroll
      for (int q = 0; q < NI; ++q) acc[q] += mb[i][j] * tcd[i][j].g[q];
#pragma unroll
  for (int q = 0; q < P; ++q) thb[q] += double(acc[q]);
  double yb[D];
#pragma unroll
  for (int j = 0; j < D; ++j) yb[j] = double(acc[P + j]);
  if (a.grad) {
#pragma unroll
    for (int q = 0; q < P; ++q) a.grad[b * P + q] = thb[q];
  }
  if (aa.grad_y0) {
#pragma unroll
    for (int j = 0; j < D; ++j) aa.grad_y0[b * D + j] = yb[j];
  }
}

}  // namespace pdq
