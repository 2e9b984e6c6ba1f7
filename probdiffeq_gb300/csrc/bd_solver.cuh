// Block-diagonal TS0 adaptive solver for high-dimensional ODEs (d up to a
// few thousand per instance), one thread-block CLUSTER per instance.
//
// Follows the reference's block-diagonal path per dimension j:
//   BlockDiagWienerIntegrated.transition  _probdiffeq/ssm_impl_blockdiag.py:406-432 (per-dim scale)
//   BlockDiagLatentCond.apply_flat / marginalise / revert  ssm_impl_blockdiag.py:19-102
//   BlockDiagOdeTs0.linearize             ssm_impl_blockdiag.py:129-144
//   residual_whitened_rms_flat (per dim)  ssm_impl_blockdiag.py:285-292
//   solver_dynamic / solver_mle / solver  _probdiffeq/solvers.py (per-dim output scale)
//   error_residual_std (error (d,), rms over d)  solvers.py:925-996
//   control, RejectionLoop with clip_dt   _ivpsolve/*.py
// The vector field couples dimensions only through the stencil of f; the
// error norm couples them through one sum over d.
//
// GB300 mapping: the instance's d dimensions are split contiguously over the
// CL CTAs of a cluster; a thread owns dimensions tid, tid + 256, ... of its
// CTA and works on one of them at a time (a runtime loop, so the register
// footprint is one dimension's and two CTAs fit on an SM).  Each attempt:
//   1. every thread extrapolates its dimensions and stages the extrapolated
//      means (all n coefficients) in its CTA's shared memory;  cluster barrier;
//   2. f at its dimensions reads the two stencil neighbours, from distributed
//      shared memory of the neighbouring CTA at the CTA boundary; the
//      per-dimension predict/update follows; the error-norm partial (a wide
//      sum: float pair in float32, double in float64) is reduced in the CTA
//      and published in shared memory;  cluster barrier;
//   3. every CTA sums the CL partials over DSMEM in rank order and takes the
//      same accept/step decision.
// The per-dimension state (mean n, lower Cholesky n(n+1)/2) lives in two
// scratch buffers in global memory (L2-resident: 64 x 4096 x 14 floats is
// 15 MB per buffer), coalesced across a warp's consecutive dimensions; the
// proposal is written to the other buffer, so an accept is a parity flip.
// Time, step size and controller follow the isotropic kernel: Wide<T> time,
// T controller, no float64 on the attempt path of the float32 kernel.
//
// FP: the fixed-point smoother (estimators_and_losses.py:473-591 with the
// block-diagonal revert / merge, ssm_impl_blockdiag.py:45-102), per
// dimension: every attempt reverts the prior transition instead of
// marginalising it and merges the backward conditional into the running one;
// the running conditionals (iso_cond_floats<NU, 1> numbers per dimension)
// live in two more parity buffers next to the state, are copied out at every
// checkpoint (exact landings) and reset to the identity; after the last step
// the backward pass marginalises each dimension's terminal state through the
// stored conditionals (Smoother.finalize, MarkovSequence.evaluate_marginals).
#pragma once

#include "iso_solver.cuh"

namespace pdq {

// Thread-block-cluster operations (those of cooperative_groups'
// cluster_group, on the device intrinsics, so that the kernel also compiles
// under NVRTC, which has no toolkit headers): the block's rank in its
// cluster, the cluster barrier (arrive with release, wait with acquire
// semantics), and the address of the same shared-memory variable in
// another block of the cluster.
// The kernel's shared memory: the dynamic part and the fixed arrays (a host
// run of the kernel body supplies per-block buffers instead).
#ifndef PDQ_BD_SMEM
#define PDQ_BD_SMEM extern __shared__ unsigned char smem_raw[]
#endif
#ifndef PDQ_BD_SHARED
#define PDQ_BD_SHARED(type, name, count) __shared__ type name[count]
#endif

struct Cluster {
  PDQ_D unsigned block_rank() const { return __clusterRelativeBlockRank(); }
  PDQ_D void sync() const {
    __cluster_barrier_arrive();
    __cluster_barrier_wait();
  }
  template <typename T>
  PDQ_D T* map_shared_rank(T* p, int rank) const {
    return static_cast<T*>(__cluster_map_shared_rank(const_cast<void*>(static_cast<const void*>(p)), unsigned(rank)));
  }
};

constexpr int kBdThreads = 256;
constexpr int kBdMaxDimsPerThread = 8;

struct BdArgs {
  int64_t B;
  int32_t S, terminal_only, solver, control, correct, d, cluster;
  int32_t ts1;  // 1: TS1 with the Jacobian diagonal along d (per-dimension H_j = [-dfj/duj, 1, 0, ...])
  int32_t state_error;  // 0: error_residual_std; 1: error_state_std (derivative 0)
  int32_t fixedpoint;   // 1: the fixed-point smoother
  double safety, factor_min, factor_max, exp_i, exp_p;
  double atol, rtol, eps, damp;
  int64_t max_attempts;
  double q1[kMaxN][kMaxN];
  float q1f[kMaxN][kMaxN];
  float safety_f, factor_min_f, factor_max_f, exp_i_f, exp_p_f;
  float atol_f, rtol_f, eps_f, damp_f;
  const double* save_at;
  const double* params;  // (B, 1): viscosity
  const double* y0;      // (B, d)
  const double* dt0;
  double* u_mean;        // (B, S_out, d, n); the fixed-point smoother writes the smoothed marginals
  double* u_chol;        // (B, S_out, d, n, n)
  double* output_scale;  // (B, S_out, d)
  double* t_out;
  int32_t* num_steps;
  int32_t* num_attempts;
  int32_t* status;
  void* workspace;       // 2 state buffers (B, ns, d) in T, then MLE sums (B, d), 8 bytes each;
                         // FP: then 2 conditional buffers (B, cf, d) and the checkpoints' (B, S - 1, cf, d) in T
  // optional fixed-point outputs (nullptr: not written): the posterior's
  // backward conditionals between consecutive checkpoints, per dimension,
  // in the reference's block-diagonal layout, and the filtering marginals
  double* cond_A;            // (B, S - 1, d, n, n)
  double* cond_noise_mean;   // (B, S - 1, d, n)
  double* cond_noise_chol;   // (B, S - 1, d, n, n), calibrated
  double* cond_to_latent;    // (B, S - 1, d, n)
  double* cond_to_observed;  // (B, S - 1, d, n)
  double* filter_mean;       // (B, S, d, n)
  double* filter_chol;       // (B, S, d, n, n), calibrated
};

// Conditional of one dimension in a strided buffer (element e of dimension g at e * d + g).
template <typename T, int NU>
PDQ_D void bd_cond_store(T* base, int64_t stride, const IsoBackward<T, NU, 1>& c) {
  constexpr int n = NU + 1;
  int o = 0;
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < n; ++j) base[(o++) * stride] = c.A[i][j];
#pragma unroll
  for (int i = 0; i < n; ++i) base[(o++) * stride] = c.xi[i][0];
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j <= i; ++j) base[(o++) * stride] = c.X[i][j];
#pragma unroll
  for (int i = 0; i < n; ++i) base[(o++) * stride] = c.tl[i];
#pragma unroll
  for (int i = 0; i < n; ++i) base[(o++) * stride] = c.to[i];
}

template <typename T, int NU>
PDQ_D void bd_cond_load(const T* base, int64_t stride, IsoBackward<T, NU, 1>& c) {
  constexpr int n = NU + 1;
  int o = 0;
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < n; ++j) c.A[i][j] = base[(o++) * stride];
#pragma unroll
  for (int i = 0; i < n; ++i) c.xi[i][0] = base[(o++) * stride];
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < n; ++j) c.X[i][j] = (j <= i) ? base[(o++) * stride] : T(0);
#pragma unroll
  for (int i = 0; i < n; ++i) c.tl[i] = base[(o++) * stride];
#pragma unroll
  for (int i = 0; i < n; ++i) c.to[i] = base[(o++) * stride];
}

template <int NU>
PDQ_HD constexpr int bd_state_rows() {
  return (NU + 1) + (NU + 1) * (NU + 2) / 2;
}

// Dynamic shared memory per CTA: staged means (n x dl), new terms and scales
// (2 x dl), current scales (dl), in T.
template <typename T, int NU>
PDQ_HD size_t bd_smem_bytes(int dl) {
  return size_t(NU + 1 + 3) * size_t(dl) * sizeof(T);
}

// Stencil fields of the block-diagonal kernel: component j of f depends on
// u_{j-1}, u_j, u_{j+1} (periodic in j), the parameters p and the grid's
// inverse spacing inv_dx = d; written once, generic over the scalar type S
// (the bulk type for the attempts, float64 jets for the Taylor-mode start):
//   struct Stencil {
//     static constexpr int P = ...;  // number of parameters
//     template <typename S, typename T>
//     PDQ_HD static S eval(const S& left, const S& mid, const S& right, const T* p, T inv_dx);
//   };
// TS1 needs the Jacobian's diagonal d f_j / d u_j; the kernel takes it from
// a stencil that declares it the same for every j (kConstantDiagonal,
// diag(p, inv_dx)), as the Burgers stencil's is.
//
// Viscous Burgers with periodic central differences (the flux-form stencil
// of benchmarks/A5_work-precision-burgers-pde.py:124-134, periodic wrap).
struct BurgersStencil {
  static constexpr int P = 1;  // viscosity
  static constexpr bool kConstantDiagonal = true;
  template <typename S, typename T>
  PDQ_HD static S eval(const S& left, const S& mid, const S& right, const T* p, T inv_dx) {
    const S flux = (right * right - left * left) * (T(0.25) * inv_dx);
    const S lap = (right - T(2) * mid + left) * (inv_dx * inv_dx);
    return -flux + p[0] * lap;
  }
  // the central-difference flux term does not involve u_j
  template <typename T>
  PDQ_HD static T diag(const T* p, T inv_dx) {
    return -(T(2) * p[0] * inv_dx * inv_dx);
  }
};

// Whether a stencil declares a constant Jacobian diagonal (TS1 available).
template <class ST, class = void>
struct StencilConstantDiagonal {
  static constexpr bool value = false;
};
template <class ST>
struct StencilConstantDiagonal<ST, decltype(void(ST::kConstantDiagonal))> {
  static constexpr bool value = ST::kConstantDiagonal;
};

template <typename T, int NU, bool FP = false, class ST = BurgersStencil>
__global__ void __launch_bounds__(kBdThreads, 2) bd_adaptive_kernel(BdArgs a) {
  constexpr int n = NU + 1;
  constexpr int NS = bd_state_rows<NU>();
  constexpr int CF = iso_cond_floats<NU, 1>();
  constexpr int OUT = 1;
  constexpr bool kNarrow = sizeof(T) == sizeof(float);
  using W = Wide<T>;
  const Cluster cluster;
  const int CL = a.cluster;
  const int rank = int(cluster.block_rank());
  const int64_t inst = blockIdx.x / CL;
  if (inst >= a.B) return;  // uniform per cluster
  const int d = a.d;
  const int dl = d / CL;
  const int j0 = rank * dl;
  const int tid = threadIdx.x;

  PDQ_BD_SMEM;
  T* mps = reinterpret_cast<T*>(smem_raw);  // [n][dl] extrapolated means of this CTA's dimensions
  T* newt = mps + n * dl;                   // [dl] whitened residual of the proposal (MLE)
  T* sig_new = newt + dl;                   // [dl] local scale of the proposal (dynamic)
  T* sig = sig_new + dl;                    // [dl] output scale of the current state
  PDQ_BD_SHARED(W, partial, 2);                  // CTA partial sums (error norm), parity
  PDQ_BD_SHARED(W, warp_sums, kBdThreads / 32);

  T* const buf0 = reinterpret_cast<T*>(a.workspace);
  T* const bufs[2] = {buf0 + inst * NS * int64_t(d), buf0 + (a.B + inst) * NS * int64_t(d)};
  W* mle_sum = reinterpret_cast<W*>(buf0 + 2 * a.B * NS * int64_t(d)) + inst * int64_t(d);
  // FP: running conditionals (parity buffers like the state) and the checkpoints'
  T* const cond0 = reinterpret_cast<T*>(reinterpret_cast<W*>(buf0 + 2 * a.B * NS * int64_t(d)) + a.B * int64_t(d));
  T* const cbufs[2] = {cond0 + inst * CF * int64_t(d), cond0 + (a.B + inst) * CF * int64_t(d)};
  T* const ckpt = cond0 + 2 * a.B * CF * int64_t(d) + inst * int64_t(a.S - 1) * CF * int64_t(d);

  constexpr int P = ST::P;
  double pd[P > 0 ? P : 1];
  T pt[P > 0 ? P : 1];
#pragma unroll
  for (int k = 0; k < P; ++k) {
    pd[k] = a.params[inst * P + k];
    pt[k] = T(pd[k]);
  }
  const T inv_dx = T(d);
  const int S = a.S;
  const int S_out = a.terminal_only ? 1 : S;
  const double* save_at = a.save_at + inst * S;

  // ---- Taylor-mode initial derivatives through the stencil (float64 jets) ----
  // coefficient k of every dimension lives in row k of buffer 0 as a
  // normalised Taylor coefficient during the recursion.
  T* st = bufs[0];
  for (int jl = tid; jl < dl; jl += kBdThreads) {
    const int g = j0 + jl;
    st[0 * d + g] = T(a.y0[inst * d + g]);
  }
  __threadfence();
  cluster.sync();
  for (int k = 0; k < NU; ++k) {
    for (int jl = tid; jl < dl; jl += kBdThreads) {
      const int g = j0 + jl;
      const int gl = (g - 1 + d) % d, gr = (g + 1) % d;
      // coefficient k of f from coefficients 0 .. k of the neighbours (the stencil on jets)
      Jet<double, NU + 1> jl_, jm, jr;
      for (int l = 0; l <= k; ++l) {
        jl_.c[l] = double(st[l * d + gl]);
        jm.c[l] = double(st[l * d + g]);
        jr.c[l] = double(st[l * d + gr]);
      }
      const Jet<double, NU + 1> fj = ST::eval(jl_, jm, jr, static_cast<const double*>(pd), double(d));
      st[(k + 1) * d + g] = T(fj.c[k] / (k + 1));
    }
    __threadfence();
    cluster.sync();
  }
  // to derivatives; Cholesky rows zero (exact initial coefficients)
  for (int jl = tid; jl < dl; jl += kBdThreads) {
    const int g = j0 + jl;
    for (int k = 0; k < n; ++k) st[k * d + g] = T(double(st[k * d + g]) * factorial(k));
    for (int r = n; r < NS; ++r) st[r * d + g] = T(0);
    mle_sum[g] = wide_from(0.0, T(0));
    sig[jl] = T(1);
    if constexpr (FP) {
      IsoBackward<T, NU, 1> id;
      iso_cond_identity(id);
      bd_cond_store<T, NU>(cbufs[0] + g, d, id);
    }
  }
  __threadfence();
  cluster.sync();

  W t = wide_from(save_at[0], T(0));
  T dt = T(a.dt0[inst]);
  T pi_prev = T(1);
  int cur = 0, num_steps = 0, attempts = 0, status = PDQ_INSTANCE_OK, num_data = 0, par = 0;
  const T damp = cst<T>(a.damp, a.damp_f);
  const T atol = cst<T>(a.atol, a.atol_f), rtol = cst<T>(a.rtol, a.rtol_f);
  const T safety = cst<T>(a.safety, a.safety_f);
  const T factor_min = cst<T>(a.factor_min, a.factor_min_f), factor_max = cst<T>(a.factor_max, a.factor_max_f);
  const T eps = cst<T>(a.eps, a.eps_f);
  T q1_out2 = T(0);
#pragma unroll
  for (int j = 0; j < n; ++j) q1_out2 += cst<T>(a.q1[OUT][j], a.q1f[OUT][j]) * cst<T>(a.q1[OUT][j], a.q1f[OUT][j]);
  const T q1_out_norm = dev_sqrt(q1_out2);
  const T q00 = cst<T>(a.q1[0][0], a.q1f[0][0]), q10 = cst<T>(a.q1[1][0], a.q1f[1][0]),
          q11 = cst<T>(a.q1[1][1], a.q1f[1][1]);

  auto before = [&](const W& x, const W& y) -> bool {
    if constexpr (kNarrow) {
      return wide_diff(y, x) > eps;
    } else {
      return x + a.eps < y;
    }
  };

  auto write_checkpoint = [&](int s_out, double tt) {
    const T* x = bufs[cur];
    const int64_t rec = inst * S_out + s_out;
    for (int jl = tid; jl < dl; jl += kBdThreads) {
      const int g = j0 + jl;
      double* um = a.u_mean + (rec * d + g) * n;
      double* uc = a.u_chol + (rec * d + g) * n * n;
      for (int i = 0; i < n; ++i) um[i] = double(x[i * d + g]);
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) uc[i * n + j] = (j <= i) ? double(x[(n + i * (i + 1) / 2 + j) * d + g]) : 0.0;
    }
    if (rank == 0 && tid == 0) {
      a.t_out[rec] = tt;
      a.num_steps[rec] = num_steps;
    }
  };
  // FP: the filtering marginal at checkpoint s (the state, before the
  // calibration, which the finalize step applies)
  auto write_filter = [&](int s) {
    if (!a.filter_mean) return;
    const T* x = bufs[cur];
    const int64_t rec = inst * S + s;
    for (int jl = tid; jl < dl; jl += kBdThreads) {
      const int g = j0 + jl;
      double* fm = a.filter_mean + (rec * d + g) * n;
      double* fc = a.filter_chol + (rec * d + g) * n * n;
      for (int i = 0; i < n; ++i) fm[i] = double(x[i * d + g]);
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) fc[i * n + j] = (j <= i) ? double(x[(n + i * (i + 1) / 2 + j) * d + g]) : 0.0;
    }
  };
  auto write_scale = [&](int s_out) {
    const int64_t rec = inst * S_out + s_out;
    for (int jl = tid; jl < dl; jl += kBdThreads) a.output_scale[rec * d + j0 + jl] = double(sig[jl]);
  };

  if (!a.terminal_only) {
    write_checkpoint(0, wide_value(t));
    for (int jl = tid; jl < dl; jl += kBdThreads) a.output_scale[(inst * S_out) * d + j0 + jl] = 1.0;
  }
  if (FP) write_filter(0);

  for (int s = 1; s < S && status == PDQ_INSTANCE_OK; ++s) {
    const W t_next = wide_from(save_at[s], T(0));
    while (before(t, t_next) && status == PDQ_INSTANCE_OK) {
      const T remaining = wide_diff(t_next, t);
      const bool clipped = !(dt < remaining);  // clip_dt
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
      T p[n], pinv[n];
      precon<T, NU>(h, p, pinv);
      const T sq_h = fast_sqrt(dev_abs(h));
      // TS1 (ssm_impl_blockdiag.py:147-183, jacobians.py:108-113): the Burgers
      // Jacobian's diagonal is d f_j / d u_j = -2 nu / dx^2 for every j (the
      // central-difference flux term does not involve u_j), so H_j = [h0, 1, 0, ...]
      // with one h0 for all dimensions
      T h0 = T(0);
      if constexpr (StencilConstantDiagonal<ST>::value) {
        if (a.ts1) h0 = -ST::diag(static_cast<const T*>(pt), inv_dx);
      }
      const T ell = a.ts1 ? observed_std_ts1<T, NU>(p[OUT], h, h0, q00, q10, q11, damp)
                          : observed_std(p[OUT], h, q1_out_norm, damp);
      // error_state_std: the conditioned unit-scale std of u is the same for
      // every dimension (one H, one unit-scale factor), so it is formed once
      const T std0 = a.state_error ? state_std0<T, NU, OUT>(a, p, h, damp, h0) : T(0);
      const T* __restrict__ x = bufs[cur];  // the two state buffers never alias
      T* __restrict__ y = bufs[cur ^ 1];

      // ---- phase 1: extrapolated means staged in shared memory ----
#pragma unroll(FP ? 1 : 2)
      for (int jl = tid; jl < dl; jl += kBdThreads) {
        const int g = j0 + jl;
        T m[n];
#pragma unroll
        for (int i = 0; i < n; ++i) m[i] = x[i * d + g];
#pragma unroll
        for (int i = 0; i < n; ++i) {
          T acc = T(0);
#pragma unroll
          for (int kk = i; kk < n; ++kk) acc += T(iwp_a<NU>(i, kk)) * pinv[kk] * m[kk];
          mps[i * dl + jl] = p[i] * acc;
        }
      }
      cluster.sync();

      // ---- phase 2: stencil, calibration, predict, update, error partial ----
      const T* ex_left = cluster.map_shared_rank(mps, (rank - 1 + CL) % CL);
      const T* ex_right = cluster.map_shared_rank(mps, (rank + 1) % CL);
      W local = wide_from(0.0, T(0));
      T pinv_abs[n];
#pragma unroll
      for (int i = 0; i < n; ++i) pinv_abs[i] = dev_abs(pinv[i]);
#pragma unroll(FP ? 1 : 2)
      for (int jl = tid; jl < dl; jl += kBdThreads) {
        const int g = j0 + jl;
        const T left = jl > 0 ? mps[jl - 1] : ex_left[dl - 1];
        const T right = jl < dl - 1 ? mps[jl + 1] : ex_right[0];
        T mp[n];
#pragma unroll
        for (int i = 0; i < n; ++i) mp[i] = mps[i * dl + jl];
        const T f = ST::eval(left, mp[0], right, static_cast<const T*>(pt), inv_dx);
        const T mobs = mp[OUT] - f;
        // per-dimension residual_whitened_rms of fx.marginalise(apply_flat(m))
        const T sigma = dev_div(dev_abs(mobs), ell);
        const T s_pred = (a.solver == PDQ_SOLVER_DYNAMIC) ? sigma : T(1);
        T L[n][n];
#pragma unroll
        for (int i = 0; i < n; ++i)
#pragma unroll
          for (int j = 0; j < n; ++j) L[i][j] = (j <= i) ? x[(n + i * (i + 1) / 2 + j) * d + g] : T(0);
        // the block-diagonal marginalise scales the factor by |p_inv| (ssm_impl_blockdiag.py:32)
        T Lp[n][n];
        if constexpr (FP) {
          // revert (ssm_impl_blockdiag.py:69-102), merge into the running conditional (:45-67)
          T mcol[n][1];
#pragma unroll
          for (int i = 0; i < n; ++i) mcol[i][0] = x[i * d + g];
          IsoBackward<T, NU, 1> cnew, bwj, merged;
          if constexpr (kNarrow) {
            iso_prior_revert<T, NU, 1>(a.q1f, mcol, L, p, pinv, s_pred * sq_h, Lp, cnew);
          } else {
            iso_prior_revert<T, NU, 1>(a.q1, mcol, L, p, pinv, s_pred * sq_h, Lp, cnew);
          }
          bd_cond_load<T, NU>(cbufs[cur] + g, d, bwj);
          iso_cond_merge(bwj, cnew, merged);
          bd_cond_store<T, NU>(cbufs[cur ^ 1] + g, d, merged);
        } else if constexpr (kNarrow) {
          iso_predict_chol<T, NU>(a.q1f, L, p, pinv_abs, s_pred * sq_h, Lp);
        } else {
          iso_predict_chol<T, NU>(a.q1, L, p, pinv_abs, s_pred * sq_h, Lp);
        }
        T gain[n], Lnew[n][n];
        const T R_Y = ts0_update<T, NU, OUT>(Lp, damp, gain, Lnew, h0);
        T mnew[n];
#pragma unroll
        for (int i = 0; i < n; ++i) mnew[i] = mp[i] - gain[i] * mobs;
        // proposal -> the other buffer
#pragma unroll
        for (int i = 0; i < n; ++i) y[i * d + g] = mnew[i];
#pragma unroll
        for (int i = 0; i < n; ++i)
#pragma unroll
          for (int j = 0; j <= i; ++j) y[(n + i * (i + 1) / 2 + j) * d + g] = Lnew[i][j];
        // error_residual_std: std = |sigma| l = |mobs|, error = std * h;
        // error_state_std: sigma_j * std0 (dt^0/0! = 1); reference max(|u0|, |u1|)
        const T err_abs = a.state_error ? dev_abs(sigma) * std0 : dev_abs(mobs) * h;
        const T ref = fmax(dev_abs(x[g]), dev_abs(mnew[0]));
        const T ratio = dev_div(err_abs, atol + rtol * ref);
        local = wide_add_sq(local, ratio);
        newt[jl] = dev_abs(mobs) * fast_rcp(dev_abs(R_Y));
        sig_new[jl] = (a.solver == PDQ_SOLVER_DYNAMIC) ? sigma : T(1);
      }
      // CTA reduction of the wide partial (warp butterflies, then warps in order)
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) local = wide_add_wide(local, wide_shfl_xor(local, off));
      if ((tid & 31) == 0) warp_sums[tid >> 5] = local;
      __syncthreads();
      if (tid == 0) {
        W sum = warp_sums[0];
#pragma unroll
        for (int w = 1; w < kBdThreads / 32; ++w) sum = wide_add_wide(sum, warp_sums[w]);
        partial[par] = sum;
      }
      cluster.sync();

      // ---- phase 3: identical decision in every CTA of the cluster ----
      W total = *cluster.map_shared_rank(&partial[par], 0);
      for (int r = 1; r < CL; ++r) total = wide_add_wide(total, *cluster.map_shared_rank(&partial[par], r));
      par ^= 1;
      const T norm2 = T(wide_hi(total)) / T(d);
      if (!(norm2 == norm2) || isinf(norm2)) {
        status = PDQ_INSTANCE_NONFINITE;
        break;
      }
      const T ep = dev_fpow(norm2, T(-0.5 / n));
      const bool accepted = wide_le(total, T(d));
      T factor;
      if (a.control == PDQ_CONTROL_INTEGRAL) {
        factor = safety * ep;
      } else {
        factor = safety * dev_fpow(ep, cst<T>(a.exp_i, a.exp_i_f)) *
                 dev_fpow(dev_div(ep, pi_prev), cst<T>(a.exp_p, a.exp_p_f));
        if (accepted) pi_prev = ep;
      }
      factor = fmax(factor_min, fmin(factor, factor_max));
      dt = factor * dt_use;
      if (accepted) {
        cur ^= 1;
        if constexpr (kNarrow) {
          t = clipped ? t_next : wide_add(t, dt_use);
        } else {
          t = t + dt_use;
        }
        ++num_steps;
#pragma unroll 1
        for (int jl = tid; jl < dl; jl += kBdThreads) {
          sig[jl] = sig_new[jl];
          if (a.solver == PDQ_SOLVER_MLE) mle_sum[j0 + jl] = wide_add_sq(mle_sum[j0 + jl], newt[jl]);
        }
        if (a.solver == PDQ_SOLVER_MLE) ++num_data;
      }
    }
    if (status != PDQ_INSTANCE_OK) break;
    // clip_dt: every checkpoint is an exact landing (interp_at_t1)
    if (!a.terminal_only || s == S - 1) {
      const int s_out = a.terminal_only ? 0 : s;
      write_checkpoint(s_out, wide_value(t));
      if (a.solver != PDQ_SOLVER_MLE) write_scale(s_out);
    }
    if constexpr (FP) {
      write_filter(s);
      // close the checkpoint's conditional, reset (estimators_and_losses.py:534-547)
      IsoBackward<T, NU, 1> c, id;
      iso_cond_identity(id);
#pragma unroll 1
      for (int jl = tid; jl < dl; jl += kBdThreads) {
        const int g = j0 + jl;
        bd_cond_load<T, NU>(cbufs[cur] + g, d, c);
        bd_cond_store<T, NU>(ckpt + int64_t(s - 1) * CF * d + g, d, c);
        bd_cond_store<T, NU>(cbufs[cur] + g, d, id);
      }
    }
  }

  // ---- fixed-point backward pass: smoothed marginals at the checkpoints ----
  if constexpr (FP) {
    if (status == PDQ_INSTANCE_OK) {
      const T* x = bufs[cur];
      auto write_marginal = [&](int s_out, int g, const T (&rm)[n][1], const T (&rL)[n][n]) {
        const int64_t rec = inst * S_out + s_out;
        double* um = a.u_mean + (rec * d + g) * n;
        double* uc = a.u_chol + (rec * d + g) * n * n;
        for (int i = 0; i < n; ++i) um[i] = double(rm[i][0]);
        for (int i = 0; i < n; ++i)
          for (int j = 0; j < n; ++j) uc[i * n + j] = double(rL[i][j]);
      };
#pragma unroll 1
      for (int jl = tid; jl < dl; jl += kBdThreads) {
        const int g = j0 + jl;
        // the posterior's conditionals (the reference's block-diagonal
        // representation per dimension, ssm_impl_blockdiag.py:16-113: the
        // revert and merge produce the same A, noise mean, noise factor,
        // to_latent and to_observed per dimension as the isotropic pieces);
        // the noise factor calibrated like the marginals
        if (a.cond_A) {
          double cal = 1.0;
          if (a.solver == PDQ_SOLVER_MLE) {
            cal = num_data > 0 ? sqrt(wide_value(mle_sum[g]) / num_data) : 0.0;
            if (a.correct) cal /= sqrt(double(num_steps));
          }
          for (int s = 1; s < S; ++s) {
            IsoBackward<T, NU, 1> c;
            bd_cond_load<T, NU>(ckpt + int64_t(s - 1) * CF * d + g, d, c);
            const int64_t cr = (inst * (S - 1) + (s - 1)) * d + g;
            for (int i = 0; i < n; ++i) {
              for (int j = 0; j < n; ++j) {
                a.cond_A[cr * n * n + i * n + j] = double(c.A[i][j]);
                a.cond_noise_chol[cr * n * n + i * n + j] = double(c.X[i][j]) * cal;
              }
              a.cond_noise_mean[cr * n + i] = double(c.xi[i][0]);
              a.cond_to_latent[cr * n + i] = double(c.tl[i]);
              a.cond_to_observed[cr * n + i] = double(c.to[i]);
            }
          }
        }
        // the terminal state itself: the last checkpoint reset the running conditional
        T rm[n][1], rL[n][n];
#pragma unroll
        for (int i = 0; i < n; ++i) {
          rm[i][0] = x[i * d + g];
#pragma unroll
          for (int j = 0; j < n; ++j) rL[i][j] = (j <= i) ? x[(n + i * (i + 1) / 2 + j) * d + g] : T(0);
        }
        if (a.terminal_only) continue;  // the terminal record is the filter's (written above)
        for (int s = S - 1; s >= 1; --s) {
          IsoBackward<T, NU, 1> c;
          bd_cond_load<T, NU>(ckpt + int64_t(s - 1) * CF * d + g, d, c);
          T pm[n][1], pL[n][n];
          iso_cond_marginalise(c, rm, rL, pm, pL);
#pragma unroll
          for (int i = 0; i < n; ++i) {
            rm[i][0] = pm[i][0];
#pragma unroll
            for (int j = 0; j < n; ++j) rL[i][j] = pL[i][j];
          }
          write_marginal(s - 1, g, rm, rL);
        }
      }
    }
  }

  // ---- finalize ----
  if (status == PDQ_INSTANCE_OK && a.solver == PDQ_SOLVER_MLE) {
    // per-dimension calibrated scale, corrected by sqrt(num_steps) (solvers.py:449-465)
    const int last = num_steps;
    for (int s = 0; s < S_out; ++s) {
      const int64_t rec = inst * S_out + s;
      for (int jl = tid; jl < dl; jl += kBdThreads) {
        const int g = j0 + jl;
        double sc = num_data > 0 ? sqrt(wide_value(mle_sum[g]) / num_data) : 0.0;
        if (a.correct) sc /= sqrt(double(last));
        a.output_scale[rec * d + g] = sc;
        double* uc = a.u_chol + (rec * d + g) * n * n;
        for (int q = 0; q < n * n; ++q) uc[q] *= sc;
      }
    }
    if (FP && a.filter_chol) {
      for (int s = 0; s < S; ++s)
        for (int jl = tid; jl < dl; jl += kBdThreads) {
          const int g = j0 + jl;
          double sc = num_data > 0 ? sqrt(wide_value(mle_sum[g]) / num_data) : 0.0;
          if (a.correct) sc /= sqrt(double(last));
          double* fc = a.filter_chol + ((inst * S + s) * d + g) * n * n;
          for (int q = 0; q < n * n; ++q) fc[q] *= sc;
        }
    }
  }
  if (status != PDQ_INSTANCE_OK) {
    const double nan = __longlong_as_double(0x7ff8000000000000ULL);
    for (int s = 0; s < S_out; ++s) {
      const int64_t rec = inst * S_out + s;
      for (int jl = tid; jl < dl; jl += kBdThreads) {
        const int g = j0 + jl;
        for (int q = 0; q < n; ++q) a.u_mean[(rec * d + g) * n + q] = nan;
        for (int q = 0; q < n * n; ++q) a.u_chol[(rec * d + g) * n * n + q] = nan;
        a.output_scale[rec * d + g] = nan;
      }
      if (rank == 0 && tid == 0) {
        a.t_out[rec] = nan;
        a.num_steps[rec] = num_steps;
      }
    }
  }
  if (rank == 0 && tid == 0) {
    a.num_attempts[inst] = attempts;
    a.status[inst] = status;
  }
  // keep every CTA's shared memory alive until the peers' last DSMEM reads
  cluster.sync();
}

}  // namespace pdq
