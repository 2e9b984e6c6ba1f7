// Dense-factorisation adaptive solver, lane-cooperative: eight lanes per IVP
// instance, the instance's state and QR workspaces in shared memory.
//
// Same algorithm, branches and references as dense_adaptive_kernel
// (dense_solver.cuh): IWP transition / revert / merge / marginalise
// (ssm_impl_dense.py:15-84, 347-363), TS0 / TS1 (ssm_impl_dense.py:237-334),
// filter / fixed-point smoother (estimators_and_losses.py:347-591),
// solver / solver_mle / solver_dynamic, error_residual_std, controllers and
// the RejectionLoop with checkpoints.
//
// The QR / revert / merge / marginalise helpers are real calls (noinline):
// inlined at every call site the kernel outgrew the instruction cache.
// Mapping: one instance per warp on lanes 0-7; lane r owns row r of every N x N matrix and rows
// r, r + 8 of the 2N-row QR workspaces; a Householder column is reduced over
// the group with three butterfly shuffles (commutative adds, so every lane
// holds the bitwise same sum), the dot products of all remaining columns are
// reduced together, and the updates are row-parallel.  Scalars (time, step,
// calibration, controller, status) are computed identically in all eight
// lanes from shared data, so control flow is uniform within a group.  One
// thread per instance left the N = 8 state (about 1.3 k values) to local
// memory and a fully unrolled code far beyond the instruction cache.
#pragma once

// The kernel's dynamic shared memory (a host run of the kernel body supplies a buffer instead).
#ifndef PDQ_DENSE_COOP_SMEM
#define PDQ_DENSE_COOP_SMEM extern __shared__ __align__(16) unsigned char coop_smem_raw[]
#endif

#include "dense_solver.cuh"

namespace pdq {

constexpr int kCoopLanes = 8;

struct Group {
  unsigned mask;
  int lane;  // 0 .. kCoopLanes - 1
  PDQ_D void sync() const { __syncwarp(mask); }
  template <typename T>
  PDQ_D T sum(T v) const {
    v += __shfl_xor_sync(mask, v, 4);
    v += __shfl_xor_sync(mask, v, 2);
    v += __shfl_xor_sync(mask, v, 1);
    return v;
  }
  template <typename T>
  PDQ_D T max(T v) const {
    v = fmax(v, __shfl_xor_sync(mask, v, 4));
    v = fmax(v, __shfl_xor_sync(mask, v, 2));
    v = fmax(v, __shfl_xor_sync(mask, v, 1));
    return v;
  }
};

// Padded leading dimensions (odd) keep the eight rows of a group in
// different shared-memory banks.
template <typename T, int N>
struct CoopCond {
  T A[N][N + 1];
  T X[N][N + 1];  // lower triangular
  T xi[N];
  T tl[N];
  T to[N];
};

template <typename T, int N>
struct CoopNormal {
  T m[N];
  T L[N][N + 1];  // lower triangular
};

template <typename T, int N, int D>
struct CoopState {
  CoopNormal<T, N> x, xi, pred, xnew;  // step_from, interp_from, prediction, proposal
  CoopCond<T, N> bw, bwi, cn, mg;      // running / interp backward conditionals, this step's, merged
  T M[2 * N][2 * N + 1];               // QR workspace
};

// Householder R factor of the R x C workspace M (rows r = lane, lane + 8, ...).
// Column norms outside [1e-30, 1e36] take the scaled path.
template <typename T, int R, int C, int LD>
__device__ __noinline__ void coop_qr(T (*M)[LD], const Group& g) {
  constexpr int RPL = (R + kCoopLanes - 1) / kCoopLanes;  // rows per lane
#pragma unroll 1
  for (int c = 0; c < C; ++c) {
    T e = T(0);
#pragma unroll
    for (int k = 0; k < RPL; ++k) {
      const int r = g.lane + k * kCoopLanes;
      if (r < R && r > c) e += M[r][c] * M[r][c];
    }
    e = g.sum(e);
    const T alpha = M[c][c];
    T nrm2 = alpha * alpha + e;
    T nrm;
    if (norm2_out_of_range(nrm2)) {
      T sc = T(0);
#pragma unroll
      for (int k = 0; k < RPL; ++k) {
        const int r = g.lane + k * kCoopLanes;
        if (r < R && r >= c) sc = fmax(sc, dev_abs(M[r][c]));
      }
      sc = g.max(sc);
      T acc = T(0);
      if (sc > T(0)) {
        const T inv = T(1) / sc;
#pragma unroll
        for (int k = 0; k < RPL; ++k) {
          const int r = g.lane + k * kCoopLanes;
          if (r < R && r >= c) acc += (M[r][c] * inv) * (M[r][c] * inv);
        }
      }
      acc = g.sum(acc);
      nrm = sc * dev_sqrt(acc);
      nrm2 = nrm > T(0) ? T(1) : T(0);
    } else {
      nrm = dev_sqrt(nrm2);
    }
    if (nrm2 > T(0)) {
      const T beta = alpha >= T(0) ? -nrm : nrm;
      const T vinv = T(1) / (alpha - beta);
      const T tau = (beta - alpha) / beta;
      // dots of the normalised reflector v = [1, M[r][c] / v0] with the later columns
      T w[C];
#pragma unroll
      for (int j = 0; j < C; ++j) {
        T acc = T(0);
        if (j > c) {
#pragma unroll
          for (int k = 0; k < RPL; ++k) {
            const int r = g.lane + k * kCoopLanes;
            if (r < R && r > c) acc += (M[r][c] * vinv) * M[r][j];
          }
        }
        w[j] = acc;
      }
#pragma unroll
      for (int j = 0; j < C; ++j)
        if (j > c) w[j] = tau * (M[c][j] + g.sum(w[j]));
      g.sync();  // every lane has read row c and column c
#pragma unroll
      for (int k = 0; k < RPL; ++k) {
        const int r = g.lane + k * kCoopLanes;
        if (r < R && r >= c) {
          const T vr = (r == c) ? T(1) : M[r][c] * vinv;
#pragma unroll
          for (int j = 0; j < C; ++j)
            if (j > c) M[r][j] -= w[j] * vr;
          M[r][c] = (r == c) ? beta : T(0);
        }
      }
    }
    g.sync();
  }
}

template <typename T, int N>
PDQ_D void coop_cond_identity(CoopCond<T, N>& c, const Group& g) {
  const int i = g.lane;
  if (i < N) {
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

template <typename T, int N>
PDQ_D void coop_cond_copy(CoopCond<T, N>& dst, const CoopCond<T, N>& src, const Group& g) {
  const int i = g.lane;
  if (i < N) {
#pragma unroll
    for (int j = 0; j < N; ++j) {
      dst.A[i][j] = src.A[i][j];
      dst.X[i][j] = src.X[i][j];
    }
    dst.xi[i] = src.xi[i];
    dst.tl[i] = src.tl[i];
    dst.to[i] = src.to[i];
  }
}

template <typename T, int N>
PDQ_D void coop_normal_copy(CoopNormal<T, N>& dst, const CoopNormal<T, N>& src, const Group& g) {
  const int i = g.lane;
  if (i < N) {
    dst.m[i] = src.m[i];
#pragma unroll
    for (int j = 0; j < N; ++j) dst.L[i][j] = src.L[i][j];
  }
}

// transition(h, s).revert(rv) / .marginalise(rv) (ssm_impl_dense.py:24-77 with :347-363)
template <typename T, int NU, int D, bool REVERT>
__device__ __noinline__ void coop_prior(const double (&q1)[kMaxN][kMaxN], const CoopNormal<T, (NU + 1) * D>& rv, T h, T scale,
                      CoopNormal<T, (NU + 1) * D>& marg, CoopCond<T, (NU + 1) * D>& cond,
                      T (*M)[2 * (NU + 1) * D + 1], const Group& g) {
  constexpr int N = (NU + 1) * D;
  T p[N], pinv[N];
  dense_precon<T, NU, D>(h, p, pinv);
  const T sq = scale * dev_sqrt(dev_abs(h));
  const int r = g.lane;
  if (r < N) {
    // row r of the top block (R_YX = (sq Q)^T) and row N + r (R_X_F = (A cl)^T, R_X = cl^T), cl = |pinv| L
#pragma unroll
    for (int c = 0; c < N; ++c) {
      const T qcr = (c % D == r % D) ? T(q1[c / D][r / D]) : T(0);
      if (REVERT) {
        M[r][c] = sq * qcr;
        M[r][N + c] = T(0);
        T acc = T(0);
#pragma unroll
        for (int k = 0; k < N; ++k)
          if (k % D == c % D) acc += T(iwp_a<NU>(c / D, k / D)) * dev_abs(pinv[k]) * rv.L[k][r];
        M[N + r][c] = acc;
        M[N + r][N + c] = dev_abs(pinv[c]) * rv.L[c][r];
      } else {
        T acc = T(0);
#pragma unroll
        for (int k = 0; k < N; ++k)
          if (k % D == c % D) acc += T(iwp_a<NU>(c / D, k / D)) * pinv[k] * rv.L[k][r];
        M[r][c] = acc;
        M[N + r][c] = sq * qcr;
      }
    }
  }
  g.sync();
  if constexpr (REVERT) {
    coop_qr<T, 2 * N, 2 * N, 2 * N + 1>(M, g);
  } else {
    coop_qr<T, 2 * N, N, 2 * N + 1>(M, g);
  }
  // mean: mobs = A (pinv * m) (every lane needs all of it for the conditional)
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
  if constexpr (REVERT) {
    // lane j: column j of G^T = R_Y^{-1} R12 (back substitution), i.e. row j of cond.A
    T gt[N];
    if (r < N) {
#pragma unroll
      for (int i = N - 1; i >= 0; --i) {
        T acc = M[i][N + r];
#pragma unroll
        for (int k = i + 1; k < N; ++k) acc -= M[i][k] * gt[k];
        gt[i] = dev_div(acc, M[i][i]);
      }
#pragma unroll
      for (int i = 0; i < N; ++i) cond.A[r][i] = gt[i];
    }
    g.sync();
    if (r < N) {
      T acc = mean_l[r];
#pragma unroll
      for (int k = 0; k < N; ++k) acc -= cond.A[r][k] * mobs[k];
      cond.xi[r] = acc;
#pragma unroll
      for (int j = 0; j < N; ++j) cond.X[r][j] = (j <= r) ? M[N + j][N + r] : T(0);
      cond.tl[r] = dev_rcp(p[r]);
      cond.to[r] = dev_rcp(pinv[r]);
    }
  }
  if (r < N) {
    marg.m[r] = p[r] * mobs[r];
#pragma unroll
    for (int j = 0; j < N; ++j) marg.L[r][j] = (j <= r) ? dev_abs(p[r]) * M[j][r] : T(0);
  }
  g.sync();
}

// outer.merge(inner) (ssm_impl_dense.py:35-49)
template <typename T, int N>
__device__ __noinline__ void coop_merge(const CoopCond<T, N>& o, const CoopCond<T, N>& in, CoopCond<T, N>& out, T (*M)[2 * N + 1],
                      const Group& g) {
  const int i = g.lane;
  if (i < N) {
    T Tv[N];
#pragma unroll
    for (int k = 0; k < N; ++k) Tv[k] = o.tl[k] * in.to[k];
#pragma unroll
    for (int j = 0; j < N; ++j) {
      T gg = T(0), r1 = T(0);
#pragma unroll
      for (int k = 0; k < N; ++k) {
        gg += o.A[i][k] * Tv[k] * in.A[k][j];
        r1 += o.A[i][k] * dev_abs(Tv[k]) * in.X[k][j];
      }
      out.A[i][j] = gg;
      M[j][i] = r1;
      M[N + j][i] = o.X[i][j];
    }
    T x = o.xi[i];
#pragma unroll
    for (int k = 0; k < N; ++k) x += o.A[i][k] * Tv[k] * in.xi[k];
    out.xi[i] = x;
    out.tl[i] = in.tl[i];
    out.to[i] = o.to[i];
  }
  g.sync();
  coop_qr<T, 2 * N, N, 2 * N + 1>(M, g);
  if (i < N) {
#pragma unroll
    for (int j = 0; j < N; ++j) out.X[i][j] = (j <= i) ? M[j][i] : T(0);
  }
  g.sync();
}

// cond.marginalise(rv) (ssm_impl_dense.py:24-33)
template <typename T, int N>
__device__ __noinline__ void coop_marginalise(const CoopCond<T, N>& c, const CoopNormal<T, N>& rv, CoopNormal<T, N>& out,
                            T (*M)[2 * N + 1], const Group& g) {
  const int r = g.lane;
  if (r < N) {
#pragma unroll
    for (int col = 0; col < N; ++col) {
      T acc = T(0);
#pragma unroll
      for (int k = 0; k < N; ++k) acc += c.A[col][k] * c.tl[k] * rv.L[k][r];
      M[r][col] = acc;
      M[N + r][col] = c.X[col][r];
    }
  }
  g.sync();
  coop_qr<T, 2 * N, N, 2 * N + 1>(M, g);
  if (r < N) {
    T acc = T(0);
#pragma unroll
    for (int k = 0; k < N; ++k) acc += c.A[r][k] * c.tl[k] * rv.m[k];
    const T m_new = c.to[r] * (acc + c.xi[r]);
    T row[N];
#pragma unroll
    for (int j = 0; j < N; ++j) row[j] = (j <= r) ? dev_abs(c.to[r]) * M[j][r] : T(0);
    g.sync();  // rv may alias out
    out.m[r] = m_new;
#pragma unroll
    for (int j = 0; j < N; ++j) out.L[r][j] = row[j];
  } else {
    g.sync();
  }
  g.sync();
}

template <typename T, int N>
PDQ_D void coop_store_cond(T* base, const CoopCond<T, N>& c, const Group& g) {
  const int i = g.lane;
  if (i < N) {
#pragma unroll
    for (int j = 0; j < N; ++j) base[i * N + j] = c.A[i][j];
    base[N * N + i] = c.xi[i];
#pragma unroll
    for (int j = 0; j <= i; ++j) base[N * N + N + i * (i + 1) / 2 + j] = c.X[i][j];
    base[N * N + N + N * (N + 1) / 2 + i] = c.tl[i];
    base[N * N + N + N * (N + 1) / 2 + N + i] = c.to[i];
  }
}

template <typename T, int N>
PDQ_D void coop_load_cond(const T* base, CoopCond<T, N>& c, const Group& g) {
  const int i = g.lane;
  if (i < N) {
#pragma unroll
    for (int j = 0; j < N; ++j) {
      c.A[i][j] = base[i * N + j];
      c.X[i][j] = (j <= i) ? base[N * N + N + i * (i + 1) / 2 + j] : T(0);
    }
    c.xi[i] = base[N * N + i];
    c.tl[i] = base[N * N + N + N * (N + 1) / 2 + i];
    c.to[i] = base[N * N + N + N * (N + 1) / 2 + N + i];
  }
  g.sync();
}

template <typename T, int N>
PDQ_D void coop_write_normal(double* mean, double* chol, const CoopNormal<T, N>& x, const Group& g) {
  const int i = g.lane;
  if (i < N) {
    mean[i] = double(x.m[i]);
#pragma unroll
    for (int j = 0; j < N; ++j) chol[i * N + j] = double(x.L[i][j]);
  }
}

template <typename T, int NU, class F, bool TS1, bool FP>
__global__ void __launch_bounds__(128) dense_coop_kernel(DenseArgs a) {
  constexpr int D = F::D, P = F::P, n = NU + 1, N = n * D;
  using State = CoopState<T, N, D>;
  PDQ_DENSE_COOP_SMEM;
  // one instance per warp, on lanes 0-7: instances take different branches
  // (accept / reject, checkpoints), and groups sharing a warp would serialise
  const int group_in_block = threadIdx.x / 32;
  if (threadIdx.x % 32 >= kCoopLanes) return;
  State& st = reinterpret_cast<State*>(coop_smem_raw)[group_in_block];
  Group g;
  g.lane = threadIdx.x % 32;
  g.mask = 0xFFu;
  const int64_t b = int64_t(blockIdx.x) * (blockDim.x / 32) + group_in_block;
  if (b >= a.B) return;  // whole group
  const int S = a.S;
  const int S_out = a.terminal_only ? 1 : S;
  const double* save_at = a.save_at + b * S;
  T* ws = FP ? reinterpret_cast<T*>(a.workspace) + b * int64_t(S - 1) * cond_floats<N>() : nullptr;
  const int lane = g.lane;

  double pd[P];
  T pt[P];
#pragma unroll
  for (int k = 0; k < P; ++k) {
    pd[k] = a.params[b * P + k];
    pt[k] = T(pd[k]);
  }
  {
    double y0[D];
#pragma unroll
    for (int j = 0; j < D; ++j) y0[j] = a.y0[b * D + j];
    double tc[n][D];
    taylor_init<F, NU>(y0, pd, tc);
    if (lane < N) {
      st.x.m[lane] = T(tc[lane / D][lane % D]);
#pragma unroll
      for (int j = 0; j < N; ++j) st.x.L[lane][j] = T(0);
    }
  }
  if constexpr (FP) {
    coop_cond_identity(st.bw, g);
    coop_cond_identity(st.bwi, g);
  }
  g.sync();
  coop_normal_copy(st.xi, st.x, g);
  g.sync();

  double t = save_at[0], ti = t, dt = a.dt0[b], pi_prev = 1.0, mle_sumsq = 0.0;
  int num_data = 0, num_steps = 0, attempts = 0, status = PDQ_INSTANCE_OK;
  T sigma_sf = T(1);
  const T damp = T(a.damp);

  if (!a.terminal_only) {
    coop_write_normal(a.u_mean + (b * S_out) * N, a.u_chol + (b * S_out) * N * N, st.x, g);
    if (lane == 0) {
      a.output_scale[b * S_out] = 1.0;
      a.t_out[b * S_out] = t;
      a.num_steps[b * S_out] = 0;
    }
  }
  if (a.filter_mean) coop_write_normal(a.filter_mean + (b * S) * N, a.filter_chol + (b * S) * N * N, st.x, g);

  for (int s = 1; s < S && status == PDQ_INSTANCE_OK; ++s) {
    const double t_next = save_at[s];
    bool cont = true;
    while (cont && status == PDQ_INSTANCE_OK) {
      if (t + a.eps < t_next) {
        bool accepted = false;
        while (!accepted) {
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
          // u = transition(h, 1).apply_flat(mean): every lane keeps the whole mean
          T mp[N];
#pragma unroll
          for (int i = 0; i < N; ++i) {
            T acc = T(0);
#pragma unroll
            for (int k = 0; k < N; ++k)
              if (k % D == i % D) acc += T(iwp_a<NU>(i / D, k / D)) * pinv[k] * st.x.m[k];
            mp[i] = p[i] * acc;
          }
          DLin<T, N, D> fx;
          dense_linearize<T, NU, F, TS1>(mp, pt, fx);
          // observed = fx.marginalise(u) (small: every lane)
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

          if constexpr (FP) {
            coop_prior<T, NU, D, true>(a.q1, st.x, h, s_pred, st.pred, st.cn, st.M, g);
          } else {
            CoopCond<T, N>& unused = st.cn;
            coop_prior<T, NU, D, false>(a.q1, st.x, h, s_pred, st.pred, unused, st.M, g);
          }

          // ---- update: fx.revert(pred), M2 = [[damp I, 0], [(J Lp)^T, Lp^T]] ----
          {
            const int rr = lane;
            if (rr < D) {
#pragma unroll
              for (int j = 0; j < D + N; ++j) st.M[rr][j] = (rr == j) ? damp : T(0);
            }
            if (rr < N) {
#pragma unroll
              for (int aa = 0; aa < D; ++aa) {
                T acc = T(0);
#pragma unroll
                for (int k = 0; k < N; ++k) acc += fx.J[aa][k] * st.pred.L[k][rr];
                st.M[D + rr][aa] = acc;
              }
#pragma unroll
              for (int c = 0; c < N; ++c) st.M[D + rr][D + c] = st.pred.L[c][rr];
            }
          }
          g.sync();
          coop_qr<T, D + N, D + N, 2 * N + 1>(st.M, g);
          // G = solve_triu(R_Y, R12)^T: every lane all D x N entries (D small)
          T ro[D];
#pragma unroll
          for (int aa = 0; aa < D; ++aa) {
            T acc = fx.b[aa];
#pragma unroll
            for (int k = 0; k < N; ++k) acc += fx.J[aa][k] * st.pred.m[k];
            ro[aa] = acc;
          }
          T xnew_mi = T(0);
          if (lane < N) {
            T gcol[D];  // G^T[:, lane]
#pragma unroll
            for (int i = D - 1; i >= 0; --i) {
              T acc = st.M[i][D + lane];
#pragma unroll
              for (int k = i + 1; k < D; ++k) acc -= st.M[i][k] * gcol[k];
              gcol[i] = dev_div(acc, st.M[i][i]);
            }
            T acc = st.pred.m[lane];
#pragma unroll
            for (int aa = 0; aa < D; ++aa) acc -= gcol[aa] * ro[aa];
            xnew_mi = acc;
            st.xnew.m[lane] = acc;
#pragma unroll
            for (int j = 0; j < N; ++j) st.xnew.L[lane][j] = (j <= lane) ? st.M[D + j][D + lane] : T(0);
          }
          g.sync();
          (void)xnew_mi;
          // error_residual_std: std of the rescaled observed = sigma * row norms of Lo
          double sumsq = 0.0;
#pragma unroll
          for (int j = 0; j < D; ++j) {
            T rn = T(0);
#pragma unroll
            for (int k = 0; k <= j; ++k) rn += Mo[k][j] * Mo[k][j];
            const T err_abs = dev_abs(sigma_loc) * dev_sqrt(rn) * h;
            const T ref = fmax(dev_abs(st.x.m[j]), dev_abs(st.xnew.m[j]));
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
            T q = T(0);
            if (a.solver == PDQ_SOLVER_MLE) {
              // new term: the observed residual whitened by R_Y (d x d)
              T wv[D];
#pragma unroll
              for (int i = 0; i < D; ++i) {
                T acc = ro[i];
#pragma unroll
                for (int k = 0; k < i; ++k) acc -= st.M[k][i] * wv[k];
                wv[i] = dev_div(acc, st.M[i][i]);
              }
#pragma unroll
              for (int i = 0; i < D; ++i) q += wv[i] * wv[i];
            }
            g.sync();  // every lane has read R_Y from M, which the merge below overwrites
            if constexpr (FP) coop_merge(st.bw, st.cn, st.mg, st.M, g);
            ti = t;
            coop_normal_copy(st.xi, st.x, g);
            if constexpr (FP) coop_cond_copy(st.bwi, st.bw, g);
            g.sync();
            t = t + dt_use;
            ++num_steps;
            coop_normal_copy(st.x, st.xnew, g);
            if constexpr (FP) coop_cond_copy(st.bw, st.mg, g);
            g.sync();
            if (a.solver == PDQ_SOLVER_MLE) {
              mle_sumsq += double(q) * (1.0 / D);
              ++num_data;
            }
            sigma_sf = (a.solver == PDQ_SOLVER_DYNAMIC) ? sigma_loc : T(1);
          }
        }
      }
      if (status != PDQ_INSTANCE_OK) break;
      const bool record = (!a.terminal_only) || (s == S - 1);
      const int s_out = a.terminal_only ? 0 : s;
      const int64_t rec = b * S_out + s_out;
      if (t + a.eps < t_next) {
        // interp_skip
      } else if (t > t_next + a.eps) {
        // interp_beyond_t1 (solvers.py:205-269)
        const T h0 = T(t_next - ti), h1 = T(t - t_next);
        if constexpr (FP) {
          // estimators_and_losses.py:549-591; st.pred holds ext_t, st.xnew ext_t1
          coop_prior<T, NU, D, true>(a.q1, st.xi, h0, sigma_sf, st.pred, st.cn, st.M, g);
          coop_merge(st.bwi, st.cn, st.mg, st.M, g);  // extrapolated_t.conditional
          coop_store_cond(ws + int64_t(s - 1) * cond_floats<N>(), st.mg, g);
          coop_prior<T, NU, D, true>(a.q1, st.pred, h1, sigma_sf, st.xnew, st.cn, st.M, g);
          coop_cond_identity(st.bwi, g);
          g.sync();
          coop_merge(st.bwi, st.cn, st.bw, st.M, g);  // extrapolated_t1.conditional -> step_from
          coop_normal_copy(st.xi, st.pred, g);        // interp_from = previous_new
          g.sync();
        } else {
          CoopCond<T, N>& unused = st.cn;
          coop_prior<T, NU, D, false>(a.q1, st.xi, h0, sigma_sf, st.pred, unused, st.M, g);
          coop_normal_copy(st.xi, st.pred, g);
          g.sync();
        }
        ti = t_next;
        if (record) {
          coop_write_normal(a.u_mean + rec * N, a.u_chol + rec * N * N, st.xi, g);
          if (lane == 0) {
            a.output_scale[rec] = double(sigma_sf);
            a.t_out[rec] = t_next;
            a.num_steps[rec] = num_steps;
          }
        }
        if (a.filter_mean) coop_write_normal(a.filter_mean + (b * S + s) * N, a.filter_chol + (b * S + s) * N * N, st.xi, g);
      } else {
        // interp_at_t1 (solvers.py:271-315)
        if constexpr (FP) {
          coop_store_cond(ws + int64_t(s - 1) * cond_floats<N>(), st.bw, g);
          g.sync();
          coop_cond_identity(st.bw, g);
          coop_cond_identity(st.bwi, g);
        }
        coop_normal_copy(st.xi, st.x, g);
        g.sync();
        ti = t;
        if (record) {
          coop_write_normal(a.u_mean + rec * N, a.u_chol + rec * N * N, st.x, g);
          if (lane == 0) {
            a.output_scale[rec] = double(sigma_sf);
            a.t_out[rec] = t;
            a.num_steps[rec] = num_steps;
          }
        }
        if (a.filter_mean) coop_write_normal(a.filter_mean + (b * S + s) * N, a.filter_chol + (b * S + s) * N * N, st.x, g);
      }
      cont = t + a.eps < t_next;
    }
  }
  __syncwarp(g.mask);

  // ---- finalize (solvers.py:439-480, 601-633, 735-767) ----
  double scale = 1.0;
  if (status == PDQ_INSTANCE_OK && a.solver == PDQ_SOLVER_MLE) {
    scale = num_data > 0 ? sqrt(mle_sumsq / num_data) : 0.0;
    if (a.correct) scale /= sqrt(double(num_steps));
  }
  if (FP && status == PDQ_INSTANCE_OK) {
    // Smoother.finalize: rv_at_t1 = posterior1.conditional.marginalise(marginal),
    // then the reverse scan of marginalise over the checkpoint conditionals
    coop_marginalise(st.bw, st.x, st.pred, st.M, g);
    for (int s = S - 1; s >= 1; --s) {
      if (!a.terminal_only || s == S - 1) {
        const int64_t rec = b * S_out + (a.terminal_only ? 0 : s);
        coop_write_normal(a.u_mean + rec * N, a.u_chol + rec * N * N, st.pred, g);
      }
      coop_load_cond(ws + int64_t(s - 1) * cond_floats<N>(), st.cn, g);
      if (a.cond_A && lane < N) {
        const int64_t cr = b * (S - 1) + (s - 1);
        const int i = lane;
        for (int j = 0; j < N; ++j) {
          a.cond_A[cr * N * N + i * N + j] = double(st.cn.A[i][j]);
          a.cond_noise_chol[cr * N * N + i * N + j] = double(st.cn.X[i][j]) * scale;
        }
        a.cond_noise_mean[cr * N + i] = double(st.cn.xi[i]);
        a.cond_to_latent[cr * N + i] = double(st.cn.tl[i]);
        a.cond_to_observed[cr * N + i] = double(st.cn.to[i]);
      }
      if (a.terminal_only) continue;
      coop_marginalise(st.cn, st.pred, st.pred, st.M, g);
      if (s == 1) coop_write_normal(a.u_mean + b * S_out * N, a.u_chol + b * S_out * N * N, st.pred, g);
    }
  }
  __syncwarp(g.mask);
  if (status == PDQ_INSTANCE_OK) {
    if (a.solver == PDQ_SOLVER_MLE) {
      for (int s = 0; s < S_out; ++s) {
        const int64_t rec = b * S_out + s;
        for (int k = lane; k < N * N; k += kCoopLanes) a.u_chol[rec * N * N + k] *= scale;
        if (lane == 0) a.output_scale[rec] = scale;
      }
      if (a.filter_chol)
        for (int k = lane; k < S * N * N; k += kCoopLanes) a.filter_chol[b * S * N * N + k] *= scale;
    }
  } else {
    const double nan = __longlong_as_double(0x7ff8000000000000ULL);
    for (int s = 0; s < S_out; ++s) {
      const int64_t rec = b * S_out + s;
      for (int k = lane; k < N; k += kCoopLanes) a.u_mean[rec * N + k] = nan;
      for (int k = lane; k < N * N; k += kCoopLanes) a.u_chol[rec * N * N + k] = nan;
      if (lane == 0) {
        a.output_scale[rec] = nan;
        a.t_out[rec] = nan;
        a.num_steps[rec] = num_steps;
      }
    }
  }
  if (lane == 0) {
    a.num_attempts[b] = attempts;
    a.status[b] = status;
  }
}

}  // namespace pdq
