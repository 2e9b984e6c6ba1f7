// Runs the isotropic adaptive kernel (iso_adaptive_kernel, one thread per
// instance, Lotka-Volterra; float64, or float32 bulk with float-pair
// accumulators) on the CPU, every instance as its own
// "thread", on buffers of exactly the sizes the library uses, so
// AddressSanitizer flags any access outside them.  The instantiations the
// library launches for TS0 with error_residual_std, with exact checkpoint
// landings (clip_dt) or with interpolation: mode 0 the filter (the lean
// instantiation), mode 1 the fixed-point smoother (its scratch of backward
// conditionals and the backward pass), mode 2 the filter with forward-mode
// sensitivities (P + d threads per instance), modes 3 and 4 the general
// filter instantiation with error_state_std, with TS0 (3) or TS1 (4, the
// Jacobian trace along d), mode 5 the terminal-value adjoint: the record
// pass (the lean filter with REC) and then the adjoint pass
// (iso_tv_bwd_kernel) for a cotangent of the terminal mean; mode 6 the
// split filter (iso_split_kernel: a covariance warp and a mean warp per
// instance, run as two host threads), mode 7 the branch-light lean filter
// (iso_lean_kernel), mode 8 the eight-lane kernel (iso_warp_kernel, each
// warp's lanes as host threads with emulated shuffles), mode 9 the split
// kernel as launched (two 32-lane warps per 32 instances, 64 host threads
// per block); modes 6 to 9 with exact landings only.
//
// Input file (whitespace-separated): precision (0 float32, 1 float64) mode nu
// B S solver control clip_dt terminal_only, then atol rtol, save_at (B x S), params (B x 4), y0 (B x 2),
// dt0 (B), Q1 ((nu + 1) x (nu + 1), row-major); mode 5 then the cotangent
// (B x (nu + 1) x 2), the record's capacity and checkpoint_every.  solver /
// control take the PDQ_SOLVER_* / PDQ_CONTROL_* codes.
// Output: per instance a line "status attempts", then per output record a
// line "t num_steps output_scale u_mean[n d] u_chol[n n]" (mode 2: followed
// by d u_mean / d params [n d 4] and d u_mean / d y0 [n d 2]; mode 5:
// followed by the gradients d <cotangent, u_mean> / d params [4] and / d y0 [2]).
#include <cstdio>
#include <cstdlib>
#include <thread>
#include <vector>

#include "iso_lean.cuh"
#include "iso_solver.cuh"
#include "iso_split.cuh"
#include "iso_warp.cuh"
#include "tv_adjoint.cuh"

thread_local pdq_host_uint3 threadIdx, blockIdx, blockDim;

using namespace pdq;

static bool read_all(FILE* in, std::vector<double>& v) {
  for (double& x : v)
    if (fscanf(in, "%lf", &x) != 1) return false;
  return true;
}

template <typename T, int NU, bool INTERP, int MODE>
static int run(FILE* in, long long B, int S, int solver, int control, int clip_dt, int terminal_only) {
  using F = LotkaVolterra;
  constexpr int n = NU + 1;
  constexpr int D = F::D;
  constexpr int P = F::P;
  std::vector<double> tol(2), save_at(B * S), params(B * P), y0(B * D), dt0(B), q1(n * n);
  if (!read_all(in, tol) || !read_all(in, save_at) || !read_all(in, params) || !read_all(in, y0) ||
      !read_all(in, dt0) || !read_all(in, q1))
    return 2;
  const int S_out = terminal_only ? 1 : S;
  std::vector<double> u_mean(B * S_out * n * D), u_chol(B * S_out * n * n), scale(B * S_out), t(B * S_out);
  std::vector<int32_t> steps(B * S_out), attempts(B), status(B);
  std::vector<double> tan_p(MODE == 2 ? B * S_out * n * D * P : 0), tan_y(MODE == 2 ? B * S_out * n * D * D : 0);
  std::vector<T> ws(MODE == 1 ? B * (S - 1) * iso_cond_floats<NU, D>() : 0);
  std::vector<double> cot(MODE == 5 ? B * n * D : 0), grad_p(MODE == 5 ? B * P : 0), grad_y(MODE == 5 ? B * D : 0);
  std::vector<T> rec;
  int cap = 0, ckpt = 0;
  if constexpr (MODE == 5) {
    if (!read_all(in, cot) || fscanf(in, "%d %d", &cap, &ckpt) != 2 || cap < 1 || ckpt < 1 || ckpt > cap) return 2;
    rec.assign(B * (tv_record_elems(NU, D, cap, ckpt) + tv_scratch_elems(NU, D, ckpt)), T(0));
  }

  IsoArgs a;
  memset(&a, 0, sizeof(a));
  a.B = B;
  a.S = S;
  a.terminal_only = terminal_only;
  a.solver = solver;
  a.control = control;
  a.clip_dt = clip_dt;
  a.correct = 1;  // solver_mle(correct_asymptotic_underconfidence=True), the default
  // control_integral / control_proportional_integral defaults (controllers.py:24-84)
  a.safety = 0.95;
  a.factor_min = 0.2;
  a.factor_max = 10.0;
  a.exp_i = 0.3;
  a.exp_p = 0.4;
  a.atol = tol[0];
  a.rtol = tol[1];
  a.eps = 1e-8;
  a.damp = 0.0;
  a.max_attempts = int64_t(1) << 20;  // pdq_config_default
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      a.q1[i][j] = q1[i * n + j];
      a.q1f[i][j] = float(q1[i * n + j]);
    }
  // float copies of the constants (read by the float32 kernels)
  a.safety_f = float(a.safety);
  a.factor_min_f = float(a.factor_min);
  a.factor_max_f = float(a.factor_max);
  a.exp_i_f = float(a.exp_i);
  a.exp_p_f = float(a.exp_p);
  a.atol_f = float(a.atol);
  a.rtol_f = float(a.rtol);
  a.eps_f = float(a.eps);
  a.damp_f = float(a.damp);
  a.save_at = save_at.data();
  a.params = params.data();
  a.y0 = y0.data();
  a.dt0 = dt0.data();
  a.u_mean = u_mean.data();
  a.u_chol = u_chol.data();
  a.output_scale = scale.data();
  a.t_out = t.data();
  a.num_steps = steps.data();
  a.num_attempts = attempts.data();
  a.status = status.data();
  if (MODE == 1) a.workspace = ws.data();
  if (MODE == 3 || MODE == 4) {
    a.state_error = 1;
    a.ts1 = MODE == 4 ? 1 : 0;
  }
  if (MODE == 2) {
    a.tan_params = tan_p.data();
    a.tan_y0 = tan_y.data();
    a.tangents = 1;
  }
  if (MODE == 5) {
    a.record = rec.data();
    a.rec_capacity = cap;
    a.rec_ckpt = ckpt;
  }

  if constexpr (MODE == 6 && !INTERP) {
    // the split kernel with one-lane warps: per instance a block of two
    // threads (the covariance and the mean warp) with their own barriers
    for (long long b = 0; b < B; ++b) {
      PdqHostBarrier bars[3];
      auto warp = [&](unsigned tid) {
        blockDim = {2, 1, 1};
        blockIdx = {uint32_t(b), 0, 0};
        threadIdx = {tid, 0, 0};
        pdq_host_barriers = bars;
        iso_split_kernel<T, NU, F, 1>(a);
        pdq_host_barriers = nullptr;
      };
      std::thread cov(warp, 0u), mean(warp, 1u);
      cov.join();
      mean.join();
    }
  }
  if constexpr (MODE == 9 && !INTERP) {
    // the split kernel as launched: 32 instances per block of two 32-lane
    // warps, all 64 lanes as host threads (the warps' __any_sync emulated
    // per warp, the named barriers and __syncthreads per block), the last
    // block ragged when B is not a multiple of 32
    const long long grid = (B + 31) / 32;
    for (long long blk = 0; blk < grid; ++blk) {
      PdqHostBarrier bars[3];
      for (auto& br : bars) br.expected = 64;
      PdqHostWarp warps[2];
      std::vector<std::thread> lanes;
      for (unsigned tid = 0; tid < 64; ++tid)
        lanes.emplace_back([&, tid] {
          blockDim = {64, 1, 1};
          blockIdx = {uint32_t(blk), 0, 0};
          threadIdx = {tid, 0, 0};
          pdq_host_barriers = bars;
          pdq_host_warp = &warps[tid / 32];
          iso_split_kernel<T, NU, F, 32>(a);
          pdq_host_warp = nullptr;
          pdq_host_barriers = nullptr;
        });
      for (auto& th : lanes) th.join();
    }
  }
  if constexpr (MODE == 8 && !INTERP) {
    // the eight-lane kernel: each warp's 32 lanes (four instances) as host
    // threads exchanging the reflectors and rotations by emulated shuffles
    const long long warps = (B * 8 + 31) / 32;
    for (long long w = 0; w < warps; ++w) {
      PdqHostWarp warp;
      std::vector<std::thread> lanes;
      for (unsigned tid = 0; tid < 32; ++tid)
        lanes.emplace_back([&, tid] {
          blockDim = {256, 1, 1};
          blockIdx = {uint32_t(w / 8), 0, 0};
          threadIdx = {uint32_t((w % 8) * 32 + tid), 0, 0};
          pdq_host_warp = &warp;
          iso_warp_kernel<T, NU, F, 8, 2>(a);
          pdq_host_warp = nullptr;
        });
      for (auto& th : lanes) th.join();
    }
  }
  const int block = 64;
  blockDim = {uint32_t(block), 1, 1};
  const long long threads = MODE == 2 ? B * (P + D) : B;
  const long long padded = (MODE == 6 || MODE >= 8) ? 0 : (threads + block - 1) / block * block;  // the launch's grid
  for (long long g = 0; g < padded; ++g) {
    blockIdx = {uint32_t(g / block), 0, 0};
    threadIdx = {uint32_t(g % block), 0, 0};
    if constexpr (MODE == 0) iso_adaptive_kernel<T, NU, F, INTERP, false, false>(a);
    if constexpr (MODE == 1) iso_adaptive_kernel<T, NU, F, INTERP, true, true>(a);
    if constexpr (MODE == 2) iso_adaptive_kernel<T, NU, F, INTERP, false, false, true>(a);
    if constexpr (MODE == 3 || MODE == 4) iso_adaptive_kernel<T, NU, F, INTERP, false, true>(a);
    if constexpr (MODE == 5 && !INTERP) iso_adaptive_kernel<T, NU, F, false, false, false, false, true>(a);
    if constexpr (MODE == 7 && !INTERP) iso_lean_kernel<T, NU, F>(a);
  }
  if constexpr (MODE == 5) {
    TvAdjArgs ta;
    ta.capacity = cap;
    ta.ckpt = ckpt;
    ta.num_steps = steps.data();
    ta.status = status.data();
    ta.cotangent = cot.data();
    ta.grad_params = grad_p.data();
    ta.grad_y0 = grad_y.data();
    ta.record = rec.data();
    ta.scratch = rec.data() + B * tv_record_elems(NU, D, cap, ckpt);
    for (long long g = 0; g < padded; ++g) {
      blockIdx = {uint32_t(g / block), 0, 0};
      threadIdx = {uint32_t(g % block), 0, 0};
      iso_tv_bwd_kernel<T, NU, F>(a, ta);
    }
  }
  for (long long b = 0; b < B; ++b) {
    printf("%d %d\n", status[b], attempts[b]);
    for (int k = 0; k < S_out; ++k) {
      const long long r = b * S_out + k;
      printf("%.17g %d %.17g", t[r], steps[r], scale[r]);
      for (int e = 0; e < n * D; ++e) printf(" %.17g", u_mean[r * n * D + e]);
      for (int e = 0; e < n * n; ++e) printf(" %.17g", u_chol[r * n * n + e]);
      if (MODE == 2) {
        for (int e = 0; e < n * D * P; ++e) printf(" %.17g", tan_p[r * n * D * P + e]);
        for (int e = 0; e < n * D * D; ++e) printf(" %.17g", tan_y[r * n * D * D + e]);
      }
      if (MODE == 5) {
        for (int e = 0; e < P; ++e) printf(" %.17g", grad_p[b * P + e]);
        for (int e = 0; e < D; ++e) printf(" %.17g", grad_y[b * D + e]);
      }
      printf("\n");
    }
  }
  return 0;
}

int main(int argc, char** argv) {
  if (argc != 2) return 2;
  FILE* in = fopen(argv[1], "r");
  if (!in) return 2;
  long long B;
  int prec, mode, nu, S, solver, control, clip_dt, terminal_only;
  if (fscanf(in, "%d %d %d %lld %d %d %d %d %d", &prec, &mode, &nu, &B, &S, &solver, &control, &clip_dt,
             &terminal_only) != 9)
    return 2;
  if (B < 1 || S < 2) return 2;
  int rc = 2;
  const bool interp = !clip_dt;
  const int args_ok = (mode >= 0 && mode <= 9) && (nu == 3 || nu == 4 || (nu == 5 && (mode == 0 || mode >= 6))) &&
                      (mode != 5 || (clip_dt && terminal_only && S == 2)) && (mode < 6 || clip_dt);
  if (!args_ok) return 2;
#define PDQ_HOST_RUN(NU_, MODE_)                                                                        \
  rc = prec ? (interp ? run<double, NU_, true, MODE_>(in, B, S, solver, control, clip_dt, terminal_only)    \
                      : run<double, NU_, false, MODE_>(in, B, S, solver, control, clip_dt, terminal_only))  \
            : (interp ? run<float, NU_, true, MODE_>(in, B, S, solver, control, clip_dt, terminal_only)     \
                      : run<float, NU_, false, MODE_>(in, B, S, solver, control, clip_dt, terminal_only))
  if (nu == 4 && mode == 0) PDQ_HOST_RUN(4, 0);
  if (nu == 3 && mode == 0) PDQ_HOST_RUN(3, 0);
  if (nu == 3 && mode == 1) PDQ_HOST_RUN(3, 1);
  if (nu == 3 && mode == 2) PDQ_HOST_RUN(3, 2);
  if (nu == 3 && mode == 3) PDQ_HOST_RUN(3, 3);
  if (nu == 3 && mode == 4) PDQ_HOST_RUN(3, 4);
  if (nu == 4 && mode == 2) PDQ_HOST_RUN(4, 2);
  if (nu == 4 && mode == 5) PDQ_HOST_RUN(4, 5);
  if (nu == 3 && mode == 5) PDQ_HOST_RUN(3, 5);
  if (nu == 4 && mode == 6) PDQ_HOST_RUN(4, 6);
  if (nu == 5 && mode == 0) PDQ_HOST_RUN(5, 0);
  if (nu == 5 && mode == 6) PDQ_HOST_RUN(5, 6);
  if (nu == 4 && mode == 7) PDQ_HOST_RUN(4, 7);
  if (nu == 3 && mode == 7) PDQ_HOST_RUN(3, 7);
  if (nu == 5 && mode == 7) PDQ_HOST_RUN(5, 7);
  if (nu == 4 && mode == 8) PDQ_HOST_RUN(4, 8);
  if (nu == 3 && mode == 8) PDQ_HOST_RUN(3, 8);
  if (nu == 4 && mode == 9) PDQ_HOST_RUN(4, 9);
  if (nu == 3 && mode == 6) PDQ_HOST_RUN(3, 6);
#undef PDQ_HOST_RUN
  fclose(in);
  return rc;
}
