// Runs the float64 dense adaptive kernel (dense_adaptive_kernel, one thread
// per instance, TS1 with the Jacobian on dual numbers) on the CPU, every
// instance as its own "thread", on buffers of exactly the sizes the library
// uses (the fixed-point smoother's scratch of backward conditionals
// included), so AddressSanitizer flags any access outside them.  With
// PDQ_HOST_DENSE_KERNEL=struct in the environment it runs the
// structure-exploiting kernel (dense_struct_kernel) with one lane per
// instance instead, its shared memory a buffer of the launch's size; with
// PDQ_HOST_DENSE_LANES=4, 8 or 16 as well, with that many lanes per instance,
// each 32-lane block's lanes as host threads (warp barriers emulated); with
// PDQ_HOST_DENSE_KERNEL=coop the lane-cooperative kernel (dense_coop_kernel,
// eight lanes per instance as host threads, shuffles emulated).
//
// Input file (whitespace-separated): field (0 Lotka-Volterra, 1 van der Pol)
// nu (2 or 3) strategy (0 filter, 1 fixed-point smoother) B S solver control
// clip_dt, then atol rtol, save_at (B x S), params (B x P), y0 (B x 2),
// dt0 (B), Q1 ((nu + 1) x (nu + 1), row-major).
// Output: per instance a line "status attempts", then per save point a line
// "t num_steps u_mean[N] u_chol[N N]", N = (nu + 1) 2.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

static std::vector<unsigned char> g_smem;  // the structure-exploiting and lane-cooperative kernels' shared memory
#define PDQ_DENSE_STRUCT_SMEM unsigned char* dense_struct_smem = g_smem.data()
#define PDQ_DENSE_COOP_SMEM unsigned char* coop_smem_raw = g_smem.data()

#include "dense_coop.cuh"
#include "dense_solver.cuh"
#include "dense_struct.cuh"

thread_local pdq_host_uint3 threadIdx, blockIdx, blockDim;

using namespace pdq;

static bool read_all(FILE* in, std::vector<double>& v) {
  for (double& x : v)
    if (fscanf(in, "%lf", &x) != 1) return false;
  return true;
}

template <int NU, class F, bool FP>
static int run(FILE* in, long long B, int S, int solver, int control, int clip_dt) {
  constexpr int n = NU + 1;
  constexpr int D = F::D;
  constexpr int N = n * D;
  std::vector<double> tol(2), save_at(B * S), params(B * F::P), y0(B * D), dt0(B), q1(n * n);
  if (!read_all(in, tol) || !read_all(in, save_at) || !read_all(in, params) || !read_all(in, y0) ||
      !read_all(in, dt0) || !read_all(in, q1))
    return 2;
  std::vector<double> u_mean(B * S * N), u_chol(B * S * N * N), scale(B * S), t(B * S);
  std::vector<int32_t> steps(B * S), attempts(B), status(B);
  std::vector<double> ws(FP ? size_t(B) * (S - 1) * cond_floats<N>() : 0);

  DenseArgs a;
  memset(&a, 0, sizeof(a));
  a.B = B;
  a.S = S;
  a.terminal_only = 0;
  a.solver = solver;
  a.control = control;
  a.clip_dt = clip_dt;
  a.correct = 1;
  a.fixedpoint = FP ? 1 : 0;
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
    for (int j = 0; j < n; ++j) a.q1[i][j] = q1[i * n + j];
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
  a.workspace = FP ? ws.data() : nullptr;

  const int block = 32;
  blockDim = {uint32_t(block), 1, 1};
  const long long padded = (B + block - 1) / block * block;  // the launch's grid
  const char* kern = getenv("PDQ_HOST_DENSE_KERNEL");
  const bool structured = kern != nullptr && strcmp(kern, "struct") == 0;
  const char* lanes_env = getenv("PDQ_HOST_DENSE_LANES");
  const int lanes = lanes_env ? atoi(lanes_env) : 1;
  if (structured && lanes > 1) {
    // the structure-exploiting kernel as launched: 32 / L instances per
    // 32-thread block, its 32 lanes as host threads meeting at the warp's
    // barriers, the blocks one after another
    if (lanes != 4 && lanes != 8 && lanes != 16) return 2;
    const int ipw = 32 / lanes;
    const long long grid = (B + ipw - 1) / ipw;
    g_smem.assign(dense_struct_smem_bytes<NU, D>(sizeof(double), lanes), 0);
    for (long long blk = 0; blk < grid; ++blk) {
      PdqHostWarp warp;
      std::vector<std::thread> threads;
      for (unsigned tid = 0; tid < 32; ++tid)
        threads.emplace_back([&, tid] {
          blockDim = {32, 1, 1};
          blockIdx = {uint32_t(blk), 0, 0};
          threadIdx = {tid, 0, 0};
          pdq_host_warp = &warp;
          if (lanes == 4) dense_struct_kernel<double, NU, F, true, FP, 4>(a);
          if (lanes == 8) dense_struct_kernel<double, NU, F, true, FP, 8>(a);
          if (lanes == 16) dense_struct_kernel<double, NU, F, true, FP, 16>(a);
          pdq_host_warp = nullptr;
        });
      for (auto& th : threads) th.join();
    }
  }
  const bool coop = kern != nullptr && strcmp(kern, "coop") == 0;
  if (coop) {
    // the lane-cooperative kernel, one instance per 32-thread block: its
    // eight lanes as host threads exchanging sums by emulated shuffles
    g_smem.assign(sizeof(CoopState<double, N, D>), 0);
    for (long long b = 0; b < B; ++b) {
      PdqHostWarp warp;
      std::vector<std::thread> threads;
      for (unsigned tid = 0; tid < unsigned(kCoopLanes); ++tid)
        threads.emplace_back([&, tid] {
          blockDim = {32, 1, 1};
          blockIdx = {uint32_t(b), 0, 0};
          threadIdx = {tid, 0, 0};
          pdq_host_warp = &warp;
          dense_coop_kernel<double, NU, F, true, FP>(a);
          pdq_host_warp = nullptr;
        });
      for (auto& th : threads) th.join();
    }
  }
  if (structured && lanes == 1) g_smem.assign(dense_struct_smem_bytes<NU, D>(sizeof(double), 1), 0);
  for (long long g = 0; g < ((structured && lanes > 1) || coop ? 0 : padded); ++g) {
    blockIdx = {uint32_t(g / block), 0, 0};
    threadIdx = {uint32_t(g % block), 0, 0};
    if (structured)
      dense_struct_kernel<double, NU, F, true, FP, 1>(a);
    else
      dense_adaptive_kernel<double, NU, F, true, FP>(a);
  }
  for (long long b = 0; b < B; ++b) {
    printf("%d %d\n", status[b], attempts[b]);
    for (int k = 0; k < S; ++k) {
      const long long r = b * S + k;
      printf("%.17g %d", t[r], steps[r]);
      for (int e = 0; e < N; ++e) printf(" %.17g", u_mean[r * N + e]);
      for (int e = 0; e < N * N; ++e) printf(" %.17g", u_chol[r * N * N + e]);
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
  int field, nu, fp, S, solver, control, clip_dt;
  if (fscanf(in, "%d %d %d %lld %d %d %d %d", &field, &nu, &fp, &B, &S, &solver, &control, &clip_dt) != 8) return 2;
  if (B < 1 || S < 2) return 2;
  int rc = 2;
  if (field == 1 && nu == 3 && fp) rc = run<3, VanDerPol, true>(in, B, S, solver, control, clip_dt);
  if (field == 0 && nu == 2 && fp) rc = run<2, LotkaVolterra, true>(in, B, S, solver, control, clip_dt);
  if (field == 0 && nu == 2 && !fp) rc = run<2, LotkaVolterra, false>(in, B, S, solver, control, clip_dt);
  fclose(in);
  return rc;
}
