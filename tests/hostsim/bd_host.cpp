// Runs the block-diagonal adaptive kernel (bd_adaptive_kernel, the Burgers
// stencil, one thread-block cluster per instance) on the CPU: every block
// of 256 threads as 256 host threads, the cluster's blocks at once, with
// __syncthreads, the warps' shuffles and the cluster's barriers and
// distributed shared memory emulated (cuda_runtime.h here), on buffers of
// exactly the sizes the library uses, so AddressSanitizer flags any access
// outside them (and ThreadSanitizer, in that build, any unordered access to
// shared memory).
//
// Input file (whitespace-separated): precision (0 float32, 1 float64)
// strategy (0 filter, 1 fixed-point smoother) B d S cluster solver ts1, then
// atol rtol, save_at (B x S), viscosity (B), y0 (B x d), dt0 (B),
// Q1 (4 x 4, row-major; nu = 3).
// Output: per instance a line "status attempts", then per save point a line
// "t num_steps u_mean[d n] u_chol[d n n]".
#include <cstdio>
#include <cstdlib>
#include <thread>
#include <vector>

#define PDQ_BD_SMEM unsigned char* smem_raw = pdq_host_block_smem()
#define PDQ_BD_SHARED(type, name, count)                   \
  type* name = reinterpret_cast<type*>(pdq_host_block_smem() + \
                                       pdq_host_cluster->fixed_offset(#name, sizeof(type) * (count)))

#include "bd_solver.cuh"

thread_local pdq_host_uint3 threadIdx, blockIdx, blockDim;

using namespace pdq;

static bool read_all(FILE* in, std::vector<double>& v) {
  for (double& x : v)
    if (fscanf(in, "%lf", &x) != 1) return false;
  return true;
}

template <typename T, bool FP>
static int run(FILE* in, long long B, int d, int S, int CL, int solver, int ts1) {
  constexpr int NU = 3, n = NU + 1;
  constexpr int NS = bd_state_rows<NU>();
  constexpr int CF = iso_cond_floats<NU, 1>();
  if (d % CL != 0 || d / CL > kBdThreads * kBdMaxDimsPerThread) return 2;
  std::vector<double> tol(2), save_at(B * S), visc(B), y0(B * d), dt0(B), q1(n * n);
  if (!read_all(in, tol) || !read_all(in, save_at) || !read_all(in, visc) || !read_all(in, y0) ||
      !read_all(in, dt0) || !read_all(in, q1))
    return 2;
  std::vector<double> u_mean(B * S * d * n), u_chol(B * S * d * n * n), scale(B * S * d), t(B * S);
  std::vector<int32_t> steps(B * S), attempts(B), status(B);
  // the workspace of pdq_workspace_size: state parity buffers, the MLE sums, FP conditionals
  size_t ws_bytes = 2 * size_t(B) * NS * size_t(d) * sizeof(T) + size_t(B) * d * 8;
  if (FP) ws_bytes += (2 + size_t(S - 1)) * size_t(B) * CF * size_t(d) * sizeof(T);
  std::vector<unsigned char> ws(ws_bytes, 0);

  BdArgs a;
  memset(&a, 0, sizeof(a));
  a.B = B;
  a.S = S;
  a.terminal_only = 0;
  a.solver = solver;
  a.control = 0;
  a.correct = 1;
  a.d = d;
  a.cluster = CL;
  a.ts1 = ts1;
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
  a.max_attempts = int64_t(1) << 20;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      a.q1[i][j] = q1[i * n + j];
      a.q1f[i][j] = float(q1[i * n + j]);
    }
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
  a.params = visc.data();
  a.y0 = y0.data();
  a.dt0 = dt0.data();
  a.u_mean = u_mean.data();
  a.u_chol = u_chol.data();
  a.output_scale = scale.data();
  a.t_out = t.data();
  a.num_steps = steps.data();
  a.num_attempts = attempts.data();
  a.status = status.data();
  a.workspace = ws.data();

  const int dl = d / CL;
  const size_t dyn = bd_smem_bytes<T, NU>(dl);
  for (long long inst = 0; inst < B; ++inst) {
    PdqHostCluster cluster;
    cluster.dim = CL;
    cluster.dynamic_bytes = (dyn + 15) / 16 * 16;
    cluster.region = cluster.dynamic_bytes + 512;
    cluster.expected = CL * kBdThreads;
    std::vector<unsigned char> smem(size_t(CL) * cluster.region, 0);
    cluster.base = smem.data();
    std::vector<PdqHostBarrier> block_bars(size_t(CL) * 3);
    for (int r = 0; r < CL; ++r) block_bars[size_t(r) * 3].expected = kBdThreads;
    std::vector<PdqHostWarp> warps(size_t(CL) * (kBdThreads / 32));
    std::vector<std::thread> threads;
    for (int r = 0; r < CL; ++r)
      for (unsigned tid = 0; tid < unsigned(kBdThreads); ++tid)
        threads.emplace_back([&, r, tid] {
          blockDim = {unsigned(kBdThreads), 1, 1};
          blockIdx = {uint32_t(inst * CL + r), 0, 0};
          threadIdx = {tid, 0, 0};
          pdq_host_cluster = &cluster;
          pdq_host_barriers = &block_bars[size_t(r) * 3];
          pdq_host_warp = &warps[size_t(r) * (kBdThreads / 32) + tid / 32];
          bd_adaptive_kernel<T, NU, FP>(a);
          pdq_host_warp = nullptr;
          pdq_host_barriers = nullptr;
          pdq_host_cluster = nullptr;
        });
    for (auto& th : threads) th.join();
  }
  for (long long b = 0; b < B; ++b) {
    printf("%d %d\n", status[b], attempts[b]);
    for (int k = 0; k < S; ++k) {
      const long long r = b * S + k;
      printf("%.17g %d", t[r], steps[r]);
      for (long long e = 0; e < (long long)d * n; ++e) printf(" %.17g", u_mean[r * d * n + e]);
      for (long long e = 0; e < (long long)d * n * n; ++e) printf(" %.17g", u_chol[r * d * n * n + e]);
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
  int prec, fp, d, S, CL, solver, ts1;
  if (fscanf(in, "%d %d %lld %d %d %d %d %d", &prec, &fp, &B, &d, &S, &CL, &solver, &ts1) != 8) return 2;
  if (B < 1 || S < 2 || d < 3 || CL < 1 || CL > 8) return 2;
  int rc = 2;
  if (prec == 1 && !fp) rc = run<double, false>(in, B, d, S, CL, solver, ts1);
  if (prec == 1 && fp) rc = run<double, true>(in, B, d, S, CL, solver, ts1);
  if (prec == 0 && !fp) rc = run<float, false>(in, B, d, S, CL, solver, ts1);
  fclose(in);
  return rc;
}
