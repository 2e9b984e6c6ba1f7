// Runs the adjoint LML kernels on the CPU (float64; float32 bulk for
// FitzHugh-Nagumo nu = 3):
// the plan kernel's single thread, then lml_adj_fwd_kernel and
// lml_adj_bwd_kernel for every sample as its own "thread" (they need no
// cooperation between threads).  Buffers have the exact sizes the library
// computes, so AddressSanitizer flags any access outside them.
//
// Input file (whitespace-separated): precision (0 float32 bulk, 1 float64)
// field nu B N save_every C average_pdfs,
// then params (B x P), y0 (B x 2), data (K x 2), std (K), cotangent (B), dt,
// Q1 ((nu + 1) x (nu + 1), row-major), K = N / save_every + 1; field 0 is
// FitzHugh-Nagumo (P = 3), field 1 Lotka-Volterra (P = 4); nu is 2 or 3.
// Output: one line per sample: status lml grad[P] grad_y0[2].
#include <cstdio>
#include <cstdlib>
#include <thread>
#include <vector>

#include "lml_adjoint.cuh"

thread_local pdq_host_uint3 threadIdx, blockIdx, blockDim;

using namespace pdq;

static bool read_all(FILE* in, std::vector<double>& v) {
  for (double& x : v)
    if (fscanf(in, "%lf", &x) != 1) return false;
  return true;
}

template <typename T, int NU, class F>
static int run(FILE* in, long long B, int N, int se, int C, int avg) {
  constexpr int P = F::P;
  constexpr int n = NU + 1;
  const int K = N / se + 1;
  std::vector<double> params(B * P), y0(B * 2), data(K * 2), stdv(K), cot(B), dt(1), q1(n * n);
  if (!read_all(in, params) || !read_all(in, y0) || !read_all(in, data) || !read_all(in, stdv) ||
      !read_all(in, cot) || !read_all(in, dt) || !read_all(in, q1))
    return 2;

  const int64_t plan_bytes = lml_plan_total_bytes(NU, N, se, int(sizeof(T)));
  const LmlAdjLayout L(NU, 2, N, se, C);
  const int64_t res_elems = int64_t(B) * L.total;
  unsigned char* plan = static_cast<unsigned char*>(calloc(plan_bytes, 1));
  T* res = static_cast<T*>(malloc(res_elems * sizeof(T)));
  // NaN everywhere: a residual read before it is written poisons the result
  for (int64_t i = 0; i < res_elems; ++i) res[i] = T(__longlong_as_double(0x7ff8000000000001LL));
  std::vector<double> lml(B), grad(B * P), gy0(B * 2);
  std::vector<int32_t> status(B);

  LmlAdjArgs aa;
  memset(&aa, 0, sizeof(aa));
  LmlArgs& a = aa.base;
  a.B = B;
  a.num_steps = N;
  a.save_every = se;
  a.average_pdfs = avg;
  a.lanes_per_sample = 1;
  a.dt = dt[0];
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) a.q1[i][j] = q1[i * n + j];
  a.params = params.data();
  a.y0 = y0.data();
  a.data = data.data();
  a.std = stdv.data();
  a.lml = lml.data();
  a.grad = grad.data();
  a.status = status.data();
  a.plan = plan;
  aa.ckpt = C;
  aa.num_ckpt = (N + C - 1) / C;
  aa.cotangent = cot.data();
  aa.grad_y0 = gy0.data();
  aa.res = res;

  blockDim = {1, 1, 1};  // the plan kernel's block as one thread
  blockIdx = {0, 0, 0};
  threadIdx = {0, 0, 0};
  lml_plan_kernel<T, NU>(a);
  blockDim = {uint32_t(kLmlThreads), 1, 1};
  const long long padded = (B + kLmlThreads - 1) / kLmlThreads * kLmlThreads;  // the launch's grid
  const bool warps = getenv("PDQ_HOST_LML_WARPS") != nullptr;  // each block's 32 lanes as threads
  for (int pass = 0; pass < 2; ++pass) {
    if (warps) {
      for (long long blk = 0; blk < padded / kLmlThreads; ++blk) {
        PdqHostWarp warp;
        std::vector<std::thread> lanes;
        for (unsigned tid = 0; tid < unsigned(kLmlThreads); ++tid)
          lanes.emplace_back([&, tid] {
            blockDim = {uint32_t(kLmlThreads), 1, 1};
            blockIdx = {uint32_t(blk), 0, 0};
            threadIdx = {tid, 0, 0};
            pdq_host_warp = &warp;
            if (pass == 0)
              lml_adj_fwd_kernel<T, NU, F>(aa);
            else
              lml_adj_bwd_kernel<T, NU, F>(aa);
            pdq_host_warp = nullptr;
          });
        for (auto& th : lanes) th.join();
      }
      continue;
    }
    for (long long t = 0; t < padded; ++t) {
      blockIdx = {uint32_t(t / kLmlThreads), 0, 0};
      threadIdx = {uint32_t(t % kLmlThreads), 0, 0};
      if (pass == 0)
        lml_adj_fwd_kernel<T, NU, F>(aa);
      else
        lml_adj_bwd_kernel<T, NU, F>(aa);
    }
  }
  for (long long b = 0; b < B; ++b) {
    printf("%d %.17g", status[b], lml[b]);
    for (int q = 0; q < P; ++q) printf(" %.17g", grad[b * P + q]);
    printf(" %.17g %.17g\n", gy0[b * 2], gy0[b * 2 + 1]);
  }
  free(plan);
  free(res);
  return 0;
}

int main(int argc, char** argv) {
  if (argc != 2) return 2;
  FILE* in = fopen(argv[1], "r");
  if (!in) return 2;
  long long B;
  int prec, field, nu, N, se, C, avg;
  if (fscanf(in, "%d %d %d %lld %d %d %d %d", &prec, &field, &nu, &B, &N, &se, &C, &avg) != 8) return 2;
  if (B < 1 || N < 1 || se < 1 || N % se != 0 || C < 1 || C > N) return 2;
  int rc = 2;
  if (prec == 1 && field == 0 && nu == 3) rc = run<double, 3, FitzHughNagumo>(in, B, N, se, C, avg);
  if (prec == 1 && field == 0 && nu == 2) rc = run<double, 2, FitzHughNagumo>(in, B, N, se, C, avg);
  if (prec == 1 && field == 1 && nu == 3) rc = run<double, 3, LotkaVolterra>(in, B, N, se, C, avg);
  if (prec == 0 && field == 0 && nu == 3) rc = run<float, 3, FitzHughNagumo>(in, B, N, se, C, avg);
  fclose(in);
  return rc;
}
