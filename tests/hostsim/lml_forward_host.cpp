// Runs the float64 forward-mode LML kernel (lml_kernel: P threads per
// parameter sample, thread k carrying d / d params[k]) on the CPU after the
// plan kernel's thread, every thread as its own "thread" (the warp's staging
// of the plan takes the one-lane host path), on buffers of exactly the sizes
// the library computes, so AddressSanitizer flags any access outside them.
//
// Input file (whitespace-separated): field nu B N save_every average_pdfs,
// then params (B x P), y0 (B x 2), data (K x 2), std (K), dt, Q1
// ((nu + 1) x (nu + 1), row-major), K = N / save_every + 1; field 0 is
// FitzHugh-Nagumo (P = 3), field 1 Lotka-Volterra (P = 4).
// Output: one line per sample: status lml grad[P].
#include <cstdio>
#include <cstdlib>
#include <thread>
#include <vector>

#include "lml_solver.cuh"

thread_local pdq_host_uint3 threadIdx, blockIdx, blockDim;

using namespace pdq;

static bool read_all(FILE* in, std::vector<double>& v) {
  for (double& x : v)
    if (fscanf(in, "%lf", &x) != 1) return false;
  return true;
}

template <int NU, class F>
static int run(FILE* in, long long B, int N, int se, int avg) {
  constexpr int P = F::P;
  constexpr int D = F::D;
  constexpr int n = NU + 1;
  const int K = N / se + 1;
  std::vector<double> params(B * P), y0(B * D), data(K * D), stdv(K), dt(1), q1(n * n);
  if (!read_all(in, params) || !read_all(in, y0) || !read_all(in, data) || !read_all(in, stdv) || !read_all(in, dt) ||
      !read_all(in, q1))
    return 2;
  const int64_t plan_bytes = lml_plan_total_bytes(NU, N, se, 8);
  // per thread: the K - 1 stored offsets xi with their tangents (n d 2 numbers each)
  const int64_t ws_elems = int64_t(B) * P * (K - 1) * n * D * 2;
  unsigned char* plan = static_cast<unsigned char*>(calloc(plan_bytes, 1));
  double* ws = static_cast<double*>(malloc(ws_elems * 8));
  std::vector<double> lml(B), grad(B * P);
  std::vector<int32_t> status(B);

  LmlArgs a;
  memset(&a, 0, sizeof(a));
  a.B = B;
  a.num_steps = N;
  a.save_every = se;
  a.average_pdfs = avg;
  a.with_gradient = 1;
  a.lanes_per_sample = P;
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
  a.workspace = ws;

  blockDim = {1, 1, 1};  // the plan kernel's block as one thread
  blockIdx = {0, 0, 0};
  threadIdx = {0, 0, 0};
  lml_plan_kernel<double, NU>(a);
  blockDim = {uint32_t(kLmlThreads), 1, 1};
  const long long threads = B * P;
  const long long padded = (threads + kLmlThreads - 1) / kLmlThreads * kLmlThreads;  // the launch's grid
  if (getenv("PDQ_HOST_LML_WARPS") != nullptr) {  // each block's 32 lanes as threads
    for (long long blk = 0; blk < padded / kLmlThreads; ++blk) {
      PdqHostWarp warp;
      std::vector<std::thread> lanes;
      for (unsigned tid = 0; tid < unsigned(kLmlThreads); ++tid)
        lanes.emplace_back([&, tid] {
          blockDim = {uint32_t(kLmlThreads), 1, 1};
          blockIdx = {uint32_t(blk), 0, 0};
          threadIdx = {tid, 0, 0};
          pdq_host_warp = &warp;
          lml_kernel<double, NU, F>(a);
          pdq_host_warp = nullptr;
        });
      for (auto& th : lanes) th.join();
    }
  } else {
    for (long long t = 0; t < padded; ++t) {
      blockIdx = {uint32_t(t / kLmlThreads), 0, 0};
      threadIdx = {uint32_t(t % kLmlThreads), 0, 0};
      lml_kernel<double, NU, F>(a);
    }
  }
  for (long long b = 0; b < B; ++b) {
    printf("%d %.17g", status[b], lml[b]);
    for (int q = 0; q < P; ++q) printf(" %.17g", grad[b * P + q]);
    printf("\n");
  }
  free(plan);
  free(ws);
  return 0;
}

int main(int argc, char** argv) {
  if (argc != 2) return 2;
  FILE* in = fopen(argv[1], "r");
  if (!in) return 2;
  long long B;
  int field, nu, N, se, avg;
  if (fscanf(in, "%d %d %lld %d %d %d", &field, &nu, &B, &N, &se, &avg) != 6) return 2;
  if (B < 1 || N < 1 || se < 1 || N % se != 0) return 2;
  int rc = 2;
  if (field == 0 && nu == 3) rc = run<3, FitzHughNagumo>(in, B, N, se, avg);
  if (field == 0 && nu == 2) rc = run<2, FitzHughNagumo>(in, B, N, se, avg);
  if (field == 1 && nu == 3) rc = run<3, LotkaVolterra>(in, B, N, se, avg);
  fclose(in);
  return rc;
}
