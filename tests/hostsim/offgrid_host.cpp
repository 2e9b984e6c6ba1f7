// Runs the off-grid marginal kernels (offgrid_iso_kernel, offgrid_dense_kernel;
// one thread per (instance, query), float64) on the CPU, every thread as its
// own "thread", on buffers of exactly the sizes the library uses, so
// AddressSanitizer flags any access outside them.
//
// Input file (whitespace-separated): ssm (0 isotropic, 2 dense) strategy
// (0 filter, 2 fixed-interval) nu B S Q d, then t (B x S), u_mean, u_chol,
// output_scale (B x S), t_query (B x Q), filter_mean and filter_chol
// (fixed-interval only), Q1 ((nu + 1) x (nu + 1), row-major).  d is the
// ODE dimension: 1 to 8 for the isotropic kernel, 2 for the dense one.
// Output: one line per query: mean (flat) chol (flat).
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "offgrid_kernels.cuh"

thread_local pdq_host_uint3 threadIdx, blockIdx, blockDim;

static bool read_all(FILE* in, std::vector<double>& v) {
  for (double& x : v)
    if (fscanf(in, "%lf", &x) != 1) return false;
  return true;
}

int main(int argc, char** argv) {
  if (argc != 2) return 2;
  FILE* in = fopen(argv[1], "r");
  if (!in) return 2;
  int ssm, strategy, nu, S, Q, d;
  long long B;
  if (fscanf(in, "%d %d %d %lld %d %d %d", &ssm, &strategy, &nu, &B, &S, &Q, &d) != 7) return 2;
  if (!(nu == 2 || nu == 3) || (ssm != 0 && ssm != 2) || B < 1 || S < 2 || Q < 1) return 2;
  if (ssm == 0 ? (d < 1 || d > 8) : d != 2) return 2;
  const int n = nu + 1, N = n * d;
  const int mean_sz = ssm == 0 ? n * d : N, chol_sz = ssm == 0 ? n * n : N * N;
  const bool fi = strategy == 2;
  std::vector<double> t(B * S), um(B * S * mean_sz), uc(B * S * chol_sz), scale(B * S), tq(B * Q);
  std::vector<double> fm(fi ? B * S * mean_sz : 0), fc(fi ? B * S * chol_sz : 0), q1(n * n);
  if (!read_all(in, t) || !read_all(in, um) || !read_all(in, uc) || !read_all(in, scale) || !read_all(in, tq) ||
      !read_all(in, fm) || !read_all(in, fc) || !read_all(in, q1))
    return 2;
  fclose(in);
  std::vector<double> mean_out(B * Q * mean_sz), chol_out(B * Q * chol_sz);

  OffgridArgs args;
  memset(&args, 0, sizeof(args));
  pdq_offgrid_args& a = args.a;
  a.ssm = ssm;
  a.strategy = strategy;
  a.num_derivatives = nu;
  a.ode_dim = d;
  a.num_instances = B;
  a.num_points = S;
  a.num_queries = Q;
  a.t = t.data();
  a.u_mean = um.data();
  a.u_chol = uc.data();
  a.filter_mean = fi ? fm.data() : nullptr;
  a.filter_chol = fi ? fc.data() : nullptr;
  a.output_scale = scale.data();
  a.t_query = tq.data();
  a.mean_out = mean_out.data();
  a.chol_out = chol_out.data();
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) args.q1[i][j] = q1[i * n + j];

  const int block = 64;
  blockDim = {uint32_t(block), 1, 1};
  const long long threads = B * Q;
  const long long padded = (threads + block - 1) / block * block;  // the launch's grid
  for (long long g = 0; g < padded; ++g) {
    blockIdx = {uint32_t(g / block), 0, 0};
    threadIdx = {uint32_t(g % block), 0, 0};
    if (ssm == 0 && nu == 2) offgrid_iso_kernel<2>(args);
    if (ssm == 0 && nu == 3) offgrid_iso_kernel<3>(args);
    if (ssm == 2 && nu == 2) offgrid_dense_kernel<2, 2>(args);
    if (ssm == 2 && nu == 3) offgrid_dense_kernel<3, 2>(args);
  }
  for (long long r = 0; r < threads; ++r) {
    for (int e = 0; e < mean_sz; ++e) printf("%.17g ", mean_out[r * mean_sz + e]);
    for (int e = 0; e < chol_sz; ++e) printf(" %.17g", chol_out[r * chol_sz + e]);
    printf("\n");
  }
  return 0;
}
