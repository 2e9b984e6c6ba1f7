// Runs the posterior-sampling kernels (sample_iso_kernel, sample_dense_kernel)
// on the CPU, every (instance, sample) as its own "thread", on buffers of
// exactly the sizes pdq_sample_markov takes, so AddressSanitizer flags any
// access outside them.
//
// Input file (whitespace-separated): ssm (0 isotropic, 2 dense) nu d S B K,
// then marginal_mean, marginal_chol, cond_A, cond_noise_mean,
// cond_noise_chol, cond_to_latent, cond_to_observed, normals, in the layouts
// of include/pdq.h (pdq_sample_args).
// Output: the samples, one line per (instance, sample).
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "sample_kernels.cuh"

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
  int ssm, nu, d, S, K;
  long long B;
  if (fscanf(in, "%d %d %d %d %lld %d", &ssm, &nu, &d, &S, &B, &K) != 6) return 2;
  const bool iso = ssm == PDQ_SSM_ISOTROPIC;
  if (!iso && ssm != PDQ_SSM_DENSE) return 2;
  const long long n = nu + 1, N = n * d;
  const long long sq = iso ? n * n : N * N, mv = iso ? n * d : N, vec = iso ? n : N;
  std::vector<double> mm(B * mv), mc(B * sq), cA(B * (S - 1) * sq), cxi(B * (S - 1) * mv), cX(B * (S - 1) * sq),
      ctl(B * (S - 1) * vec), cto(B * (S - 1) * vec), z(B * K * S * vec), out(B * K * S * (iso ? n * d : N));
  if (!read_all(in, mm) || !read_all(in, mc) || !read_all(in, cA) || !read_all(in, cxi) || !read_all(in, cX) ||
      !read_all(in, ctl) || !read_all(in, cto) || !read_all(in, z))
    return 2;
  fclose(in);
  pdq_sample_args a;
  a.ssm = ssm;
  a.num_derivatives = nu;
  a.ode_dim = d;
  a.num_points = S;
  a.num_instances = B;
  a.num_samples = K;
  a.marginal_mean = mm.data();
  a.marginal_chol = mc.data();
  a.cond_A = cA.data();
  a.cond_noise_mean = cxi.data();
  a.cond_noise_chol = cX.data();
  a.cond_to_latent = ctl.data();
  a.cond_to_observed = cto.data();
  a.normals = z.data();
  a.samples = out.data();
  const int block = 128;
  blockDim = {uint32_t(block), 1, 1};
  const long long padded = (B * K + block - 1) / block * block;  // the launch's grid
  for (long long g = 0; g < padded; ++g) {
    blockIdx = {uint32_t(g / block), 0, 0};
    threadIdx = {uint32_t(g % block), 0, 0};
    if (iso)
      pdq::sample_iso_kernel(a);
    else
      pdq::sample_dense_kernel(a);
  }
  const long long per = S * (iso ? n * d : N);
  for (long long t = 0; t < B * K; ++t) {
    for (long long e = 0; e < per; ++e) printf("%s%.17g", e ? " " : "", out[t * per + e]);
    printf("\n");
  }
  return 0;
}
