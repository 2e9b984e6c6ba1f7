// Host side of the C ABI declared in include/pdq.h: validation, constants of
// the IWP prior, and dispatch to the solver kernels.
#include <math.h>
#include <string.h>

#include "pdq_nvtx.h"
#include "bd_launch.cuh"
#include "dense_launch.cuh"
#include "offgrid.h"
#include "lml_adj_launch.cuh"
#include "lml_launch.cuh"
#include "iso_launch.cuh"
#include "iso_split_launch.cuh"
#include "nvrtc_fields.h"
#include "tv_launch.cuh"
#include "pdq.h"

namespace {

// Lower square root (non-negative diagonal) of flip(Hilbert(n)):
// (Q Q^T)[i][j] = 1 / (2 nu + 1 - i - j).  This is the Q_1d of
// system_matrices_1d_iwp (_probdiffeq/utilities.py:57-71); the Cholesky
// factor is unique, computed here in long double.
void iwp_q1(int nu, double (&q)[pdq::kMaxN][pdq::kMaxN]) {
  const int n = nu + 1;
  long double c[pdq::kMaxN][pdq::kMaxN] = {};
  for (int i = 0; i < n; ++i) {
    for (int j = 0; j <= i; ++j) {
      long double s = 1.0L / (long double)(2 * nu + 1 - i - j);
      for (int k = 0; k < j; ++k) s -= c[i][k] * c[j][k];
      if (i == j)
        c[i][j] = sqrtl(s > 0 ? s : 0);
      else
        c[i][j] = c[j][j] > 0 ? s / c[j][j] : 0;
    }
  }
  for (int i = 0; i < pdq::kMaxN; ++i)
    for (int j = 0; j < pdq::kMaxN; ++j) q[i][j] = (i < n && j <= i) ? (double)c[i][j] : 0.0;
}

int field_dim(int field) {
  if (field >= PDQ_FIELD_USER_BASE) return pdq_user_field_dim(field);
  switch (field) {
    case PDQ_FIELD_LOTKA_VOLTERRA:
    case PDQ_FIELD_VAN_DER_POL:
    case PDQ_FIELD_FITZHUGH_NAGUMO:
      return 2;
    case PDQ_FIELD_BURGERS:
      return -1;  // any
    default:
      return 0;
  }
}

pdq_status validate_common(const pdq_config* c) {
  if (c == nullptr) return PDQ_ERROR_INVALID_VALUE;
  if (c->abi_version != PDQ_ABI_VERSION) return PDQ_ERROR_ABI_VERSION;
  if (c->num_derivatives < 1 || c->num_derivatives > 5) return PDQ_ERROR_UNSUPPORTED;
  const int d = field_dim(c->field);
  if (d == 0) return PDQ_ERROR_INVALID_VALUE;
  if (d > 0 && c->ode_dim != d) return PDQ_ERROR_INVALID_VALUE;
  if (c->precision != PDQ_PRECISION_F32 && c->precision != PDQ_PRECISION_F64) return PDQ_ERROR_INVALID_VALUE;
  if (c->solver < PDQ_SOLVER_PLAIN || c->solver > PDQ_SOLVER_DYNAMIC) return PDQ_ERROR_INVALID_VALUE;
  if (c->control != PDQ_CONTROL_INTEGRAL && c->control != PDQ_CONTROL_PROPORTIONAL_INTEGRAL)
    return PDQ_ERROR_INVALID_VALUE;
  if (c->error != PDQ_ERROR_RESIDUAL_STD && c->error != PDQ_ERROR_STATE_STD) return PDQ_ERROR_INVALID_VALUE;
  if (!(c->atol >= 0) || !(c->rtol >= 0) || !(c->atol + c->rtol > 0)) return PDQ_ERROR_INVALID_VALUE;
  if (!(c->eps >= 0) || !(c->damp >= 0)) return PDQ_ERROR_INVALID_VALUE;
  if (!(c->factor_min > 0) || !(c->factor_max >= c->factor_min) || !(c->safety > 0)) return PDQ_ERROR_INVALID_VALUE;
  if (c->max_attempts < 1) return PDQ_ERROR_INVALID_VALUE;
  if (c->reserved0 != 0) return PDQ_ERROR_INVALID_VALUE;
  // a registered stencil serves the block-diagonal kernel only
  if (c->field >= PDQ_FIELD_USER_BASE && pdq_user_field_is_stencil(c->field) && c->ssm != PDQ_SSM_BLOCKDIAG)
    return PDQ_ERROR_UNSUPPORTED;
  // launch shapes any mapping accepts (each mapping checks its own subset)
  const int ipb = c->instances_per_block;
  if (!(ipb == 0 || (ipb >= 1 && ipb <= 4) || ipb == 8 || ipb == 16 || ipb == 32 || ipb == 64))
    return PDQ_ERROR_INVALID_VALUE;
  return PDQ_SUCCESS;
}

// The isotropic kernels' arguments from the configuration and the solve's
// buffers (the mapping, the posterior outputs and the record stay zero).
void iso_args_fill(const pdq_config* c, const pdq_adaptive_args* args, pdq::IsoArgs& a) {
  memset(&a, 0, sizeof(a));
  a.B = args->num_instances;
  a.S = args->num_save_at;
  a.terminal_only = args->terminal_only ? 1 : 0;
  a.solver = c->solver;
  a.control = c->control;
  a.clip_dt = c->clip_dt ? 1 : 0;
  a.correct = c->correct_asymptotic_underconfidence ? 1 : 0;
  a.ts1 = c->constraint == PDQ_CONSTRAINT_TS1 ? 1 : 0;
  a.state_error = c->error == PDQ_ERROR_STATE_STD ? 1 : 0;
  a.safety = c->safety;
  a.factor_min = c->factor_min;
  a.factor_max = c->factor_max;
  a.exp_i = c->exponent_integral;
  a.exp_p = c->exponent_proportional;
  a.atol = c->atol;
  a.rtol = c->rtol;
  a.eps = c->eps;
  a.damp = c->damp;
  a.max_attempts = c->max_attempts;
  iwp_q1(c->num_derivatives, a.q1);
  for (int i = 0; i < pdq::kMaxN; ++i)
    for (int j = 0; j < pdq::kMaxN; ++j) a.q1f[i][j] = float(a.q1[i][j]);
  a.safety_f = float(a.safety);
  a.factor_min_f = float(a.factor_min);
  a.factor_max_f = float(a.factor_max);
  a.exp_i_f = float(a.exp_i);
  a.exp_p_f = float(a.exp_p);
  a.atol_f = float(a.atol);
  a.rtol_f = float(a.rtol);
  a.eps_f = float(a.eps);
  a.damp_f = float(a.damp);
  a.save_at = args->save_at;
  a.params = args->params;
  a.y0 = args->y0;
  a.dt0 = args->dt0;
  a.u_mean = args->u_mean;
  a.u_chol = args->u_chol;
  a.output_scale = args->output_scale;
  a.t_out = args->t;
  a.num_steps = args->num_steps;
  a.num_attempts = args->num_attempts;
  a.status = args->status;
}

// The terminal-value adjoint's configuration rules (include/pdq.h).
pdq_status terminal_check(const pdq_config* c) {
  const pdq_status st = validate_common(c);
  if (st != PDQ_SUCCESS) return st;
  if (c->ssm != PDQ_SSM_ISOTROPIC || c->constraint != PDQ_CONSTRAINT_TS0 || c->strategy != PDQ_STRATEGY_FILTER ||
      c->error != PDQ_ERROR_RESIDUAL_STD || !c->clip_dt || c->damp != 0.0 ||
      (c->solver != PDQ_SOLVER_PLAIN && c->solver != PDQ_SOLVER_MLE) || c->field >= PDQ_FIELD_USER_BASE ||
      c->kernel_variant > 1)
    return PDQ_ERROR_UNSUPPORTED;
  if (!(c->instances_per_block == 0 || c->instances_per_block == 64)) return PDQ_ERROR_INVALID_VALUE;
  return PDQ_SUCCESS;
}

using TvLaunch = cudaError_t (*)(const pdq::IsoArgs&, const pdq::TvAdjArgs*, int, cudaStream_t);

TvLaunch tv_launcher(const pdq_config* c) {
  const bool f64 = c->precision == PDQ_PRECISION_F64;
  switch (c->field) {
    case PDQ_FIELD_LOTKA_VOLTERRA: return f64 ? pdq_launch_tv_lv_f64 : pdq_launch_tv_lv_f32;
    case PDQ_FIELD_VAN_DER_POL: return f64 ? pdq_launch_tv_vdp_f64 : pdq_launch_tv_vdp_f32;
    case PDQ_FIELD_FITZHUGH_NAGUMO: return f64 ? pdq_launch_tv_fhn_f64 : pdq_launch_tv_fhn_f32;
    default: return nullptr;
  }
}

// Bytes of the record and, after it at a 256-byte boundary, the adjoint pass's scratch.
void terminal_sizes(const pdq_config* c, int64_t B, int32_t capacity, int32_t ckpt, size_t* rec_bytes,
                    size_t* total) {
  const size_t elem = c->precision == PDQ_PRECISION_F64 ? 8 : 4;
  const size_t rec = size_t(B) * size_t(pdq::tv_record_elems(c->num_derivatives, c->ode_dim, capacity, ckpt)) * elem;
  *rec_bytes = (rec + 255) / 256 * 256;
  *total = *rec_bytes + size_t(B) * size_t(pdq::tv_scratch_elems(c->num_derivatives, c->ode_dim, ckpt)) * elem;
}

}  // namespace

extern "C" {

uint32_t pdq_abi_version(void) { return PDQ_ABI_VERSION; }

const char* pdq_status_string(pdq_status s) {
  switch (s) {
    case PDQ_SUCCESS: return "success";
    case PDQ_ERROR_INVALID_VALUE: return "invalid value";
    case PDQ_ERROR_UNSUPPORTED: return "unsupported configuration";
    case PDQ_ERROR_CUDA: return "CUDA error";
    case PDQ_ERROR_WORKSPACE: return "workspace too small";
    case PDQ_ERROR_ABI_VERSION: return "ABI version mismatch";
    case PDQ_ERROR_STATIC_SCRATCH: return "problem exceeds the library's static scratch array";
    case PDQ_ERROR_COMPILE: return "run-time compilation of the vector field failed";
    default: return "unknown status";
  }
}

pdq_status pdq_config_default(pdq_config* c, int32_t ssm, int32_t field, int32_t num_derivatives, int32_t ode_dim) {
  if (c == nullptr) return PDQ_ERROR_INVALID_VALUE;
  memset(c, 0, sizeof(*c));
  c->abi_version = PDQ_ABI_VERSION;
  c->ssm = ssm;
  c->constraint = PDQ_CONSTRAINT_TS0;
  c->strategy = PDQ_STRATEGY_FILTER;
  c->solver = PDQ_SOLVER_DYNAMIC;
  c->error = PDQ_ERROR_RESIDUAL_STD;
  c->control = PDQ_CONTROL_INTEGRAL;
  c->precision = PDQ_PRECISION_F32;
  c->field = field;
  c->num_derivatives = num_derivatives;
  c->ode_dim = ode_dim;
  c->clip_dt = 1;
  c->correct_asymptotic_underconfidence = 1;
  c->safety = 0.95;
  c->factor_min = 0.2;
  c->factor_max = 10.0;
  c->exponent_integral = 0.3;
  c->exponent_proportional = 0.4;
  c->atol = 1e-6;
  c->rtol = 1e-6;
  c->eps = 1e-8;
  c->damp = 0.0;
  c->max_attempts = 1 << 20;
  return PDQ_SUCCESS;
}

pdq_status pdq_workspace_size(const pdq_config* c, int64_t num_instances, int32_t num_save_at, size_t* bytes) {
  if (bytes == nullptr) return PDQ_ERROR_INVALID_VALUE;
  pdq_status st = validate_common(c);
  if (st != PDQ_SUCCESS) return st;
  if (num_instances < 0 || num_save_at < 2) return PDQ_ERROR_INVALID_VALUE;
  *bytes = 0;
  if (c->ssm == PDQ_SSM_BLOCKDIAG) {
    const size_t elem = c->precision == PDQ_PRECISION_F64 ? 8 : 4;
    const int nu = c->num_derivatives;
    const size_t rows = size_t(nu + 1) + size_t(nu + 1) * (nu + 2) / 2;
    *bytes = 2 * size_t(num_instances) * rows * size_t(c->ode_dim) * elem + size_t(num_instances) * c->ode_dim * 8;
    if (c->strategy == PDQ_STRATEGY_FIXEDPOINT) {
      // running conditionals (2 parity buffers) and one per checkpoint interval, per dimension
      const size_t n = size_t(nu + 1);
      const size_t cf = n * n + n + n * (n + 1) / 2 + 2 * n;
      *bytes += (2 + size_t(num_save_at - 1)) * size_t(num_instances) * cf * size_t(c->ode_dim) * elem;
    }
  }
  if (c->ssm == PDQ_SSM_ISOTROPIC && c->strategy == PDQ_STRATEGY_FIXEDPOINT) {
    const int n = c->num_derivatives + 1, d = c->ode_dim;
    const size_t floats = size_t(n) * n + size_t(n) * d + size_t(n) * (n + 1) / 2 + 2 * size_t(n);
    const size_t elem = c->precision == PDQ_PRECISION_F64 ? 8 : 4;
    *bytes = size_t(num_instances) * size_t(num_save_at - 1) * floats * elem;
  }
  if (c->ssm == PDQ_SSM_DENSE && c->strategy == PDQ_STRATEGY_FIXEDPOINT) {
    const int N = (c->num_derivatives + 1) * c->ode_dim;
    const size_t floats = size_t(N) * N + N + size_t(N) * (N + 1) / 2 + 2 * N;
    const size_t elem = c->precision == PDQ_PRECISION_F64 ? 8 : 4;
    *bytes = size_t(num_instances) * size_t(num_save_at - 1) * floats * elem;
  }
  return PDQ_SUCCESS;
}

pdq_status pdq_solve_adaptive(const pdq_config* c, const pdq_adaptive_args* args, void* workspace,
                              size_t workspace_bytes, void* stream_ptr) {
  pdq::NvtxRange nvtx_range("pdq_solve_adaptive");
  (void)workspace;
  (void)workspace_bytes;
  pdq_status st = validate_common(c);
  if (st != PDQ_SUCCESS) return st;
  if (args == nullptr || args->num_instances < 0 || args->num_save_at < 2) return PDQ_ERROR_INVALID_VALUE;
  if (args->num_instances == 0) return PDQ_SUCCESS;
  if (!args->save_at || !args->params || !args->y0 || !args->dt0 || !args->u_mean || !args->u_chol ||
      !args->output_scale || !args->t || !args->num_steps || !args->num_attempts || !args->status)
    return PDQ_ERROR_INVALID_VALUE;
  cudaStream_t stream = static_cast<cudaStream_t>(stream_ptr);

  if (c->ssm == PDQ_SSM_ISOTROPIC) {
    if (c->constraint != PDQ_CONSTRAINT_TS0 && c->constraint != PDQ_CONSTRAINT_TS1) return PDQ_ERROR_INVALID_VALUE;
    if (c->strategy != PDQ_STRATEGY_FILTER && c->strategy != PDQ_STRATEGY_FIXEDPOINT) return PDQ_ERROR_INVALID_VALUE;
    const bool fp = c->strategy == PDQ_STRATEGY_FIXEDPOINT;
    if (fp) {
      size_t need = 0;
      pdq_workspace_size(c, args->num_instances, args->num_save_at, &need);
      if (workspace == nullptr || workspace_bytes < need) return PDQ_ERROR_WORKSPACE;
    }
    pdq::IsoArgs a;
    iso_args_fill(c, args, a);
    const bool interp = !c->clip_dt;
    if (c->kernel_variant < 0 || c->kernel_variant > 4) return PDQ_ERROR_INVALID_VALUE;
    if (c->kernel_variant == 4) {
      // a covariance warp and a mean warp per 32 instances: the lean filter
      // (TS0 without damping, error_residual_std, exact landings), solver none or mle
      if (!c->clip_dt || a.ts1 || a.state_error || fp || a.damp != 0.0 || c->solver == PDQ_SOLVER_DYNAMIC ||
          args->u_mean_d_params || args->u_mean_d_y0 || c->field >= PDQ_FIELD_USER_BASE)
        return PDQ_ERROR_UNSUPPORTED;
      if (c->instances_per_block != 0) return PDQ_ERROR_INVALID_VALUE;
      using SplitLaunch = cudaError_t (*)(const pdq::IsoArgs&, int, cudaStream_t);
      const bool f64 = c->precision == PDQ_PRECISION_F64;
      SplitLaunch launch = nullptr;
      switch (c->field) {
        case PDQ_FIELD_LOTKA_VOLTERRA: launch = f64 ? pdq_launch_iso_split_lv_f64 : pdq_launch_iso_split_lv_f32; break;
        case PDQ_FIELD_VAN_DER_POL: launch = f64 ? pdq_launch_iso_split_vdp_f64 : pdq_launch_iso_split_vdp_f32; break;
        case PDQ_FIELD_FITZHUGH_NAGUMO:
          launch = f64 ? pdq_launch_iso_split_fhn_f64 : pdq_launch_iso_split_fhn_f32;
          break;
        default: return PDQ_ERROR_UNSUPPORTED;
      }
      return launch(a, c->num_derivatives, stream) == cudaSuccess ? PDQ_SUCCESS : PDQ_ERROR_CUDA;
    }
    // 0 (auto) and 1: one thread per instance; 2 / 3: the lane-cooperative
    // kernel (8 lanes per instance) with <= 128 / <= 85 registers per lane,
    // for exact checkpoint landings only
    const bool warp = c->clip_dt && c->kernel_variant >= 2;
    if (c->kernel_variant >= 2 && (!c->clip_dt || a.ts1 || a.state_error || fp)) return PDQ_ERROR_UNSUPPORTED;
    a.tan_params = args->u_mean_d_params;
    a.tan_y0 = args->u_mean_d_y0;
    a.tangents = (a.tan_params || a.tan_y0) ? 1 : 0;
    if (a.tangents && (a.ts1 || a.state_error || fp || c->kernel_variant >= 2 || c->field >= PDQ_FIELD_USER_BASE))
      return PDQ_ERROR_UNSUPPORTED;
    const int ipb = c->instances_per_block;
    if (warp ? !(ipb == 0 || ipb == 8 || ipb == 16 || ipb == 32) : !(ipb == 0 || ipb == 32 || ipb == 64))
      return PDQ_ERROR_INVALID_VALUE;
    a.instances_per_block = ipb;
    a.workspace = workspace;
    if (fp) {
      a.cond_A = args->cond_A;
      a.cond_noise_mean = args->cond_noise_mean;
      a.cond_noise_chol = args->cond_noise_chol;
      a.cond_to_latent = args->cond_to_latent;
      a.cond_to_observed = args->cond_to_observed;
      a.filter_mean = args->filter_mean;
      a.filter_chol = args->filter_chol;
      if ((a.cond_A || a.filter_mean) && (!a.cond_A || !a.cond_noise_mean || !a.cond_noise_chol || !a.cond_to_latent ||
                                          !a.cond_to_observed || !a.filter_mean || !a.filter_chol))
        return PDQ_ERROR_INVALID_VALUE;
    }
    const int block = warp ? -(c->kernel_variant == 2 ? 2 : 3) : (ipb > 0 ? ipb : 64);
    const bool f64 = c->precision == PDQ_PRECISION_F64;
    cudaError_t err;
    if (c->field >= PDQ_FIELD_USER_BASE) {
      if (warp) return PDQ_ERROR_UNSUPPORTED;
      err = pdq_launch_iso_user(a, c->field, f64, c->num_derivatives, interp, fp, stream, block);
      return err == cudaSuccess ? PDQ_SUCCESS : (err == cudaErrorInvalidSource ? PDQ_ERROR_COMPILE : PDQ_ERROR_CUDA);
    }
    using IsoLaunch = cudaError_t (*)(const pdq::IsoArgs&, int, bool, cudaStream_t, int);
    IsoLaunch launch = nullptr;
    switch (c->field) {
      case PDQ_FIELD_LOTKA_VOLTERRA:
        launch = fp ? (f64 ? pdq_launch_iso_fp_lv_f64 : pdq_launch_iso_fp_lv_f32)
                    : (f64 ? pdq_launch_iso_lv_f64 : pdq_launch_iso_lv_f32);
        break;
      case PDQ_FIELD_VAN_DER_POL:
        launch = fp ? (f64 ? pdq_launch_iso_fp_vdp_f64 : pdq_launch_iso_fp_vdp_f32)
                    : (f64 ? pdq_launch_iso_vdp_f64 : pdq_launch_iso_vdp_f32);
        break;
      case PDQ_FIELD_FITZHUGH_NAGUMO:
        launch = fp ? (f64 ? pdq_launch_iso_fp_fhn_f64 : pdq_launch_iso_fp_fhn_f32)
                    : (f64 ? pdq_launch_iso_fhn_f64 : pdq_launch_iso_fhn_f32);
        break;
      default:
        return PDQ_ERROR_UNSUPPORTED;
    }
    err = launch(a, c->num_derivatives, interp, stream, block);
    return err == cudaSuccess ? PDQ_SUCCESS : PDQ_ERROR_CUDA;
  }
  if (c->ssm == PDQ_SSM_BLOCKDIAG) {
    // the Burgers stencil, or a registered one (pdq_register_stencil; TS0 only)
    const bool user_stencil = c->field >= PDQ_FIELD_USER_BASE && pdq_user_field_is_stencil(c->field);
    if (c->field != PDQ_FIELD_BURGERS && !user_stencil) return PDQ_ERROR_UNSUPPORTED;
    if (user_stencil && c->constraint != PDQ_CONSTRAINT_TS0) return PDQ_ERROR_UNSUPPORTED;
    if (c->instances_per_block != 0) return PDQ_ERROR_INVALID_VALUE;  // one cluster per instance
    if (args->u_mean_d_params || args->u_mean_d_y0) return PDQ_ERROR_UNSUPPORTED;
    if (c->constraint != PDQ_CONSTRAINT_TS0 && c->constraint != PDQ_CONSTRAINT_TS1) return PDQ_ERROR_INVALID_VALUE;
    if (c->strategy != PDQ_STRATEGY_FILTER && c->strategy != PDQ_STRATEGY_FIXEDPOINT) return PDQ_ERROR_INVALID_VALUE;
    if (!c->clip_dt) return PDQ_ERROR_UNSUPPORTED;  // checkpoints by exact landing only
    const bool any_post = args->cond_A || args->cond_noise_mean || args->cond_noise_chol || args->cond_to_latent ||
                          args->cond_to_observed || args->filter_mean || args->filter_chol;
    const bool all_post = args->cond_A && args->cond_noise_mean && args->cond_noise_chol && args->cond_to_latent &&
                          args->cond_to_observed && args->filter_mean && args->filter_chol;
    if (any_post && c->strategy != PDQ_STRATEGY_FIXEDPOINT) return PDQ_ERROR_UNSUPPORTED;  // a smoother's posterior
    if (any_post && !all_post) return PDQ_ERROR_INVALID_VALUE;
    if (c->num_derivatives < 2 || c->num_derivatives > 4) return PDQ_ERROR_UNSUPPORTED;
    const int d = c->ode_dim;
    if (d < 3) return PDQ_ERROR_INVALID_VALUE;
    const int CL = pdq::bd_cluster_size(d);
    if (d % CL != 0 || d / CL > pdq::kBdThreads * pdq::kBdMaxDimsPerThread) return PDQ_ERROR_UNSUPPORTED;
    size_t need = 0;
    pdq_workspace_size(c, args->num_instances, args->num_save_at, &need);
    if (workspace == nullptr || workspace_bytes < need) return PDQ_ERROR_WORKSPACE;
    pdq::BdArgs a;
    memset(&a, 0, sizeof(a));
    a.B = args->num_instances;
    a.S = args->num_save_at;
    a.terminal_only = args->terminal_only ? 1 : 0;
    a.solver = c->solver;
    a.control = c->control;
    a.correct = c->correct_asymptotic_underconfidence ? 1 : 0;
    a.d = d;
    a.cluster = CL;
    a.ts1 = c->constraint == PDQ_CONSTRAINT_TS1 ? 1 : 0;
    a.state_error = c->error == PDQ_ERROR_STATE_STD ? 1 : 0;
    a.fixedpoint = c->strategy == PDQ_STRATEGY_FIXEDPOINT ? 1 : 0;
    if (any_post) {
      a.cond_A = args->cond_A;
      a.cond_noise_mean = args->cond_noise_mean;
      a.cond_noise_chol = args->cond_noise_chol;
      a.cond_to_latent = args->cond_to_latent;
      a.cond_to_observed = args->cond_to_observed;
      a.filter_mean = args->filter_mean;
      a.filter_chol = args->filter_chol;
    }
    a.safety = c->safety;
    a.factor_min = c->factor_min;
    a.factor_max = c->factor_max;
    a.exp_i = c->exponent_integral;
    a.exp_p = c->exponent_proportional;
    a.atol = c->atol;
    a.rtol = c->rtol;
    a.eps = c->eps;
    a.damp = c->damp;
    a.max_attempts = c->max_attempts;
    iwp_q1(c->num_derivatives, a.q1);
    for (int i = 0; i < pdq::kMaxN; ++i)
      for (int j = 0; j < pdq::kMaxN; ++j) a.q1f[i][j] = float(a.q1[i][j]);
    a.safety_f = float(a.safety);
    a.factor_min_f = float(a.factor_min);
    a.factor_max_f = float(a.factor_max);
    a.exp_i_f = float(a.exp_i);
    a.exp_p_f = float(a.exp_p);
    a.atol_f = float(a.atol);
    a.rtol_f = float(a.rtol);
    a.eps_f = float(a.eps);
    a.damp_f = float(a.damp);
    a.save_at = args->save_at;
    a.params = args->params;
    a.y0 = args->y0;
    a.dt0 = args->dt0;
    a.u_mean = args->u_mean;
    a.u_chol = args->u_chol;
    a.output_scale = args->output_scale;
    a.t_out = args->t;
    a.num_steps = args->num_steps;
    a.num_attempts = args->num_attempts;
    a.status = args->status;
    a.workspace = workspace;
    if (user_stencil) {
      const cudaError_t err =
          pdq_launch_bd_user(a, c->field, c->precision == PDQ_PRECISION_F64, c->num_derivatives, stream);
      return err == cudaSuccess ? PDQ_SUCCESS : (err == cudaErrorInvalidSource ? PDQ_ERROR_COMPILE : PDQ_ERROR_CUDA);
    }
    const cudaError_t err = c->precision == PDQ_PRECISION_F64
                                ? pdq_launch_bd_burgers_f64(a, c->num_derivatives, stream)
                                : pdq_launch_bd_burgers_f32(a, c->num_derivatives, stream);
    return err == cudaSuccess ? PDQ_SUCCESS : PDQ_ERROR_CUDA;
  }
  if (c->ssm == PDQ_SSM_DENSE) {
    // kernel_variant 1: one thread per instance; 2: eight lanes per instance; 3 / 4 / 5: the
    // structure-exploiting kernel with four / eight / sixteen lanes per instance; 0: 4 unless
    // error_state_std or a run-time field asks for 1 (error_state_std: the thread-per-instance mapping only)
    const bool state_std = c->error == PDQ_ERROR_STATE_STD;
    const bool user_field = c->field >= PDQ_FIELD_USER_BASE;
    if (c->kernel_variant < 0 || c->kernel_variant > 5) return PDQ_ERROR_INVALID_VALUE;
    if ((state_std || user_field) && c->kernel_variant >= 2) return PDQ_ERROR_UNSUPPORTED;
    const int variant = c->kernel_variant != 0 ? c->kernel_variant : ((state_std || user_field) ? 1 : 4);
    if (args->u_mean_d_params || args->u_mean_d_y0) return PDQ_ERROR_UNSUPPORTED;
    {
      const int ipb = c->instances_per_block;
      const bool ok = variant == 2 ? (ipb >= 0 && ipb <= 4)
                                   : (variant >= 3 ? ipb == 0 : (ipb == 0 || ipb == 8 || ipb == 16 || ipb == 32));
      if (!ok) return PDQ_ERROR_INVALID_VALUE;
    }
    if (c->num_derivatives < 2 || c->num_derivatives > 3) return PDQ_ERROR_UNSUPPORTED;
    if (c->constraint != PDQ_CONSTRAINT_TS0 && c->constraint != PDQ_CONSTRAINT_TS1) return PDQ_ERROR_INVALID_VALUE;
    if (c->strategy != PDQ_STRATEGY_FILTER && c->strategy != PDQ_STRATEGY_FIXEDPOINT) return PDQ_ERROR_INVALID_VALUE;
    const bool fp = c->strategy == PDQ_STRATEGY_FIXEDPOINT;
    size_t need = 0;
    pdq_workspace_size(c, args->num_instances, args->num_save_at, &need);
    if (need > 0 && (workspace == nullptr || workspace_bytes < need)) return PDQ_ERROR_WORKSPACE;
    const bool any_cond = args->cond_A || args->cond_noise_mean || args->cond_noise_chol || args->cond_to_latent ||
                          args->cond_to_observed;
    const bool all_cond = args->cond_A && args->cond_noise_mean && args->cond_noise_chol && args->cond_to_latent &&
                          args->cond_to_observed;
    if (any_cond && (!all_cond || !fp || args->terminal_only)) return PDQ_ERROR_INVALID_VALUE;
    if ((args->filter_mean == nullptr) != (args->filter_chol == nullptr)) return PDQ_ERROR_INVALID_VALUE;
    pdq::DenseArgs a;
    memset(&a, 0, sizeof(a));
    a.B = args->num_instances;
    a.S = args->num_save_at;
    a.terminal_only = args->terminal_only ? 1 : 0;
    a.solver = c->solver;
    a.control = c->control;
    a.clip_dt = c->clip_dt ? 1 : 0;
    a.correct = c->correct_asymptotic_underconfidence ? 1 : 0;
    a.fixedpoint = fp ? 1 : 0;
    a.state_error = c->error == PDQ_ERROR_STATE_STD ? 1 : 0;
    a.instances_per_block = c->instances_per_block;
    a.safety = c->safety;
    a.factor_min = c->factor_min;
    a.factor_max = c->factor_max;
    a.exp_i = c->exponent_integral;
    a.exp_p = c->exponent_proportional;
    a.atol = c->atol;
    a.rtol = c->rtol;
    a.eps = c->eps;
    a.damp = c->damp;
    a.max_attempts = c->max_attempts;
    iwp_q1(c->num_derivatives, a.q1);
    a.save_at = args->save_at;
    a.params = args->params;
    a.y0 = args->y0;
    a.dt0 = args->dt0;
    a.u_mean = args->u_mean;
    a.u_chol = args->u_chol;
    a.output_scale = args->output_scale;
    a.t_out = args->t;
    a.num_steps = args->num_steps;
    a.num_attempts = args->num_attempts;
    a.status = args->status;
    a.cond_A = args->cond_A;
    a.cond_noise_mean = args->cond_noise_mean;
    a.cond_noise_chol = args->cond_noise_chol;
    a.cond_to_latent = args->cond_to_latent;
    a.cond_to_observed = args->cond_to_observed;
    a.filter_mean = args->filter_mean;
    a.filter_chol = args->filter_chol;
    a.workspace = workspace;
    const bool ts1 = c->constraint == PDQ_CONSTRAINT_TS1;
    const bool f64 = c->precision == PDQ_PRECISION_F64;
    const int block = variant == 2 ? 0 : variant;  // the launchers' mapping code
    cudaError_t err;
    if (user_field) {  // run-time fields: one thread per instance
      err = pdq_launch_dense_user(a, c->field, f64, c->num_derivatives, ts1, fp, stream);
      return err == cudaSuccess ? PDQ_SUCCESS : (err == cudaErrorInvalidSource ? PDQ_ERROR_COMPILE : PDQ_ERROR_CUDA);
    }
    if (variant >= 4) {  // eight / sixteen lanes per instance (own translation units)
      using DenseLanes = cudaError_t (*)(const pdq::DenseArgs&, int, bool, bool, int, cudaStream_t);
      DenseLanes launch = nullptr;
      switch (c->field) {
        case PDQ_FIELD_LOTKA_VOLTERRA:
          launch = f64 ? pdq_launch_dense_lanes_lv_f64 : pdq_launch_dense_lanes_lv_f32;
          break;
        case PDQ_FIELD_VAN_DER_POL:
          launch = f64 ? pdq_launch_dense_lanes_vdp_f64 : pdq_launch_dense_lanes_vdp_f32;
          break;
        case PDQ_FIELD_FITZHUGH_NAGUMO:
          launch = f64 ? pdq_launch_dense_lanes_fhn_f64 : pdq_launch_dense_lanes_fhn_f32;
          break;
        default: return PDQ_ERROR_UNSUPPORTED;
      }
      const int lanes = variant == 4 ? 8 : 16;
      return launch(a, c->num_derivatives, ts1, fp, lanes, stream) == cudaSuccess ? PDQ_SUCCESS : PDQ_ERROR_CUDA;
    }
    switch (c->field) {
      case PDQ_FIELD_LOTKA_VOLTERRA:
        err = f64 ? pdq_launch_dense_lv_f64(a, c->num_derivatives, ts1, fp, stream, block)
                  : pdq_launch_dense_lv_f32(a, c->num_derivatives, ts1, fp, stream, block);
        break;
      case PDQ_FIELD_VAN_DER_POL:
        err = f64 ? pdq_launch_dense_vdp_f64(a, c->num_derivatives, ts1, fp, stream, block)
                  : pdq_launch_dense_vdp_f32(a, c->num_derivatives, ts1, fp, stream, block);
        break;
      case PDQ_FIELD_FITZHUGH_NAGUMO:
        err = f64 ? pdq_launch_dense_fhn_f64(a, c->num_derivatives, ts1, fp, stream, block)
                  : pdq_launch_dense_fhn_f32(a, c->num_derivatives, ts1, fp, stream, block);
        break;
      default:
        return PDQ_ERROR_UNSUPPORTED;
    }
    return err == cudaSuccess ? PDQ_SUCCESS : PDQ_ERROR_CUDA;
  }
  return PDQ_ERROR_UNSUPPORTED;
}

static pdq_status lml_check(const pdq_config* c, int64_t B, int32_t num_steps, int32_t save_every) {
  pdq_status st = validate_common(c);
  if (st != PDQ_SUCCESS) return st;
  if (c->ssm != PDQ_SSM_ISOTROPIC || c->constraint != PDQ_CONSTRAINT_TS0 || c->strategy != PDQ_STRATEGY_FIXEDPOINT ||
      c->solver != PDQ_SOLVER_PLAIN)
    return PDQ_ERROR_UNSUPPORTED;
  if (c->num_derivatives < 2 || c->num_derivatives > 3) return PDQ_ERROR_UNSUPPORTED;
  const bool user = c->field >= PDQ_FIELD_USER_BASE;
  if (user) {  // a registered run-time field of the configuration's dimension
    if (pdq_user_field_dim(c->field) != c->ode_dim || pdq_user_field_params(c->field) < 1) return PDQ_ERROR_INVALID_VALUE;
  } else if (c->field != PDQ_FIELD_FITZHUGH_NAGUMO && c->field != PDQ_FIELD_LOTKA_VOLTERRA) {
    return PDQ_ERROR_UNSUPPORTED;
  }
  if (c->instances_per_block != 0) return PDQ_ERROR_INVALID_VALUE;
  if (c->field == PDQ_FIELD_LOTKA_VOLTERRA && c->precision != PDQ_PRECISION_F64) return PDQ_ERROR_UNSUPPORTED;
  if (B < 0 || num_steps < 1 || save_every < 1 || num_steps % save_every != 0) return PDQ_ERROR_INVALID_VALUE;
  return PDQ_SUCCESS;
}

static int lml_num_params(const pdq_config* c) {
  if (c->field >= PDQ_FIELD_USER_BASE) return pdq_user_field_params(c->field);
  return c->field == PDQ_FIELD_FITZHUGH_NAGUMO ? 3 : 4;
}

// Workspace: the shared covariance plan (key + tables, rounded to 256 bytes),
// then per thread (P threads per sample, one tangent each) the backward
// conditionals' offsets xi (values and tangents) at the observations.
static size_t lml_plan_bytes(const pdq_config* c, int32_t num_steps, int32_t save_every) {
  const int elem = c->precision == PDQ_PRECISION_F64 ? 8 : 4;
  return size_t(pdq::lml_plan_total_bytes(c->num_derivatives, num_steps, save_every, elem));
}

static size_t lml_bytes(const pdq_config* c, int64_t B, int32_t num_steps, int32_t save_every) {
  const int n = c->num_derivatives + 1, d = c->ode_dim;
  const int P = lml_num_params(c);
  const size_t per = size_t(n) * d * 2;
  const size_t elem = c->precision == PDQ_PRECISION_F64 ? 8 : 4;
  return lml_plan_bytes(c, num_steps, save_every) + size_t(B) * size_t(P) * size_t(num_steps / save_every) * per * elem;
}

pdq_status pdq_lml_workspace_size(const pdq_config* c, int64_t B, int32_t num_steps, int32_t save_every, size_t* bytes) {
  if (bytes == nullptr) return PDQ_ERROR_INVALID_VALUE;
  pdq_status st = lml_check(c, B, num_steps, save_every);
  if (st != PDQ_SUCCESS) return st;
  *bytes = lml_bytes(c, B, num_steps, save_every);
  return PDQ_SUCCESS;
}

pdq_status pdq_lml_fixed_grid(const pdq_config* c, const pdq_lml_args* args, void* workspace, size_t workspace_bytes,
                              void* stream_ptr) {
  pdq::NvtxRange nvtx_range("pdq_lml_fixed_grid");
  if (args == nullptr) return PDQ_ERROR_INVALID_VALUE;
  pdq_status st = lml_check(c, args->num_instances, args->num_steps, args->save_every);
  if (st != PDQ_SUCCESS) return st;
  if (args->num_instances == 0) return PDQ_SUCCESS;
  if (!args->params || !args->y0 || !args->data || !args->std || !args->lml || !args->status ||
      (args->with_gradient && !args->grad) || !(args->dt > 0))
    return PDQ_ERROR_INVALID_VALUE;
  if (workspace == nullptr || workspace_bytes < lml_bytes(c, args->num_instances, args->num_steps, args->save_every))
    return PDQ_ERROR_WORKSPACE;
  pdq::LmlArgs a;
  memset(&a, 0, sizeof(a));
  a.B = args->num_instances;
  a.num_steps = args->num_steps;
  a.save_every = args->save_every;
  a.average_pdfs = args->average_pdfs ? 1 : 0;
  a.with_gradient = args->with_gradient ? 1 : 0;
  a.lanes_per_sample = args->with_gradient ? lml_num_params(c) : 1;
  a.t0 = args->t0;
  a.dt = args->dt;
  a.damp = c->damp;
  iwp_q1(c->num_derivatives, a.q1);
  a.params = args->params;
  a.y0 = args->y0;
  a.data = args->data;
  a.std = args->std;
  a.lml = args->lml;
  a.grad = args->with_gradient ? args->grad : nullptr;
  a.status = args->status;
  a.plan = workspace;
  a.workspace = static_cast<unsigned char*>(workspace) + lml_plan_bytes(c, args->num_steps, args->save_every);
  cudaStream_t stream = static_cast<cudaStream_t>(stream_ptr);
  cudaError_t err;
  if (c->field >= PDQ_FIELD_USER_BASE) {
    err = pdq_launch_lml_user(a, c->field, c->precision == PDQ_PRECISION_F64, c->num_derivatives, stream);
    return err == cudaSuccess ? PDQ_SUCCESS : (err == cudaErrorInvalidSource ? PDQ_ERROR_COMPILE : PDQ_ERROR_CUDA);
  }
  if (c->field == PDQ_FIELD_FITZHUGH_NAGUMO)
    err = c->precision == PDQ_PRECISION_F64 ? pdq_launch_lml_fhn_f64(a, c->num_derivatives, stream)
                                            : pdq_launch_lml_fhn_f32(a, c->num_derivatives, stream);
  else
    err = pdq_launch_lml_lv_f64(a, c->num_derivatives, stream);
  return err == cudaSuccess ? PDQ_SUCCESS : PDQ_ERROR_CUDA;
}


// ---- adjoint (reverse-mode) LML: pdq_lml_fwd / pdq_lml_bwd ----

// Steps between stored states: the caller's, or round(sqrt(num_steps)).
static int32_t lml_adj_ckpt(int32_t num_steps, int32_t checkpoint_every) {
  if (checkpoint_every != 0) return checkpoint_every;
  const int32_t c = int32_t(lround(sqrt(double(num_steps))));
  return c < 1 ? 1 : c;
}

static pdq_status lml_adj_check(const pdq_config* c, int64_t B, int32_t num_steps, int32_t save_every,
                                int32_t checkpoint_every) {
  pdq_status st = lml_check(c, B, num_steps, save_every);
  if (st != PDQ_SUCCESS) return st;
  if (checkpoint_every < 0 || checkpoint_every > num_steps) return PDQ_ERROR_INVALID_VALUE;
  return PDQ_SUCCESS;
}

// Workspace: the shared covariance plan (the layout pdq_lml_fixed_grid uses),
// then the residuals of every sample (lml_adjoint.cuh).
static size_t lml_adj_bytes(const pdq_config* c, int64_t B, int32_t num_steps, int32_t save_every, int32_t ckpt) {
  const size_t elem = c->precision == PDQ_PRECISION_F64 ? 8 : 4;
  const pdq::LmlAdjLayout L(c->num_derivatives, c->ode_dim, num_steps, save_every, ckpt);
  return lml_plan_bytes(c, num_steps, save_every) + size_t(B) * size_t(L.total) * elem;
}

pdq_status pdq_lml_adjoint_workspace_size(const pdq_config* c, int64_t B, int32_t num_steps, int32_t save_every,
                                          int32_t checkpoint_every, size_t* bytes) {
  if (bytes == nullptr) return PDQ_ERROR_INVALID_VALUE;
  pdq_status st = lml_adj_check(c, B, num_steps, save_every, checkpoint_every);
  if (st != PDQ_SUCCESS) return st;
  *bytes = lml_adj_bytes(c, B, num_steps, save_every, lml_adj_ckpt(num_steps, checkpoint_every));
  return PDQ_SUCCESS;
}

static pdq_status lml_adj_launch(const pdq_config* c, const pdq_lml_adjoint_args* args, void* workspace,
                                 size_t workspace_bytes, void* stream_ptr, bool backward) {
  if (args == nullptr) return PDQ_ERROR_INVALID_VALUE;
  const pdq_lml_args& l = args->lml;
  pdq_status st = lml_adj_check(c, l.num_instances, l.num_steps, l.save_every, args->checkpoint_every);
  if (st != PDQ_SUCCESS) return st;
  if (args->reserved0 != 0) return PDQ_ERROR_INVALID_VALUE;
  if (l.num_instances == 0) return PDQ_SUCCESS;
  if (!l.params || !l.y0 || !l.data || !l.std || !l.status || !(l.dt > 0)) return PDQ_ERROR_INVALID_VALUE;
  if (!backward && !l.lml) return PDQ_ERROR_INVALID_VALUE;
  if (backward && !l.grad && !args->grad_y0) return PDQ_ERROR_INVALID_VALUE;
  const int32_t ckpt = lml_adj_ckpt(l.num_steps, args->checkpoint_every);
  if (workspace == nullptr || reinterpret_cast<uintptr_t>(workspace) % 16 != 0 ||
      workspace_bytes < lml_adj_bytes(c, l.num_instances, l.num_steps, l.save_every, ckpt))
    return PDQ_ERROR_WORKSPACE;
  pdq::LmlAdjArgs aa;
  memset(&aa, 0, sizeof(aa));
  pdq::LmlArgs& a = aa.base;
  a.B = l.num_instances;
  a.num_steps = l.num_steps;
  a.save_every = l.save_every;
  a.average_pdfs = l.average_pdfs ? 1 : 0;
  a.with_gradient = 0;
  a.lanes_per_sample = 1;
  a.t0 = l.t0;
  a.dt = l.dt;
  a.damp = c->damp;
  iwp_q1(c->num_derivatives, a.q1);
  a.params = l.params;
  a.y0 = l.y0;
  a.data = l.data;
  a.std = l.std;
  a.lml = l.lml;
  a.grad = l.grad;
  a.status = l.status;
  a.plan = workspace;
  a.workspace = nullptr;
  aa.ckpt = ckpt;
  aa.num_ckpt = int32_t((int64_t(l.num_steps) + ckpt - 1) / ckpt);
  aa.cotangent = args->cotangent;
  aa.grad_y0 = args->grad_y0;
  aa.res = static_cast<unsigned char*>(workspace) + lml_plan_bytes(c, l.num_steps, l.save_every);
  cudaStream_t stream = static_cast<cudaStream_t>(stream_ptr);
  cudaError_t err;
  if (c->field >= PDQ_FIELD_USER_BASE) {
    err = pdq_launch_lml_adj_user(aa, c->field, c->precision == PDQ_PRECISION_F64, c->num_derivatives, backward, stream);
    return err == cudaSuccess ? PDQ_SUCCESS : (err == cudaErrorInvalidSource ? PDQ_ERROR_COMPILE : PDQ_ERROR_CUDA);
  }
  if (c->field == PDQ_FIELD_FITZHUGH_NAGUMO)
    err = c->precision == PDQ_PRECISION_F64 ? pdq_launch_lml_adj_fhn_f64(aa, c->num_derivatives, backward, stream)
                                            : pdq_launch_lml_adj_fhn_f32(aa, c->num_derivatives, backward, stream);
  else
    err = pdq_launch_lml_adj_lv_f64(aa, c->num_derivatives, backward, stream);
  return err == cudaSuccess ? PDQ_SUCCESS : PDQ_ERROR_CUDA;
}

pdq_status pdq_lml_fwd(const pdq_config* c, const pdq_lml_adjoint_args* args, void* workspace, size_t workspace_bytes,
                       void* stream) {
  pdq::NvtxRange nvtx_range("pdq_lml_fwd");
  return lml_adj_launch(c, args, workspace, workspace_bytes, stream, false);
}

pdq_status pdq_lml_bwd(const pdq_config* c, const pdq_lml_adjoint_args* args, void* workspace, size_t workspace_bytes,
                       void* stream) {
  pdq::NvtxRange nvtx_range("pdq_lml_bwd");
  return lml_adj_launch(c, args, workspace, workspace_bytes, stream, true);
}

}  // extern "C"

extern "C" pdq_status pdq_terminal_record_size(const pdq_config* c, int64_t B, int32_t capacity,
                                               int32_t checkpoint_every, size_t* bytes) {
  if (bytes == nullptr) return PDQ_ERROR_INVALID_VALUE;
  const pdq_status st = terminal_check(c);
  if (st != PDQ_SUCCESS) return st;
  if (B < 0 || capacity < 1 || checkpoint_every < 1 || checkpoint_every > capacity) return PDQ_ERROR_INVALID_VALUE;
  size_t rec = 0;
  terminal_sizes(c, B, capacity, checkpoint_every, &rec, bytes);
  return PDQ_SUCCESS;
}

extern "C" pdq_status pdq_terminal_fwd(const pdq_config* c, const pdq_adaptive_args* args, int32_t capacity,
                                       int32_t checkpoint_every, void* record, size_t record_bytes, void* stream_ptr) {
  pdq::NvtxRange nvtx_range("pdq_terminal_fwd");
  const pdq_status st = terminal_check(c);
  if (st != PDQ_SUCCESS) return st;
  if (args == nullptr || args->num_instances < 0 || args->num_save_at != 2 || !args->terminal_only)
    return PDQ_ERROR_INVALID_VALUE;
  if (capacity < 1 || checkpoint_every < 1 || checkpoint_every > capacity) return PDQ_ERROR_INVALID_VALUE;
  if (args->u_mean_d_params || args->u_mean_d_y0 || args->cond_A || args->filter_mean) return PDQ_ERROR_UNSUPPORTED;
  if (args->num_instances == 0) return PDQ_SUCCESS;
  if (!args->save_at || !args->params || !args->y0 || !args->dt0 || !args->u_mean || !args->u_chol ||
      !args->output_scale || !args->t || !args->num_steps || !args->num_attempts || !args->status)
    return PDQ_ERROR_INVALID_VALUE;
  size_t rec = 0, need = 0;
  terminal_sizes(c, args->num_instances, capacity, checkpoint_every, &rec, &need);
  if (record == nullptr || record_bytes < need || (reinterpret_cast<uintptr_t>(record) & 15) != 0)
    return PDQ_ERROR_WORKSPACE;
  pdq::IsoArgs a;
  iso_args_fill(c, args, a);
  a.record = record;
  a.rec_capacity = capacity;
  a.rec_ckpt = checkpoint_every;
  const TvLaunch launch = tv_launcher(c);
  if (launch == nullptr) return PDQ_ERROR_UNSUPPORTED;
  const cudaError_t err = launch(a, nullptr, c->num_derivatives, static_cast<cudaStream_t>(stream_ptr));
  return err == cudaSuccess ? PDQ_SUCCESS : PDQ_ERROR_CUDA;
}

extern "C" pdq_status pdq_terminal_bwd(const pdq_config* c, const pdq_terminal_adjoint_args* t, void* record,
                                       size_t record_bytes, void* stream_ptr) {
  pdq::NvtxRange nvtx_range("pdq_terminal_bwd");
  const pdq_status st = terminal_check(c);
  if (st != PDQ_SUCCESS) return st;
  if (t == nullptr || t->num_instances < 0) return PDQ_ERROR_INVALID_VALUE;
  if (t->capacity < 1 || t->checkpoint_every < 1 || t->checkpoint_every > t->capacity) return PDQ_ERROR_INVALID_VALUE;
  if (t->num_instances == 0) return PDQ_SUCCESS;
  if (!t->params || !t->y0 || !t->num_steps || !t->status || !t->cotangent) return PDQ_ERROR_INVALID_VALUE;
  size_t rec = 0, need = 0;
  terminal_sizes(c, t->num_instances, t->capacity, t->checkpoint_every, &rec, &need);
  if (record == nullptr || record_bytes < need || (reinterpret_cast<uintptr_t>(record) & 15) != 0)
    return PDQ_ERROR_WORKSPACE;
  pdq_adaptive_args args;
  memset(&args, 0, sizeof(args));
  args.num_instances = t->num_instances;
  args.num_save_at = 2;
  args.terminal_only = 1;
  args.params = t->params;
  args.y0 = t->y0;
  pdq::IsoArgs a;
  iso_args_fill(c, &args, a);
  pdq::TvAdjArgs ta;
  ta.capacity = t->capacity;
  ta.ckpt = t->checkpoint_every;
  ta.num_steps = t->num_steps;
  ta.status = t->status;
  ta.cotangent = t->cotangent;
  ta.grad_params = t->grad_params;
  ta.grad_y0 = t->grad_y0;
  ta.record = record;
  ta.scratch = static_cast<unsigned char*>(record) + rec;
  const TvLaunch launch = tv_launcher(c);
  if (launch == nullptr) return PDQ_ERROR_UNSUPPORTED;
  const cudaError_t err = launch(a, &ta, c->num_derivatives, static_cast<cudaStream_t>(stream_ptr));
  return err == cudaSuccess ? PDQ_SUCCESS : PDQ_ERROR_CUDA;
}

extern "C" pdq_status pdq_offgrid_marginals(const pdq_offgrid_args* args, void* stream) {
  pdq::NvtxRange nvtx_range("pdq_offgrid_marginals");
  if (args == nullptr) return PDQ_ERROR_INVALID_VALUE;
  const pdq_offgrid_args& a = *args;
  if (a.num_instances < 0 || a.num_points < 1 || a.num_queries < 0 || a.ode_dim < 1) return PDQ_ERROR_INVALID_VALUE;
  if (a.strategy == PDQ_STRATEGY_FIXEDPOINT) return PDQ_ERROR_UNSUPPORTED;
  if (a.strategy != PDQ_STRATEGY_FILTER && a.strategy != PDQ_STRATEGY_FIXEDINTERVAL) return PDQ_ERROR_INVALID_VALUE;
  if (a.ssm == PDQ_SSM_ISOTROPIC) {
    if (a.num_derivatives < 1 || a.num_derivatives > 5 || a.ode_dim > 64) return PDQ_ERROR_UNSUPPORTED;
  } else if (a.ssm == PDQ_SSM_DENSE) {
    if (a.num_derivatives < 2 || a.num_derivatives > 3 || a.ode_dim != 2) return PDQ_ERROR_UNSUPPORTED;
  } else {
    return PDQ_ERROR_UNSUPPORTED;
  }
  if (a.num_instances * int64_t(a.num_queries) == 0) return PDQ_SUCCESS;
  if (!a.t || !a.u_mean || !a.u_chol || !a.output_scale || !a.t_query || !a.mean_out || !a.chol_out ||
      (a.strategy == PDQ_STRATEGY_FIXEDINTERVAL && (!a.filter_mean || !a.filter_chol)))
    return PDQ_ERROR_INVALID_VALUE;
  double q1[pdq::kMaxN][pdq::kMaxN];
  iwp_q1(a.num_derivatives, q1);
  const cudaError_t e = pdq_launch_offgrid(a, q1, static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? PDQ_SUCCESS : PDQ_ERROR_CUDA;
}
