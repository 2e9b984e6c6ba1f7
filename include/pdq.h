/*
 * pdq.h -- C ABI of the GB300 probabilistic-IVP hot path.
 *
 * The reference (pnkraemer/probdiffeq) is pure JAX and has no FFI; its
 * "operator API" is the set of Python constructors and the ivpsolve entry
 * points.  Each function below replaces one of those entry points for a
 * batch of independent IVP instances (the reference's jax.vmap over a solve):
 *
 *   pdq_solve_adaptive  <- ivpsolve.solve_adaptive_save_at / solve_adaptive_terminal_values
 *                          (probdiffeq/_ivpsolve/solvers_via_adaptive_steps.py:16-148)
 *                          with the solver, strategy, constraint, error estimator
 *                          and controller chosen in pdq_config
 *                          (probdiffeq/_probdiffeq/solvers.py:318-767, 850-996;
 *                           probdiffeq/_ivpsolve/controllers.py:24-84)
 *
 * Conventions:
 *   - every pointer in the argument structs is a DEVICE pointer unless
 *     stated otherwise; the caller owns all buffers;
 *   - float64 in and out; the arithmetic precision is pdq_config.precision;
 *   - launches are asynchronous on the given stream; no allocation, no
 *     synchronisation inside the calls;
 *   - configuration errors return a non-zero pdq_status before any launch;
 *     run-time failures are reported per instance in the status array
 *     (never a trap);
 *   - the first call of an entry point on a device may raise the context's
 *     per-thread stack limit for its kernels (a one-time, synchronising
 *     cudaDeviceSetLimit); make it before capturing a stream into a graph,
 *     later calls only enqueue launches;
 *   - every entry point opens an NVTX range named after itself (visible to
 *     ncu --nvtx and Nsight Systems).
 */
#ifndef PDQ_H_
#define PDQ_H_

#if defined(__CUDACC_RTC__)
/* runtime compilation (NVRTC) of the solver templates with a user vector
 * field: no C library headers there */
typedef int int32_t;
typedef unsigned int uint32_t;
typedef long long int64_t;
typedef unsigned long long uint64_t;
typedef unsigned long size_t;
#else
#include <stddef.h>
#include <stdint.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define PDQ_ABI_VERSION 2u

typedef enum pdq_status {
  PDQ_SUCCESS = 0,
  PDQ_ERROR_INVALID_VALUE = 1,
  PDQ_ERROR_UNSUPPORTED = 2,
  PDQ_ERROR_CUDA = 3,
  PDQ_ERROR_WORKSPACE = 4,
  PDQ_ERROR_ABI_VERSION = 5,
  PDQ_ERROR_STATIC_SCRATCH = 6,
  PDQ_ERROR_COMPILE = 7
} pdq_status;

/* State-space factorisation (probdiffeq/_probdiffeq/ssm_impl_*.py). */
enum { PDQ_SSM_ISOTROPIC = 0, PDQ_SSM_BLOCKDIAG = 1, PDQ_SSM_DENSE = 2 };
/* Linearisation: constraint_ode_ts0 / constraint_ode_ts1 (ssm_impl_api.py:520-558). */
enum { PDQ_CONSTRAINT_TS0 = 0, PDQ_CONSTRAINT_TS1 = 1 };
/* strategy_filter / strategy_smoother_fixedpoint (estimators_and_losses.py:347-591). */
enum { PDQ_STRATEGY_FILTER = 0, PDQ_STRATEGY_FIXEDPOINT = 1,
       PDQ_STRATEGY_FIXEDINTERVAL = 2 /* pdq_offgrid_marginals only: a solve on a grid lowers the
                                          fixed-interval smoother to FIXEDPOINT with every grid point
                                          a checkpoint */ };
/* solver / solver_mle / solver_dynamic (solvers.py:318-767). */
enum { PDQ_SOLVER_PLAIN = 0, PDQ_SOLVER_MLE = 1, PDQ_SOLVER_DYNAMIC = 2 };
/* error_residual_std (solvers.py:850-996) / error_state_std (solvers.py:999-1098, derivative_idx 0). */
enum { PDQ_ERROR_RESIDUAL_STD = 0, PDQ_ERROR_STATE_STD = 1 };
/* control_integral / control_proportional_integral (controllers.py:24-84). */
enum { PDQ_CONTROL_INTEGRAL = 0, PDQ_CONTROL_PROPORTIONAL_INTEGRAL = 1 };
/* Bulk arithmetic precision.  Time, calibration and error-norm sums are float64 in
 * PDQ_PRECISION_F64 and float pairs (48-bit significand) in PDQ_PRECISION_F32. */
enum { PDQ_PRECISION_F32 = 0, PDQ_PRECISION_F64 = 1 };
/* Registered device vector fields (autonomous, first order). */
enum {
  PDQ_FIELD_LOTKA_VOLTERRA = 0, /* params (a, b, c, d), d = 2 */
  PDQ_FIELD_VAN_DER_POL = 1,    /* params (mu), d = 2 */
  PDQ_FIELD_FITZHUGH_NAGUMO = 2,/* params (a, b, c), d = 2 */
  PDQ_FIELD_BURGERS = 3,        /* params (nu), periodic grid, any d */
  PDQ_FIELD_USER_BASE = 1000    /* ids returned by pdq_register_field */
};

/* Per-instance run-time status. */
enum {
  PDQ_INSTANCE_OK = 0,
  PDQ_INSTANCE_MAX_STEPS = 1,   /* attempt bound reached before the last checkpoint */
  PDQ_INSTANCE_DT_UNDERFLOW = 2,/* step size collapsed below 1e-14 * max(1, |t|) */
  PDQ_INSTANCE_NONFINITE = 3,   /* NaN or Inf in the error norm or the state */
  PDQ_INSTANCE_RECORD_FULL = 4  /* pdq_terminal_fwd: more accepted steps than the record holds
                                   (the solve itself finished; rerun with a larger capacity) */
};

typedef struct pdq_config {
  uint32_t abi_version;   /* must equal PDQ_ABI_VERSION */
  int32_t ssm;            /* PDQ_SSM_* */
  int32_t constraint;     /* PDQ_CONSTRAINT_* */
  int32_t strategy;       /* PDQ_STRATEGY_* */
  int32_t solver;         /* PDQ_SOLVER_* */
  int32_t error;          /* PDQ_ERROR_* */
  int32_t control;        /* PDQ_CONTROL_* */
  int32_t precision;      /* PDQ_PRECISION_* */
  int32_t field;          /* PDQ_FIELD_* */
  int32_t num_derivatives;/* nu; the state holds nu + 1 Taylor coefficients */
  int32_t ode_dim;        /* d */
  int32_t clip_dt;        /* RejectionLoop clip_dt (solvers_via_adaptive_steps.py:300-301) */
  int32_t correct_asymptotic_underconfidence; /* solver_mle (solvers.py:456-457) */
  int32_t kernel_variant;  /* isotropic mapping: 0 auto, 1 one thread per instance,
                              2 / 3 eight lanes per instance with <= 128 / <= 85 registers (clip_dt only),
                              4 a covariance warp and a mean warp per 32 instances (the filter with
                              TS0, no damping, error_residual_std, clip_dt, solver none or mle);
                              dense: 0 auto (4, or 1 for error_state_std and run-time fields),
                              1 one thread per instance, 2 eight lanes per instance,
                              3 / 4 / 5 structure-exploiting QRs on four / eight / sixteen lanes
                              per instance */
  double safety, factor_min, factor_max;           /* controller (defaults 0.95, 0.2, 10) */
  double exponent_integral, exponent_proportional; /* PI controller (0.3, 0.4) */
  double atol, rtol, eps, damp;                    /* solve(...) arguments */
  int64_t max_attempts;   /* bound on step attempts per instance (the reference has none) */
  int32_t instances_per_block; /* instances per CTA; 0: default.  Isotropic: 32 or 64 (one thread
                                  each; default 64), 8, 16 or 32 (eight lanes each; default 32);
                                  dense: 8, 16 or 32 (one thread each; default 32), 1 to 4 (eight
                                  lanes each; default 4), 0 for variant 3 (eight instances per
                                  32-thread CTA); block-diagonal: 0 */
  int32_t reserved0;      /* 0 */
} pdq_config;

typedef struct pdq_adaptive_args {
  int64_t num_instances;  /* B */
  int32_t num_save_at;    /* S >= 2; save_at[b][0] = t0 */
  int32_t terminal_only;  /* 1: write only the last checkpoint (solve_adaptive_terminal_values) */
  const double* save_at;  /* (B, S) checkpoint times, strictly increasing per instance */
  const double* params;   /* (B, P) vector-field parameters */
  const double* y0;       /* (B, d) initial values; Taylor-mode derivatives are computed on device */
  const double* dt0;      /* (B,) initial step */
  /* outputs; S_out = terminal_only ? 1 : S */
  double* u_mean;         /* isotropic (B, S_out, n, d); dense (B, S_out, n*d) */
  double* u_chol;         /* isotropic (B, S_out, n, n); dense (B, S_out, n*d, n*d) */
  double* output_scale;   /* (B, S_out) */
  double* t;              /* (B, S_out) time of each output */
  int32_t* num_steps;     /* (B, S_out) accepted steps up to each output */
  int32_t* num_attempts;  /* (B,) total attempts (accepted + rejected) */
  int32_t* status;        /* (B,) PDQ_INSTANCE_* */
  /* optional outputs of the fixed-point smoother (NULL: not written; all or
   * none): the posterior's backward conditional between consecutive
   * checkpoints and the filtering marginals.  Dense, N = n*d: shapes below;
   * isotropic: cond_A (B, S-1, n, n), cond_noise_mean (B, S-1, n, d),
   * cond_noise_chol (B, S-1, n, n), cond_to_* (B, S-1, n), filter_mean
   * (B, S, n, d), filter_chol (B, S, n, n). */
  double* cond_A;           /* (B, S-1, N, N) */
  double* cond_noise_mean;  /* (B, S-1, N) */
  double* cond_noise_chol;  /* (B, S-1, N, N) */
  double* cond_to_latent;   /* (B, S-1, N) */
  double* cond_to_observed; /* (B, S-1, N) */
  double* filter_mean;      /* (B, S, N) filtering marginals at the checkpoints */
  double* filter_chol;      /* (B, S, N, N) */
  /* optional forward-mode sensitivities of the mean records (NULL: not
   * computed; isotropic TS0 filter with error_residual_std, built-in fields):
   * d u_mean / d params (B, S_out, n, d, P) and d u_mean / d y0
   * (B, S_out, n, d, d), through the Taylor-mode initialisation and every
   * accepted step, with the step sizes held constant (the reference stops
   * gradients through dt).  The covariance of a TS0 solve does not depend on
   * params or y0 (H = e_1), so u_chol has no sensitivity apart from the MLE
   * output scale, which is not differentiated here.  The launch runs P + d
   * threads per instance. */
  double* u_mean_d_params;
  double* u_mean_d_y0;
} pdq_adaptive_args;

typedef struct pdq_lml_args {
  int64_t num_instances;  /* B parameter samples */
  int32_t num_steps;      /* fixed grid of num_steps steps of size dt from t0 */
  int32_t save_every;     /* one observation every save_every steps (num_steps % save_every == 0) */
  int32_t average_pdfs;   /* loss_lml_timeseries(average_pdfs=...) */
  int32_t with_gradient;  /* 1: also write d lml / d params */
  double t0, dt;
  const double* params;   /* (B, P) vector-field parameters */
  const double* y0;       /* (B, d) initial values */
  const double* data;     /* (num_obs, d), num_obs = num_steps / save_every + 1, at t0 + k save_every dt */
  const double* std;      /* (num_obs,) observation noise standard deviations */
  double* lml;            /* (B,) log-marginal likelihood */
  double* grad;           /* (B, P) gradient, written if with_gradient */
  int32_t* status;        /* (B,) PDQ_INSTANCE_* */
} pdq_lml_args;

/* ABI version compiled into the library. */
#if !defined(__CUDACC_RTC__)
uint32_t pdq_abi_version(void);
#endif

/* Human-readable name of a status code (static storage). */
#if !defined(__CUDACC_RTC__)
const char* pdq_status_string(pdq_status status);
#endif

/* Fill a config with the reference's defaults for the given factorisation:
 * filter strategy, solver_dynamic, error_residual_std, control_integral,
 * TS0, float32 bulk, clip_dt 1, eps 1e-8, damp 0, atol = rtol = 1e-6. */
#if !defined(__CUDACC_RTC__)
pdq_status pdq_config_default(pdq_config* config, int32_t ssm, int32_t field, int32_t num_derivatives, int32_t ode_dim);
#endif

/* Device scratch the solve needs, in bytes (0 for configurations without scratch). */
#if !defined(__CUDACC_RTC__)
pdq_status pdq_workspace_size(const pdq_config* config, int64_t num_instances, int32_t num_save_at, size_t* bytes);
#endif

/* Adaptive solve of B independent instances; see the file header. */
#if !defined(__CUDACC_RTC__)
pdq_status pdq_solve_adaptive(const pdq_config* config, const pdq_adaptive_args* args, void* workspace,
                              size_t workspace_bytes, void* stream);
#endif

/* Device scratch of pdq_lml_fixed_grid in bytes.  Its leading part holds
 * the covariance plan shared by all parameter samples (with TS0, the
 * uncalibrated solver and a fixed step the covariances do not depend on the
 * parameters), keyed by (dt, damp, num_steps, save_every, nu, precision)
 * and a bit-exact copy of the per-observation noise std: a call whose key
 * equals the one stored in the workspace reuses the plan, so
 * a caller that writes into the workspace between calls must zero its first
 * 256 bytes. */
#if !defined(__CUDACC_RTC__)
pdq_status pdq_lml_workspace_size(const pdq_config* config, int64_t num_instances, int32_t num_steps, int32_t save_every,
                                  size_t* bytes);
#endif

/* Log-marginal likelihood of time-series data, and its gradient with respect
 * to the vector-field parameters, for B parameter samples:
 *   an isotropic TS0 solve with the uncalibrated solver and the fixed-point
 *   smoother on a fixed grid whose every save_every-th point is an
 *   observation (checkpoint reset, estimators_and_losses.py:534-547), then
 *   loss_lml_timeseries on the resulting backward Markov sequence
 *   (probdiffeq/_probdiffeq/estimators_and_losses.py:53-105, 180-218).
 * The gradient follows the reference's differentiation rules (qr_r's custom
 * JVP, probdiffeq/backend/linalg.py:13-37; no gradient through dt).
 * config: ssm isotropic, constraint TS0, strategy fixedpoint, solver plain. */
#if !defined(__CUDACC_RTC__)
pdq_status pdq_lml_fixed_grid(const pdq_config* config, const pdq_lml_args* args, void* workspace, size_t workspace_bytes,
                              void* stream);
#endif

/* The same LML with its gradient by reverse mode (an adjoint pass), split
 * into the forward and backward halves of a custom VJP: the counterpart of
 * jax.vjp / jax.grad of loss_lml_timeseries through solve_fixed_grid with
 * the fixed-point smoother (probdiffeq/_probdiffeq/estimators_and_losses.py:
 * 53-105, 180-218, 526-547; probdiffeq/_ivpsolve/solvers_via_fixed_steps.py:
 * 11-34), i.e. the fwd/bwd pair a jax.custom_vjp or torch.autograd.Function
 * binds.  pdq_lml_fwd writes lml and status and leaves in the workspace what
 * the backward pass needs: the state every checkpoint_every steps (sqrt(N)
 * checkpointing: 0 selects round(sqrt(num_steps))), the backward
 * conditionals' offsets and the LML recursion's innovations.  pdq_lml_bwd
 * then reads them (same args, same workspace, untouched in between),
 * recomputes each segment of checkpoint_every steps from its checkpoint and
 * differentiates it in reverse, writing
 *   lml.grad (B, P) = cotangent * d lml / d params   (if not NULL)
 *   grad_y0  (B, d) = cotangent * d lml / d y0       (if not NULL)
 * (cotangent NULL: ones).  Samples whose status is not PDQ_INSTANCE_OK get
 * NaN gradients.  The derivative is the forward-mode one of
 * pdq_lml_fixed_grid (the same rules), at a cost independent of P.
 * lml.with_gradient is ignored.  The workspace must be 16-byte aligned. */
typedef struct pdq_lml_adjoint_args {
  pdq_lml_args lml;          /* inputs, lml / status (written by fwd, status read by bwd), grad (bwd) */
  int32_t checkpoint_every;  /* steps between stored states, 0 <= C <= num_steps (0: round(sqrt(num_steps))) */
  int32_t reserved0;         /* 0 */
  const double* cotangent;   /* (B,) d loss / d lml for pdq_lml_bwd, or NULL for ones */
  double* grad_y0;           /* (B, d) output of pdq_lml_bwd, or NULL */
} pdq_lml_adjoint_args;

#if !defined(__CUDACC_RTC__)
pdq_status pdq_lml_adjoint_workspace_size(const pdq_config* config, int64_t num_instances, int32_t num_steps,
                                          int32_t save_every, int32_t checkpoint_every, size_t* bytes);
pdq_status pdq_lml_fwd(const pdq_config* config, const pdq_lml_adjoint_args* args, void* workspace,
                       size_t workspace_bytes, void* stream);
pdq_status pdq_lml_bwd(const pdq_config* config, const pdq_lml_adjoint_args* args, void* workspace,
                       size_t workspace_bytes, void* stream);
#endif

/* Reverse-mode (adjoint) gradient of adaptive terminal values, split into
 * the forward and backward halves of a custom VJP: the counterpart of
 * jax.vjp / jax.grad through solve_adaptive_terminal_values with its
 * stop-gradient on the step size (probdiffeq/_ivpsolve/
 * solvers_via_adaptive_steps.py:16-43, 294-301).
 * pdq_terminal_fwd solves exactly as pdq_solve_adaptive (same args, same
 * outputs) and records in `record`, per instance, the size of every accepted
 * step and the state before every checkpoint_every-th one, for at most
 * `capacity` accepted steps; an instance that takes more finishes its solve
 * and reports PDQ_INSTANCE_RECORD_FULL (rerun with capacity >= its
 * num_steps).  pdq_terminal_bwd then reads the record (same config, same
 * capacity and checkpoint_every, record untouched in between), recomputes
 * each segment of checkpoint_every steps from its state and differentiates
 * the mean recursion in reverse, writing
 *   grad_params (B, P) = sum over (i, j) of cotangent[b, i, j] d u_mean[b, i, j] / d params
 *   grad_y0     (B, d) = the same for d / d y0
 * for the terminal mean u_mean (B, 1, n, d) (its Taylor coefficients at t1).
 * Instances whose forward status is not PDQ_INSTANCE_OK get NaN gradients.
 * config: ssm isotropic, constraint TS0, strategy filter, error
 * residual_std, clip_dt, damp 0, solver plain or mle (whose prediction runs
 * at unit scale, so the gains do not depend on the parameters), built-in
 * field; args: terminal_only, two save points; kernel_variant 0 or 1.  The
 * record must be 16-byte aligned. */
typedef struct pdq_terminal_adjoint_args {
  int64_t num_instances;     /* B, as in the forward call */
  int32_t capacity;          /* accepted steps the record holds per instance, >= 1 */
  int32_t checkpoint_every;  /* accepted steps between stored states, 1 <= C <= capacity */
  const double* params;      /* (B, P), as in the forward call */
  const double* y0;          /* (B, d), as in the forward call */
  const int32_t* num_steps;  /* (B,) the forward call's num_steps (accepted steps to t1) */
  const int32_t* status;     /* (B,) the forward call's status */
  const double* cotangent;   /* (B, n, d) d loss / d u_mean at t1 */
  double* grad_params;       /* (B, P) output, or NULL */
  double* grad_y0;           /* (B, d) output, or NULL */
} pdq_terminal_adjoint_args;

#if !defined(__CUDACC_RTC__)
pdq_status pdq_terminal_record_size(const pdq_config* config, int64_t num_instances, int32_t capacity,
                                    int32_t checkpoint_every, size_t* bytes);
pdq_status pdq_terminal_fwd(const pdq_config* config, const pdq_adaptive_args* args, int32_t capacity,
                            int32_t checkpoint_every, void* record, size_t record_bytes, void* stream);
pdq_status pdq_terminal_bwd(const pdq_config* config, const pdq_terminal_adjoint_args* args, void* record,
                            size_t record_bytes, void* stream);
#endif

/* Size of the scratch array inside the library used by pdq_lml_fixed_grid_static. */
#define PDQ_LML_STATIC_SCRATCH_BYTES (32u * 1024u * 1024u)

/* pdq_lml_fixed_grid without any allocation, for callers that cannot call
 * cudaMalloc (plugin hosts that pass only input and output buffers, such as
 * custom-call interfaces without a scratch operand, and loops whose
 * allocation policy forbids it).  No counterpart in the
 * reference: it is an addition of this library.  The scratch is a 32 MiB
 * array inside the library (held on every GPU that loads it, until exit);
 * problems whose scratch (pdq_lml_workspace_size) exceeds
 * PDQ_LML_STATIC_SCRATCH_BYTES return PDQ_ERROR_STATIC_SCRATCH before any
 * launch.  The first call on a device looks up the array's device address, so
 * make it before any stream capture.  All calls share the array: calls whose
 * launches overlap on the GPU race.  Allocates nothing (no cudaMalloc or
 * cudaFree). */
#if !defined(__CUDACC_RTC__)
pdq_status pdq_lml_fixed_grid_static(const pdq_config* config, const pdq_lml_args* args, void* stream);
#endif

/* Posterior samples of a fixed-point smoother solution, MarkovSequence.sample
 * (probdiffeq/_probdiffeq/estimators_and_losses.py:233-273): draw the last
 * point from its marginal, then walk the backward conditionals to the first
 * point with cond.apply_flat (mean to_observed * (A (to_latent * x)) +
 * noise_mean, factor |to_observed| noise_chol).  The standard-normal draws
 * come in `normals`; as in the reference's isotropic sample_flat, one
 * n-vector per point is shared by the d dimensions.  Device pointers. */
typedef struct pdq_sample_args {
  int32_t ssm;              /* PDQ_SSM_ISOTROPIC or PDQ_SSM_DENSE */
  int32_t num_derivatives;  /* nu; n = nu + 1 */
  int32_t ode_dim;          /* d; dense N = n * d */
  int32_t num_points;       /* S: the marginal at point S-1 and S-1 conditionals */
  int64_t num_instances;    /* B */
  int32_t num_samples;      /* K per instance */
  const double* marginal_mean;     /* iso (B, n, d) | dense (B, N): the marginal at the last point */
  const double* marginal_chol;     /* iso (B, n, n) | dense (B, N, N) */
  const double* cond_A;            /* as in pdq_adaptive_args */
  const double* cond_noise_mean;
  const double* cond_noise_chol;
  const double* cond_to_latent;
  const double* cond_to_observed;
  const double* normals;           /* iso (B, K, S, n) | dense (B, K, S, N) */
  double* samples;                 /* iso (B, K, S, n, d) | dense (B, K, S, N) */
} pdq_sample_args;

#if !defined(__CUDACC_RTC__)
pdq_status pdq_sample_markov(const pdq_sample_args* args, void* stream);
#endif

/* Marginals at off-grid times of a solution on a grid: solver.offgrid_marginals
 * (probdiffeq/_probdiffeq/solvers.py:149-203).  For each query t the
 * interval comes from searchsorted(t_grid, t) = index; the transitions from
 * t_grid[index-1] to t and from t to t_grid[index] use output_scale[index].
 *   PDQ_STRATEGY_FILTER: the marginal at index-1 predicted to t
 *     (estimators_and_losses.py:403-414);
 *   PDQ_STRATEGY_FIXEDINTERVAL: the filtering marginal at index-1 reverted
 *     to t, that reverted to t_grid[index], and the smoothed marginal at
 *     index marginalised through the resulting backward conditional
 *     (estimators_and_losses.py:674-709).
 * PDQ_STRATEGY_FIXEDPOINT returns PDQ_ERROR_UNSUPPORTED (the reference raises
 * NotImplementedError).  A query on a grid point returns that point's
 * marginal; one outside [t_grid[0], t_grid[S-1]] (or NaN) returns NaN.
 * Float64; isotropic (nu 1..5, d <= 64) and dense (nu 2..3, d = 2).  Device
 * pointers; one thread per (instance, query).  A block-diagonal solution is
 * d independent one-dimensional models with per-dimension output scales:
 * pass it as PDQ_SSM_ISOTROPIC with ode_dim 1 and B * d instances (instance
 * b * d + j = dimension j of instance b, its mean (S, n, 1), factor
 * (S, n, n) and output scale (S) taken from that dimension). */
typedef struct pdq_offgrid_args {
  int32_t ssm;              /* PDQ_SSM_ISOTROPIC or PDQ_SSM_DENSE */
  int32_t strategy;         /* PDQ_STRATEGY_FILTER or PDQ_STRATEGY_FIXEDINTERVAL */
  int32_t num_derivatives;  /* nu; n = nu + 1 */
  int32_t ode_dim;          /* d; dense N = n * d */
  int64_t num_instances;    /* B */
  int32_t num_points;       /* S grid points per instance (t0 included) */
  int32_t num_queries;      /* Q query times per instance */
  const double* t;             /* (B, S) the grid, increasing */
  const double* u_mean;        /* iso (B, S, n, d) | dense (B, S, N): marginals at the grid points */
  const double* u_chol;        /* iso (B, S, n, n) | dense (B, S, N, N) */
  const double* filter_mean;   /* FIXEDINTERVAL: filtering marginals at the grid points, shapes as u_* */
  const double* filter_chol;
  const double* output_scale;  /* (B, S) */
  const double* t_query;       /* (B, Q) */
  double* mean_out;            /* iso (B, Q, n, d) | dense (B, Q, N) */
  double* chol_out;            /* iso (B, Q, n, n) | dense (B, Q, N, N) */
} pdq_offgrid_args;

#if !defined(__CUDACC_RTC__)
pdq_status pdq_offgrid_marginals(const pdq_offgrid_args* args, void* stream);
#endif

/* Register a vector field given as CUDA C++ source, compiled at run time
 * (NVRTC) into the isotropic solver.  Replaces passing a Python callable to
 * probdiffeq.ode (probdiffeq/_probdiffeq/problems.py:283-295); the registry
 * of device functors is the boundary's plugin seam for new models.
 * `source` defines, at namespace scope,
 *   struct Field {
 *     static constexpr int D = <state dimension>, P = <number of parameters>;
 *     template <typename S, typename T> PDQ_HD static void eval(const S* u, const T* p, S* out);
 *   };
 * generic over the scalar S (float, double, Taylor jets, dual numbers).  On
 * success *field_id (>= PDQ_FIELD_USER_BASE) goes into pdq_config.field
 * (isotropic and dense factorisations -- the dense TS1 Jacobian comes from the
 * same definition; dim and num_params must match D and P).
 * Compiler diagnostics are copied to `log` (host buffer, may be NULL);
 * errors return PDQ_ERROR_COMPILE.  The source is validated by compiling one
 * variant now; each variant used later is compiled and loaded on first use
 * (so the first solve of a variant takes seconds, then it is cached).
 * Host pointers; thread-safe. */
#if !defined(__CUDACC_RTC__)
pdq_status pdq_register_field(const char* name, const char* source, int32_t dim, int32_t num_params,
                              int32_t* field_id, char* log, size_t log_bytes);
#endif

/* Register a stencil field for the block-diagonal kernel (any d, periodic
 * grid), compiled at run time like pdq_register_field.  `source` defines
 *   struct Stencil {
 *     static constexpr int P = <number of parameters>;
 *     template <typename S, typename T>
 *     PDQ_HD static S eval(const S& left, const S& mid, const S& right, const T* p, T inv_dx);
 *   };
 * component j of f from u_{j-1}, u_j, u_{j+1} (indices mod d), the
 * parameters and inv_dx = d, generic over the scalar S (the bulk type, and
 * float64 Taylor jets for the Taylor-mode start); the built-in Burgers field
 * is such a stencil.  The id goes into pdq_config.field with ssm
 * PDQ_SSM_BLOCKDIAG (TS0; num_params must match P); other factorisations
 * reject it. */
#if !defined(__CUDACC_RTC__)
pdq_status pdq_register_stencil(const char* name, const char* source, int32_t num_params, int32_t* field_id,
                                char* log, size_t log_bytes);
#endif

#ifdef __cplusplus
}
#endif

#endif /* PDQ_H_ */
