// XLA FFI handlers over the C ABI (include/pdq.h): the custom calls a JAX
// process registers with jax.ffi.register_ffi_target to run the solver
// kernels from jitted code, and the forward / backward halves its
// jax.custom_vjp binds.  Built (by probdiffeq_gb300/build.py) only where
// jaxlib's headers (xla/ffi/api/ffi.h) are present, and linked against
// libpdq_gb300.so.  Each handler fills pdq_config from the call's attributes
// and the argument structs from the FFI buffers, then calls the entry point
// on the FFI stream; a non-zero pdq_status becomes an FFI error carrying
// pdq_status_string.
//
// Handlers (operands; results; attributes):
//   PdqSolveAdaptive   save_at (B, S), params (B, P), y0 (B, d), dt0 (B);
//                      u_mean, u_chol, output_scale, t, num_steps, num_attempts,
//                      status, workspace (u8, pdq_workspace_size bytes);
//                      config attributes, terminal_only
//   PdqLmlFwd          params (B, P), y0 (B, d), data (K, d), std (K);
//                      lml (B), status (B), workspace (u8, pdq_lml_adjoint_workspace_size);
//                      config attributes, t0, dt, num_steps, save_every, average_pdfs, checkpoint_every
//   PdqLmlBwd          params, y0, data, std, status, workspace, cotangent (B);
//                      grad_params (B, P), grad_y0 (B, d); the same attributes
//   PdqTerminalFwd     save_at (B, 2), params, y0, dt0;
//                      u_mean, u_chol, output_scale, t, num_steps, num_attempts, status,
//                      record (u8, pdq_terminal_record_size); config attributes, capacity, checkpoint_every
//   PdqTerminalBwd     params, y0, num_steps, status, record, cotangent (B, n, d);
//                      grad_params, grad_y0; config attributes, capacity, checkpoint_every
// Config attributes: ssm, field, num_derivatives, ode_dim, constraint,
// strategy, solver, precision, error, control, clip_dt (int32) and atol,
// rtol (double); everything else keeps pdq_config_default's value.
//
// The workspaces and the record are results of the forward calls, so XLA
// allocates them and keeps them alive as residuals of the custom VJP until
// the backward call reads them: the entry points themselves allocate nothing.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>

#include "pdq.h"
#include "xla/ffi/api/ffi.h"

namespace ffi = xla::ffi;

namespace {

struct ConfigAttrs {
  int32_t ssm, field, num_derivatives, ode_dim, constraint, strategy, solver, precision, error, control, clip_dt;
  double atol, rtol;
};

ffi::Error make_config(const ConfigAttrs& a, pdq_config* c) {
  pdq_status st = pdq_config_default(c, a.ssm, a.field, a.num_derivatives, a.ode_dim);
  if (st != PDQ_SUCCESS) return ffi::Error(ffi::ErrorCode::kInvalidArgument, pdq_status_string(st));
  c->constraint = a.constraint;
  c->strategy = a.strategy;
  c->solver = a.solver;
  c->precision = a.precision;
  c->error = a.error;
  c->control = a.control;
  c->clip_dt = a.clip_dt;
  c->atol = a.atol;
  c->rtol = a.rtol;
  return ffi::Error::Success();
}

ffi::Error status_error(pdq_status st) {
  if (st == PDQ_SUCCESS) return ffi::Error::Success();
  return ffi::Error(ffi::ErrorCode::kInternal, pdq_status_string(st));
}

#define PDQ_CONFIG_ATTRS                                                                                            \
  .Attr<int32_t>("ssm").Attr<int32_t>("field").Attr<int32_t>("num_derivatives").Attr<int32_t>("ode_dim")           \
      .Attr<int32_t>("constraint").Attr<int32_t>("strategy").Attr<int32_t>("solver").Attr<int32_t>("precision")    \
      .Attr<int32_t>("error").Attr<int32_t>("control").Attr<int32_t>("clip_dt").Attr<double>("atol")              \
      .Attr<double>("rtol")

#define PDQ_CONFIG_PARAMS                                                                                          \
  int32_t ssm, int32_t field, int32_t num_derivatives, int32_t ode_dim, int32_t constraint, int32_t strategy,      \
      int32_t solver, int32_t precision, int32_t error, int32_t control, int32_t clip_dt, double atol, double rtol

#define PDQ_CONFIG_VALUES \
  ConfigAttrs { ssm, field, num_derivatives, ode_dim, constraint, strategy, solver, precision, error, control, clip_dt, atol, rtol }

void fill_solve_args(pdq_adaptive_args* a, ffi::Buffer<ffi::F64> save_at, ffi::Buffer<ffi::F64> params,
                     ffi::Buffer<ffi::F64> y0, ffi::Buffer<ffi::F64> dt0, ffi::ResultBuffer<ffi::F64>& u_mean,
                     ffi::ResultBuffer<ffi::F64>& u_chol, ffi::ResultBuffer<ffi::F64>& output_scale,
                     ffi::ResultBuffer<ffi::F64>& t, ffi::ResultBuffer<ffi::S32>& num_steps,
                     ffi::ResultBuffer<ffi::S32>& num_attempts, ffi::ResultBuffer<ffi::S32>& status) {
  std::memset(a, 0, sizeof(*a));
  a->num_instances = int64_t(y0.dimensions()[0]);
  a->num_save_at = int32_t(save_at.dimensions()[1]);
  a->save_at = save_at.typed_data();
  a->params = params.typed_data();
  a->y0 = y0.typed_data();
  a->dt0 = dt0.typed_data();
  a->u_mean = u_mean->typed_data();
  a->u_chol = u_chol->typed_data();
  a->output_scale = output_scale->typed_data();
  a->t = t->typed_data();
  a->num_steps = num_steps->typed_data();
  a->num_attempts = num_attempts->typed_data();
  a->status = status->typed_data();
}

ffi::Error SolveAdaptiveImpl(cudaStream_t stream, ffi::Buffer<ffi::F64> save_at, ffi::Buffer<ffi::F64> params,
                             ffi::Buffer<ffi::F64> y0, ffi::Buffer<ffi::F64> dt0, ffi::ResultBuffer<ffi::F64> u_mean,
                             ffi::ResultBuffer<ffi::F64> u_chol, ffi::ResultBuffer<ffi::F64> output_scale,
                             ffi::ResultBuffer<ffi::F64> t, ffi::ResultBuffer<ffi::S32> num_steps,
                             ffi::ResultBuffer<ffi::S32> num_attempts, ffi::ResultBuffer<ffi::S32> status,
                             ffi::ResultBuffer<ffi::U8> workspace, PDQ_CONFIG_PARAMS, int32_t terminal_only) {
  pdq_config c;
  ffi::Error e = make_config(PDQ_CONFIG_VALUES, &c);
  if (e.failure()) return e;
  pdq_adaptive_args a;
  fill_solve_args(&a, save_at, params, y0, dt0, u_mean, u_chol, output_scale, t, num_steps, num_attempts, status);
  a.terminal_only = terminal_only;
  return status_error(pdq_solve_adaptive(&c, &a, workspace->untyped_data(), workspace->size_bytes(), stream));
}

void fill_lml_args(pdq_lml_adjoint_args* a, ffi::Buffer<ffi::F64> params, ffi::Buffer<ffi::F64> y0,
                   ffi::Buffer<ffi::F64> data, ffi::Buffer<ffi::F64> std_, double t0, double dt, int32_t num_steps,
                   int32_t save_every, int32_t average_pdfs, int32_t checkpoint_every) {
  std::memset(a, 0, sizeof(*a));
  a->lml.num_instances = int64_t(y0.dimensions()[0]);
  a->lml.num_steps = num_steps;
  a->lml.save_every = save_every;
  a->lml.average_pdfs = average_pdfs;
  a->lml.t0 = t0;
  a->lml.dt = dt;
  a->lml.params = params.typed_data();
  a->lml.y0 = y0.typed_data();
  a->lml.data = data.typed_data();
  a->lml.std = std_.typed_data();
  a->checkpoint_every = checkpoint_every;
}

ffi::Error LmlFwdImpl(cudaStream_t stream, ffi::Buffer<ffi::F64> params, ffi::Buffer<ffi::F64> y0,
                      ffi::Buffer<ffi::F64> data, ffi::Buffer<ffi::F64> std_, ffi::ResultBuffer<ffi::F64> lml,
                      ffi::ResultBuffer<ffi::S32> status, ffi::ResultBuffer<ffi::U8> workspace, PDQ_CONFIG_PARAMS,
                      double t0, double dt, int32_t num_steps, int32_t save_every, int32_t average_pdfs,
                      int32_t checkpoint_every) {
  pdq_config c;
  ffi::Error e = make_config(PDQ_CONFIG_VALUES, &c);
  if (e.failure()) return e;
  pdq_lml_adjoint_args a;
  fill_lml_args(&a, params, y0, data, std_, t0, dt, num_steps, save_every, average_pdfs, checkpoint_every);
  a.lml.lml = lml->typed_data();
  a.lml.status = status->typed_data();
  return status_error(pdq_lml_fwd(&c, &a, workspace->untyped_data(), workspace->size_bytes(), stream));
}

ffi::Error LmlBwdImpl(cudaStream_t stream, ffi::Buffer<ffi::F64> params, ffi::Buffer<ffi::F64> y0,
                      ffi::Buffer<ffi::F64> data, ffi::Buffer<ffi::F64> std_, ffi::Buffer<ffi::S32> status,
                      ffi::Buffer<ffi::U8> workspace, ffi::Buffer<ffi::F64> cotangent,
                      ffi::ResultBuffer<ffi::F64> grad_params, ffi::ResultBuffer<ffi::F64> grad_y0, PDQ_CONFIG_PARAMS,
                      double t0, double dt, int32_t num_steps, int32_t save_every, int32_t average_pdfs,
                      int32_t checkpoint_every) {
  pdq_config c;
  ffi::Error e = make_config(PDQ_CONFIG_VALUES, &c);
  if (e.failure()) return e;
  pdq_lml_adjoint_args a;
  fill_lml_args(&a, params, y0, data, std_, t0, dt, num_steps, save_every, average_pdfs, checkpoint_every);
  a.lml.status = const_cast<int32_t*>(status.typed_data());  // read by the backward half only
  a.lml.grad = grad_params->typed_data();
  a.cotangent = cotangent.typed_data();
  a.grad_y0 = grad_y0->typed_data();
  // the workspace is an operand here (the forward call's result), passed on unchanged
  return status_error(pdq_lml_bwd(&c, &a, const_cast<uint8_t*>(workspace.typed_data()), workspace.size_bytes(), stream));
}

ffi::Error TerminalFwdImpl(cudaStream_t stream, ffi::Buffer<ffi::F64> save_at, ffi::Buffer<ffi::F64> params,
                           ffi::Buffer<ffi::F64> y0, ffi::Buffer<ffi::F64> dt0, ffi::ResultBuffer<ffi::F64> u_mean,
                           ffi::ResultBuffer<ffi::F64> u_chol, ffi::ResultBuffer<ffi::F64> output_scale,
                           ffi::ResultBuffer<ffi::F64> t, ffi::ResultBuffer<ffi::S32> num_steps,
                           ffi::ResultBuffer<ffi::S32> num_attempts, ffi::ResultBuffer<ffi::S32> status,
                           ffi::ResultBuffer<ffi::U8> record, PDQ_CONFIG_PARAMS, int32_t capacity,
                           int32_t checkpoint_every) {
  pdq_config c;
  ffi::Error e = make_config(PDQ_CONFIG_VALUES, &c);
  if (e.failure()) return e;
  pdq_adaptive_args a;
  fill_solve_args(&a, save_at, params, y0, dt0, u_mean, u_chol, output_scale, t, num_steps, num_attempts, status);
  a.terminal_only = 1;
  return status_error(
      pdq_terminal_fwd(&c, &a, capacity, checkpoint_every, record->untyped_data(), record->size_bytes(), stream));
}

ffi::Error TerminalBwdImpl(cudaStream_t stream, ffi::Buffer<ffi::F64> params, ffi::Buffer<ffi::F64> y0,
                           ffi::Buffer<ffi::S32> num_steps, ffi::Buffer<ffi::S32> status, ffi::Buffer<ffi::U8> record,
                           ffi::Buffer<ffi::F64> cotangent, ffi::ResultBuffer<ffi::F64> grad_params,
                           ffi::ResultBuffer<ffi::F64> grad_y0, PDQ_CONFIG_PARAMS, int32_t capacity,
                           int32_t checkpoint_every) {
  pdq_config c;
  ffi::Error e = make_config(PDQ_CONFIG_VALUES, &c);
  if (e.failure()) return e;
  pdq_terminal_adjoint_args a;
  std::memset(&a, 0, sizeof(a));
  a.num_instances = int64_t(y0.dimensions()[0]);
  a.capacity = capacity;
  a.checkpoint_every = checkpoint_every;
  a.params = params.typed_data();
  a.y0 = y0.typed_data();
  a.num_steps = num_steps.typed_data();
  a.status = status.typed_data();
  a.cotangent = cotangent.typed_data();
  a.grad_params = grad_params->typed_data();
  a.grad_y0 = grad_y0->typed_data();
  return status_error(
      pdq_terminal_bwd(&c, &a, const_cast<uint8_t*>(record.typed_data()), record.size_bytes(), stream));
}

}  // namespace

XLA_FFI_DEFINE_HANDLER_SYMBOL(PdqSolveAdaptive, SolveAdaptiveImpl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::S32>>()
                                  .Ret<ffi::Buffer<ffi::S32>>()
                                  .Ret<ffi::Buffer<ffi::S32>>()
                                  .Ret<ffi::Buffer<ffi::U8>>() PDQ_CONFIG_ATTRS.Attr<int32_t>("terminal_only"));

XLA_FFI_DEFINE_HANDLER_SYMBOL(PdqLmlFwd, LmlFwdImpl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::S32>>()
                                  .Ret<ffi::Buffer<ffi::U8>>() PDQ_CONFIG_ATTRS.Attr<double>("t0")
                                  .Attr<double>("dt")
                                  .Attr<int32_t>("num_steps")
                                  .Attr<int32_t>("save_every")
                                  .Attr<int32_t>("average_pdfs")
                                  .Attr<int32_t>("checkpoint_every"));

XLA_FFI_DEFINE_HANDLER_SYMBOL(PdqLmlBwd, LmlBwdImpl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::S32>>()
                                  .Arg<ffi::Buffer<ffi::U8>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>() PDQ_CONFIG_ATTRS.Attr<double>("t0")
                                  .Attr<double>("dt")
                                  .Attr<int32_t>("num_steps")
                                  .Attr<int32_t>("save_every")
                                  .Attr<int32_t>("average_pdfs")
                                  .Attr<int32_t>("checkpoint_every"));

XLA_FFI_DEFINE_HANDLER_SYMBOL(PdqTerminalFwd, TerminalFwdImpl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::S32>>()
                                  .Ret<ffi::Buffer<ffi::S32>>()
                                  .Ret<ffi::Buffer<ffi::S32>>()
                                  .Ret<ffi::Buffer<ffi::U8>>() PDQ_CONFIG_ATTRS.Attr<int32_t>("capacity")
                                  .Attr<int32_t>("checkpoint_every"));

XLA_FFI_DEFINE_HANDLER_SYMBOL(PdqTerminalBwd, TerminalBwdImpl,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Arg<ffi::Buffer<ffi::S32>>()
                                  .Arg<ffi::Buffer<ffi::S32>>()
                                  .Arg<ffi::Buffer<ffi::U8>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>()
                                  .Ret<ffi::Buffer<ffi::F64>>() PDQ_CONFIG_ATTRS.Attr<int32_t>("capacity")
                                  .Attr<int32_t>("checkpoint_every"));
