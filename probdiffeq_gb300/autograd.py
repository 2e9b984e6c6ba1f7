"""The LML kernel as a ``torch.autograd.Function``.

``lml(params, y0, data, std, ...)`` returns the log-marginal likelihood of
each parameter sample.  Two gradient modes, the torch counterpart of the
reference's ``jax.grad`` of ``loss_lml_timeseries``
(probdiffeq/_probdiffeq/estimators_and_losses.py:53-105):

* ``mode="forward"`` (``pdq_lml_fixed_grid``): the forward launch computes the
  parameter gradient with forward-mode tangents (one direction per thread);
  the backward multiplies the incoming cotangent into it, no second launch.
* ``mode="adjoint"`` (``pdq_lml_fwd`` / ``pdq_lml_bwd``): the forward launch
  computes the value and stores sqrt(N)-checkpointed residuals; the backward
  launch runs the adjoint pass for the incoming cotangent and gives the
  gradient with respect to ``params`` and ``y0``, at a cost independent of
  the number of parameters.
"""

import torch

from . import _native, ensemble

__all__ = ["lml", "terminal_values"]


class _LmlFixedGrid(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params, y0, data, std, cfg, t0, dt, num_steps, save_every, average_pdfs, stream):
        out = _native.lml_fixed_grid(
            cfg, params.detach().contiguous(), y0.detach().contiguous(), data.contiguous(), std.contiguous(),
            t0=t0, dt=dt, num_steps=num_steps, save_every=save_every, average_pdfs=average_pdfs,
            gradient=ctx.needs_input_grad[0], stream=stream,
        )
        ctx.save_for_backward(out["grad"] if out.get("grad") is not None else torch.empty(0))
        ctx.mark_non_differentiable(out["status"])
        return out["lml"], out["status"]

    @staticmethod
    def backward(ctx, g_lml, g_status):
        (grad,) = ctx.saved_tensors
        g_params = g_lml[:, None] * grad if ctx.needs_input_grad[0] else None
        return g_params, None, None, None, None, None, None, None, None, None, None


class _LmlAdjoint(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params, y0, data, std, cfg, t0, dt, num_steps, save_every, average_pdfs, checkpoint_every,
                stream):
        fwd = _native.lml_fwd(
            cfg, params.detach().contiguous(), y0.detach().contiguous(), data.contiguous(), std.contiguous(),
            t0=t0, dt=dt, num_steps=num_steps, save_every=save_every, average_pdfs=average_pdfs,
            checkpoint_every=checkpoint_every, stream=stream,
        )
        ctx.mark_non_differentiable(fwd["status"])
        if ctx.needs_input_grad[0] or ctx.needs_input_grad[1]:
            ctx.fwd = fwd
        else:
            _native.lml_release(fwd)  # no backward will come: the workspace serves the next call
        return fwd["lml"], fwd["status"]

    @staticmethod
    def backward(ctx, g_lml, g_status):
        want_p, want_y0 = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
        # one backward per forward: the workspace (with its plan) goes back to
        # the pool for the next forward call on this stream
        out = _native.lml_bwd(ctx.fwd, g_lml, params_grad=want_p, y0_grad=want_y0, release=True)
        return (out["grad"], out["grad_y0"], None, None, None, None, None, None, None, None, None, None)


def lml(params, y0, data, std, *, field="fitzhugh_nagumo", num_derivatives=3, dt, num_steps, save_every,
        t0=0.0, average_pdfs=False, precision="float64", damp=0.0, mode="forward", checkpoint_every=0, stream=None):
    """Differentiable LML of observations under the fixed-point-smoother posterior.

    params (B, P) float64 CUDA tensor (``requires_grad`` for gradients), y0 (B, d),
    data (num_steps // save_every + 1, d), std (same length).  Returns
    (lml (B,), status (B,) int32); ``lml.sum().backward()`` fills ``params.grad``
    (and, with ``mode="adjoint"``, ``y0.grad``).  ``checkpoint_every`` (adjoint
    mode): steps between stored states, 0 for round(sqrt(num_steps)).
    Gradients with respect to data and std are not provided.
    """
    if num_steps % save_every != 0 or data.shape[0] != num_steps // save_every + 1:
        raise ValueError("The standard deviation container differs from what was expected.")
    cfg = ensemble.make_config(field=field, num_derivatives=num_derivatives, ode_dim=y0.shape[-1], ssm="isotropic",
                               constraint="ts0", strategy="fixedpoint", solver="none", precision=precision, damp=damp)
    if mode == "adjoint":
        return _LmlAdjoint.apply(params, y0, data, std, cfg, float(t0), float(dt), int(num_steps), int(save_every),
                                 bool(average_pdfs), int(checkpoint_every), stream)
    if mode != "forward":
        raise ValueError(f"unknown gradient mode {mode!r} (expected 'forward' or 'adjoint')")
    return _LmlFixedGrid.apply(params, y0, data, std, cfg, float(t0), float(dt), int(num_steps), int(save_every),
                               bool(average_pdfs), stream)


class _TerminalValues(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params, y0, cfg, t0, t1, dt0, stream):
        grad = ctx.needs_input_grad[0] or ctx.needs_input_grad[1]
        out = ensemble.solve_ensemble(cfg, params=params.detach().contiguous(), y0=y0.detach().contiguous(),
                                      save_at=torch.tensor([float(t0), float(t1)], dtype=torch.float64), dt0=dt0,
                                      terminal_only=True, device=y0.device, stream=stream, sensitivities=grad)
        if grad:
            ctx.save_for_backward(out["u_mean_d_params"][:, 0], out["u_mean_d_y0"][:, 0])
        ctx.mark_non_differentiable(out["status"])
        return out["u_mean"][:, 0], out["status"]

    @staticmethod
    def backward(ctx, g_mean, g_status):
        d_params, d_y0 = ctx.saved_tensors
        g_params = torch.einsum("bij,bijk->bk", g_mean, d_params) if ctx.needs_input_grad[0] else None
        g_y0 = torch.einsum("bij,bijk->bk", g_mean, d_y0) if ctx.needs_input_grad[1] else None
        return g_params, g_y0, None, None, None, None, None


class _TerminalValuesAdjoint(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params, y0, cfg, t0, t1, dt0, stream, capacity, checkpoint_every):
        p, y = params.detach().contiguous(), y0.detach().contiguous()
        B = y.shape[0]
        save_at = torch.tensor([float(t0), float(t1)], dtype=torch.float64, device=y.device).expand(B, 2).contiguous()
        dt = torch.as_tensor(dt0, dtype=torch.float64, device=y.device).expand(B).contiguous()
        out = _native.terminal_fwd(cfg, save_at, p, y, dt, capacity=capacity, checkpoint_every=checkpoint_every,
                                   stream=stream)
        ctx.cfg, ctx.fwd, ctx.inputs, ctx.stream = cfg, out, (p, y), stream
        ctx.mark_non_differentiable(out["status"])
        return out["u_mean"][:, 0], out["status"]

    @staticmethod
    def backward(ctx, g_mean, g_status):
        p, y = ctx.inputs
        gp, gy = _native.terminal_bwd(ctx.cfg, ctx.fwd, p, y, g_mean, params_grad=ctx.needs_input_grad[0],
                                      y0_grad=ctx.needs_input_grad[1], stream=ctx.stream)
        return gp, gy, None, None, None, None, None, None, None


def terminal_values(params, y0, *, t0, t1, field="lotka_volterra", num_derivatives=4, solver="mle", atol=1e-6,
                    rtol=1e-6, dt0=0.1, precision="float64", stream=None, mode="forward", capacity=None,
                    checkpoint_every=None):
    """Differentiable terminal values of an isotropic TS0 filter solve.

    params (B, P) and y0 (B, d) float64 CUDA tensors (``requires_grad`` for
    gradients).  Returns (u_mean (B, n, d) -- the Taylor coefficients at t1 --,
    status (B,) int32): the counterpart of ``jax.grad`` through
    ``solve_adaptive_terminal_values`` with its stop-gradient on the step size
    (probdiffeq/_ivpsolve/solvers_via_adaptive_steps.py:16-43, 294-301).

    mode "forward": the backward pass contracts the cotangent with the
    forward-mode sensitivities the same launch computed (P + d threads per
    instance).  mode "adjoint": the forward pass records the accepted steps
    (``pdq_terminal_fwd``; ``capacity`` accepted steps per instance, None for
    a guess and one rerun if it was too small; the state every
    ``checkpoint_every`` steps, None for sqrt(capacity)), the backward pass
    differentiates them in reverse (``pdq_terminal_bwd``) at a cost
    independent of P + d.  The adjoint takes solver "none" or "mle".
    """
    cfg = ensemble.make_config(field=field, num_derivatives=num_derivatives, ode_dim=y0.shape[-1], ssm="isotropic",
                               constraint="ts0", strategy="filter", solver=solver, precision=precision, atol=atol,
                               rtol=rtol, clip_dt=True)
    if mode == "adjoint":
        return _TerminalValuesAdjoint.apply(params, y0, cfg, float(t0), float(t1), dt0, stream, capacity,
                                            checkpoint_every)
    if mode != "forward":
        raise ValueError(f"unknown gradient mode {mode!r} (expected 'forward' or 'adjoint')")
    return _TerminalValues.apply(params, y0, cfg, float(t0), float(t1), dt0, stream)
