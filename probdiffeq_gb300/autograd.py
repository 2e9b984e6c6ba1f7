"""The LML kernel as a ``torch.autograd.Function``.

``lml(params, y0, data, std, ...)`` returns the log-marginal likelihood of
each parameter sample (one native launch, the same C ABI as
``pdq_lml_fixed_grid``); its backward multiplies the incoming cotangent into
the parameter gradient that the forward launch already computed (forward-mode
tangents inside the kernel, one direction per thread), so ``loss.backward()``
through it costs no second launch.  This is the torch counterpart of the
reference's ``jax.grad`` of ``loss_lml_timeseries``
(probdiffeq/_probdiffeq/estimators_and_losses.py:53-105).
"""

import torch

from . import _native, ensemble

__all__ = ["lml"]


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


def lml(params, y0, data, std, *, field="fitzhugh_nagumo", num_derivatives=3, dt, num_steps, save_every,
        t0=0.0, average_pdfs=False, precision="float64", damp=0.0, stream=None):
    """Differentiable LML of observations under the fixed-point-smoother posterior.

    params (B, P) float64 CUDA tensor (``requires_grad`` for gradients), y0 (B, d),
    data (num_steps // save_every + 1, d), std (same length).  Returns
    (lml (B,), status (B,) int32); ``lml.sum().backward()`` fills ``params.grad``.
    Gradients with respect to y0, data and std are not provided.
    """
    if num_steps % save_every != 0 or data.shape[0] != num_steps // save_every + 1:
        raise ValueError("The standard deviation container differs from what was expected.")
    cfg = ensemble.make_config(field=field, num_derivatives=num_derivatives, ode_dim=y0.shape[-1], ssm="isotropic",
                               constraint="ts0", strategy="fixedpoint", solver="none", precision=precision, damp=damp)
    return _LmlFixedGrid.apply(params, y0, data, std, cfg, float(t0), float(dt), int(num_steps), int(save_every),
                               bool(average_pdfs), stream)
