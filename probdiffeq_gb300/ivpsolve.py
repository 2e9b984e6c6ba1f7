"""IVP solve loops, mirroring ``probdiffeq.ivpsolve``.

Same entry points as ``probdiffeq/_ivpsolve/solvers_via_adaptive_steps.py:16-148``,
``solvers_via_fixed_steps.py:11-34`` and ``controllers.py:24-84``.  Each
``solve(...)`` lowers the constructor objects to one ``pdq_config`` and runs
the whole batch (the reference's ``jax.vmap`` axis = the leading axis of the
initial values / parameters) in one native call on the current CUDA stream.
Errors the reference raises at trace time (shapes, unsuitable strategies)
are raised here before any launch; run-time failures are reported per
instance in ``Solution.status`` (0 ok, 1 max attempts, 2 dt underflow,
3 non-finite).
"""

import dataclasses
import warnings
from typing import Any

import torch

from . import _native, ensemble
from .probdiffeq import Prior, lower

__all__ = [
    "control_integral",
    "control_proportional_integral",
    "solve_adaptive_terminal_values",
    "solve_adaptive_save_at",
    "solve_fixed_grid",
    "lml_fixed_grid",
    "Solution",
    "Normal",
]


@dataclasses.dataclass(frozen=True)
class control_integral:
    """Integral controller (controllers.py:66-84)."""

    safety: float = 0.95
    factor_min: float = 0.2
    factor_max: float = 10.0


@dataclasses.dataclass(frozen=True)
class control_proportional_integral:
    """Proportional-integral controller (controllers.py:24-63)."""

    safety: float = 0.95
    factor_min: float = 0.2
    factor_max: float = 10.0
    exponent_integral: float = 0.3
    exponent_proportional: float = 0.4


@dataclasses.dataclass
class Normal:
    """Marginals with the reference's flat layouts (``mean_flat``, ``cholesky_flat``)."""

    mean_flat: torch.Tensor
    cholesky_flat: torch.Tensor
    ssm: str

    @property
    def mean(self):
        """Taylor coefficients as a list [u, u', ...] (the reference's pytree)."""
        if self.ssm == "isotropic":
            return [self.mean_flat[..., i, :] for i in range(self.mean_flat.shape[-2])]
        if self.ssm == "blockdiag":
            return [self.mean_flat[..., i] for i in range(self.mean_flat.shape[-1])]
        raise AttributeError("dense means are flat; use mean_flat")

    @property
    def std(self):
        """Row norms of the Cholesky factor (ssm_impl_*.py std)."""
        return torch.sqrt((self.cholesky_flat**2).sum(-1))


@dataclasses.dataclass
class Solution:
    """ProbabilisticSolution (solvers.py:33-69) with per-instance diagnostics."""

    t: torch.Tensor
    u: Normal
    output_scale: torch.Tensor
    num_steps: torch.Tensor
    num_attempts: torch.Tensor
    status: torch.Tensor
    posterior: Any = None
    ode_dim: Any = None


def _prior_inputs(prior):
    if not isinstance(prior, Prior):
        raise TypeError("u must be a prior from state_space_model_*().prior_wiener_integrated(...)")
    tc = prior.tcoeffs
    y0 = tc.y0 if tc.y0.ndim == 2 else tc.y0[None]
    params = tc.field.params
    params = params if params.ndim == 2 else params[None].expand(y0.shape[0], -1)
    if params.shape[0] != y0.shape[0]:
        raise ValueError("the batch axes of the initial values and the parameters differ")
    return y0, params


def _run(prior, solver, error, control, save_at, *, atol, rtol, dt0, eps, damp, clip_dt, terminal_only, precision,
         device, posterior=False, stream=None):
    if prior.ssm != solver.constraint.ssm:
        raise ValueError("the prior and the constraint come from different state-space models")
    if solver.constraint.field is not prior.tcoeffs.field and solver.constraint.field.name != prior.tcoeffs.field.name:
        raise ValueError("the constraint and the Taylor coefficients use different vector fields")
    y0, params = _prior_inputs(prior)
    cfg = lower(solver, error, control, num_derivatives=prior.num_derivatives, y0=y0, precision=precision, atol=atol,
                rtol=rtol, clip_dt=clip_dt, eps=eps, damp=damp)
    B = y0.shape[0]
    save_at = torch.as_tensor(save_at, dtype=torch.float64)
    S = save_at.shape[-1]
    outs = _native.alloc_outputs(cfg, B, S, terminal_only, device, posterior=posterior)
    out = ensemble.solve_ensemble(cfg, params=params, y0=y0, save_at=save_at, dt0=dt0, terminal_only=terminal_only,
                                  device=device, stream=stream, outputs=outs)
    post = {k: out[k] for k in _native.OPTIONAL_OUTPUTS if k in out} or None
    return Solution(
        t=out["t"],
        u=Normal(out["u_mean"], out["u_chol"], prior.ssm),
        output_scale=out["output_scale"],
        num_steps=out["num_steps"],
        num_attempts=out["num_attempts"],
        status=out["status"],
        posterior=post,
        ode_dim=y0.shape[-1],
    )


def solve_adaptive_terminal_values(solver, error, control=None, clip_dt=True, *, precision="float32", device="cuda"):
    """Terminal values of an IVP (solvers_via_adaptive_steps.py:16-43)."""

    def solve(u, /, *, t0, t1, atol, rtol, dt0=0.1, eps=1e-8, damp=0.0, stream=None):
        save_at = torch.tensor([float(t0), float(t1)], dtype=torch.float64)
        return _run(u, solver, error, control, save_at, atol=atol, rtol=rtol, dt0=dt0, eps=eps, damp=damp,
                    clip_dt=clip_dt, terminal_only=True, precision=precision, device=device, stream=stream)

    return solve


def solve_adaptive_save_at(*, solver, error, control=None, clip_dt=False, warn=True, precision="float32",
                           device="cuda", posterior=False):
    """Solution on a grid of checkpoints (solvers_via_adaptive_steps.py:46-148)."""
    if not solver.is_suitable_for_save_at and warn:
        warnings.warn(f"Solver {solver} should not be used in solve_adaptive_save_at.", stacklevel=2)

    def solve(u, save_at, atol, rtol, dt0=0.1, eps=1e-8, damp=0.0, stream=None):
        return _run(u, solver, error, control, save_at, atol=atol, rtol=rtol, dt0=dt0, eps=eps, damp=damp,
                    clip_dt=clip_dt, terminal_only=False, precision=precision, device=device,
                    posterior=posterior, stream=stream)

    return solve


def solve_fixed_grid(*, solver, precision="float32", device="cuda"):
    """Solution on a fixed grid (solvers_via_fixed_steps.py:11-34).

    Realised as the adaptive loop with the grid as checkpoints, clip_dt and an
    error norm that always accepts (atol = inf): every step is clipped to the
    next grid point, so the steps are exactly diff(grid) -- the equivalence
    the reference pins in tests/test_ivpsolve/test_solve_fixed_grid.py:17-54.
    """
    if not solver.is_suitable_for_save_every_step:
        warnings.warn(f"Solver {solver} should not be used in solve_fixed_grid (fixedpoint).", stacklevel=2)
    if solver.strategy.name == "fixedinterval":
        # every grid point is a checkpoint: the fixed-point conditionals are the per-step ones
        strategy = type(solver.strategy)()
        strategy._on_grid = True
        solver = dataclasses.replace(solver, strategy=strategy)

    def solve(u, /, *, grid, damp=0.0, posterior=None, stream=None):
        # the fixed-interval smoother keeps its posterior (off-grid marginals need the filtering marginals)
        posterior = solver.strategy.name == "fixedinterval" if posterior is None else posterior
        grid = torch.as_tensor(grid, dtype=torch.float64)
        span = float((grid[..., -1] - grid[..., 0]).abs().max())
        # eps far above the rounding of t, far below any grid spacing
        eps = 1e-12 * max(1.0, float(grid.abs().max()))
        return _run(u, solver, None, control_integral(factor_max=1e30), grid, atol=float("inf"), rtol=0.0,
                    dt0=10.0 * span + 1.0, eps=eps, damp=damp, clip_dt=True, terminal_only=False,
                    precision=precision, device=device, posterior=posterior, stream=stream)

    return solve


def lml_fixed_grid(prior, data, std, *, dt, num_steps, save_every, loss=None, gradient=True, precision="float64",
                   t0=0.0, device="cuda", stream=None, checkpoint_every=0):
    """LML of observations under the fixed-point-smoother posterior, and d LML / d params.

    The fixed grid t0 + k dt, k = 0..num_steps, observed at every save_every-th
    point (t0 included); loss_lml_timeseries semantics
    (estimators_and_losses.py:53-105) with the uncalibrated solver and TS0.
    ``gradient``: True (or "forward") for forward-mode tangents in the same
    launch, "adjoint" for the reverse-mode pair pdq_lml_fwd / pdq_lml_bwd
    (sqrt(N) step checkpointing, ``checkpoint_every`` steps between stored
    states, 0 for round(sqrt(num_steps))), False for the value only.
    Returns (lml (B,), grad (B, P) or None, status (B,)); with "adjoint" a
    fourth item, d LML / d y0 (B, d).
    """
    if gradient not in (True, False, "forward", "adjoint"):
        raise ValueError(f"gradient must be True, False, 'forward' or 'adjoint', not {gradient!r}")
    from .probdiffeq import loss_lml_timeseries

    loss = loss_lml_timeseries() if loss is None else loss
    y0, params = _prior_inputs(prior)
    cfg = ensemble.make_config(field=prior.tcoeffs.field.name, num_derivatives=prior.num_derivatives, ode_dim=y0.shape[-1],
                               ssm=prior.ssm, constraint="ts0", strategy="fixedpoint", solver="none", precision=precision)
    data = torch.as_tensor(data, dtype=torch.float64)
    std = torch.as_tensor(std, dtype=torch.float64)
    if std.ndim == 0:
        std = std.expand(data.shape[0])
    if num_steps % save_every != 0 or data.shape[0] != num_steps // save_every + 1:
        raise ValueError("The standard deviation container differs from what was expected.")
    dev = torch.device(device)
    params, y0 = params.to(dev).contiguous(), y0.to(dev).contiguous()
    data, std = data.to(dev).contiguous(), std.to(dev).contiguous()
    if gradient == "adjoint":
        fwd = _native.lml_fwd(cfg, params, y0, data, std, t0=t0, dt=dt, num_steps=num_steps, save_every=save_every,
                              average_pdfs=loss.average_pdfs, checkpoint_every=checkpoint_every, stream=stream)
        bwd = _native.lml_bwd(fwd, None, params_grad=True, y0_grad=True, release=True)
        return fwd["lml"], bwd["grad"], fwd["status"], bwd["grad_y0"]
    out = _native.lml_fixed_grid(
        cfg, params, y0, data, std, t0=t0, dt=dt, num_steps=num_steps, save_every=save_every,
        average_pdfs=loss.average_pdfs, gradient=bool(gradient), stream=stream,
    )
    return out["lml"], out.get("grad"), out["status"]
