"""Batched solves of many independent IVP instances on one GPU.

``solve_ensemble`` is the tensor-level entry point: one row of ``params`` and
``y0`` per instance (the reference's ``jax.vmap`` over a solve).  Host
tensors are copied to the device, the native solver runs on the current CUDA
stream, and device tensors are returned.
"""

import torch

from . import _native

DEFAULT_MAX_ATTEMPTS = 1 << 20


# Instance-to-thread mappings by name (include/pdq.h kernel_variant): the
# isotropic kernels (one thread, eight lanes with two register budgets, a
# covariance warp and a mean warp per 32 instances) and the dense ones (one
# thread, eight cooperative lanes, the structure-exploiting kernel on four,
# eight or sixteen lanes).
_VARIANTS = {
    "isotropic": {"auto": 0, "thread": 1, "lanes": 2, "lanes_compact": 3, "split": 4},
    "dense": {"auto": 0, "thread": 1, "lanes": 2, "struct": 3, "struct8": 4, "struct16": 5},
}


def _kernel_variant(ssm, kernel_variant):
    if isinstance(kernel_variant, str):
        names = _VARIANTS.get(ssm, {"auto": 0})
        if kernel_variant not in names:
            raise ValueError(f"kernel_variant {kernel_variant!r} for ssm {ssm!r}: one of {sorted(names)}")
        return names[kernel_variant]
    return int(kernel_variant)


def make_config(
    *,
    field,
    num_derivatives,
    ode_dim,
    ssm="isotropic",
    constraint="ts0",
    strategy="filter",
    solver="dynamic",
    control="integral",
    precision="float32",
    atol=1e-6,
    rtol=1e-6,
    clip_dt=True,
    eps=1e-8,
    damp=0.0,
    correct_asymptotic_underconfidence=True,
    safety=0.95,
    factor_min=0.2,
    factor_max=10.0,
    exponent_integral=0.3,
    exponent_proportional=0.4,
    max_attempts=DEFAULT_MAX_ATTEMPTS,
    kernel_variant=0,
    error="residual_std",
    instances_per_block=0,
):
    """Build a ``pdq_config`` (include/pdq.h) from keyword arguments."""
    cfg = _native.config_default(ssm, field, num_derivatives, ode_dim)
    cfg.constraint = _native.CONSTRAINT[constraint]
    cfg.strategy = _native.STRATEGY[strategy]
    cfg.solver = _native.SOLVER[solver]
    cfg.control = _native.CONTROL[control]
    cfg.error = _native.ERROR[error]
    cfg.precision = _native.PRECISION[precision]
    cfg.atol, cfg.rtol, cfg.eps, cfg.damp = float(atol), float(rtol), float(eps), float(damp)
    cfg.clip_dt = 1 if clip_dt else 0
    cfg.correct_asymptotic_underconfidence = 1 if correct_asymptotic_underconfidence else 0
    cfg.safety, cfg.factor_min, cfg.factor_max = float(safety), float(factor_min), float(factor_max)
    cfg.exponent_integral, cfg.exponent_proportional = float(exponent_integral), float(exponent_proportional)
    cfg.max_attempts = int(max_attempts)
    cfg.kernel_variant = _kernel_variant(ssm, kernel_variant)
    cfg.instances_per_block = int(instances_per_block)
    return cfg


def _dev(x, device, B=None, cols=None):
    t = torch.as_tensor(x, dtype=torch.float64)
    if B is not None and t.ndim == 1 and cols is not None and t.shape[0] == cols:
        t = t.expand(B, cols)
    return t.to(device, non_blocking=True).contiguous()


def solve_ensemble(cfg, *, params, y0, save_at, dt0=0.1, terminal_only=True, device="cuda", stream=None, outputs=None,
                   autotune=False, sensitivities=False):
    """Solve B instances; returns the dict of output device tensors.

    params (B, P), y0 (B, d), save_at (S,) shared or (B, S) per instance,
    dt0 scalar or (B,).  Output layout as in include/pdq.h.  ``autotune``:
    pick the instance-to-thread mapping and instances per CTA by timing the
    candidates on this batch (once per configuration and batch-size class;
    ``probdiffeq_gb300.autotune``).  ``sensitivities`` (isotropic TS0 filter):
    also d u_mean / d params and d u_mean / d y0 by forward mode
    (``u_mean_d_params`` (B, S_out, n, d, P), ``u_mean_d_y0`` (B, S_out, n, d, d)).
    """
    y0 = _dev(y0, device)
    B = y0.shape[0]
    params = _dev(params, device)
    if params.ndim == 1:
        params = params.expand(B, params.shape[0]).contiguous()
    save_at = torch.as_tensor(save_at, dtype=torch.float64)
    if save_at.ndim == 1:
        save_at = save_at.expand(B, save_at.shape[0])
    save_at = save_at.to(device, non_blocking=True).contiguous()
    dt0 = torch.as_tensor(dt0, dtype=torch.float64)
    if dt0.ndim == 0:
        dt0 = dt0.expand(B)
    dt0 = dt0.to(device, non_blocking=True).contiguous()
    S = save_at.shape[1]
    if outputs is None:
        outputs = _native.alloc_outputs(cfg, B, S, terminal_only, device,
                                        num_params=params.shape[1] if sensitivities else None)
    if autotune:
        from . import autotune as tuner

        cfg = tuner.tuned_config(cfg, save_at, params, y0, dt0, terminal_only, stream=stream)
    _native.solve_adaptive(cfg, save_at, params, y0, dt0, terminal_only, outputs, stream=stream)
    return outputs
