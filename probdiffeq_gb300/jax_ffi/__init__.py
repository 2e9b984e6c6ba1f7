"""JAX bindings of the C ABI through XLA FFI custom calls.

Needs jax with a CUDA jaxlib (and jaxlib's FFI headers to build the handler
library); nothing here runs without them, and importing this module does not
import jax.  ``register()`` builds ``libpdq_jax_ffi.so``
(``probdiffeq_gb300.build.build_jax_ffi``, the handlers of
``jax_ffi/ffi_pdq.cc``) and registers them as CUDA FFI targets.  Then:

* ``solve_adaptive(cfg, save_at, params, y0, dt0, terminal_only)`` -- the
  solve as one custom call (``pdq_solve_adaptive``);
* ``terminal_values(cfg, params, y0, t0, t1, dt0, capacity, checkpoint_every)``
  -- a ``jax.custom_vjp`` whose forward half is ``pdq_terminal_fwd`` (the
  record is the residual) and whose backward half is ``pdq_terminal_bwd``,
  the counterpart of ``jax.grad`` through ``solve_adaptive_terminal_values``
  (probdiffeq/_ivpsolve/solvers_via_adaptive_steps.py:16-43, 294-301);
* ``lml(cfg, params, y0, data, std, t0, dt, num_steps, save_every)`` -- the
  same for ``pdq_lml_fwd`` / ``pdq_lml_bwd`` (loss_lml_timeseries through
  solve_fixed_grid, estimators_and_losses.py:53-105, 180-218).

``cfg`` is a ``pdq_config`` from ``probdiffeq_gb300.ensemble.make_config``;
the handlers rebuild it from the fields passed as call attributes.
"""

import ctypes

import numpy as np

__all__ = ["register", "solve_adaptive", "terminal_values", "lml"]

_TARGETS = ("PdqSolveAdaptive", "PdqLmlFwd", "PdqLmlBwd", "PdqTerminalFwd", "PdqTerminalBwd")
_registered = False


def register():
    """Build the handler library and register its targets with JAX (once)."""
    global _registered
    if _registered:
        return
    import jax

    from .. import build

    path = build.build_jax_ffi()
    if path is None:
        raise RuntimeError("jaxlib's FFI headers (xla/ffi/api/ffi.h) were not found: the handlers cannot be built")
    lib = ctypes.CDLL(path)
    for name in _TARGETS:
        jax.ffi.register_ffi_target(name, jax.ffi.pycapsule(getattr(lib, name)), platform="CUDA")
    _registered = True


def _config_attrs(cfg):
    i32 = np.int32
    return dict(ssm=i32(cfg.ssm), field=i32(cfg.field), num_derivatives=i32(cfg.num_derivatives),
                ode_dim=i32(cfg.ode_dim), constraint=i32(cfg.constraint), strategy=i32(cfg.strategy),
                solver=i32(cfg.solver), precision=i32(cfg.precision), error=i32(cfg.error), control=i32(cfg.control),
                clip_dt=i32(cfg.clip_dt), atol=np.float64(cfg.atol), rtol=np.float64(cfg.rtol))


def _solve_shapes(cfg, B, S, terminal_only, record_bytes=None, workspace_bytes=0):
    import jax
    import jax.numpy as jnp

    n, d = cfg.num_derivatives + 1, cfg.ode_dim
    So = 1 if terminal_only else S
    if cfg.ssm == 0:  # isotropic: (n, d) means, (n, n) factors
        mean, chol = (B, So, n, d), (B, So, n, n)
    elif cfg.ssm == 1:  # block-diagonal: (d, n) and (d, n, n)
        mean, chol = (B, So, d, n), (B, So, d, n, n)
    else:
        mean, chol = (B, So, n * d), (B, So, n * d, n * d)
    f64, i32 = jnp.float64, jnp.int32
    shapes = [jax.ShapeDtypeStruct(mean, f64), jax.ShapeDtypeStruct(chol, f64), jax.ShapeDtypeStruct((B, So), f64),
              jax.ShapeDtypeStruct((B, So), f64), jax.ShapeDtypeStruct((B, So), i32), jax.ShapeDtypeStruct((B,), i32),
              jax.ShapeDtypeStruct((B,), i32)]
    nbytes = workspace_bytes if record_bytes is None else record_bytes
    shapes.append(jax.ShapeDtypeStruct((max(1, nbytes),), jnp.uint8))
    return shapes


def solve_adaptive(cfg, save_at, params, y0, dt0, terminal_only=True):
    """(u_mean, u_chol, output_scale, t, num_steps, num_attempts, status) of ``pdq_solve_adaptive``."""
    import jax

    from .. import _native

    register()
    B, S = y0.shape[0], save_at.shape[1]
    ws = _native.workspace_size(cfg, B, S)
    call = jax.ffi.ffi_call("PdqSolveAdaptive", _solve_shapes(cfg, B, S, terminal_only, workspace_bytes=ws))
    out = call(save_at, params, y0, dt0, **_config_attrs(cfg), terminal_only=np.int32(bool(terminal_only)))
    return tuple(out[:7])


def terminal_values(cfg, params, y0, t0, t1, dt0=0.1, capacity=2048, checkpoint_every=None):
    """Terminal means (B, n, d) with the adjoint as their VJP; instances whose
    accepted steps exceed ``capacity`` get status PDQ_INSTANCE_RECORD_FULL."""
    import jax
    import jax.numpy as jnp

    from .. import _native

    register()
    B = y0.shape[0]
    C = int(checkpoint_every) if checkpoint_every else max(1, round(capacity ** 0.5))
    nbytes = _native.terminal_record_size(cfg, B, capacity, C)
    attrs = dict(_config_attrs(cfg), capacity=np.int32(capacity), checkpoint_every=np.int32(C))
    save_at = jnp.broadcast_to(jnp.asarray([t0, t1], dtype=jnp.float64), (B, 2))
    dt = jnp.full((B,), dt0, dtype=jnp.float64)

    def fwd_call(p, y):
        out = jax.ffi.ffi_call("PdqTerminalFwd", _solve_shapes(cfg, B, 2, True, record_bytes=nbytes))(
            save_at, p, y, dt, **attrs)
        return out[0][:, 0], out[4][:, 0], out[6], out[7]  # mean, num_steps, status, record

    @jax.custom_vjp
    def f(p, y):
        return fwd_call(p, y)[0]

    def f_fwd(p, y):
        mean, steps, status, record = fwd_call(p, y)
        return mean, (p, y, steps, status, record)

    def f_bwd(res, g):
        p, y, steps, status, record = res
        shapes = (jax.ShapeDtypeStruct(p.shape, jnp.float64), jax.ShapeDtypeStruct(y.shape, jnp.float64))
        gp, gy = jax.ffi.ffi_call("PdqTerminalBwd", shapes)(p, y, steps, status, record, g, **attrs)
        return gp, gy

    f.defvjp(f_fwd, f_bwd)
    return f(params, y0)


def lml(cfg, params, y0, data, std, t0, dt, num_steps, save_every, average_pdfs=False, checkpoint_every=0):
    """LML (B,) of the data with the hand-written adjoint as its VJP."""
    import jax
    import jax.numpy as jnp

    from .. import _native

    register()
    B = y0.shape[0]
    nbytes = _native.lml_adjoint_workspace_bytes(cfg, B, num_steps, save_every, checkpoint_every)
    attrs = dict(_config_attrs(cfg), t0=np.float64(t0), dt=np.float64(dt), num_steps=np.int32(num_steps),
                 save_every=np.int32(save_every), average_pdfs=np.int32(bool(average_pdfs)),
                 checkpoint_every=np.int32(checkpoint_every))
    fwd_shapes = (jax.ShapeDtypeStruct((B,), jnp.float64), jax.ShapeDtypeStruct((B,), jnp.int32),
                  jax.ShapeDtypeStruct((nbytes,), jnp.uint8))

    @jax.custom_vjp
    def f(p, y):
        return jax.ffi.ffi_call("PdqLmlFwd", fwd_shapes)(p, y, data, std, **attrs)[0]

    def f_fwd(p, y):
        value, status, ws = jax.ffi.ffi_call("PdqLmlFwd", fwd_shapes)(p, y, data, std, **attrs)
        return value, (p, y, status, ws)

    def f_bwd(res, g):
        p, y, status, ws = res
        shapes = (jax.ShapeDtypeStruct(p.shape, jnp.float64), jax.ShapeDtypeStruct(y.shape, jnp.float64))
        gp, gy = jax.ffi.ffi_call("PdqLmlBwd", shapes)(p, y, data, std, status, ws, g, **attrs)
        return gp, gy

    f.defvjp(f_fwd, f_bwd)
    return f(params, y0)
