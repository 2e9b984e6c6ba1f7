"""Parity of the block-diagonal cluster CUDA solver (viscous Burgers) (GPU).

Configuration of the high-dimensional batch: periodic viscous Burgers with
central differences, initial condition a sum of 8 random Fourier modes with
amplitudes ~ N(0, 1/k^2), IWP with 3 derivatives, TS0 blockdiag filter,
per-dimension dynamic calibration, error_residual_std, integral control,
terminal values (clip_dt).

Parity against the oracle runs at d = 64 (the oracle loops over dimensions
in Python), on short horizons and on the configuration's t in [0, 1]; the full size d = 4096 (a 4-CTA cluster per instance) is checked
against scipy's DOP853 on the same semi-discretisation (the reference's own
accuracy tests compare against a classical solver) and float32 against
float64.  At d = 4096 the viscous term is stiff (largest eigenvalue
4 nu / dx^2 = 6.7e5), so explicit-type TS0 steps are ~1e-6 long; the
full-size checks use the horizon [0, 2e-3] (hundreds of steps).

Tolerances: float64 -- solution 1e-8, rows 1e-5, covariances 1e-5,
per-dimension output scales 1e-6, steps +-1; float32 -- solution 1e-3; the
per-dimension std of u within max(2, 4 r) of float64, r >= 1 the largest
ratio the oracle itself shows when run in float32 (float32 cannot carry
these covariances: the reference algorithm in single precision deviates the
same way); steps within max(2 %, 2x the float32 oracle's difference, 1).
"""

import math

import numpy as np
import pytest
import scipy.integrate
import torch

from oracle import problems, solvers, ssm

pytestmark = pytest.mark.gpu

NU_VISC = 0.01


def burgers_ic(d, seed):
    g = np.random.default_rng(seed)
    x = np.arange(d) / d
    k = np.arange(1, 9)
    amp = g.normal(0.0, 1.0 / k)
    phase = g.uniform(0.0, 2 * np.pi, size=8)
    return (amp[:, None] * np.sin(2 * np.pi * k[:, None] * x[None, :] + phase[:, None])).sum(axis=0)


def oracle_bd(u0, t1, solver="dynamic", atol=1e-4, rtol=1e-4, dtype=torch.float64, constraint="ts0"):
    p = torch.tensor([NU_VISC], dtype=torch.float64)
    tc = problems.taylor_derivatives(problems.burgers, torch.tensor(u0), p, 3).to(dtype)
    S = ssm.BdSSM()
    prior = S.prior_wiener_integrated(tc)
    pt = p.to(dtype)
    vf = lambda u, t: problems.burgers(u[0], pt)  # noqa: E731
    c = S.constraint_ode_ts1(vf) if constraint == "ts1" else S.constraint_ode_ts0(vf)
    cls = {"dynamic": solvers.SolverDynamic, "mle": solvers.SolverMLE, "none": solvers.SolverPlain}[solver]
    return solvers.solve_adaptive_terminal_values(
        cls(solvers.StrategyFilter(), c), solvers.ErrorResidualStd(c), prior, 0.0, t1, atol, rtol, dt0=0.1 * t1
    )


def gpu_bd(u0s, t1, precision, solver="dynamic", atol=1e-4, rtol=1e-4, constraint="ts0"):
    from probdiffeq_gb300 import ensemble

    u0s = torch.as_tensor(np.asarray(u0s), dtype=torch.float64)
    B, d = u0s.shape
    cfg = ensemble.make_config(field="burgers", num_derivatives=3, ode_dim=d, ssm="blockdiag", solver=solver,
                               precision=precision, atol=atol, rtol=rtol, clip_dt=True, constraint=constraint)
    out = ensemble.solve_ensemble(cfg, params=torch.full((B, 1), NU_VISC, dtype=torch.float64), y0=u0s,
                                  save_at=torch.tensor([0.0, t1], dtype=torch.float64), dt0=0.1 * t1)
    torch.cuda.synchronize()
    return {k: v.cpu() for k, v in out.items() if not k.startswith("_") and v is not None}


def rel(a, b):
    return float((a - b).abs().max() / b.abs().max().clamp_min(1e-300))


def compare(out, b, res, tol):
    o = res.u[-1]  # BdNormal: mean (d, n), chol (d, n, n)
    gm, gc = out["u_mean"][b, 0], out["u_chol"][b, 0]
    err_u = rel(gm[:, 0], o.mean[:, 0])
    err_rows = max(rel(gm[:, i], o.mean[:, i]) for i in range(o.mean.shape[1]))
    cg = gc @ gc.transpose(-1, -2)
    co = o.cholesky @ o.cholesky.transpose(-1, -2)
    err_cov = max(rel(cg[j], co[j]) for j in range(co.shape[0]))
    msg = f"u {err_u:.2e} rows {err_rows:.2e} cov {err_cov:.2e}"
    assert err_u <= tol["u"], msg
    if tol.get("f32"):
        # float32 cannot carry these covariances; std of u per dimension within 2x
        assert torch.isfinite(gc).all(), msg
        sg, so = cg[:, 0, 0].sqrt(), co[:, 0, 0].sqrt()
        f = tol["std_factor"]
        assert bool(((sg >= so / f) & (sg <= f * so)).all()), (msg, f, float((sg / so).min()), float((sg / so).max()))
    else:
        assert err_rows <= tol["rows"], msg
        assert err_cov <= tol["cov"], msg
    allowed = max(1, math.ceil(tol["steps"] * res.num_steps[-1]), tol.get("steps_abs", 0))
    assert abs(int(out["num_steps"][b, 0]) - res.num_steps[-1]) <= allowed


@pytest.mark.parametrize("precision", ["float64", "float32"])
@pytest.mark.parametrize("solver", ["dynamic", "mle"])
def test_burgers_small_vs_oracle(solver, precision):
    d, t1 = 64, 0.05
    u0s = [burgers_ic(d, s) for s in (1, 2)]
    out = gpu_bd(u0s, t1, precision, solver=solver)
    assert (out["status"] == 0).all()
    for b, u0 in enumerate(u0s):
        res = oracle_bd(u0, t1, solver=solver)
        if precision == "float64":
            tol = dict(u=1e-8, rows=1e-5, cov=1e-5, steps=0.0)
        else:
            r32 = oracle_bd(u0, t1, solver=solver, dtype=torch.float32)
            c64, c32 = res.u[-1].cholesky, r32.u[-1].cholesky.double()
            ratio = ((c32 @ c32.transpose(-1, -2))[:, 0, 0] / (c64 @ c64.transpose(-1, -2))[:, 0, 0]).sqrt()
            r = float(torch.maximum(ratio, 1.0 / ratio).max())
            dsteps = abs(int(r32.num_steps[-1]) - int(res.num_steps[-1]))
            tol = dict(u=1e-3, std_factor=max(2.0, 4.0 * r), steps=0.02, steps_abs=2 * dsteps, f32=True)
        compare(out, b, res, tol)
        if precision == "float64":
            assert rel(out["output_scale"][b, 0], torch.as_tensor(res.output_scale[-1]).reshape(-1)) < 1e-6


def burgers_rhs(d):
    dx = 1.0 / d

    def f(t, u):
        left, right = np.roll(u, 1), np.roll(u, -1)
        return -(right**2 - left**2) / (4 * dx) + NU_VISC * (right - 2 * u + left) / dx**2

    return f


T_FULL = 2e-3


def test_burgers_d64_full_horizon_vs_oracle():
    """The configuration's horizon t in [0, 1] at d = 64, where the oracle
    finishes (about 950 attempts): float64 kernel vs the oracle with the
    float64 tolerances, the float32 kernel's solution within 1e-3 of the
    oracle and its step count within 2 %."""
    d, t1 = 64, 1.0
    u0 = burgers_ic(d, 1)
    res = oracle_bd(u0, t1)
    o64 = gpu_bd([u0], t1, "float64")
    o32 = gpu_bd([u0], t1, "float32")
    assert int(o64["status"][0]) == 0 and int(o32["status"][0]) == 0
    compare(o64, 0, res, dict(u=1e-8, rows=1e-5, cov=1e-5, steps=0.0))
    assert rel(o64["output_scale"][0, 0], torch.as_tensor(res.output_scale[-1]).reshape(-1)) < 1e-6
    err = rel(o32["u_mean"][0, 0][:, 0], res.u[-1].mean[:, 0])
    assert err < 1e-3, err
    assert abs(int(o32["num_steps"][0, 0]) - res.num_steps[-1]) <= max(1, math.ceil(0.02 * res.num_steps[-1]))


@pytest.mark.parametrize("precision", ["float64", "float32"])
def test_burgers_full_size_vs_classical_solver(precision):
    """d = 4096, rtol = atol = 1e-4: terminal u against DOP853 (rtol 1e-10)."""
    d = 4096
    u0s = [burgers_ic(d, s) for s in (3, 4)]
    out = gpu_bd(u0s, T_FULL, precision)
    assert (out["status"] == 0).all()
    for b, u0 in enumerate(u0s):
        ref = scipy.integrate.solve_ivp(burgers_rhs(d), (0.0, T_FULL), u0, method="DOP853", rtol=1e-10, atol=1e-10).y[:, -1]
        u = out["u_mean"][b, 0, :, 0].numpy()
        err = np.abs(u - ref).max() / np.abs(ref).max()
        assert err < 2e-3, err  # global error of an rtol = 1e-4 local-error controller


def test_burgers_f32_matches_f64_full_size():
    """Float32 bulk reaches the float64 solution in about as many steps: at
    d = 4096 the TS0 step is bound by the stencil's stiffness (4 nu / dx^2 =
    6.7e5), not by the error estimate's noise: float32 took 9 % more attempts
    than float64 on the 64-instance batch over t in [0, 0.02] (bounded here by
    2x on the shorter horizon, where the start-up steps weigh more).  (Carrying
    u in float pairs with the stencil in float-pair arithmetic left the count
    unchanged and cost 20 % per attempt, so the kernel does not.)"""
    d = 4096
    u0s = [burgers_ic(d, 5)]
    o32 = gpu_bd(u0s, T_FULL, "float32")
    o64 = gpu_bd(u0s, T_FULL, "float64")
    assert (o32["status"] == 0).all() and (o64["status"] == 0).all()
    err = rel(o32["u_mean"][0, 0, :, 0], o64["u_mean"][0, 0, :, 0])
    assert err < 1e-3, err
    assert int(o32["num_steps"][0, 0]) <= 2 * int(o64["num_steps"][0, 0])


@pytest.mark.parametrize("precision", ["float64", "float32"])
def test_burgers_ts1_diagonal_vs_oracle(precision):
    """Block-diagonal TS1 (the Jacobian's diagonal along d, ssm_impl_blockdiag.py:147-183) at d = 64."""
    d, t1 = 64, 0.05
    u0s = [burgers_ic(d, s) for s in (1, 2)]
    out = gpu_bd(u0s, t1, precision, constraint="ts1")
    assert (out["status"] == 0).all()
    for b, u0 in enumerate(u0s):
        res = oracle_bd(u0, t1, constraint="ts1")
        if precision == "float64":
            compare(out, b, res, dict(u=1e-8, rows=1e-5, cov=1e-5, steps=0.0))
            assert rel(out["output_scale"][b, 0], torch.as_tensor(res.output_scale[-1]).reshape(-1)) < 1e-6
        else:
            err = rel(out["u_mean"][b, 0][:, 0], res.u[-1].mean[:, 0])
            assert err < 1e-3, err


def test_burgers_ts1_full_size_takes_far_fewer_steps():
    """At d = 4096 the diagonal TS1 operator carries the stiff -2 nu / dx^2 term:
    the solve on [0, 2e-3] needs a fraction of TS0's steps and still matches
    DOP853 to the accuracy of an rtol = 1e-4 controller."""
    d = 4096
    u0s = [burgers_ic(d, 3)]
    o0 = gpu_bd(u0s, T_FULL, "float64")
    o1 = gpu_bd(u0s, T_FULL, "float64", constraint="ts1")
    assert (o0["status"] == 0).all() and (o1["status"] == 0).all()
    ref = scipy.integrate.solve_ivp(burgers_rhs(d), (0.0, T_FULL), u0s[0], method="DOP853", rtol=1e-10, atol=1e-10).y[:, -1]
    err = np.abs(o1["u_mean"][0, 0, :, 0].numpy() - ref).max() / np.abs(ref).max()
    assert err < 2e-3, err
    assert int(o1["num_steps"][0, 0]) * 4 < int(o0["num_steps"][0, 0]), (int(o1["num_steps"][0, 0]), int(o0["num_steps"][0, 0]))


def test_burgers_error_state_std_vs_oracle():
    """error_state_std with per-dimension calibration (solvers.py:999-1098), d = 64, float64."""
    from probdiffeq_gb300 import ensemble

    d, t1 = 64, 0.05
    u0s = [burgers_ic(d, s) for s in (1, 2)]
    u0t = torch.as_tensor(np.asarray(u0s), dtype=torch.float64)
    cfg = ensemble.make_config(field="burgers", num_derivatives=3, ode_dim=d, ssm="blockdiag", solver="dynamic",
                               precision="float64", atol=1e-4, rtol=1e-4, clip_dt=True, error="state_std")
    out = ensemble.solve_ensemble(cfg, params=torch.full((2, 1), NU_VISC, dtype=torch.float64), y0=u0t,
                                  save_at=torch.tensor([0.0, t1], dtype=torch.float64), dt0=0.1 * t1)
    torch.cuda.synchronize()
    out = {k: v.cpu() for k, v in out.items() if not k.startswith("_") and v is not None}
    assert (out["status"] == 0).all()
    p = torch.tensor([NU_VISC], dtype=torch.float64)
    for b, u0 in enumerate(u0s):
        tc = problems.taylor_derivatives(problems.burgers, torch.tensor(u0), p, 3)
        S = ssm.BdSSM()
        c = S.constraint_ode_ts0(lambda u, t: problems.burgers(u[0], p))
        res = solvers.solve_adaptive_terminal_values(solvers.SolverDynamic(solvers.StrategyFilter(), c),
                                                     solvers.ErrorStateStd(c), S.prior_wiener_integrated(tc),
                                                     0.0, t1, 1e-4, 1e-4, dt0=0.1 * t1)
        compare(out, b, res, dict(u=1e-8, rows=1e-5, cov=1e-5, steps=0.0))


def compare_record(gm, gc, o, tol):
    err_u = rel(gm[:, 0], o.mean[:, 0])
    err_rows = max(rel(gm[:, i], o.mean[:, i]) for i in range(o.mean.shape[1]))
    cg = gc @ gc.transpose(-1, -2)
    co = o.cholesky @ o.cholesky.transpose(-1, -2)
    if float(co.abs().max()) == 0.0:  # the exact initial coefficients at t0
        err_cov = float(cg.abs().max())
    else:
        err_cov = max(rel(cg[j], co[j]) for j in range(co.shape[0]) if float(co[j].abs().max()) > 0)
    msg = f"u {err_u:.2e} rows {err_rows:.2e} cov {err_cov:.2e}"
    assert err_u <= tol["u"] and err_rows <= tol["rows"] and err_cov <= tol["cov"], msg


@pytest.mark.parametrize("solver", ["dynamic", "mle"])
def test_burgers_fixedpoint_smoother_vs_oracle(solver):
    """strategy_smoother_fixedpoint in the block-diagonal kernel (estimators_and_losses.py:473-591,
    ssm_impl_blockdiag.py:45-102): smoothed marginals at every checkpoint, d = 64, float64."""
    from probdiffeq_gb300 import ensemble

    d, t1 = 64, 0.05
    save_at = np.linspace(0.0, t1, 5)
    u0s = [burgers_ic(d, s) for s in (3, 4)]
    u0t = torch.as_tensor(np.asarray(u0s), dtype=torch.float64)
    cfg = ensemble.make_config(field="burgers", num_derivatives=3, ode_dim=d, ssm="blockdiag", solver=solver,
                               strategy="fixedpoint", precision="float64", atol=1e-4, rtol=1e-4, clip_dt=True)
    out = ensemble.solve_ensemble(cfg, params=torch.full((2, 1), NU_VISC, dtype=torch.float64), y0=u0t,
                                  save_at=torch.tensor(save_at), dt0=0.1 * t1, terminal_only=False)
    torch.cuda.synchronize()
    out = {k: v.cpu() for k, v in out.items() if not k.startswith("_") and v is not None}
    assert (out["status"] == 0).all()
    p = torch.tensor([NU_VISC], dtype=torch.float64)
    cls = {"dynamic": solvers.SolverDynamic, "mle": solvers.SolverMLE}[solver]
    for b, u0 in enumerate(u0s):
        tc = problems.taylor_derivatives(problems.burgers, torch.tensor(u0), p, 3)
        S = ssm.BdSSM()
        c = S.constraint_ode_ts0(lambda u, t: problems.burgers(u[0], p))
        res = solvers.solve_adaptive_save_at(cls(solvers.StrategyFixedPoint(), c), solvers.ErrorResidualStd(c),
                                             S.prior_wiener_integrated(tc), save_at, 1e-4, 1e-4, clip_dt=True,
                                             dt0=0.1 * t1)
        steps_o = [0] + list(res.num_steps)
        for s in range(len(save_at)):
            compare_record(out["u_mean"][b, s], out["u_chol"][b, s], res.u[s], dict(u=1e-8, rows=1e-5, cov=1e-5))
            assert int(out["num_steps"][b, s]) == steps_o[s]


def test_burgers_fixedpoint_full_size_float32():
    """d = 4096 in float32: the smoothed terminal record is the filter's, the
    smoothed t0 record the exact initial coefficients, all records finite."""
    from probdiffeq_gb300 import ensemble

    d, t1 = 4096, 2e-4
    u0s = [burgers_ic(d, s) for s in (1, 2)]
    u0t = torch.as_tensor(np.asarray(u0s), dtype=torch.float64)
    outs = {}
    for strategy in ("filter", "fixedpoint"):
        cfg = ensemble.make_config(field="burgers", num_derivatives=3, ode_dim=d, ssm="blockdiag", solver="dynamic",
                                   strategy=strategy, precision="float32", atol=1e-4, rtol=1e-4, clip_dt=True,
                                   max_attempts=1 << 26)
        outs[strategy] = ensemble.solve_ensemble(cfg, params=torch.full((2, 1), NU_VISC, dtype=torch.float64),
                                                 y0=u0t, save_at=torch.linspace(0.0, t1, 4, dtype=torch.float64),
                                                 dt0=0.1 * t1, terminal_only=False)
        torch.cuda.synchronize()
    f, s = outs["filter"], outs["fixedpoint"]
    assert (s["status"] == 0).all()
    assert torch.equal(s["num_steps"], f["num_steps"])
    assert torch.isfinite(s["u_mean"]).all() and torch.isfinite(s["u_chol"]).all()
    # float32: the smoother predicts through the revert's 2n x 2n QR, the filter through the 2n x n one
    assert rel(s["u_mean"][:, -1, :, 0].cpu(), f["u_mean"][:, -1, :, 0].cpu()) < 1e-3
    assert rel(s["u_mean"][:, 0, :, 0].cpu(), u0t) < 1e-5
