"""Parity of the dense-factorisation CUDA solver against the oracle (GPU).

Configuration of the stiff dense batch: van der Pol (first order), IWP with 3
derivatives, TS1 with the analytic Jacobian, fixed-point smoother with
save_at checkpoints, dynamic calibration, error_residual_std, integral
control.  The oracle's step count grows quickly with mu (48 / 3.5e3 / 1e5
accepted steps for mu = 1 / 10 / 100), so parity runs at small mu.

Tolerances (relative to the largest entry per Taylor-coefficient row and of
L L^T): float64 -- solution 1e-8, rows 1e-5, covariance 1e-5, steps +-1;
float32 -- solution 1e-3 and the std of u within a factor 2 (float32 cannot
carry these covariances: the oracle itself deviates by tens of percent in
float32), steps within 2 % (+-1).
"""

import math

import numpy as np
import pytest
import torch

from oracle import problems, solvers, ssm

pytestmark = pytest.mark.gpu


def oracle_vdp(mu, save_at, strategy="fixedpoint", constraint="ts1", solver="dynamic", atol=1e-5, rtol=1e-5, dtype=torch.float64,
               error="residual_std"):
    p = torch.tensor([mu], dtype=torch.float64)
    y0 = torch.tensor([2.0, 0.0], dtype=torch.float64)
    tc = problems.taylor_derivatives(problems.van_der_pol, y0, p, 3).to(dtype)
    pt = p.to(dtype)
    D = ssm.DenseSSM()
    prior = D.prior_wiener_integrated(tc)
    vf = lambda u, t: problems.van_der_pol(u[0], pt)
    jac = lambda u, t: problems.jacobian(problems.van_der_pol, u, pt)
    c = D.constraint_ode_ts1(vf, jac, 2) if constraint == "ts1" else D.constraint_ode_ts0(vf, 2)
    strat = solvers.StrategyFixedPoint() if strategy == "fixedpoint" else solvers.StrategyFilter()
    cls = {"dynamic": solvers.SolverDynamic, "mle": solvers.SolverMLE, "none": solvers.SolverPlain}[solver]
    err = solvers.ErrorStateStd(c) if error == "state_std" else solvers.ErrorResidualStd(c)
    return solvers.solve_adaptive_save_at(cls(strat, c), err, prior, save_at, atol, rtol)


def gpu_dense(field, params, y0, save_at, precision, strategy="fixedpoint", constraint="ts1", solver="dynamic",
              atol=1e-5, rtol=1e-5, nu=3, posterior=True, clip_dt=False, terminal_only=False, variant=0,
              error="residual_std"):
    from probdiffeq_gb300 import _native, ensemble

    cfg = ensemble.make_config(
        field=field, num_derivatives=nu, ode_dim=2, ssm="dense", constraint=constraint, strategy=strategy,
        solver=solver, precision=precision, atol=atol, rtol=rtol, clip_dt=clip_dt, kernel_variant=variant,
        error=error,
    )
    params = torch.as_tensor(params, dtype=torch.float64)
    y0 = torch.as_tensor(y0, dtype=torch.float64)
    save_at = torch.as_tensor(save_at, dtype=torch.float64)
    B, S = y0.shape[0], save_at.shape[-1]
    outs = _native.alloc_outputs(cfg, B, S, terminal_only, "cuda", posterior=posterior and strategy == "fixedpoint" and not terminal_only)
    out = ensemble.solve_ensemble(cfg, params=params, y0=y0, save_at=save_at, dt0=0.1, terminal_only=terminal_only, outputs=outs)
    torch.cuda.synchronize()
    return {k: v.cpu() for k, v in out.items() if not k.startswith("_") and v is not None}


def rel(a, b):
    return float((a - b).abs().max() / b.abs().max().clamp_min(1e-300))


def row_rel(g, o, d=2):
    g, o = g.reshape(-1, d), o.reshape(-1, d)
    return max(rel(g[i], o[i]) for i in range(o.shape[0]))


def check(gm, gc, o, tol):
    err_u = rel(gm[:2], o.mean[:2])
    err_rows = row_rel(gm, o.mean)
    co = o.cholesky @ o.cholesky.T
    cg = gc @ gc.T
    err_cov = rel(cg, co)
    msg = f"u {err_u:.2e} rows {err_rows:.2e} cov {err_cov:.2e}"
    assert err_u <= tol["u"], msg
    if tol.get("f32"):
        # float32 cannot carry these covariances; assert the std of u within 2x
        assert torch.isfinite(gc).all(), msg
        for j in range(2):
            s_g, s_o = float(cg[j, j].sqrt()), float(co[j, j].sqrt())
            assert 0.5 * s_o <= s_g <= 2.0 * s_o or s_o < 1e-6 * float(o.mean[:2].abs().max()), (s_g, s_o, msg)
    else:
        assert err_rows <= tol["rows"], msg
        assert err_cov <= tol["cov"], msg


def f32_tol(o64, o32):
    rows = row_rel(o32.mean.double(), o64.mean)
    c32 = o32.cholesky.double()
    cov = rel(c32 @ c32.T, o64.cholesky @ o64.cholesky.T)
    return dict(u=1e-3, rows=max(5e-2, 4 * rows), cov=max(5e-2, 4 * cov), f32=True)


TOL64 = dict(u=1e-8, rows=1e-5, cov=1e-5)


VARIANTS = {"thread": 1, "lanes": 2, "struct": 3, "struct8": 4, "struct16": 5}


@pytest.mark.parametrize("variant", ["thread", "lanes", "struct", "struct8", "struct16"])
@pytest.mark.parametrize("precision", ["float64", "float32"])
@pytest.mark.parametrize("mu", [1.0, 3.0])
def test_vdp_fixedpoint_ts1_save_at(mu, precision, variant):
    """Smoothed marginals at the checkpoints, the backward pass included, for
    both instance-to-thread mappings."""
    save_at = np.linspace(0.0, 2.0 * mu, 8)
    res = oracle_vdp(mu, save_at)
    out = gpu_dense("van_der_pol", [[mu]], [[2.0, 0.0]], save_at, precision, variant=VARIANTS[variant])
    assert int(out["status"][0]) == 0
    if precision == "float32":
        r32 = oracle_vdp(mu, save_at, dtype=torch.float32)
    steps_o = [0] + list(res.num_steps)
    for s in range(len(save_at)):
        tol = TOL64 if precision == "float64" else f32_tol(res.u[s], r32.u[s])
        check(out["u_mean"][0, s], out["u_chol"][0, s], res.u[s], tol)
        allowed = 1 if precision == "float64" else max(1, math.ceil(0.02 * steps_o[s]))
        assert abs(int(out["num_steps"][0, s]) - steps_o[s]) <= allowed
    if precision == "float64":
        # the backward conditionals of the smoother posterior
        for k, c in enumerate(res.posterior["conditionals"]):
            assert rel(out["cond_A"][0, k], c.A) < 1e-6
            assert rel(out["cond_noise_mean"][0, k], c.noise.mean) < 1e-6
            X = out["cond_noise_chol"][0, k]
            assert rel(X @ X.T, c.noise.cholesky @ c.noise.cholesky.T) < 1e-5
            assert rel(out["cond_to_latent"][0, k], c.to_latent) < 1e-6  # 1/p: ~h^-3, sensitive to t rounding
            assert rel(out["cond_to_observed"][0, k], c.to_observed) < 1e-6
        # filtering marginals at the checkpoints
        for s, f in enumerate(res.posterior["filtering"]):
            assert rel(out["filter_mean"][0, s], f.mean) < 1e-6


@pytest.mark.parametrize("variant", ["thread", "lanes", "struct", "struct8", "struct16"])
def test_vdp_filter_ts0_and_mle(variant):
    """Dense TS0 with the filter and MLE calibration, float64."""
    save_at = np.linspace(0.0, 2.0, 5)
    res = oracle_vdp(1.0, save_at, strategy="filter", constraint="ts0", solver="mle")
    out = gpu_dense("van_der_pol", [[1.0]], [[2.0, 0.0]], save_at, "float64", strategy="filter", constraint="ts0", solver="mle",
                    variant=VARIANTS[variant])
    assert int(out["status"][0]) == 0
    for s in range(len(save_at)):
        check(out["u_mean"][0, s], out["u_chol"][0, s], res.u[s], TOL64)


@pytest.mark.parametrize("solver,strategy", [("dynamic", "fixedpoint"), ("mle", "filter")])
def test_vdp_error_state_std(solver, strategy):
    """error_state_std (solvers.py:999-1098) in the dense factorisation: the
    posterior std of u after conditioning the unit-scale extrapolation on
    the TS1 linearisation, float64, vs the oracle's ErrorStateStd."""
    mu = 2.0
    save_at = np.linspace(0.0, 2.0 * mu, 6)
    res = oracle_vdp(mu, save_at, strategy=strategy, solver=solver, error="state_std")
    out = gpu_dense("van_der_pol", [[mu]], [[2.0, 0.0]], save_at, "float64", strategy=strategy, solver=solver,
                    error="state_std", posterior=False)
    assert int(out["status"][0]) == 0
    steps_o = [0] + list(res.num_steps)
    for s in range(len(save_at)):
        check(out["u_mean"][0, s], out["u_chol"][0, s], res.u[s], TOL64)
        assert abs(int(out["num_steps"][0, s]) - steps_o[s]) <= 1
    # the lane mappings do not implement it
    from probdiffeq_gb300 import _native

    for variant in (2, 3, 4, 5):
        with pytest.raises(_native.NativeError):
            gpu_dense("van_der_pol", [[mu]], [[2.0, 0.0]], save_at, "float64", error="state_std", variant=variant)


def test_dense_equals_isotropic_on_lotka_volterra():
    """TS0 with kron-structured priors: dense and isotropic agree
    (tests/test_probdiffeq/test_calibration/test_dynamic_across_factorisations.py:10-64)."""
    from probdiffeq_gb300 import ensemble

    params = torch.tensor([[0.5, 0.05, 0.5, 0.05]], dtype=torch.float64)
    y0 = torch.tensor([[20.0, 20.0]], dtype=torch.float64)
    save_at = torch.tensor([0.0, 5.0], dtype=torch.float64)
    dn = gpu_dense("lotka_volterra", params, y0, save_at, "float64", strategy="filter", constraint="ts0",
                   atol=1e-6, rtol=1e-6, nu=3, clip_dt=True, terminal_only=True)
    cfg = ensemble.make_config(field="lotka_volterra", num_derivatives=3, ode_dim=2, solver="dynamic", precision="float64")
    iso = ensemble.solve_ensemble(cfg, params=params, y0=y0, save_at=save_at)
    torch.cuda.synchronize()
    assert int(dn["num_steps"][0, 0]) == int(iso["num_steps"][0, 0].item())
    assert rel(dn["u_mean"][0, 0], iso["u_mean"][0, 0].cpu().reshape(-1)) < 1e-9
    Ld = dn["u_chol"][0, 0]
    Li = iso["u_chol"][0, 0].cpu()
    Ci = torch.kron(Li @ Li.T, torch.eye(2, dtype=torch.float64))
    assert rel(Ld @ Ld.T, Ci) < 1e-7


@pytest.mark.parametrize("variant", ["thread", "lanes", "struct", "struct8", "struct16"])
def test_dense_batch_and_workspace_errors(variant):
    """Several instances in one launch (five: a partly filled block for the
    lane mappings); too small a workspace is rejected before launch."""
    import ctypes

    from probdiffeq_gb300 import _native, ensemble

    mus = [1.0, 1.5, 2.0, 1.25, 1.75]
    save_at = np.linspace(0.0, 2.0, 4)
    out = gpu_dense("van_der_pol", [[m] for m in mus], [[2.0, 0.0]] * len(mus), save_at, "float64", posterior=False,
                    variant=VARIANTS[variant])
    for b, mu in enumerate(mus):
        res = oracle_vdp(mu, np.linspace(0.0, 2.0, 4))
        check(out["u_mean"][b, -1], out["u_chol"][b, -1], res.u[-1], TOL64)
    cfg = ensemble.make_config(field="van_der_pol", num_derivatives=3, ode_dim=2, ssm="dense", constraint="ts1", strategy="fixedpoint")
    assert _native.workspace_size(cfg, 3, 4) > 0
    args = _native.PdqAdaptiveArgs()
    args.num_instances, args.num_save_at = 3, 4
    dummy = torch.zeros(64, dtype=torch.float64, device="cuda")
    for k in ("save_at", "params", "y0", "dt0", "u_mean", "u_chol", "output_scale", "t", "num_steps", "num_attempts", "status"):
        setattr(args, k, ctypes.c_void_p(dummy.data_ptr()))
    st = _native.load().pdq_solve_adaptive(ctypes.byref(cfg), ctypes.byref(args), ctypes.c_void_p(dummy.data_ptr()), 8, None)
    assert st == 4  # PDQ_ERROR_WORKSPACE, nothing launched


@pytest.mark.parametrize("precision", ["float64", "float32"])
def test_vdp_mu30_100_save_points_matches_fixture(precision):
    """The stiff configuration's solver at mu = 30 with its 100 save points
    (the oracle's 1.9e4 accepted steps, 3.2e4 attempts; the oracle output is
    the committed fixture ``tests/golden/vdp_dense_mu30.json``), the default
    (structure-exploiting) kernel.  Float64: the live-oracle tolerances at
    every save point.  Float32: matched accuracy -- its error against the
    exact solution (scipy Radau, rtol = atol = 1e-12) within 2x the float64
    oracle's own error against it, in the median and at the maximum over the
    save points (the solver's error at rtol 1e-5 reaches several percent at
    the relaxation oscillations' fast transitions; the kernel carries the
    mean's rows 0 and 1 and the residual in float pairs, without which
    float32 measured 2.3x / 3.1x), and accepted steps within 2 %."""
    import scipy.integrate

    from tests.golden import make_golden

    gold = make_golden.load("vdp_dense_mu30.json")
    mu = gold["mu"][0]
    save_at = np.asarray(gold["save_at"][0])
    rec = gold["records"][0]
    out = gpu_dense("van_der_pol", [[mu]], [gold["y0"]], save_at, precision)
    assert int(out["status"][0]) == 0
    steps_o = [0] + list(rec["num_steps"])
    if precision == "float32":
        truth = scipy.integrate.solve_ivp(
            lambda t, u: [u[1], mu * ((1 - u[0] ** 2) * u[1] - u[0])], (0.0, save_at[-1]), gold["y0"],
            method="Radau", rtol=1e-12, atol=1e-12, t_eval=save_at,
            jac=lambda t, u: [[0.0, 1.0], [mu * (-2 * u[0] * u[1] - 1), mu * (1 - u[0] ** 2)]]).y.T
        scale = np.abs(truth).max(axis=1)
        e32 = np.abs(out["u_mean"][0, :, :2].numpy() - truth).max(axis=1) / scale
        e64 = np.abs(np.array([m[:2] for m in rec["u_mean"]]) - truth).max(axis=1) / scale
        assert np.median(e32) <= 2 * np.median(e64), (np.median(e32), np.median(e64))
        assert e32.max() <= 2 * e64.max(), (e32.max(), e64.max())
    for s in range(len(save_at)):
        om = torch.tensor(rec["u_mean"][s], dtype=torch.float64)
        oc = torch.tensor(rec["u_chol"][s], dtype=torch.float64)
        gm, gc = out["u_mean"][0, s], out["u_chol"][0, s]
        if precision == "float64":
            assert rel(gm[:2], om[:2]) <= 1e-8, s
            assert row_rel(gm, om) <= 1e-5, s
            assert rel(gc @ gc.T, oc @ oc.T) <= 1e-5, s
            allowed = 1
        else:
            assert torch.isfinite(gc).all()
            allowed = max(1, math.ceil(0.02 * steps_o[s]))
        assert abs(int(out["num_steps"][0, s]) - steps_o[s]) <= allowed, (s, int(out["num_steps"][0, s]), steps_o[s])
