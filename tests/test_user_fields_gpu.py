"""Run-time compiled vector fields in the isotropic and dense solvers (GPU).

* The Lotka--Volterra source, registered at run time, reproduces the
  built-in Lotka--Volterra kernel (same templates, same arithmetic) exactly,
  in float32 and float64, for the filter and the fixed-point smoother.
* Fields without a built-in counterpart (Brusselator, the three-dimensional
  Lorenz system) match the oracle with a Python definition of the same field
  (float64: solution 1e-9, rows 1e-6, covariance 1e-6, steps +-1).
* The LML kernels (forward mode; the adjoint pair with its covariance plan)
  compiled for a registered field: FitzHugh--Nagumo reproduces the built-in
  kernels bit for bit, Brusselator matches the oracle's reverse mode.
* The block-diagonal cluster kernel compiled for a registered stencil: the
  Burgers stencil reproduces the built-in kernel bit for bit (filter and
  fixed-point smoother, d = 64 and 4096, float32 and float64), Allen--Cahn
  matches the oracle at d = 64.
"""

import numpy as np
import pytest
import torch

from oracle import problems, solvers, ssm
from probdiffeq_gb300 import _native, ensemble
from tests import user_fields
from tests.test_iso_gpu import compare_record, lv_instances, tolerances

pytestmark = pytest.mark.gpu


def _solve(field, params, y0, save_at, precision, strategy="filter", clip_dt=True, nu=4, solver="mle", tol=1e-6):
    cfg = ensemble.make_config(field=field, num_derivatives=nu, ode_dim=y0.shape[1], solver=solver, precision=precision,
                               atol=tol, rtol=tol, clip_dt=clip_dt, strategy=strategy)
    out = ensemble.solve_ensemble(cfg, params=params, y0=y0, save_at=torch.tensor(save_at, dtype=torch.float64),
                                  dt0=0.1, terminal_only=False)
    torch.cuda.synchronize()
    return {k: v.cpu() for k, v in out.items() if not k.startswith("_") and v is not None}


@pytest.mark.parametrize("strategy", ["filter", "fixedpoint"])
@pytest.mark.parametrize("precision", ["float32", "float64"])
def test_runtime_lotka_volterra_equals_the_builtin_kernel(precision, strategy):
    if "gpu_test_lv" not in _native.FIELD:
        _native.register_field("gpu_test_lv", user_fields.LOTKA_VOLTERRA, 2, 4)
    params, y0 = lv_instances(33, seed=9)
    save_at = [0.0, 3.0, 7.5]
    a = _solve("lotka_volterra", params, y0, save_at, precision, strategy=strategy, clip_dt=strategy == "filter")
    b = _solve("gpu_test_lv", params, y0, save_at, precision, strategy=strategy, clip_dt=strategy == "filter")
    for k in ("u_mean", "u_chol", "output_scale", "t", "num_steps", "num_attempts", "status"):
        assert torch.equal(a[k], b[k]), k


@pytest.mark.parametrize("case", ["brusselator", "lorenz"])
def test_runtime_fields_match_the_oracle(case):
    source, fn, params, y0, t1 = {
        "brusselator": (user_fields.BRUSSELATOR, user_fields.brusselator, [[1.0, 3.0], [1.2, 2.5]],
                        [[1.5, 3.0], [1.0, 2.0]], 5.0),
        "lorenz": (user_fields.LORENZ, user_fields.lorenz, [[10.0, 28.0, 8.0 / 3.0], [10.0, 20.0, 2.0]],
                   [[1.0, 1.0, 1.0], [-2.0, 0.5, 10.0]], 1.0),
    }[case]
    name = "gpu_test_" + case
    if name not in _native.FIELD:
        _native.register_field(name, source, len(y0[0]), len(params[0]))
    params = torch.tensor(params, dtype=torch.float64)
    y0 = torch.tensor(y0, dtype=torch.float64)
    save_at = [0.0, t1]
    out = _solve(name, params, y0, save_at, "float64", nu=3, solver="dynamic", tol=1e-6)
    assert (out["status"] == 0).all()
    for b in range(2):
        tc = problems.taylor_derivatives(fn, y0[b], params[b], 3)
        S = ssm.IsoSSM()
        c = S.constraint_ode_ts0(lambda u, t, p=params[b]: fn(u[0], p))
        res = solvers.solve_adaptive_save_at(solvers.SolverDynamic(solvers.StrategyFilter(), c),
                                             solvers.ErrorResidualStd(c), S.prior_wiener_integrated(tc), save_at,
                                             1e-6, 1e-6, clip_dt=True, dt0=0.1)
        o = res.u[-1]
        compare_record(out["u_mean"][b, -1], out["u_chol"][b, -1], o.mean, o.cholesky, out["num_steps"][b, -1],
                       res.num_steps[-1], tolerances("float64"))


def _solve_dense(field, params, y0, save_at, precision, constraint="ts1", strategy="fixedpoint", solver="dynamic",
                 tol=1e-6, nu=3, variant=0):
    cfg = ensemble.make_config(field=field, num_derivatives=nu, ode_dim=y0.shape[1], ssm="dense", constraint=constraint,
                               strategy=strategy, solver=solver, precision=precision, atol=tol, rtol=tol,
                               clip_dt=False, kernel_variant=variant)
    out = ensemble.solve_ensemble(cfg, params=params, y0=y0, save_at=torch.tensor(save_at, dtype=torch.float64),
                                  dt0=0.1, terminal_only=False)
    torch.cuda.synchronize()
    return {k: v.cpu() for k, v in out.items() if not k.startswith("_") and v is not None}


def test_runtime_lotka_volterra_equals_the_builtin_dense_kernel(precision="float32"):
    """The dense TS1 fixed-point kernel instantiated at run time for the
    Lotka--Volterra source (run-time fields take the thread-per-instance
    kernel) equals the built-in thread-per-instance kernel bit for bit
    (float32; each dense variant takes about a minute of NVRTC compilation on
    first use)."""
    if "gpu_test_lv" not in _native.FIELD:
        _native.register_field("gpu_test_lv", user_fields.LOTKA_VOLTERRA, 2, 4)
    params, y0 = lv_instances(9, seed=11)
    save_at = [0.0, 2.0, 5.0]
    a = _solve_dense("lotka_volterra", params, y0, save_at, precision, variant=1)
    b = _solve_dense("gpu_test_lv", params, y0, save_at, precision)
    for k in ("u_mean", "u_chol", "output_scale", "t", "num_steps", "num_attempts", "status"):
        assert torch.equal(a[k], b[k]), k


def test_runtime_lorenz_dense_ts1_matches_the_oracle():
    """Lorenz-63 (d = 3, N = 12) in the dense factorisation with TS1 (the
    Jacobian by dual numbers from the registered source), fixed-point
    smoother, float64, vs the oracle with the Jacobian by torch autograd.
    Lorenz-63 is chaotic: over [0, 0.5] the tolerances are solution 1e-7,
    rows / covariances 1e-4, steps +-1."""
    if "gpu_test_lorenz" not in _native.FIELD:
        _native.register_field("gpu_test_lorenz", user_fields.LORENZ, 3, 3)
    params = torch.tensor([[10.0, 28.0, 8.0 / 3.0], [10.0, 20.0, 2.0]], dtype=torch.float64)
    y0 = torch.tensor([[1.0, 1.0, 1.0], [-2.0, 0.5, 10.0]], dtype=torch.float64)
    save_at = [0.0, 0.25, 0.5]
    out = _solve_dense("gpu_test_lorenz", params, y0, save_at, "float64")
    assert (out["status"] == 0).all()
    for b in range(2):
        tc = problems.taylor_derivatives(user_fields.lorenz, y0[b], params[b], 3)
        S = ssm.DenseSSM()
        vf = lambda u, t, p=params[b]: user_fields.lorenz(u[0], p)  # noqa: E731
        jac = lambda u, t, p=params[b]: problems.jacobian(user_fields.lorenz, u, p)  # noqa: E731
        c = S.constraint_ode_ts1(vf, jac, 3)
        res = solvers.solve_adaptive_save_at(solvers.SolverDynamic(solvers.StrategyFixedPoint(), c),
                                             solvers.ErrorResidualStd(c), S.prior_wiener_integrated(tc), save_at,
                                             1e-6, 1e-6, dt0=0.1)
        steps_o = [0] + list(res.num_steps)
        for s in range(len(save_at)):
            o = res.u[s]
            m, L = out["u_mean"][b, s], out["u_chol"][b, s]
            mo, Co = o.to_multivariate_normal()
            assert float((m[:3] - mo[:3]).abs().max() / mo[:3].abs().max()) < 1e-7
            assert float((m - mo).abs().max() / mo.abs().max()) < 1e-4
            C = L @ L.T
            assert float((C - Co).abs().max() / Co.abs().max().clamp_min(1e-300)) < 1e-4
            assert abs(int(out["num_steps"][b, s]) - steps_o[s]) <= 1


def _lml_calls(field, precision, thetas, data, num_steps, y0):
    """Forward-mode LML + gradient and the adjoint pair for ``field``."""
    f64 = dict(dtype=torch.float64, device="cuda")
    B = thetas.shape[0]
    cfg = ensemble.make_config(field=field, num_derivatives=3, ode_dim=2, strategy="fixedpoint", solver="none",
                               precision=precision)
    th, y = thetas.to(**f64), torch.as_tensor(y0, **f64).expand(B, 2).contiguous()
    d = torch.as_tensor(data, **f64)
    std = torch.full((d.shape[0],), 0.01, **f64)
    fm = _native.lml_fixed_grid(cfg, th, y, d, std, t0=0.0, dt=0.01, num_steps=num_steps, save_every=10,
                                average_pdfs=False, gradient=True)
    fwd = _native.lml_fwd(cfg, th, y, d, std, t0=0.0, dt=0.01, num_steps=num_steps, save_every=10)
    bwd = _native.lml_bwd(fwd, None, y0_grad=True)
    torch.cuda.synchronize()
    return {"lml": fm["lml"].cpu(), "grad": fm["grad"].cpu(), "status": fm["status"].cpu(),
            "adj_lml": fwd["lml"].cpu(), "adj_grad": bwd["grad"].cpu(), "adj_grad_y0": bwd["grad_y0"].cpu()}


@pytest.mark.parametrize("precision", ["float32", "float64"])
def test_runtime_field_lml_equals_the_builtin_kernels(precision):
    """The LML kernels (forward mode, and the adjoint pair with its plan)
    compiled at run time for a registered FitzHugh--Nagumo source reproduce
    the built-in FitzHugh--Nagumo kernels bit for bit."""
    from tests import lml_problem

    if "gpu_test_fhn" not in _native.FIELD:
        _native.register_field("gpu_test_fhn", user_fields.FITZHUGH_NAGUMO, 2, 3)
    num_steps, data = lml_problem.observations(t1=2.0)
    thetas = torch.tensor(lml_problem.theta_samples(40, seed=5), dtype=torch.float64)
    a = _lml_calls("fitzhugh_nagumo", precision, thetas, data, num_steps, lml_problem.U0)
    b = _lml_calls("gpu_test_fhn", precision, thetas, data, num_steps, lml_problem.U0)
    assert (a["status"] == 0).all()
    for k in a:
        assert torch.equal(a[k], b[k]), k


def test_runtime_field_lml_matches_the_oracle():
    """A field without a built-in LML kernel (Brusselator, two parameters):
    LML and gradient through the run-time kernels against the oracle's
    reverse mode (float64: LML 1e-9, gradient 1e-6 of its norm)."""
    from oracle import lml as oracle_lml

    if "gpu_test_brusselator" not in _native.FIELD:
        _native.register_field("gpu_test_brusselator", user_fields.BRUSSELATOR, 2, 2)
    y0 = [1.5, 3.0]
    thetas = torch.tensor([[1.0, 3.0], [1.1, 2.8]], dtype=torch.float64)
    num_steps = 200
    t_obs = np.arange(num_steps // 10 + 1) * 0.1
    data = np.stack([1.5 + 0.1 * np.sin(t_obs), 3.0 - 0.2 * t_obs], axis=1)
    out = _lml_calls("gpu_test_brusselator", "float64", thetas, data, num_steps, y0)
    assert (out["status"] == 0).all()
    for b in range(2):
        lml, g, _ = oracle_lml.lml_value_and_grads(thetas[b].numpy(), np.array(y0), data, 0.01, num_steps, 10, 0.01,
                                                   field=user_fields.brusselator)
        assert abs(float(out["lml"][b]) - lml) <= 1e-9 * abs(lml), (b, float(out["lml"][b]), lml)
        assert np.abs(out["grad"][b].numpy() - g).max() <= 1e-6 * np.linalg.norm(g), b
        assert np.abs(out["adj_grad"][b].numpy() - g).max() <= 1e-6 * np.linalg.norm(g), b


def _bd(field, u0s, t1, precision, strategy="filter", param=0.01):
    u0s = torch.as_tensor(np.asarray(u0s), dtype=torch.float64)
    B, d = u0s.shape
    cfg = ensemble.make_config(field=field, num_derivatives=3, ode_dim=d, ssm="blockdiag", solver="dynamic",
                               strategy=strategy, precision=precision, atol=1e-4, rtol=1e-4, clip_dt=True)
    out = ensemble.solve_ensemble(cfg, params=torch.full((B, 1), param, dtype=torch.float64), y0=u0s,
                                  save_at=torch.tensor([0.0, t1], dtype=torch.float64), dt0=0.1 * t1)
    torch.cuda.synchronize()
    return {k: v.cpu() for k, v in out.items() if not k.startswith("_") and v is not None}


@pytest.mark.parametrize("precision", ["float32", "float64"])
@pytest.mark.parametrize("strategy,d,t1", [("filter", 64, 0.05), ("fixedpoint", 64, 0.05), ("filter", 4096, 2e-4)])
def test_runtime_stencil_equals_the_builtin_burgers_kernel(precision, strategy, d, t1):
    """The block-diagonal cluster kernel compiled at run time for a
    registered Burgers stencil reproduces the built-in Burgers kernel bit for
    bit (the same template, the same arithmetic)."""
    from tests.test_blockdiag_gpu import burgers_ic

    if "gpu_test_burgers_stencil" not in _native.FIELD:
        _native.register_stencil("gpu_test_burgers_stencil", user_fields.BURGERS_STENCIL, 1)
    u0s = [burgers_ic(d, s) for s in (1, 2)]
    a = _bd("burgers", u0s, t1, precision, strategy)
    b = _bd("gpu_test_burgers_stencil", u0s, t1, precision, strategy)
    assert (a["status"] == 0).all()
    for k in a:
        assert torch.equal(a[k], b[k]), k


def test_runtime_stencil_allen_cahn_matches_the_oracle():
    """A stencil without a built-in counterpart (Allen--Cahn, eps^2 = 0.01) at
    d = 64 against the oracle's block-diagonal TS0 filter with the same field
    in Python (float64: solution 1e-8, the higher Taylor rows 1e-3 -- measured
    1.5e-4: the small third-derivative row carries the rounding of the
    preconditioned update relative to its own scale --, covariances 1e-3,
    measured 1.5e-4, steps +-1)."""
    from oracle import problems, solvers, ssm

    if "gpu_test_allen_cahn" not in _native.FIELD:
        _native.register_stencil("gpu_test_allen_cahn", user_fields.ALLEN_CAHN_STENCIL, 1)
    d, t1 = 64, 0.5
    x = np.arange(d) / d
    u0s = [0.5 * np.sin(2 * np.pi * x) + 0.1 * np.cos(4 * np.pi * x), 0.3 * np.cos(2 * np.pi * x) - 0.2]
    out = _bd("gpu_test_allen_cahn", u0s, t1, "float64")
    assert (out["status"] == 0).all()
    p = torch.tensor([0.01], dtype=torch.float64)
    for b, u0 in enumerate(u0s):
        tc = problems.taylor_derivatives(user_fields.allen_cahn, torch.tensor(u0), p, 3)
        S = ssm.BdSSM()
        c = S.constraint_ode_ts0(lambda u, t: user_fields.allen_cahn(u[0], p))
        res = solvers.solve_adaptive_terminal_values(solvers.SolverDynamic(solvers.StrategyFilter(), c),
                                                     solvers.ErrorResidualStd(c), S.prior_wiener_integrated(tc),
                                                     0.0, t1, 1e-4, 1e-4, dt0=0.1 * t1)
        o = res.u[-1]
        gm, gc = out["u_mean"][b, 0], out["u_chol"][b, 0]
        rel = lambda g, w: float((g - w).abs().max() / w.abs().max().clamp_min(1e-300))  # noqa: E731
        assert rel(gm[:, 0], o.mean[:, 0]) <= 1e-8
        assert max(rel(gm[:, i], o.mean[:, i]) for i in range(4)) <= 1e-3
        cg, co = gc @ gc.transpose(-1, -2), o.cholesky @ o.cholesky.transpose(-1, -2)
        assert max(rel(cg[j], co[j]) for j in range(d)) <= 1e-3
        assert abs(int(out["num_steps"][b, 0]) - res.num_steps[-1]) <= 1
