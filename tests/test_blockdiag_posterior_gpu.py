"""The block-diagonal fixed-point smoother's posterior (GPU): its backward
conditionals and filtering marginals as outputs, the fixed-interval
off-grid marginals built on them through the drop-in API, and posterior
samples.

Periodic viscous Burgers (the high-dimensional configuration's problem) at
d = 16 on t in [0, 0.05], IWP nu = 3, TS0, float64, against the oracle's
block-diagonal smoother (ssm_impl_blockdiag.py:16-113 per dimension,
estimators_and_losses.py:437-591): conditionals A, noise mean, to_latent,
to_observed within 1e-6, the noise covariance X X^T within 1e-5 (the parity
tests' float64 tolerances), filtering marginals within 1e-6 / 1e-5.
"""

import numpy as np
import pytest
import torch

from oracle import problems, solvers, ssm
from tests.test_blockdiag_gpu import NU_VISC, burgers_ic

pytestmark = pytest.mark.gpu

D, T1 = 16, 0.05


def rel(a, b):
    a, b = torch.as_tensor(a, dtype=torch.float64), torch.as_tensor(b, dtype=torch.float64)
    return float((a - b).abs().max() / b.abs().max().clamp_min(1e-300))


def gpu_smoother(u0s, save_at, solver):
    from probdiffeq_gb300 import _native, ensemble

    u0t = torch.as_tensor(np.asarray(u0s), dtype=torch.float64)
    B = u0t.shape[0]
    cfg = ensemble.make_config(field="burgers", num_derivatives=3, ode_dim=D, ssm="blockdiag", solver=solver,
                               strategy="fixedpoint", precision="float64", atol=1e-4, rtol=1e-4, clip_dt=True)
    outs = _native.alloc_outputs(cfg, B, len(save_at), False, "cuda", posterior=True)
    out = ensemble.solve_ensemble(cfg, params=torch.full((B, 1), NU_VISC, dtype=torch.float64), y0=u0t,
                                  save_at=torch.tensor(save_at), dt0=0.1 * T1, terminal_only=False, outputs=outs)
    torch.cuda.synchronize()
    return {k: v.cpu() for k, v in out.items() if not k.startswith("_") and v is not None}


def oracle_smoother(u0, save_at, solver):
    p = torch.tensor([NU_VISC], dtype=torch.float64)
    tc = problems.taylor_derivatives(problems.burgers, torch.tensor(u0), p, 3)
    S = ssm.BdSSM()
    c = S.constraint_ode_ts0(lambda u, t: problems.burgers(u[0], p))
    cls = {"dynamic": solvers.SolverDynamic, "mle": solvers.SolverMLE}[solver]
    return solvers.solve_adaptive_save_at(cls(solvers.StrategyFixedPoint(), c), solvers.ErrorResidualStd(c),
                                          S.prior_wiener_integrated(tc), save_at, 1e-4, 1e-4, clip_dt=True, dt0=0.1 * T1)


@pytest.mark.parametrize("solver", ["dynamic", "mle"])
def test_blockdiag_smoother_posterior_matches_the_oracle(solver):
    save_at = np.linspace(0.0, T1, 4)
    u0s = [burgers_ic(D, s) for s in (5, 6)]
    out = gpu_smoother(u0s, save_at, solver)
    assert (out["status"] == 0).all()
    for b, u0 in enumerate(u0s):
        res = oracle_smoother(u0, save_at, solver)
        for k, c in enumerate(res.posterior["conditionals"]):
            assert rel(out["cond_A"][b, k], c.A) < 1e-6, (b, k)
            assert rel(out["cond_noise_mean"][b, k], c.noise.mean) < 1e-6, (b, k)
            X = out["cond_noise_chol"][b, k]
            Xo = c.noise.cholesky
            assert rel(X @ X.transpose(-1, -2), Xo @ Xo.transpose(-1, -2)) < 1e-5, (b, k)
            assert rel(out["cond_to_latent"][b, k], c.to_latent) < 1e-6, (b, k)
            assert rel(out["cond_to_observed"][b, k], c.to_observed) < 1e-6, (b, k)
        for s, f in enumerate(res.posterior["filtering"]):
            assert rel(out["filter_mean"][b, s], f.mean) < 1e-6, (b, s)
            L = out["filter_chol"][b, s]
            assert rel(L @ L.transpose(-1, -2), f.cholesky @ f.cholesky.transpose(-1, -2)) < 1e-5, (b, s)


def test_blockdiag_fixed_interval_offgrid_through_the_api():
    """solve_fixed_grid with strategy_smoother_fixedinterval on a block-diagonal
    model (the posterior's filtering marginals come from the kernel), then
    offgrid_marginals (solvers.py:149-203) against the oracle's."""
    from probdiffeq_gb300 import ivpsolve, probdiffeq

    grid = np.linspace(0.0, T1, 6)
    queries = np.array([0.004, 0.013, 0.031, 0.047])
    u0 = burgers_ic(D, 7)
    vf = probdiffeq.ode("burgers", torch.tensor([NU_VISC], dtype=torch.float64))
    y0 = torch.tensor(u0, dtype=torch.float64)[None]
    tcoeffs, _ = probdiffeq.jetexpand_ode_padded_scan(num=3)(vf, (y0,), t=0.0)
    S_ = probdiffeq.state_space_model_blockdiag()
    solver = probdiffeq.solver_dynamic(strategy=probdiffeq.strategy_smoother_fixedinterval(),
                                       constraint=S_.constraint_ode_ts0(vf))
    sol = ivpsolve.solve_fixed_grid(solver=solver, precision="float64")(S_.prior_wiener_integrated(tcoeffs),
                                                                       grid=torch.tensor(grid))
    torch.cuda.synchronize()
    assert (sol.status == 0).all() and sol.posterior is not None and "filter_mean" in sol.posterior
    out = solver.offgrid_marginals(torch.tensor(queries), solution=sol)
    torch.cuda.synchronize()

    p = torch.tensor([NU_VISC], dtype=torch.float64)
    tc = problems.taylor_derivatives(problems.burgers, torch.tensor(u0), p, 3)
    So = ssm.BdSSM()
    c = So.constraint_ode_ts0(lambda u, t: problems.burgers(u[0], p))
    prior = So.prior_wiener_integrated(tc)
    res = solvers.solve_grid_save_every_point(solvers.SolverDynamic(solvers.StrategyFixedPoint(), c), prior, grid)
    o_solver = solvers.SolverDynamic(solvers.StrategyFixedInterval(), c)
    for q, t in enumerate(queries):
        o = solvers.offgrid_marginals(o_solver, float(t), res, prior)
        L = out.cholesky_flat[0, q].cpu()
        assert rel(out.mean_flat[0, q].cpu(), o.mean) < 1e-8, q
        assert rel(L @ L.transpose(-1, -2), o.cholesky @ o.cholesky.transpose(-1, -2)) < 1e-6, q
