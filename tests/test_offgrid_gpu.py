"""Off-grid marginals (solver.offgrid_marginals, solvers.py:149-203) on the GPU.

The oracle's off-grid marginals are pinned to the reference's dense-output
test (tests/test_oracle_offgrid.py).  Here the GPU solves on a grid
(``solve_fixed_grid``: every grid point a checkpoint, the fixed-interval
smoother's posterior) and its off-grid marginals are compared with the
oracle's on the same grid (``solve_grid_save_every_point``).  Float64;
tolerances: means 1e-9, covariances 1e-7 relative.
"""

import numpy as np
import pytest
import torch

from oracle import problems, solvers, ssm
from probdiffeq_gb300 import ivpsolve, probdiffeq

pytestmark = pytest.mark.gpu

LV = torch.tensor([0.5, 0.05, 0.5, 0.05], dtype=torch.float64)
STRATEGIES = {
    "filter": (solvers.StrategyFilter, solvers.StrategyFilter, probdiffeq.strategy_filter),
    "smoother": (solvers.StrategyFixedInterval, solvers.StrategyFixedPoint, probdiffeq.strategy_smoother_fixedinterval),
}
SOLVERS = {"dynamic": (solvers.SolverDynamic, probdiffeq.solver_dynamic), "mle": (solvers.SolverMLE, probdiffeq.solver_mle)}


def rel(a, b):
    a, b = torch.as_tensor(a, dtype=torch.float64), torch.as_tensor(b, dtype=torch.float64)
    return float((a - b).abs().max() / b.abs().max().clamp_min(1e-300))


def oracle_setup(kind, nu=2, y0=(20.0, 20.0)):
    tc = problems.taylor_derivatives(problems.lotka_volterra, torch.tensor(y0, dtype=torch.float64), LV, nu)
    S = ssm.IsoSSM() if kind == "isotropic" else ssm.DenseSSM()
    vf = lambda u, t: problems.lotka_volterra(u[0], LV)  # noqa: E731
    jac = lambda u, t: problems.jacobian(problems.lotka_volterra, u, LV)  # noqa: E731
    c = S.constraint_ode_ts1(vf, jac, 2) if kind == "dense" else S.constraint_ode_ts1(vf)
    return S.prior_wiener_integrated(tc), c


def gpu_solution(kind, strategy, solver_kind, grid, nu=2, y0=((20.0, 20.0),)):
    y0 = torch.tensor(y0, dtype=torch.float64)
    vf = probdiffeq.ode("lotka_volterra", LV)
    tcoeffs, _ = probdiffeq.jetexpand_ode_padded_scan(num=nu)(vf, (y0,), t=0.0)
    S_ = probdiffeq.state_space_model_isotropic() if kind == "isotropic" else probdiffeq.state_space_model_dense()
    iwp = S_.prior_wiener_integrated(tcoeffs)
    solver = SOLVERS[solver_kind][1](strategy=STRATEGIES[strategy][2](), constraint=S_.constraint_ode_ts1(vf))
    sol = ivpsolve.solve_fixed_grid(solver=solver, precision="float64")(iwp, grid=torch.as_tensor(grid))
    torch.cuda.synchronize()
    assert (sol.status == 0).all()
    return solver, sol


def covariance(kind, mean, chol):
    C = chol @ chol.T
    if kind == "isotropic":
        return mean.reshape(-1), torch.kron(C, torch.eye(2, dtype=torch.float64))
    return mean, C


def check(kind, gm, gc, o):
    mo, Co = o.to_multivariate_normal()
    m, C = covariance(kind, gm.cpu(), gc.cpu())
    assert rel(m, mo) < 1e-9, (rel(m, mo), m, mo)
    assert rel(C, Co) < 1e-7, rel(C, Co)


def oracle_grid_solution(kind, strategy, solver_kind, grid, y0=(20.0, 20.0)):
    prior, c = oracle_setup(kind, y0=y0)
    cls = SOLVERS[solver_kind][0]
    on_grid = solvers.StrategyFilter() if strategy == "filter" else solvers.StrategyFixedPoint()
    res = solvers.solve_grid_save_every_point(cls(on_grid, c), prior, grid)
    return cls(STRATEGIES[strategy][0](), c), res, prior


@pytest.mark.parametrize("solver_kind", ["dynamic", "mle"])
@pytest.mark.parametrize("strategy", ["filter", "smoother"])
@pytest.mark.parametrize("kind", ["isotropic", "dense"])
def test_offgrid_marginals_match_oracle(kind, strategy, solver_kind):
    """An adaptive step grid (the oracle's save-every-step times for
    rtol = atol = 1e-2) and queries between its points."""
    prior, c = oracle_setup(kind)
    every = solvers.solve_adaptive_save_every_step(
        SOLVERS[solver_kind][0](solvers.StrategyFilter(), c), solvers.ErrorResidualStd(c), prior, 0.0, 2.0, 1e-2, 1e-2)
    grid = np.asarray(every.t)
    rng = np.random.default_rng(0)
    k = rng.integers(1, len(grid), size=6)
    queries = grid[k - 1] + rng.uniform(0.05, 0.95, size=6) * (grid[k] - grid[k - 1])

    solver, sol = gpu_solution(kind, strategy, solver_kind, grid)
    out = solver.offgrid_marginals(torch.tensor(queries), solution=sol)
    o_solver, res, o_prior = oracle_grid_solution(kind, strategy, solver_kind, grid)
    for q, t in enumerate(queries):
        o = solvers.offgrid_marginals(o_solver, float(t), res, o_prior)
        check(kind, out.mean_flat[0, q], out.cholesky_flat[0, q], o)


@pytest.mark.parametrize("kind", ["isotropic", "dense"])
def test_offgrid_marginals_batch_grid_points_and_outside(kind):
    """Per-instance queries (B, Q); a query on a grid point returns that
    point's marginal; outside the grid's span NaN."""
    grid = torch.linspace(0.0, 2.0, 9, dtype=torch.float64)
    y0 = ((20.0, 20.0), (15.0, 25.0), (30.0, 12.0))
    solver, sol = gpu_solution(kind, "smoother", "dynamic", grid, y0=y0)
    tq = torch.tensor([[0.1, 0.75, 1.9], [0.5, 1.0, 2.5], [-0.1, 0.33, 1.75]], dtype=torch.float64)
    out = solver.offgrid_marginals(tq, solution=sol)
    torch.cuda.synchronize()
    assert out.mean_flat.shape[:2] == (3, 3)
    # grid points 1.0 (index 4) and 1.75 (index 7)
    assert torch.equal(out.mean_flat[1, 1], sol.u.mean_flat[1, 4])
    assert torch.equal(out.cholesky_flat[2, 2], sol.u.cholesky_flat[2, 7])
    assert torch.isnan(out.mean_flat[1, 2]).all() and torch.isnan(out.mean_flat[2, 0]).all()
    assert torch.isfinite(out.mean_flat[0]).all() and torch.isfinite(out.cholesky_flat[0]).all()
    # a scalar query drops the query axis and matches the batched call
    one = solver.offgrid_marginals(0.33, solution=sol)
    assert one.mean_flat.shape[0] == 3
    assert torch.equal(one.mean_flat[2], out.mean_flat[2, 1])
    # every instance against the oracle on its own initial value
    for b in range(3):
        o_solver, res, o_prior = oracle_grid_solution(kind, "smoother", "dynamic", grid, y0=y0[b])
        for q in range(3):
            t = float(tq[b, q])
            if 0.0 < t < 2.0 and not bool((grid == t).any()):
                check(kind, out.mean_flat[b, q], out.cholesky_flat[b, q], solvers.offgrid_marginals(o_solver, t, res, o_prior))


def test_offgrid_marginals_errors():
    grid = torch.linspace(0.0, 1.0, 5, dtype=torch.float64)
    y0 = torch.tensor([[20.0, 20.0]], dtype=torch.float64)
    vf = probdiffeq.ode("lotka_volterra", LV)
    tcoeffs, _ = probdiffeq.jetexpand_ode_padded_scan(num=2)(vf, (y0,), t=0.0)
    S_ = probdiffeq.state_space_model_isotropic()
    iwp = S_.prior_wiener_integrated(tcoeffs)
    fp = probdiffeq.solver_dynamic(strategy=probdiffeq.strategy_smoother_fixedpoint(), constraint=S_.constraint_ode_ts0(vf))
    with pytest.raises(NotImplementedError):
        fp.offgrid_marginals(0.3, solution=None)
    fi = probdiffeq.solver_dynamic(strategy=probdiffeq.strategy_smoother_fixedinterval(), constraint=S_.constraint_ode_ts0(vf))
    sol = ivpsolve.solve_fixed_grid(solver=fi, precision="float64")(iwp, grid=grid, posterior=False)
    with pytest.raises(ValueError, match="filtering marginals"):
        fi.offgrid_marginals(0.3, solution=sol)


@pytest.mark.parametrize("strategy", ["filter", "smoother"])
def test_blockdiag_offgrid_marginals_match_oracle(strategy):
    """Block-diagonal grid solutions (the oracle's, for two initial values,
    moved to the device) through the isotropic kernel as B * d instances of
    dimension 1, against the oracle's block-diagonal off-grid marginals."""
    from tests.test_offgrid_blockdiag_cpu import NU, Y0S, api_solution, oracle_grid

    grid = np.linspace(0.0, 2.0, 9)
    queries = np.array([0.1, 0.6, 1.3, 1.9])
    oracles = [oracle_grid(strategy, "dynamic", grid, y0) for y0 in Y0S]
    sol = api_solution([res for _, res, _ in oracles], strategy, grid)
    sol.t, sol.output_scale = sol.t.cuda(), sol.output_scale.cuda()
    sol.u = ivpsolve.Normal(sol.u.mean_flat.cuda(), sol.u.cholesky_flat.cuda(), "blockdiag")
    if sol.posterior is not None:
        sol.posterior = {k: v.cuda() for k, v in sol.posterior.items()}
    S_ = probdiffeq.state_space_model_blockdiag()
    strat = probdiffeq.strategy_filter() if strategy == "filter" else probdiffeq.strategy_smoother_fixedinterval()
    solver = probdiffeq.solver_dynamic(strategy=strat, constraint=S_.constraint_ode_ts1(probdiffeq.ode("lotka_volterra", LV)))
    out = solver.offgrid_marginals(torch.tensor(queries), solution=sol)
    torch.cuda.synchronize()
    assert tuple(out.mean_flat.shape) == (len(Y0S), len(queries), 2, NU + 1)
    for b, (o_solver, res, o_prior) in enumerate(oracles):
        for q, t in enumerate(queries):
            o = solvers.offgrid_marginals(o_solver, float(t), res, o_prior)
            L = out.cholesky_flat[b, q].cpu()
            assert rel(out.mean_flat[b, q].cpu(), o.mean) < 1e-9, (b, q)
            assert rel(L @ L.transpose(-1, -2), o.cholesky @ o.cholesky.transpose(-1, -2)) < 1e-7, (b, q)
