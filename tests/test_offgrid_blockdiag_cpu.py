"""Off-grid marginals of block-diagonal solutions, on the CPU.

A block-diagonal model is d independent one-dimensional models, one per ODE
dimension, each transitioned with its own output scale
(ssm_impl_blockdiag.py:406-432), so ``solver.offgrid_marginals`` of a
block-diagonal grid solution runs on the isotropic kernel as B * d instances
of dimension 1.  Here the native call is replaced by a host run of that
kernel (``tests/hostsim/offgrid_host.cpp``, compiled under AddressSanitizer
and UBSan), and what the public ``offgrid_marginals`` returns is compared
with the oracle's block-diagonal off-grid marginals -- pinned to the
reference's dense-output test in all three factorisations by
``tests/test_oracle_offgrid.py`` -- on the oracle's own block-diagonal grid
solutions of Lotka--Volterra (TS1, rtol = atol = 1e-2 step grid, dynamic and
MLE calibration).  Two instances with different initial values share the
grid, so a mix-up of instances or dimensions in the reshaping shows.
Tolerances as for the kernels on the GPU: means 1e-9, covariances 1e-7
relative.
"""

import numpy as np
import pytest
import torch

from oracle import problems, solvers, ssm
from probdiffeq_gb300 import _native, ivpsolve, probdiffeq
from tests import hostsim

from .test_oracle_equivalence import LV_P, lv

Y0S = ((20.0, 20.0), (10.0, 15.0))
NU = 2
ORACLE_SOLVERS = {"dynamic": solvers.SolverDynamic, "mle": solvers.SolverMLE}
API_SOLVERS = {"dynamic": probdiffeq.solver_dynamic, "mle": probdiffeq.solver_mle}
API_STRATEGIES = {"filter": probdiffeq.strategy_filter, "smoother": probdiffeq.strategy_smoother_fixedinterval}


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    return hostsim.compile_harness("offgrid_host.cpp", tmp_path_factory.mktemp("hostsim") / "offgrid_host")


def q1_iwp(nu):
    n = nu + 1
    H = np.array([[1.0 / (2 * nu + 1 - i - j) for j in range(n)] for i in range(n)])
    return np.linalg.cholesky(H)


def rel(a, b):
    a, b = np.asarray(a, dtype=float), np.asarray(b, dtype=float)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def bd_setup(y0):
    tc = problems.taylor_derivatives(problems.lotka_volterra, torch.tensor(y0, dtype=torch.float64), LV_P, NU)
    S = ssm.BdSSM()
    return S.prior_wiener_integrated(tc), S.constraint_ode_ts1(lv)


def host_offgrid(harness, workdir):
    """Stand-in for ``_native.offgrid_marginals``: the isotropic kernel's body
    run on the CPU, with the native call's argument checks for ode_dim 1."""

    def offgrid(ssm_, strategy, num_derivatives, ode_dim, t, u_mean, u_chol, output_scale, t_query,
                filter_mean=None, filter_chol=None, stream=None):
        assert ssm_ == "isotropic" and ode_dim == 1
        B, S = t.shape
        Q = t_query.shape[1]
        n = num_derivatives + 1
        assert tuple(u_mean.shape) == (B, S, n, 1) and tuple(u_chol.shape) == (B, S, n, n)
        assert tuple(output_scale.shape) == (B, S) and t_query.shape[0] == B
        parts = [t, u_mean, u_chol, output_scale, t_query]
        if strategy == "fixedinterval":
            assert tuple(filter_mean.shape) == (B, S, n, 1) and tuple(filter_chol.shape) == (B, S, n, n)
            parts += [filter_mean, filter_chol]
        flat = np.concatenate([np.asarray(p, dtype=float).reshape(-1) for p in parts] + [q1_iwp(num_derivatives).ravel()])
        head = [0, _native.OFFGRID_STRATEGY[strategy], num_derivatives, B, S, Q, 1]
        path = workdir / "input.txt"
        path.write_text(" ".join(str(v) for v in head) + " " + " ".join(repr(float(v)) for v in flat))
        lines = hostsim.run_harness(harness, path)
        vals = torch.tensor([[float(x) for x in line.split()] for line in lines], dtype=torch.float64)
        assert tuple(vals.shape) == (B * Q, n + n * n)
        return vals[:, :n].reshape(B, Q, n, 1), vals[:, n:].reshape(B, Q, n, n)

    return offgrid


def oracle_grid(strategy, solver_kind, grid, y0):
    prior, c = bd_setup(y0)
    cls = ORACLE_SOLVERS[solver_kind]
    on_grid = solvers.StrategyFilter() if strategy == "filter" else solvers.StrategyFixedPoint()
    res = solvers.solve_grid_save_every_point(cls(on_grid, c), prior, grid)
    query_strategy = solvers.StrategyFilter() if strategy == "filter" else solvers.StrategyFixedInterval()
    return cls(query_strategy, c), res, prior


def api_solution(results, strategy, grid):
    """The grid solutions as one batched ``ivpsolve.Solution`` with the
    library's block-diagonal layouts."""
    S = len(grid)

    def stack(marginals):
        return (torch.stack([torch.stack([m.mean for m in ms]) for ms in marginals]),
                torch.stack([torch.stack([m.cholesky for m in ms]) for ms in marginals]))

    marg = [r.u if strategy == "smoother" else r.posterior for r in results]
    mean, chol = stack(marg)
    scale = torch.stack([torch.stack([torch.as_tensor(r.output_scale[min(s, len(r.output_scale) - 1)])
                                      for s in range(S)]) for r in results])
    post = None
    if strategy == "smoother":
        fm, fc = stack([r.posterior["filtering"] for r in results])
        post = {"filter_mean": fm, "filter_chol": fc}
    B = len(results)
    t = torch.tensor(grid, dtype=torch.float64).expand(B, -1).contiguous()
    return ivpsolve.Solution(t=t, u=ivpsolve.Normal(mean, chol, "blockdiag"), output_scale=scale,
                             num_steps=torch.zeros((B, S), dtype=torch.int32), num_attempts=torch.zeros(B, dtype=torch.int32),
                             status=torch.zeros(B, dtype=torch.int32), posterior=post, ode_dim=2)


@pytest.mark.parametrize("solver_kind", ["dynamic", "mle"])
@pytest.mark.parametrize("strategy", ["filter", "smoother"])
def test_blockdiag_offgrid_marginals_match_oracle(harness, tmp_path, monkeypatch, strategy, solver_kind):
    prior, c = bd_setup(Y0S[0])
    every = solvers.solve_adaptive_save_every_step(
        ORACLE_SOLVERS[solver_kind](solvers.StrategyFilter(), c), solvers.ErrorResidualStd(c), prior, 0.0, 2.0,
        1e-2, 1e-2)
    grid = np.asarray(every.t)
    rng = np.random.default_rng(0)
    k = rng.integers(1, len(grid), size=6)
    queries = grid[k - 1] + rng.uniform(0.05, 0.95, size=6) * (grid[k] - grid[k - 1])
    oracles = [oracle_grid(strategy, solver_kind, grid, y0) for y0 in Y0S]
    sol = api_solution([res for _, res, _ in oracles], strategy, grid)

    monkeypatch.setattr(_native, "offgrid_marginals", host_offgrid(harness, tmp_path))
    S_ = probdiffeq.state_space_model_blockdiag()
    solver = API_SOLVERS[solver_kind](strategy=API_STRATEGIES[strategy](),
                                      constraint=S_.constraint_ode_ts1(probdiffeq.ode("lotka_volterra", LV_P)))
    out = solver.offgrid_marginals(torch.tensor(queries), solution=sol)
    assert tuple(out.mean_flat.shape) == (len(Y0S), len(queries), 2, NU + 1)
    assert tuple(out.cholesky_flat.shape) == (len(Y0S), len(queries), 2, NU + 1, NU + 1)
    for b, (o_solver, res, o_prior) in enumerate(oracles):
        for q, t in enumerate(queries):
            o = solvers.offgrid_marginals(o_solver, float(t), res, o_prior)
            L = out.cholesky_flat[b, q]
            assert rel(out.mean_flat[b, q], o.mean) < 1e-9, (b, q)
            assert rel(L @ L.transpose(-1, -2), o.cholesky @ o.cholesky.transpose(-1, -2)) < 1e-7, (b, q)

    one = solver.offgrid_marginals(float(queries[0]), solution=sol)  # a scalar query: no query axis
    assert torch.equal(one.mean_flat, out.mean_flat[:, 0])


def test_blockdiag_offgrid_checks_the_output_scale_shape():
    """An output scale without the per-dimension axis is rejected
    (ssm_impl_blockdiag.py:412-418 raises on the wrong shape)."""
    grid = np.linspace(0.0, 1.0, 4)
    _, res, _ = oracle_grid("filter", "dynamic", grid, Y0S[0])
    sol = api_solution([res], "filter", grid)
    sol.output_scale = sol.output_scale[..., 0]
    S_ = probdiffeq.state_space_model_blockdiag()
    solver = probdiffeq.solver_dynamic(strategy=probdiffeq.strategy_filter(),
                                       constraint=S_.constraint_ode_ts1(probdiffeq.ode("lotka_volterra", LV_P)))
    with pytest.raises(ValueError, match="wrong shape"):
        solver.offgrid_marginals(0.5, solution=sol)


def test_blockdiag_offgrid_per_instance_queries(harness, tmp_path, monkeypatch):
    """(B, Q) query times that differ between instances, on a uniform grid:
    each instance's dimensions see that instance's queries."""
    grid = np.linspace(0.0, 2.0, 9)
    tq = torch.tensor([[0.1, 0.6, 1.9], [0.4, 1.1, 1.6]], dtype=torch.float64)
    oracles = [oracle_grid("filter", "mle", grid, y0) for y0 in Y0S]
    sol = api_solution([res for _, res, _ in oracles], "filter", grid)
    monkeypatch.setattr(_native, "offgrid_marginals", host_offgrid(harness, tmp_path))
    S_ = probdiffeq.state_space_model_blockdiag()
    solver = probdiffeq.solver_mle(strategy=probdiffeq.strategy_filter(),
                                   constraint=S_.constraint_ode_ts1(probdiffeq.ode("lotka_volterra", LV_P)))
    out = solver.offgrid_marginals(tq, solution=sol)
    for b, (o_solver, res, o_prior) in enumerate(oracles):
        for q in range(tq.shape[1]):
            o = solvers.offgrid_marginals(o_solver, float(tq[b, q]), res, o_prior)
            L = out.cholesky_flat[b, q]
            assert rel(out.mean_flat[b, q], o.mean) < 1e-9, (b, q)
            assert rel(L @ L.transpose(-1, -2), o.cholesky @ o.cholesky.transpose(-1, -2)) < 1e-7, (b, q)
