"""The off-grid marginal kernels run on the CPU against the oracle.

``tests/hostsim/offgrid_host.cpp`` compiles ``offgrid_kernels.cuh`` with
the host compiler under AddressSanitizer and UBSan.  Its inputs are the
oracle's own grid solution (an adaptive save-every-step grid of
Lotka--Volterra at rtol = atol = 1e-2, TS1, dynamic and MLE calibration),
so the comparison with the oracle's ``offgrid_marginals`` isolates the
kernel's arithmetic: means within 1e-9, covariances within 1e-7 relative
(the GPU test's tolerances), for the filter and the fixed-interval
smoother in the isotropic and dense factorisations.
"""

import numpy as np
import pytest

from oracle import solvers
from tests import hostsim
from tests.test_offgrid_gpu import SOLVERS, oracle_grid_solution, oracle_setup


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


@pytest.mark.parametrize("solver_kind", ["dynamic", "mle"])
@pytest.mark.parametrize("strategy", ["filter", "smoother"])
@pytest.mark.parametrize("kind", ["isotropic", "dense"])
def test_host_offgrid_kernels_match_oracle(harness, tmp_path, kind, strategy, solver_kind):
    prior, c = oracle_setup(kind)
    every = solvers.solve_adaptive_save_every_step(
        SOLVERS[solver_kind][0](solvers.StrategyFilter(), c), solvers.ErrorResidualStd(c), prior, 0.0, 2.0, 1e-2, 1e-2)
    grid = np.asarray(every.t)
    rng = np.random.default_rng(0)
    k = rng.integers(1, len(grid), size=6)
    queries = grid[k - 1] + rng.uniform(0.05, 0.95, size=6) * (grid[k] - grid[k - 1])
    o_solver, res, o_prior = oracle_grid_solution(kind, strategy, solver_kind, grid)
    S, Q, nu = len(grid), len(queries), 2
    marg = res.u if strategy == "smoother" else res.posterior
    u_mean = np.concatenate([m.mean.reshape(-1).numpy() for m in marg])
    u_chol = np.concatenate([m.cholesky.reshape(-1).numpy() for m in marg])
    scales = [float(res.output_scale[min(s, len(res.output_scale) - 1)]) for s in range(S)]
    parts = [grid, u_mean, u_chol, scales, queries]
    if strategy == "smoother":
        filt = res.posterior["filtering"]
        parts += [np.concatenate([m.mean.reshape(-1).numpy() for m in filt]),
                  np.concatenate([m.cholesky.reshape(-1).numpy() for m in filt])]
    parts.append(q1_iwp(nu).ravel())
    head = [0 if kind == "isotropic" else 2, 0 if strategy == "filter" else 2, nu, 1, S, Q, 2]
    path = tmp_path / "input.txt"
    path.write_text(" ".join(str(v) for v in head) + " " + " ".join(repr(float(v)) for v in np.concatenate(parts)))
    lines = hostsim.run_harness(harness, path)
    assert len(lines) == Q
    n, d = nu + 1, 2
    for q, t in enumerate(queries):
        vals = np.array([float(x) for x in lines[q].split()])
        o = solvers.offgrid_marginals(o_solver, float(t), res, o_prior)
        mo, Co = o.to_multivariate_normal()
        if kind == "isotropic":
            m = vals[:n * d]
            L = vals[n * d:].reshape(n, n)
            C = np.kron(L @ L.T, np.eye(d))
        else:
            N = n * d
            m = vals[:N]
            L = vals[N:].reshape(N, N)
            C = L @ L.T
        assert rel(m, mo.numpy()) < 1e-9, (q, rel(m, mo.numpy()))
        assert rel(C, Co.numpy()) < 1e-7, (q, rel(C, Co.numpy()))
