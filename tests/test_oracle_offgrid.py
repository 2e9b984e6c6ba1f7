"""Pin the oracle's off-grid marginals to the reference's dense-output test.

tests/test_probdiffeq/test_dense_output/test_offgrid_marginals_vs_solve_and_save_at.py:48-87:
the off-grid marginals of a save-every-step solution (filter, or the
fixed-interval smoother) equal the save_at solution (filter, or the
fixed-point smoother) at the same points -- LV on [0, 2], two derivatives,
TS1, dynamic calibration, rtol = atol = 1e-2, all three factorisations.
"""

import numpy as np
import pytest
import torch

from oracle import problems, solvers, ssm

from .test_oracle_equivalence import LV_P, allclose, lv, lv_jac, make_ssm

STRATEGIES = {
    "filter": (solvers.StrategyFilter, solvers.StrategyFilter),
    "smoother": (solvers.StrategyFixedInterval, solvers.StrategyFixedPoint),
}


def ts1(S, kind):
    return S.constraint_ode_ts1(lv, lv_jac, 2) if kind == "dense" else S.constraint_ode_ts1(lv)


def covariance(rv):
    m, C = rv.to_multivariate_normal()
    return m, C


@pytest.mark.parametrize("strategy", ["filter", "smoother"])
@pytest.mark.parametrize("kind", ["isotropic", "blockdiag", "dense"])
def test_offgrid_marginals_match_save_at(kind, strategy):
    tc = problems.taylor_derivatives(problems.lotka_volterra, torch.tensor([20.0, 20.0]), LV_P, 2)
    S = make_ssm(kind)
    prior = S.prior_wiener_integrated(tc)
    c = ts1(S, kind)
    error = solvers.ErrorResidualStd(c)
    every_step, save_at = STRATEGIES[strategy]
    ts = np.linspace(0.0, 2.0, 5)

    solver = solvers.SolverDynamic(every_step(), c)
    every = solvers.solve_adaptive_save_every_step(solver, error, prior, 0.0, 2.0, 1e-2, 1e-2)
    interpolated = [solvers.offgrid_marginals(solver, float(t), every, prior) for t in ts[1:-1]]

    sa = solvers.solve_adaptive_save_at(solvers.SolverDynamic(save_at(), c), error, prior, ts, 1e-2, 1e-2)
    for a, b in zip(interpolated, sa.u[1:-1]):
        m1, C1 = covariance(a)
        m2, C2 = covariance(b)
        assert allclose(m1, m2)
        assert allclose(C1, C2)


def test_offgrid_marginals_reject_the_fixed_point_smoother():
    """solvers.py:163-164: only strategies suitable for off-grid marginals."""
    tc = problems.taylor_derivatives(problems.lotka_volterra, torch.tensor([20.0, 20.0]), LV_P, 2)
    S = ssm.IsoSSM()
    prior = S.prior_wiener_integrated(tc)
    c = S.constraint_ode_ts0(lv)
    solver = solvers.SolverDynamic(solvers.StrategyFixedPoint(), c)
    res = solvers.solve_adaptive_save_at(solver, solvers.ErrorResidualStd(c), prior, np.linspace(0.0, 1.0, 3), 1e-2, 1e-2)
    with pytest.raises(NotImplementedError):
        solvers.offgrid_marginals(solver, 0.3, res, prior)
