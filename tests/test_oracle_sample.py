"""The oracle's MarkovSequence.sample (oracle/markov.py) on the CPU.

The reference's test (tests/test_probdiffeq/test_sample.py) solves
Lotka--Volterra with the fixed-point smoother (nu = 2, 12 save points,
atol = rtol = 1e-2) in the three factorisations and checks the sample
shapes; here the same solve through the oracle, the shapes, and that the
samples reproduce the smoothed marginals (3000 draws: every Taylor
coefficient's sample mean within 5 standard errors, its std within 10 %).
"""

import math

import pytest
import torch

from oracle import markov, problems, solvers, ssm

LV = torch.tensor([0.5, 0.05, 0.5, 0.05], dtype=torch.float64)
Y0 = torch.tensor([20.0, 20.0], dtype=torch.float64)


def _smoother_solution(kind):
    tc = problems.taylor_derivatives(problems.lotka_volterra, Y0, LV, 2)
    S = {"isotropic": ssm.IsoSSM, "blockdiag": ssm.BdSSM, "dense": ssm.DenseSSM}[kind]()
    vf = lambda u, t: problems.lotka_volterra(u[0], LV)  # noqa: E731
    c = S.constraint_ode_ts0(vf, 2) if kind == "dense" else S.constraint_ode_ts0(vf)
    save_at = torch.linspace(0.0, 2.0, 12, dtype=torch.float64).tolist()
    return solvers.solve_adaptive_save_at(solvers.SolverPlain(solvers.StrategyFixedPoint(), c),
                                          solvers.ErrorResidualStd(c), S.prior_wiener_integrated(tc), save_at,
                                          1e-2, 1e-2)


def _base_shape(normal):
    if isinstance(normal, ssm.IsoNormal):
        return (normal.cholesky.shape[0],)
    if isinstance(normal, ssm.BdNormal):
        return tuple(normal.mean.shape)
    return (normal.mean.shape[0],)


@pytest.mark.parametrize("kind", ["isotropic", "blockdiag", "dense"])
def test_oracle_samples_have_the_state_shape_and_the_smoothed_marginals(kind):
    res = _smoother_solution(kind)
    conds = res.posterior["conditionals"]
    marginal = res.u[-1]
    S = len(conds) + 1
    g = torch.Generator().manual_seed(0)
    K = 3000
    draws = []
    for _ in range(K):
        z = [torch.randn(_base_shape(marginal), dtype=torch.float64, generator=g) for _ in range(S)]
        draws.append(torch.stack(markov.sample_backward(marginal, conds, z)))
    smp = torch.stack(draws)  # (K, S, *state)
    assert tuple(smp.shape[2:]) == tuple(res.u[0].mean.shape)
    for s in range(S):
        m, L = res.u[s].mean, res.u[s].cholesky
        var = torch.diagonal(L @ L.transpose(-1, -2), dim1=-2, dim2=-1)
        sd = torch.sqrt(var)
        if kind == "isotropic":
            sd = sd[:, None].expand_as(m)
        ok = sd > 1e-9 * m.abs().max()
        emp_m, emp_sd = smp[:, s].mean(0), smp[:, s].std(0)
        if not bool(ok.any()):  # an exact marginal (the initial point): every draw is its mean
            assert float((smp[:, s] - m).abs().max()) <= 1e-9 * float(m.abs().max()), s
            continue
        zs = ((emp_m - m).abs() / (sd / math.sqrt(K)))[ok]
        assert float(zs.max()) < 5.0, (s, float(zs.max()))
        assert float(((emp_sd - sd).abs() / sd)[ok].max()) < 0.1, s
