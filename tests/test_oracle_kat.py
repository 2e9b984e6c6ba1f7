"""Pin the oracle to the reference's own known-answer tests.

Each test restates a reference test (cited) against the oracle.  Tolerances
follow ``probdiffeq/backend/testing.py:54-111``: atol = sqrt(eps),
rtol = 10 sqrt(eps) of the dtype (float64 here).
"""

import math

import numpy as np
import pytest
import torch

from oracle import linalg, problems, solvers, ssm

TOL = math.sqrt(np.finfo(np.float64).eps)


def allclose(a, b, atol=TOL, rtol=10 * TOL):
    a, b = torch.as_tensor(a, dtype=torch.float64), torch.as_tensor(b, dtype=torch.float64)
    assert a.shape == b.shape, (a.shape, b.shape)
    return bool(torch.allclose(a, b, atol=atol, rtol=rtol))


def _A_Q_expected(dt):
    A = torch.tensor(
        [[1.0, dt, dt**2 / 2.0, dt**3 / 6.0], [0.0, 1.0, dt, dt**2 / 2.0], [0.0, 0.0, 1.0, dt], [0.0, 0.0, 0.0, 1.0]]
    )
    h = abs(dt)
    Q = torch.tensor(
        [
            [h**7 / 252.0, h**6 / 72.0, h**5 / 30.0, h**4 / 24.0],
            [h**6 / 72.0, h**5 / 20.0, h**4 / 8.0, h**3 / 6.0],
            [h**5 / 30.0, h**4 / 8.0, h**3 / 3.0, h**2 / 2.0],
            [h**4 / 24.0, h**3 / 6.0, h**2 / 2.0, h**1 / 1.0],
        ]
    )
    return A, Q


@pytest.mark.parametrize("factory", ["isotropic", "dense"])
@pytest.mark.parametrize("dt", [1.234, -1.234])
def test_iwp_transitions_1d(factory, dt):
    """tests/test_probdiffeq/test_priors/test_wiener_integrated.py:12-43."""
    tc = torch.tensor([2.0, 3.0, 4.0, 5.0])[:, None]
    S = ssm.IsoSSM() if factory == "isotropic" else ssm.DenseSSM()
    cond = S.prior_wiener_integrated(tc).transition(dt, 1.0).preconditioner_apply()
    A_exp, Q_exp = _A_Q_expected(dt)
    assert allclose(cond.A, A_exp)
    q, Q = cond.noise.to_multivariate_normal()
    assert allclose(q, torch.zeros(4))
    assert allclose(Q, Q_exp)


@pytest.mark.parametrize("dt", [1.234, -1.234])
def test_iwp_transitions_1d_blockdiag(dt):
    """tests/test_probdiffeq/test_priors/test_wiener_integrated.py:47-81."""
    tc = torch.tensor([2.0, 3.0, 4.0, 5.0])[:, None]
    cond = ssm.BdSSM().prior_wiener_integrated(tc).transition(dt, torch.ones(1)).preconditioner_apply()
    A_exp, Q_exp = _A_Q_expected(dt)
    assert allclose(cond.A, A_exp[None])
    q, Q = cond.noise.to_multivariate_normal()
    assert allclose(q, torch.zeros(4))
    assert allclose(Q, Q_exp)


@pytest.mark.parametrize("factory", ["isotropic", "dense", "blockdiag"])
def test_output_scale_covariances(factory):
    """tests/test_probdiffeq/test_priors/test_output_scales.py:93-123 (default and custom scale)."""
    tc = torch.ones((2, 1))
    Q_exp = 1.0 / torch.tensor([[3.0, 2.0], [2.0, 1.0]])
    if factory == "isotropic":
        prior = ssm.IsoSSM().prior_wiener_integrated(tc, output_scale=123.45)
        cond = prior.transition(1.0, 9.876)
    elif factory == "blockdiag":
        prior = ssm.BdSSM().prior_wiener_integrated(tc, output_scale=123.45 * torch.ones(1))
        cond = prior.transition(1.0, 9.876 * torch.ones(1))
    else:
        prior = ssm.DenseSSM().prior_wiener_integrated(tc)
        prior.Q = prior.Q * 123.45
        cond = prior.transition(1.0, 9.876)
    _, cov = cond.noise.to_multivariate_normal()
    assert allclose(cov, (9.876 * 123.45) ** 2 * Q_exp)


def _some_array(shape, seed):
    g = torch.Generator().manual_seed(seed)
    return torch.randn(shape, generator=g, dtype=torch.float64)


@pytest.mark.parametrize("HCshape, Cshape, Xshape", [((4, 3), (3, 3), (4, 4)), ((2, 3), (3, 3), (2, 2))])
@pytest.mark.parametrize("solve", ["triu", "lstsq"])
def test_revert_conditional(HCshape, Cshape, Xshape, solve):
    """tests/test_util/test_cholesky_util.py:9-33: revert vs explicit Kalman S, K, C1."""
    HC = _some_array(HCshape, 1) + 1.0
    C = _some_array(Cshape, 2) + 2.0
    X = _some_array(Xshape, 3) + 3.0 + torch.eye(Xshape[0])
    S = HC @ HC.T + X @ X.T
    K = C @ HC.T @ torch.linalg.inv(S)
    C1 = C @ C.T - K @ S @ K.T
    st = linalg.solve_triu if solve == "triu" else linalg.lstsq_svd
    extra, (bw, g) = ssm.revert_conditional(HC.T, C.T, X.T, st)
    assert allclose(extra.T @ extra, S)
    assert allclose(g, K)
    assert allclose(bw.T @ bw, C1)


def test_revert_conditional_gradient_finite_at_zero():
    """tests/test_util/test_cholesky_util.py:41-58: no NaN in jacrev at zero covariance."""
    C = torch.zeros((3, 3), requires_grad=True)
    HC = torch.zeros((2, 3), requires_grad=True)
    X = (_some_array((2, 2), 4) + 3.0 + torch.eye(2)).requires_grad_(True)
    extra, (bw, g) = ssm.revert_conditional(HC.T, C.T, X.T, linalg.solve_triu)
    (extra.sum() + bw.sum() + g.sum()).backward()
    for t in (C, HC, X):
        assert torch.isfinite(t.grad).all()


def _random_variable(factory):
    """tests/test_probdiffeq/test_logpdf.py:56-74 (IWP noise with random values)."""
    tc = torch.ones((5, 3))
    std = torch.ones(5) if factory == "isotropic" else torch.ones((5, 3))
    if factory == "isotropic":
        prior = ssm.IsoSSM().prior_wiener_integrated(tc, std=std)
        rv = prior.transition(0.1, 1.0).noise
        g = torch.Generator().manual_seed(1)
        return ssm.IsoNormal(torch.randn(rv.mean.shape, generator=g), torch.randn(rv.cholesky.shape, generator=g))
    if factory == "blockdiag":
        prior = ssm.BdSSM().prior_wiener_integrated(tc, std=std)
        rv = prior.transition(0.1, torch.ones(3)).noise
        g = torch.Generator().manual_seed(1)
        return ssm.BdNormal(torch.randn(rv.mean.shape, generator=g), torch.randn(rv.cholesky.shape, generator=g))
    prior = ssm.DenseSSM().prior_wiener_integrated(tc, std=std)
    rv = prior.transition(0.1, 1.0).noise
    g = torch.Generator().manual_seed(1)
    return ssm.DenseNormal(torch.randn(rv.mean.shape, generator=g), torch.randn(rv.cholesky.shape, generator=g), 3)


@pytest.mark.parametrize("factory", ["isotropic", "dense", "blockdiag"])
def test_logpdf_matches_multivariate_normal(factory):
    """tests/test_probdiffeq/test_logpdf.py:9-29."""
    from scipy.stats import multivariate_normal

    rv = _random_variable(factory)
    mean, cov = rv.to_multivariate_normal()
    pdf1 = rv.logpdf(torch.ones_like(rv.mean))
    pdf2 = multivariate_normal.logpdf(np.ones(mean.shape[0]), mean.numpy(), cov.numpy())
    assert allclose(pdf1, pdf2)


def test_controllers_pi_equivalent_to_i():
    """tests/test_ivpsolve/test_controllers.py:7-26."""
    pi = solvers.ControlPI(exponent_integral=1.0, exponent_proportional=0.0)
    ic = solvers.ControlIntegral()
    dt, x = 0.1428, pi.init(0.1428)
    for _ in range(4):
        dt, x = pi.apply(dt, x, 3.142)
    dt2, y = 0.1428, ic.init(0.1428)
    for _ in range(4):
        dt2, y = ic.apply(dt2, y, 3.142)
    assert allclose(dt, dt2)


def test_taylor_init_lotka_volterra_closed_form():
    """Taylor-mode derivatives (jet_expansion_algorithms.py:49-103) against hand-derived ones."""
    a, b, c, d = 0.5, 0.05, 0.5, 0.05
    p = torch.tensor([a, b, c, d])
    y = torch.tensor([20.0, 20.0])
    tc = problems.taylor_derivatives(problems.lotka_volterra, y, p, 2)
    f = lambda y: torch.stack([a * y[0] - b * y[0] * y[1], -c * y[1] + d * y[0] * y[1]])
    J = torch.func.jacfwd(f)(y)
    assert allclose(tc[0], y)
    assert allclose(tc[1], f(y))
    assert allclose(tc[2], J @ f(y))
    # third derivative: u''' = J u'' + f''(u', u')
    tc3 = problems.taylor_derivatives(problems.lotka_volterra, y, p, 3)
    H = torch.func.jacfwd(torch.func.jacfwd(f))(y)
    u1, u2 = f(y), J @ f(y)
    assert allclose(tc3[3], J @ u2 + torch.einsum("ijk,j,k->i", H, u1, u1))


def test_cholesky_hilbert_and_system_matrices():
    """util/cholesky_util.py:106-176 and _probdiffeq/utilities.py:57-71."""
    for n in range(1, 7):
        L = ssm.cholesky_hilbert(n)
        Hm = torch.tensor([[1.0 / (i + j + 1) for j in range(n)] for i in range(n)])
        assert allclose(L @ L.T, Hm)
        A, Q = ssm.system_matrices_1d_iwp(n - 1)
        fH = torch.flip(Hm, dims=(0, 1))
        assert allclose(Q @ Q.T, fH)
        assert bool((torch.diagonal(Q) >= 0).all())
        assert allclose(torch.triu(Q, 1), torch.zeros((n, n)))
