"""Pin the oracle to the reference's equivalence and accuracy tests.

Each test restates a reference test (cited).  Tolerances follow
``probdiffeq/backend/testing.py:83-111`` unless the reference test states
its own.
"""

import math

import numpy as np
import pytest
import scipy.integrate
import torch

from oracle import problems, solvers, ssm

TOL = math.sqrt(np.finfo(np.float64).eps)
LV_P = torch.tensor([0.5, 0.05, 0.5, 0.05])


def allclose(a, b, atol=TOL, rtol=10 * TOL):
    a, b = torch.as_tensor(a, dtype=torch.float64), torch.as_tensor(b, dtype=torch.float64)
    assert a.shape == b.shape, (a.shape, b.shape)
    return bool(torch.allclose(a, b, atol=atol, rtol=rtol))


def lv(u, t):
    return problems.lotka_volterra(u[0], LV_P)


def lv_jac(u, t):
    return problems.jacobian(problems.lotka_volterra, u, LV_P)


def make_ssm(kind):
    return {"isotropic": ssm.IsoSSM, "blockdiag": ssm.BdSSM, "dense": ssm.DenseSSM}[kind]()


def ts0(S, kind, vf=lv, d=2):
    return S.constraint_ode_ts0(vf, d) if kind == "dense" else S.constraint_ode_ts0(vf)


def lv_reference(t1, y0=(20.0, 20.0)):
    f = lambda t, y: [0.5 * y[0] - 0.05 * y[0] * y[1], -0.5 * y[1] + 0.05 * y[0] * y[1]]
    return scipy.integrate.solve_ivp(f, (0.0, t1), list(y0), method="DOP853", rtol=1e-13, atol=1e-13).y[:, -1]


@pytest.mark.parametrize("kind", ["isotropic", "blockdiag", "dense"])
def test_terminal_values_match_reference_solver(kind):
    """tests/test_ivpsolve/test_solve_adaptive_terminal_values.py:15-51 (LV on [0, 2])."""
    tc = problems.taylor_derivatives(problems.lotka_volterra, torch.tensor([20.0, 20.0]), LV_P, 4)
    S = make_ssm(kind)
    prior = S.prior_wiener_integrated(tc)
    c = ts0(S, kind)
    solver = solvers.SolverDynamic(solvers.StrategyFixedPoint(), c)
    res = solvers.solve_adaptive_terminal_values(solver, solvers.ErrorResidualStd(c), prior, 0.0, 2.0, 1e-3, 1e-3)
    u = solvers.coeff(res.u[-1], 0)
    # the reference runs in float32: allclose tolerances are sqrt(eps32)
    tol32 = math.sqrt(np.finfo(np.float32).eps)
    assert allclose(u, lv_reference(2.0), atol=tol32, rtol=10 * tol32)
    assert abs(res.t[-1] - 2.0) < 1e-12


@pytest.mark.parametrize("kind", ["isotropic", "blockdiag", "dense"])
def test_fixed_grid_matches_adaptive_grid(kind):
    """tests/test_ivpsolve/test_solve_fixed_grid.py:17-54."""
    tc = problems.taylor_derivatives(problems.lotka_volterra, torch.tensor([20.0, 20.0]), LV_P, 2)
    S = make_ssm(kind)
    prior = S.prior_wiener_integrated(tc)
    c = ts0(S, kind)
    solver = solvers.SolverMLE(solvers.StrategyFilter(), c)
    ad = solvers.solve_adaptive_save_every_step(solver, solvers.ErrorResidualStd(c), prior, 0.0, 2.0, 1e-2, 1e-2, clip_dt=True)
    grid, u, _, scales, steps = solvers.solve_fixed_grid(solver, prior, ad.t)
    assert len(u) == len(ad.u)
    for a, b in zip(u, ad.u):
        assert allclose(a.mean, b.mean)
        assert allclose(a.cholesky @ a.cholesky.transpose(-1, -2), b.cholesky @ b.cholesky.transpose(-1, -2))
    assert steps == ad.num_steps


@pytest.mark.parametrize("kind", ["isotropic", "blockdiag", "dense"])
def test_fixedpoint_equals_fixedinterval_on_same_grid(kind):
    """tests/test_probdiffeq/test_strategies/test_smoother_fixedinterval_vs_fixedpoint.py:50-86."""
    tc = problems.taylor_derivatives(problems.lotka_volterra, torch.tensor([20.0, 20.0]), LV_P, 2)
    S = make_ssm(kind)
    prior = S.prior_wiener_integrated(tc)
    c = ts0(S, kind)
    err = solvers.ErrorResidualStd(c)
    sm = solvers.solve_adaptive_save_every_step(
        solvers.SolverPlain(solvers.StrategyFixedInterval(), c), err, prior, 0.0, 2.0, 1e-3, 1e-3, dt0=0.1
    )
    fp = solvers.solve_adaptive_save_at(
        solvers.SolverPlain(solvers.StrategyFixedPoint(), c), err, prior, sm.t, 1e-3, 1e-3, dt0=0.1
    )
    assert allclose(torch.tensor(fp.t), torch.tensor(sm.t))
    assert fp.num_steps == sm.num_steps
    for a, b in zip(fp.u, sm.u):
        assert allclose(a.mean, b.mean)
        assert allclose(a.cholesky @ a.cholesky.transpose(-1, -2), b.cholesky @ b.cholesky.transpose(-1, -2))
    # backward conditionals implement the same transitions after preconditioner_apply
    for c1, c2 in zip(fp.posterior["conditionals"], sm.posterior["conditionals"]):
        p1, p2 = c1.preconditioner_apply(), c2.preconditioner_apply()
        assert allclose(p1.A, p2.A)
        assert allclose(p1.noise.mean, p2.noise.mean)
        n1, n2 = p1.noise.cholesky, p2.noise.cholesky
        assert allclose(n1 @ n1.transpose(-1, -2), n2 @ n2.transpose(-1, -2))


@pytest.mark.parametrize("strategy", [solvers.StrategyFilter, solvers.StrategyFixedInterval, solvers.StrategyFixedPoint])
def test_mle_changes_scale_not_mean(strategy):
    """tests/test_probdiffeq/test_calibration/test_mle.py:94-110."""
    tc = problems.taylor_derivatives(problems.lotka_volterra, torch.tensor([20.0, 20.0]), LV_P, 2)
    S = ssm.IsoSSM()
    prior = S.prior_wiener_integrated(tc, std=1e-6 * torch.ones(3))
    c = S.constraint_ode_ts0(lv)
    out = []
    for Sv in (solvers.SolverPlain, solvers.SolverMLE):
        s = Sv(strategy(), c)
        out.append(solvers.solve_adaptive_terminal_values(s, solvers.ErrorResidualStd(c), prior, 0.0, 2.0, 1e-2, 1e-2))
    un, mle = out
    assert not allclose(un.output_scale[-1], mle.output_scale[-1])
    assert not allclose(un.u[-1].std(), mle.u[-1].std())
    assert allclose(solvers.coeff(un.u[-1], 0), solvers.coeff(mle.u[-1], 0), rtol=1e-3)


def test_dense_equals_isotropic_on_isotropic_ode():
    """tests/test_probdiffeq/test_calibration/test_dynamic_across_factorisations.py:10-64.

    TS0 variant (isotropic TS1 via Jacobian traces is not part of this path):
    for an isotropic vector field the dense (kron-structured) and isotropic
    solvers with dynamic calibration must agree.
    """
    g = torch.Generator().manual_seed(1)
    scalar = torch.randn((), generator=g)
    u0 = torch.randn(5, generator=g)

    def vf(u, t):
        return scalar * u[0] + t

    tc = torch.stack([u0, scalar * u0, scalar * scalar * u0 + 1.0])  # u, u', u'' at t=0
    ts = np.linspace(0.0, 10.0, 7)
    outs = []
    for S in (ssm.DenseSSM(), ssm.IsoSSM()):
        prior = S.prior_wiener_integrated(tc)
        c = S.constraint_ode_ts0(vf, 5) if isinstance(S, ssm.DenseSSM) else S.constraint_ode_ts0(vf)
        solver = solvers.SolverDynamic(solvers.StrategyFixedPoint(), c)
        res = solvers.solve_adaptive_save_at(solver, solvers.ErrorStateStd(c), prior, ts, 1e-1, 1e-1)
        outs.append(res)
    dn, iso = outs
    for a, b in zip(dn.u, iso.u):
        ma, Ca = a.to_multivariate_normal()
        mb, Cb = b.to_multivariate_normal()
        # dense is coefficient-major (u, u', ...), isotropic is (n, d) -> same order
        assert allclose(ma, mb)
        assert allclose(Ca, Cb)
    for sa, sb in zip(dn.output_scale, iso.output_scale):
        assert allclose(sa, sb)


def test_blockdiag_equals_per_dimension_dense_on_diagonal_ode():
    """tests/test_probdiffeq/test_calibration/test_dynamic_across_factorisations.py:67-145.

    On a diagonal ODE with a fixed grid, the block-diagonal solver equals d
    independent one-dimensional dense solvers.
    """
    g = torch.Generator().manual_seed(2)
    lam = -torch.rand(3, generator=g)
    u0 = torch.randn(3, generator=g)
    grid = np.linspace(0.0, 1.0, 6)
    tc = torch.stack([u0, lam * u0, lam * lam * u0])
    S = ssm.BdSSM()
    c = S.constraint_ode_ts0(lambda u, t: lam * u[0])
    _, ubd, _, _, _ = solvers.solve_fixed_grid(solvers.SolverDynamic(solvers.StrategyFilter(), c), S.prior_wiener_integrated(tc), grid)
    for j in range(3):
        D = ssm.DenseSSM()
        cj = D.constraint_ode_ts0(lambda u, t, j=j: lam[j] * u[0], 1)
        _, ud, _, _, _ = solvers.solve_fixed_grid(
            solvers.SolverDynamic(solvers.StrategyFilter(), cj), D.prior_wiener_integrated(tc[:, j : j + 1]), grid
        )
        for a, b in zip(ubd, ud):
            assert allclose(a.mean[j], b.mean)
            assert allclose(a.cholesky[j] @ a.cholesky[j].T, b.cholesky @ b.cholesky.T)


def test_dense_ts1_equals_isotropic_ts1_on_isotropic_ode():
    """tests/test_probdiffeq/test_calibration/test_dynamic_across_factorisations.py:10-64 with TS1.

    For an isotropic field f(u) = s u + t the dense TS1 operator is
    [-s I, I, 0] and the isotropic one, the Jacobian trace along d divided by
    d (ssm_impl_isotropic.py:320-355), is [-s, 1, 0]: the solvers agree.
    """
    g = torch.Generator().manual_seed(1)
    scalar = torch.randn((), generator=g)
    u0 = torch.randn(5, generator=g)

    def vf(u, t):
        return scalar * u[0] + t

    tc = torch.stack([u0, scalar * u0, scalar * scalar * u0 + 1.0])
    ts = np.linspace(0.0, 10.0, 7)
    outs = []
    for S in (ssm.DenseSSM(), ssm.IsoSSM()):
        prior = S.prior_wiener_integrated(tc)
        if isinstance(S, ssm.DenseSSM):
            c = S.constraint_ode_ts1(vf, lambda u, t: scalar * torch.eye(5, dtype=u.dtype), 5)
        else:
            c = S.constraint_ode_ts1(vf)
        solver = solvers.SolverDynamic(solvers.StrategyFixedPoint(), c)
        outs.append(solvers.solve_adaptive_save_at(solver, solvers.ErrorResidualStd(c), prior, ts, 1e-3, 1e-3))
    dn, iso = outs
    assert dn.num_steps == iso.num_steps
    for a, b in zip(dn.u, iso.u):
        ma, Ca = a.to_multivariate_normal()
        mb, Cb = b.to_multivariate_normal()
        assert allclose(ma, mb)
        assert allclose(Ca, Cb)


def test_blockdiag_ts1_equals_per_dimension_dense_ts1_on_diagonal_ode():
    """tests/test_probdiffeq/test_calibration/test_dynamic_across_factorisations.py:67-145 (TS1, fixed grid).

    The block-diagonal TS1 operators are the Jacobian's diagonal along d
    (ssm_impl_blockdiag.py:147-183); on a diagonal field they equal the d
    one-dimensional dense TS1 operators.
    """
    g = torch.Generator().manual_seed(2)
    lam = -torch.rand(3, generator=g)
    u0 = torch.randn(3, generator=g)
    grid = np.linspace(0.0, 1.0, 6)
    tc = torch.stack([u0, lam * u0, lam * lam * u0])
    S = ssm.BdSSM()
    c = S.constraint_ode_ts1(lambda u, t: lam * u[0] + t)
    _, ubd, _, _, _ = solvers.solve_fixed_grid(solvers.SolverDynamic(solvers.StrategyFilter(), c), S.prior_wiener_integrated(tc), grid)
    for j in range(3):
        D = ssm.DenseSSM()
        cj = D.constraint_ode_ts1(lambda u, t, j=j: lam[j] * u[0] + t, lambda u, t, j=j: lam[j].reshape(1, 1).to(u.dtype), 1)
        _, ud, _, _, _ = solvers.solve_fixed_grid(
            solvers.SolverDynamic(solvers.StrategyFilter(), cj), D.prior_wiener_integrated(tc[:, j : j + 1]), grid
        )
        for a, b in zip(ubd, ud):
            assert allclose(a.mean[j], b.mean)
            assert allclose(a.cholesky[j] @ a.cholesky[j].T, b.cholesky @ b.cholesky.T)


def test_ts1_differs_from_ts0_only_through_the_jacobian_term():
    """With a field whose Jacobian trace is zero (f(u) = (u1, -u0)) TS1 reduces to TS0."""
    u0 = torch.tensor([1.0, 0.5], dtype=torch.float64)

    def vf(u, t):
        return torch.stack([u[0][1], -u[0][0]])

    tc = torch.stack([u0, vf(u0[None], 0.0), -u0, -vf(u0[None], 0.0)])
    S = ssm.IsoSSM()
    res = []
    for c in (S.constraint_ode_ts0(vf), S.constraint_ode_ts1(vf)):
        res.append(solvers.solve_adaptive_terminal_values(
            solvers.SolverMLE(solvers.StrategyFilter(), c), solvers.ErrorResidualStd(c), S.prior_wiener_integrated(tc),
            0.0, 2.0, 1e-6, 1e-6))
    assert res[0].num_steps[-1] == res[1].num_steps[-1]
    assert allclose(res[0].u[-1].mean, res[1].u[-1].mean)


@pytest.mark.parametrize("solver_name", ["none", "mle", "dynamic"])
@pytest.mark.parametrize("strategy", ["filter", "smoother"])
def test_behaviour_close_to_t1(strategy, solver_name):
    """test_dense_output/test_behaviour_close_to_t1.py:58-94: dense TS1 on
    Lotka--Volterra (nu = 2, tol 1e-1, 30 save points between t0 and the
    second-to-last point of the save-every-step grid); solving with the last
    save point removed leaves every other marginal unchanged -- for the
    smoother this checks that marginals close to t1 are informed by the
    overstepped state."""
    cls = {"none": solvers.SolverPlain, "mle": solvers.SolverMLE, "dynamic": solvers.SolverDynamic}[solver_name]
    S = make_ssm("dense")
    tc = problems.taylor_derivatives(problems.lotka_volterra, torch.tensor([20.0, 20.0]), LV_P, 2)
    prior = S.prior_wiener_integrated(tc)
    c = S.constraint_ode_ts1(lv, lv_jac, 2)
    every_strategy = solvers.StrategyFilter() if strategy == "filter" else solvers.StrategyFixedInterval()
    at_strategy = solvers.StrategyFilter() if strategy == "filter" else solvers.StrategyFixedPoint()
    every = solvers.solve_adaptive_save_every_step(cls(every_strategy, c), solvers.ErrorResidualStd(c), prior, 0.0, 2.0,
                                                   1e-1, 1e-1)
    ts = np.linspace(float(every.t[0]), float(every.t[-2]), 30)
    full = solvers.solve_adaptive_save_at(cls(at_strategy, c), solvers.ErrorResidualStd(c), prior, ts, 1e-1, 1e-1)
    cut = solvers.solve_adaptive_save_at(cls(at_strategy, c), solvers.ErrorResidualStd(c), prior, ts[:-1], 1e-1, 1e-1)
    assert len(full.u) == 30 and len(cut.u) == 29
    for a, b in zip(full.u[:-1], cut.u):
        ma, Ca = a.to_multivariate_normal()
        mb, Cb = b.to_multivariate_normal()
        assert allclose(ma, mb) and allclose(Ca, Cb)


def lv_reference_at(ts, y0=(20.0, 20.0)):
    f = lambda t, y: [0.5 * y[0] - 0.05 * y[0] * y[1], -0.5 * y[1] + 0.05 * y[0] * y[1]]
    return scipy.integrate.solve_ivp(f, (0.0, float(ts[-1])), list(y0), t_eval=ts, method="DOP853", rtol=1e-13,
                                     atol=1e-13).y.T


@pytest.mark.parametrize("solver_name", ["none", "mle", "dynamic"])
@pytest.mark.parametrize("strategy", ["filter", "fixedpoint"])
@pytest.mark.parametrize("kind", ["isotropic", "blockdiag", "dense"])
def test_save_at_matches_reference_solver(kind, strategy, solver_name):
    """tests/test_ivpsolve/test_solve_adaptive_save_at.py:202-247: seven save
    points on Lotka--Volterra, rtol = atol = 1e-4, against a high-accuracy
    classical solution (there odeint at 1e-7, here DOP853 at 1e-13) with the
    float32 allclose tolerances the reference's test runs under.  The
    reference test uses error_norm_rms_then_scale; the restatement has the
    default error_norm_scale_then_rms, the normalisation the kernels
    implement."""
    cls = {"none": solvers.SolverPlain, "mle": solvers.SolverMLE, "dynamic": solvers.SolverDynamic}[solver_name]
    strat = solvers.StrategyFilter() if strategy == "filter" else solvers.StrategyFixedPoint()
    tc = problems.taylor_derivatives(problems.lotka_volterra, torch.tensor([20.0, 20.0]), LV_P, 4)
    S = make_ssm(kind)
    c = ts0(S, kind)
    save_at = np.linspace(0.0, 2.0, 7)
    res = solvers.solve_adaptive_save_at(cls(strat, c), solvers.ErrorResidualStd(c), S.prior_wiener_integrated(tc),
                                         save_at, 1e-4, 1e-4)
    got = torch.stack([solvers.coeff(u, 0) for u in res.u])
    tol32 = math.sqrt(np.finfo(np.float32).eps)
    assert allclose(got, lv_reference_at(save_at), atol=tol32, rtol=10 * tol32)
