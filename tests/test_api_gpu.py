"""The drop-in constructor API (probdiffeq_gb300.probdiffeq / .ivpsolve) on the GPU.

Written like the reference's own tests: build the solver from constructor
objects, call ``solve``, compare with the oracle (float64, tolerances as in
tests/test_iso_gpu.py: solution 1e-9, steps +-1).
"""

import numpy as np
import pytest
import torch

from oracle import problems, solvers, ssm
from probdiffeq_gb300 import ivpsolve, probdiffeq

pytestmark = pytest.mark.gpu

LV = torch.tensor([0.5, 0.05, 0.5, 0.05], dtype=torch.float64)


def oracle_terminal(y0, t1, solver_cls, nu=4, tol=1e-6):
    tc = problems.taylor_derivatives(problems.lotka_volterra, torch.tensor(y0), LV, nu)
    S = ssm.IsoSSM()
    c = S.constraint_ode_ts0(lambda u, t: problems.lotka_volterra(u[0], LV))
    return solvers.solve_adaptive_terminal_values(solver_cls(solvers.StrategyFilter(), c), solvers.ErrorResidualStd(c),
                                                  S.prior_wiener_integrated(tc), 0.0, t1, tol, tol)


def test_quickstart_style_terminal_values_batch():
    """test_solve_adaptive_terminal_values.py:15-51 pattern, with a batch of 3 initial values."""
    y0 = torch.tensor([[20.0, 20.0], [15.0, 25.0], [30.0, 12.0]], dtype=torch.float64)
    vf = probdiffeq.ode("lotka_volterra", LV)
    tcoeffs, _ = probdiffeq.jetexpand_ode_padded_scan(num=4)(vf, (y0,), t=0.0)
    ssm_ = probdiffeq.state_space_model_isotropic()
    iwp = ssm_.prior_wiener_integrated(tcoeffs)
    ts0 = ssm_.constraint_ode_ts0(vf)
    solver = probdiffeq.solver_mle(strategy=probdiffeq.strategy_filter(), constraint=ts0)
    error = probdiffeq.error_residual_std(constraint=ts0)
    solve = ivpsolve.solve_adaptive_terminal_values(solver, error, precision="float64")
    sol = solve(iwp, t0=0.0, t1=10.0, atol=1e-6, rtol=1e-6)
    torch.cuda.synchronize()
    assert (sol.status == 0).all()
    for b in range(3):
        res = oracle_terminal(y0[b], 10.0, solvers.SolverMLE)
        u = sol.u.mean[0][b, 0].cpu()
        ref = res.u[-1].mean[0]
        assert float((u - ref).abs().max() / ref.abs().max()) < 1e-9
        assert abs(int(sol.num_steps[b, 0]) - res.num_steps[-1]) <= 1


def test_fixed_grid_matches_oracle_save_every_step():
    """test_solve_fixed_grid.py:17-54 across implementations: the oracle's adaptive grid, solved on the GPU."""
    y0 = torch.tensor([20.0, 20.0], dtype=torch.float64)
    tc = problems.taylor_derivatives(problems.lotka_volterra, y0, LV, 2)
    S = ssm.IsoSSM()
    c = S.constraint_ode_ts0(lambda u, t: problems.lotka_volterra(u[0], LV))
    ad = solvers.solve_adaptive_save_every_step(solvers.SolverMLE(solvers.StrategyFilter(), c), solvers.ErrorResidualStd(c),
                                                S.prior_wiener_integrated(tc), 0.0, 2.0, 1e-2, 1e-2, clip_dt=True)
    vf = probdiffeq.ode("lotka_volterra", LV)
    tcoeffs, _ = probdiffeq.jetexpand_ode_padded_scan(num=2)(vf, (y0,), t=0.0)
    ssm_ = probdiffeq.state_space_model_isotropic()
    solver = probdiffeq.solver_mle(strategy=probdiffeq.strategy_filter(), constraint=ssm_.constraint_ode_ts0(vf))
    sol = ivpsolve.solve_fixed_grid(solver=solver, precision="float64")(ssm_.prior_wiener_integrated(tcoeffs), grid=np.asarray(ad.t))
    torch.cuda.synchronize()
    assert int(sol.status[0]) == 0
    for s, o in enumerate(ad.u):
        m = sol.u.mean_flat[0, s].cpu()
        L = sol.u.cholesky_flat[0, s].cpu()
        assert float((m - o.mean).abs().max() / o.mean.abs().max()) < 1e-9
        C, Co = L @ L.T, o.cholesky @ o.cholesky.T
        assert float((C - Co).abs().max() / Co.abs().max().clamp_min(1e-300)) < 1e-7
    assert [int(x) for x in sol.num_steps[0, 1:].cpu()] == ad.num_steps


def test_api_errors_are_raised_before_launch():
    vf = probdiffeq.ode("lotka_volterra", LV)
    with pytest.raises(ValueError):
        probdiffeq.ode("lotka_volterra", torch.ones(3))
    with pytest.raises(ValueError):
        probdiffeq.ode("no_such_field", torch.ones(1))
    iso, dense = probdiffeq.state_space_model_isotropic(), probdiffeq.state_space_model_dense()
    with pytest.raises(NotImplementedError):
        iso.constraint_ode_ts1(vf, taylor_point="map")
    tcoeffs, _ = probdiffeq.jetexpand_ode_padded_scan(num=3)(vf, (torch.tensor([20.0, 20.0]),))
    prior = iso.prior_wiener_integrated(tcoeffs)
    solver = probdiffeq.solver_dynamic(strategy=probdiffeq.strategy_filter(), constraint=dense.constraint_ode_ts0(vf))
    solve = ivpsolve.solve_adaptive_terminal_values(solver, probdiffeq.error_residual_std(constraint=solver.constraint))
    with pytest.raises(ValueError):
        solve(prior, t0=0.0, t1=1.0, atol=1e-6, rtol=1e-6)


def test_lml_through_the_api():
    from tests import lml_problem

    num_steps, data = lml_problem.observations(t1=2.0)
    thetas = torch.tensor(lml_problem.theta_samples(2, seed=1), dtype=torch.float64)
    vf = probdiffeq.ode("fitzhugh_nagumo", thetas)
    y0 = torch.tensor(np.tile(lml_problem.U0, (2, 1)), dtype=torch.float64)
    tcoeffs, _ = probdiffeq.jetexpand_ode_padded_scan(num=3)(vf, (y0,))
    prior = probdiffeq.state_space_model_isotropic().prior_wiener_integrated(tcoeffs)
    lml, grad, status = ivpsolve.lml_fixed_grid(prior, data, lml_problem.STD, dt=0.01, num_steps=num_steps, save_every=10,
                                                loss=probdiffeq.loss_lml_timeseries(average_pdfs=False))
    torch.cuda.synchronize()
    assert (status == 0).all()
    from tests.test_lml_gpu import oracle_lml

    v, g = oracle_lml(thetas[0].numpy(), data, 0.01, num_steps, 10)
    assert abs(float(lml[0]) - v) <= 1e-9 * abs(v)
    assert np.abs(grad[0].cpu().numpy() - g).max() <= 1e-6 * np.linalg.norm(g)


@pytest.mark.parametrize("ssm_name", ["isotropic", "dense"])
def test_fixed_grid_fixedinterval_smoother_and_posterior_samples(ssm_name):
    """solve_fixed_grid with strategy_smoother_fixedinterval (estimators_and_losses.py:594-717),
    then posterior samples.

    The reference's solve_fixed_grid hands the last state -- whose backward
    conditional is the last step's, not the identity that Smoother.finalize
    assumes (estimators_and_losses.py:455-458) -- to finalize, so its
    terminal marginal is not the filter's; the smoother's posterior on the
    grid is what the reference's save-every-step path computes, and equals
    the fixed-point smoother with a checkpoint at every grid point
    (test_smoother_fixedinterval_vs_fixedpoint.py).  That is the comparison.
    """
    from probdiffeq_gb300 import markov

    y0 = torch.tensor([[20.0, 20.0]], dtype=torch.float64)
    vf = probdiffeq.ode("lotka_volterra", LV)
    tcoeffs, _ = probdiffeq.jetexpand_ode_padded_scan(num=3)(vf, (y0,), t=0.0)
    S_ = probdiffeq.state_space_model_isotropic() if ssm_name == "isotropic" else probdiffeq.state_space_model_dense()
    iwp = S_.prior_wiener_integrated(tcoeffs)
    ts0 = S_.constraint_ode_ts0(vf)
    solver = probdiffeq.solver_mle(strategy=probdiffeq.strategy_smoother_fixedinterval(), constraint=ts0)
    grid = torch.linspace(0.0, 2.0, 11, dtype=torch.float64)
    sol = ivpsolve.solve_fixed_grid(solver=solver, precision="float64")(iwp, grid=grid, posterior=True)
    torch.cuda.synchronize()
    assert (sol.status == 0).all()

    tc = problems.taylor_derivatives(problems.lotka_volterra, y0[0], LV, 3)
    So = ssm.IsoSSM() if ssm_name == "isotropic" else ssm.DenseSSM()
    vfo = lambda u, t: problems.lotka_volterra(u[0], LV)  # noqa: E731
    c = So.constraint_ode_ts0(vfo) if ssm_name == "isotropic" else So.constraint_ode_ts0(vfo, 2)
    uo = solvers.solve_fixed_steps_save_at(solvers.SolverMLE(solvers.StrategyFixedPoint(), c),
                                           So.prior_wiener_integrated(tc), 0.0, 0.2, 10, 1)[0]
    for s, o in enumerate(uo):
        mo, Co = o.to_multivariate_normal()
        m = sol.u.mean_flat[0, s].cpu().reshape(-1)
        L = sol.u.cholesky_flat[0, s].cpu()
        C = L @ L.T
        if ssm_name == "isotropic":
            C = torch.kron(C, torch.eye(2, dtype=torch.float64))
        assert float((m - mo).abs().max() / mo.abs().max()) < 1e-9
        assert float((C - Co).abs().max() / Co.abs().max().clamp_min(1e-300)) < 1e-7
    smp = markov.sample(sol, 7, generator=torch.Generator(device="cuda").manual_seed(3))
    assert smp.shape[:3] == (1, 7, 11) and torch.isfinite(smp).all()
