"""Forward-mode sensitivities of the isotropic mean records on the GPU.

d u_mean / d params and d u_mean / d y0 (``pdq_adaptive_args.u_mean_d_*``,
``ensemble.solve_ensemble(..., sensitivities=True)``,
``autograd.terminal_values``) against the oracle's torch reverse mode
through the same solve (step sizes and the dynamic scale detached, as the
reference stops gradients through them), and against central finite
differences on a fixed grid (where the step sequence cannot change).
Float64; tolerances relative to the largest entry: 1e-9 vs the oracle on a
grid, 1e-8 (Lotka-Volterra) or 1e-5 (rounding-sensitive step sequences) with
adaptive steps, 1e-4 vs finite differences (the accuracy target for gradients).
"""

import pytest
import torch

from oracle import problems, solvers, ssm
from probdiffeq_gb300 import autograd, ensemble

pytestmark = pytest.mark.gpu

CASES = {
    "lotka_volterra": (torch.tensor([[0.5, 0.05, 0.5, 0.05], [0.55, 0.045, 0.48, 0.052]], dtype=torch.float64),
                       torch.tensor([[20.0, 20.0], [15.0, 25.0]], dtype=torch.float64), 5.0),
    "fitzhugh_nagumo": (torch.tensor([[0.2, 0.2, 3.0], [0.25, 0.15, 2.8]], dtype=torch.float64),
                        torch.tensor([[-1.0, 1.0], [-0.8, 1.2]], dtype=torch.float64), 4.0),
}
SOLVERS = {"mle": solvers.SolverMLE, "dynamic": solvers.SolverDynamic, "none": solvers.SolverPlain}


def oracle_jacobians(field, params, y0, save_at, solver, nu, clip_dt, grid=False, every=1):
    """Jacobians of every mean record with respect to params and y0 (torch reverse mode);
    ``grid``: a step to every save_at point instead of the adaptive loop."""
    fn = problems.FIELDS[field]
    p = params.clone().requires_grad_(True)
    y = y0.clone().requires_grad_(True)
    tc = problems.taylor_derivatives(fn, y, p, nu)
    S = ssm.IsoSSM()
    c = S.constraint_ode_ts0(lambda u, t: fn(u[0], p))
    sol = SOLVERS[solver](solvers.StrategyFilter(), c)
    if grid:
        res = solvers.solve_grid_save_every_point(sol, S.prior_wiener_integrated(tc), save_at.tolist())
    else:
        res = solvers.solve_adaptive_save_at(sol, solvers.ErrorResidualStd(c), S.prior_wiener_integrated(tc),
                                             save_at.numpy(), 1e-6, 1e-6, clip_dt=clip_dt)
    out = []
    steps = [0] + list(res.num_steps)
    for k, (rec, num) in enumerate(zip(res.u, steps)):
        if k % every:
            out.append(None)
            continue
        m = rec.mean
        jp = torch.zeros(m.shape + p.shape, dtype=torch.float64)
        jy = torch.zeros(m.shape + y.shape, dtype=torch.float64)
        for i in range(m.shape[0]):
            for j in range(m.shape[1]):
                if not m[i, j].requires_grad:
                    continue
                gp, gy = torch.autograd.grad(m[i, j], (p, y), retain_graph=True, allow_unused=True)
                jp[i, j] = gp if gp is not None else 0.0
                jy[i, j] = gy if gy is not None else 0.0
        out.append((m.detach(), jp, jy, num))
    return out


def rel(a, b):
    return float((a - b).abs().max() / b.abs().max().clamp_min(1e-300))


@pytest.mark.parametrize("solver", ["mle", "dynamic", "none"])
@pytest.mark.parametrize("field", ["lotka_volterra", "fitzhugh_nagumo"])
def test_sensitivities_match_oracle_reverse_mode_on_a_grid(field, solver):
    """A step to every grid point (atol = inf, clip_dt): the same step sequence
    in both, so values and sensitivities agree to rounding."""
    params, y0, t1 = CASES[field]
    # fixed steps of 0.05 on LV; on FHN 0.012 up to t = 1.2 (the fixed-step dynamic
    # solve, oracle included, blows up beyond t = 1.6 at steps of 0.04)
    grid = torch.linspace(0.0, t1 if field == "lotka_volterra" else 1.2, 101, dtype=torch.float64)
    cfg = ensemble.make_config(field=field, num_derivatives=3, ode_dim=2, solver=solver, precision="float64",
                               atol=float("inf"), rtol=0.0, clip_dt=True, factor_max=1e30)
    out = ensemble.solve_ensemble(cfg, params=params, y0=y0, save_at=grid, dt0=100.0, terminal_only=False,
                                  sensitivities=True)
    torch.cuda.synchronize()
    assert (out["status"] == 0).all()
    for b in range(params.shape[0]):
        recs = oracle_jacobians(field, params[b], y0[b], grid, solver, 3, True, grid=True, every=10)
        # FHN with dynamic calibration on this grid (output scales up to ~600): a one-ulp
        # parameter change moves the oracle's own solution by up to 5e-9
        tol_v, tol_g = (1e-7, 1e-6) if (field, solver) == ("fitzhugh_nagumo", "dynamic") else (1e-10, 1e-9)
        for s, rec in enumerate(recs):
            if rec is None:
                continue
            m, jp, jy, _ = rec
            assert rel(out["u_mean"][b, s].cpu(), m) < tol_v, s
            assert rel(out["u_mean_d_params"][b, s].cpu(), jp) < tol_g, (s, rel(out["u_mean_d_params"][b, s].cpu(), jp))
            assert rel(out["u_mean_d_y0"][b, s].cpu(), jy) < tol_g, (s, rel(out["u_mean_d_y0"][b, s].cpu(), jy))


@pytest.mark.parametrize("clip_dt", [True, False])
@pytest.mark.parametrize("solver", ["mle", "dynamic", "none"])
@pytest.mark.parametrize("field", ["lotka_volterra", "fitzhugh_nagumo"])
def test_sensitivities_match_oracle_reverse_mode(field, solver, clip_dt):
    """Adaptive steps.  The step sizes are continuous functions of rounded
    error estimates: on FitzHugh-Nagumo with MLE a one-ulp change of the
    parameters moves the oracle's own solution by 7e-8, so the bar is the
    solver tolerance (values 1e-6, sensitivities 1e-5); Lotka-Volterra holds
    the rounding-level bar."""
    params, y0, t1 = CASES[field]
    save_at = torch.linspace(0.0, t1, 4, dtype=torch.float64)
    nu = 3
    cfg = ensemble.make_config(field=field, num_derivatives=nu, ode_dim=2, solver=solver, precision="float64",
                               atol=1e-6, rtol=1e-6, clip_dt=clip_dt)
    out = ensemble.solve_ensemble(cfg, params=params, y0=y0, save_at=save_at, terminal_only=False, sensitivities=True)
    torch.cuda.synchronize()
    assert (out["status"] == 0).all()
    for b in range(params.shape[0]):
        recs = oracle_jacobians(field, params[b], y0[b], save_at, solver, nu, clip_dt)
        for s, (m, jp, jy, num) in enumerate(recs):
            # rounding may flip one accept decision (steps +-1): the records then differ at the
            # solver tolerance; with the oracle's step count they agree to rounding
            same = int(out["num_steps"][b, s]) == num
            assert abs(int(out["num_steps"][b, s]) - num) <= 1
            tol_v, tol_g = (1e-9, 1e-8) if same and field == "lotka_volterra" else (1e-6, 1e-5)
            assert rel(out["u_mean"][b, s].cpu(), m) < tol_v, (s, same)
            assert rel(out["u_mean_d_params"][b, s].cpu(), jp) < tol_g, (s, same, rel(out["u_mean_d_params"][b, s].cpu(), jp))
            assert rel(out["u_mean_d_y0"][b, s].cpu(), jy) < tol_g, (s, same, rel(out["u_mean_d_y0"][b, s].cpu(), jy))


def test_sensitivities_match_central_finite_differences_on_a_fixed_grid():
    """Every step lands on the grid (atol = inf, clip_dt): the solution is a
    smooth function of params and y0, so central differences are exact to O(h^2)."""
    params, y0, _ = CASES["lotka_volterra"]
    grid = torch.linspace(0.0, 4.0, 41, dtype=torch.float64)

    def solve(p, y, sens=False):
        cfg = ensemble.make_config(field="lotka_volterra", num_derivatives=4, ode_dim=2, solver="none",
                                   precision="float64", atol=float("inf"), rtol=0.0, clip_dt=True,
                                   factor_max=1e30)
        o = ensemble.solve_ensemble(cfg, params=p, y0=y, save_at=grid, dt0=100.0, terminal_only=True,
                                    sensitivities=sens)
        torch.cuda.synchronize()
        assert (o["status"] == 0).all() and (o["num_steps"][:, 0] == 40).all()
        return o

    base = solve(params, y0, sens=True)
    h = 1e-6
    for k in range(4):
        e = torch.zeros_like(params)
        e[:, k] = h * params[:, k]
        fd = (solve(params + e, y0)["u_mean"] - solve(params - e, y0)["u_mean"])[:, 0].cpu() / (2 * e[:, k, None, None])
        got = base["u_mean_d_params"][:, 0, :, :, k].cpu()
        assert rel(got, fd) < 1e-4, (k, rel(got, fd))
    for j in range(2):
        e = torch.zeros_like(y0)
        e[:, j] = h * y0[:, j]
        fd = (solve(params, y0 + e)["u_mean"] - solve(params, y0 - e)["u_mean"])[:, 0].cpu() / (2 * e[:, j, None, None])
        got = base["u_mean_d_y0"][:, 0, :, :, j].cpu()
        assert rel(got, fd) < 1e-4, (j, rel(got, fd))


def test_terminal_values_autograd_function():
    """loss.backward() through autograd.terminal_values equals the oracle's gradient."""
    params, y0, t1 = CASES["lotka_volterra"]
    p = params.cuda().requires_grad_(True)
    y = y0.cuda().requires_grad_(True)
    w = torch.randn((2, 5, 2), generator=torch.Generator().manual_seed(0), dtype=torch.float64)
    mean, status = autograd.terminal_values(p, y, t0=0.0, t1=t1, num_derivatives=4, solver="mle")
    (mean * w.cuda()).sum().backward()
    assert (status == 0).all()
    for b in range(2):
        recs = oracle_jacobians("lotka_volterra", params[b], y0[b], torch.tensor([0.0, t1], dtype=torch.float64),
                                "mle", 4, True)
        _, jp, jy, _ = recs[-1]
        assert rel(p.grad[b].cpu(), torch.einsum("ij,ijk->k", w[b], jp)) < 1e-8
        assert rel(y.grad[b].cpu(), torch.einsum("ij,ijk->k", w[b], jy)) < 1e-8


def test_sensitivities_float32_and_unsupported_configurations():
    from probdiffeq_gb300 import _native

    params, y0, t1 = CASES["lotka_volterra"]
    cfg = ensemble.make_config(field="lotka_volterra", num_derivatives=4, ode_dim=2, solver="mle", precision="float32")
    o32 = ensemble.solve_ensemble(cfg, params=params, y0=y0, save_at=torch.tensor([0.0, t1]), sensitivities=True)
    cfg = ensemble.make_config(field="lotka_volterra", num_derivatives=4, ode_dim=2, solver="mle", precision="float64")
    o64 = ensemble.solve_ensemble(cfg, params=params, y0=y0, save_at=torch.tensor([0.0, t1]), sensitivities=True)
    torch.cuda.synchronize()
    assert rel(o32["u_mean_d_params"][:, :, 0].cpu(), o64["u_mean_d_params"][:, :, 0].cpu()) < 1e-2
    for kw in (dict(constraint="ts1"), dict(strategy="fixedpoint"), dict(error="state_std")):
        cfg = ensemble.make_config(field="lotka_volterra", num_derivatives=4, ode_dim=2, precision="float64", **kw)
        with pytest.raises(_native.NativeError):
            ensemble.solve_ensemble(cfg, params=params, y0=y0, save_at=torch.tensor([0.0, t1]), sensitivities=True)
