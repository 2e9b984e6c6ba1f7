"""Log-marginal likelihood and its parameter gradient on the GPU vs the oracle.

The oracle runs the same pipeline in float64 on the CPU (fixed-point smoother
on the fixed grid with checkpoint resets, loss_lml_timeseries with
average_pdfs=False) and differentiates it with PyTorch autograd using the
reference's qr_r rule (Q held constant, backend/linalg.py:13-37); central
finite differences pin both.  Tolerances: float64 -- LML 1e-9 relative,
gradient 1e-6 relative to its norm (and vs finite differences 1e-4, the
accuracy target for gradients); float32 -- LML 1e-3, gradient 5e-2 relative.
"""

import numpy as np
import pytest
import torch

from oracle import linalg, problems, solvers, ssm
from tests import lml_problem

pytestmark = pytest.mark.gpu


def oracle_lml(theta, data, dt, num_steps, save_every, requires_grad=True):
    linalg.set_qr_derivative("reference")
    th = torch.tensor(theta, dtype=torch.float64, requires_grad=requires_grad)
    tc = problems.taylor_derivatives(problems.fitzhugh_nagumo, torch.tensor(lml_problem.U0), th, 3)
    S = ssm.IsoSSM()
    prior = S.prior_wiener_integrated(tc)
    c = S.constraint_ode_ts0(lambda u, t: problems.fitzhugh_nagumo(u[0], th))
    solver = solvers.SolverPlain(solvers.StrategyFixedPoint(), c)
    _, post = solvers.solve_fixed_steps_save_at(solver, prior, 0.0, dt, num_steps, save_every)
    d = torch.tensor(data, dtype=torch.float64)
    lml = solvers.loss_lml_timeseries(list(d), post, lml_problem.STD * torch.ones(d.shape[0]), average_pdfs=False)
    if not requires_grad:
        return float(lml.detach()), None
    (g,) = torch.autograd.grad(lml, th)
    return float(lml.detach()), g.numpy()


def gpu_lml(thetas, data, dt, num_steps, save_every, precision):
    from probdiffeq_gb300 import _native, ensemble

    cfg = ensemble.make_config(field="fitzhugh_nagumo", num_derivatives=3, ode_dim=2, ssm="isotropic",
                               strategy="fixedpoint", solver="none", precision=precision)
    B = len(thetas)
    dev = "cuda"
    f64 = dict(dtype=torch.float64, device=dev)
    out = _native.lml_fixed_grid(
        cfg, torch.tensor(np.asarray(thetas), **f64), torch.tensor(np.tile(lml_problem.U0, (B, 1)), **f64),
        torch.tensor(data, **f64), torch.full((data.shape[0],), lml_problem.STD, **f64),
        t0=0.0, dt=dt, num_steps=num_steps, save_every=save_every, average_pdfs=False, gradient=True,
    )
    torch.cuda.synchronize()
    return out["lml"].cpu().numpy(), out["grad"].cpu().numpy(), out["status"].cpu().numpy()


@pytest.mark.parametrize("precision", ["float64", "float32"])
def test_lml_and_gradient_short_horizon(precision):
    dt, save_every = 0.01, 10
    num_steps, data = lml_problem.observations(t1=2.0, dt=dt, save_every=save_every)
    thetas = lml_problem.theta_samples(3, seed=1)
    lml, grad, status = gpu_lml(thetas, data, dt, num_steps, save_every, precision)
    assert (status == 0).all()
    for b, th in enumerate(thetas):
        v, g = oracle_lml(th, data, dt, num_steps, save_every)
        if precision == "float64":
            assert abs(lml[b] - v) <= 1e-9 * abs(v), (lml[b], v)
            assert np.abs(grad[b] - g).max() <= 1e-6 * np.linalg.norm(g), (grad[b], g)
        else:
            assert abs(lml[b] - v) <= 1e-3 * abs(v), (lml[b], v)
            assert np.abs(grad[b] - g).max() <= 5e-2 * np.linalg.norm(g), (grad[b], g)


def test_gradient_matches_central_finite_differences():
    """Accuracy target: forward-mode gradients within 1e-4 relative of central FD (float64)."""
    dt, save_every = 0.01, 10
    num_steps, data = lml_problem.observations(t1=2.0, dt=dt, save_every=save_every)
    th = lml_problem.theta_samples(1, seed=2)[0]
    eps = 1e-5
    probe = [th]
    for i in range(3):
        for sgn in (1, -1):
            e = np.zeros(3)
            e[i] = sgn * eps
            probe.append(th + e)
    lml, grad, status = gpu_lml(probe, data, dt, num_steps, save_every, "float64")
    assert (status == 0).all()
    fd = np.array([(lml[1 + 2 * i] - lml[2 + 2 * i]) / (2 * eps) for i in range(3)])
    assert np.abs(grad[0] - fd).max() <= 1e-4 * np.linalg.norm(fd), (grad[0], fd)


def test_full_horizon_values_match_oracle():
    """t in [0, 20], 2000 steps, 201 observations (the benchmark configuration), float64."""
    dt, save_every = 0.01, 10
    num_steps, data = lml_problem.observations(t1=20.0, dt=dt, save_every=save_every)
    thetas = lml_problem.theta_samples(2, seed=3)
    lml, grad, status = gpu_lml(thetas, data, dt, num_steps, save_every, "float64")
    assert (status == 0).all()
    v, g = oracle_lml(thetas[0], data, dt, num_steps, save_every)
    assert abs(lml[0] - v) <= 1e-8 * abs(v), (lml[0], v)
    assert np.abs(grad[0] - g).max() <= 1e-5 * np.linalg.norm(g), (grad[0], g)
