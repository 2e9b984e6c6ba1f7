"""Adjoint (reverse-mode) LML gradient, pdq_lml_fwd / pdq_lml_bwd, on the GPU.

Checked against the forward-mode kernel (pdq_lml_fixed_grid, the same
derivative rules), the oracle differentiated by PyTorch autograd (the
reference's qr_r rule, backend/linalg.py:13-37) and central finite
differences, over sqrt(N), ragged, single-step and single-segment checkpoint
spacings.  Tolerances: float64 -- adjoint vs forward mode 1e-9 relative to
the gradient's norm, vs the oracle 1e-6 (short horizon) / 1e-5 (2000 steps),
vs central differences 1e-4 (the accuracy target for gradients); float32 -- 5e-2 vs the
float64 oracle, as for the forward-mode kernel.
"""

import numpy as np
import pytest
import torch

from tests import lml_problem
from tests.lml_oracle import lml_value_and_grads as oracle_with_y0
from tests.test_lml_gpu import gpu_lml, oracle_lml

pytestmark = pytest.mark.gpu

F64 = dict(dtype=torch.float64, device="cuda")


def fhn_config(precision):
    from probdiffeq_gb300 import ensemble

    return ensemble.make_config(field="fitzhugh_nagumo", num_derivatives=3, ode_dim=2, ssm="isotropic",
                                strategy="fixedpoint", solver="none", precision=precision)


def adjoint(thetas, y0s, data, dt, num_steps, save_every, precision, checkpoint_every=0, average_pdfs=False,
            cotangent=None, cfg=None):
    from probdiffeq_gb300 import _native

    cfg = cfg or fhn_config(precision)
    fwd = _native.lml_fwd(cfg, torch.tensor(np.asarray(thetas), **F64), torch.tensor(np.asarray(y0s), **F64),
                          torch.tensor(data, **F64), torch.full((data.shape[0],), lml_problem.STD, **F64),
                          t0=0.0, dt=dt, num_steps=num_steps, save_every=save_every, average_pdfs=average_pdfs,
                          checkpoint_every=checkpoint_every)
    cot = None if cotangent is None else torch.tensor(np.asarray(cotangent), **F64)
    out = _native.lml_bwd(fwd, cot, params_grad=True, y0_grad=True)
    torch.cuda.synchronize()
    return (fwd["lml"].cpu().numpy(), out["grad"].cpu().numpy(), out["grad_y0"].cpu().numpy(),
            fwd["status"].cpu().numpy(), fwd)


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("checkpoint_every", [0, 1, 7, 2000])
def test_adjoint_equals_forward_mode_full_horizon(checkpoint_every):
    """2000 steps, 201 observations (the benchmark grid), float64: the same
    value and gradient as the forward-mode kernel for every checkpoint
    spacing (0 = round(sqrt(2000)) = 45; 7 leaves a ragged last segment)."""
    dt, save_every = 0.01, 10
    num_steps, data = lml_problem.observations(t1=20.0, dt=dt, save_every=save_every)
    thetas = lml_problem.theta_samples(5, seed=4)
    y0s = np.tile(lml_problem.U0, (5, 1))
    v, g, _, st, _ = adjoint(thetas, y0s, data, dt, num_steps, save_every, "float64", checkpoint_every)
    v_fm, g_fm, st_fm = gpu_lml(thetas, data, dt, num_steps, save_every, "float64")
    assert (st == 0).all() and (st_fm == 0).all()
    for b in range(5):
        assert abs(v[b] - v_fm[b]) <= 1e-12 * abs(v_fm[b]), (v[b], v_fm[b])
        assert rel(g[b], g_fm[b]) <= 1e-9, (g[b], g_fm[b])


@pytest.mark.parametrize("precision", ["float64", "float32"])
def test_adjoint_matches_oracle_autograd(precision):
    """Short horizon (200 steps): value, d/d params and d/d y0 against the
    oracle's reverse mode, with perturbed initial values and a cotangent."""
    dt, save_every = 0.01, 10
    num_steps, data = lml_problem.observations(t1=2.0, dt=dt, save_every=save_every)
    thetas = lml_problem.theta_samples(3, seed=1)
    y0s = np.tile(lml_problem.U0, (3, 1)) + np.array([[0.0, 0.0], [0.1, -0.05], [-0.02, 0.03]])
    cot = np.array([1.0, -0.5, 2.0])
    v, g, gy, st, _ = adjoint(thetas, y0s, data, dt, num_steps, save_every, precision, 14, cotangent=cot)
    assert (st == 0).all()
    tol_v, tol_g = (1e-9, 1e-6) if precision == "float64" else (1e-3, 5e-2)
    for b in range(3):
        ov, og, ogy = oracle_with_y0(thetas[b], y0s[b], data, dt, num_steps, save_every)
        assert abs(v[b] - ov) <= tol_v * abs(ov), (v[b], ov)
        assert rel(g[b], cot[b] * og) <= tol_g, (g[b], cot[b] * og)
        assert rel(gy[b], cot[b] * ogy) <= tol_g, (gy[b], cot[b] * ogy)


def test_adjoint_full_horizon_matches_oracle():
    dt, save_every = 0.01, 10
    num_steps, data = lml_problem.observations(t1=20.0, dt=dt, save_every=save_every)
    th = lml_problem.theta_samples(1, seed=3)
    v, g, gy, st, _ = adjoint(th, lml_problem.U0[None, :], data, dt, num_steps, save_every, "float64")
    assert st[0] == 0
    ov, og, ogy = oracle_with_y0(th[0], lml_problem.U0, data, dt, num_steps, save_every)
    assert abs(v[0] - ov) <= 1e-8 * abs(ov)
    assert rel(g[0], og) <= 1e-5 and rel(gy[0], ogy) <= 1e-5, (g[0], og, gy[0], ogy)


def test_adjoint_matches_central_finite_differences():
    """Accuracy target: the adjoint gradient within 1e-4 relative of central
    differences of the LML, for the parameters and the initial values."""
    dt, save_every = 0.01, 10
    num_steps, data = lml_problem.observations(t1=2.0, dt=dt, save_every=save_every)
    th = lml_problem.theta_samples(1, seed=2)[0]
    y0 = lml_problem.U0.copy()
    eps = 1e-5
    thetas, y0s = [th], [y0]
    for i in range(3):
        for sgn in (1, -1):
            e = np.zeros(3)
            e[i] = sgn * eps
            thetas.append(th + e)
            y0s.append(y0)
    for i in range(2):
        for sgn in (1, -1):
            e = np.zeros(2)
            e[i] = sgn * eps
            thetas.append(th)
            y0s.append(y0 + e)
    v, g, gy, st, _ = adjoint(np.array(thetas), np.array(y0s), data, dt, num_steps, save_every, "float64")
    assert (st == 0).all()
    fd = np.array([(v[1 + 2 * i] - v[2 + 2 * i]) / (2 * eps) for i in range(3)])
    fdy = np.array([(v[7 + 2 * i] - v[8 + 2 * i]) / (2 * eps) for i in range(2)])
    assert rel(g[0], fd) <= 1e-4, (g[0], fd)
    assert rel(gy[0], fdy) <= 1e-4, (gy[0], fdy)


def test_average_pdfs_cotangent_and_repeated_backward():
    """average_pdfs divides the gradient by the number of observations (as the
    forward-mode kernel's running mean does); the cotangent scales it; a
    second backward call on the same residuals gives the same bits."""
    from probdiffeq_gb300 import _native

    dt, save_every = 0.01, 10
    num_steps, data = lml_problem.observations(t1=2.0, dt=dt, save_every=save_every)
    thetas = lml_problem.theta_samples(4, seed=5)
    y0s = np.tile(lml_problem.U0, (4, 1))
    v, g, _, st, fwd = adjoint(thetas, y0s, data, dt, num_steps, save_every, "float64", average_pdfs=True)
    cfg = fhn_config("float64")
    out = _native.lml_fixed_grid(cfg, torch.tensor(thetas, **F64), torch.tensor(y0s, **F64), torch.tensor(data, **F64),
                                 torch.full((data.shape[0],), lml_problem.STD, **F64), t0=0.0, dt=dt,
                                 num_steps=num_steps, save_every=save_every, average_pdfs=True, gradient=True)
    torch.cuda.synchronize()
    assert (st == 0).all()
    assert np.allclose(v, out["lml"].cpu().numpy(), rtol=1e-12, atol=0)
    g_fm = out["grad"].cpu().numpy()
    for b in range(4):
        assert rel(g[b], g_fm[b]) <= 1e-9
    cot = torch.tensor([2.0, -1.0, 0.5, 0.0], **F64)
    again = _native.lml_bwd(fwd, cot, params_grad=True, y0_grad=True)
    twice = _native.lml_bwd(fwd, cot, params_grad=True, y0_grad=True)
    torch.cuda.synchronize()
    assert torch.equal(again["grad"], twice["grad"]) and torch.equal(again["grad_y0"], twice["grad_y0"])
    scaled = again["grad"].cpu().numpy()
    for b in range(4):
        assert np.allclose(scaled[b], float(cot[b]) * g[b], rtol=1e-12, atol=1e-300)


@pytest.mark.parametrize("B", [1, 33])
def test_ragged_batches_equal_single_samples(B):
    """Batch sizes that do not fill a warp give every sample the result it
    gets alone."""
    dt, save_every = 0.01, 10
    num_steps, data = lml_problem.observations(t1=2.0, dt=dt, save_every=save_every)
    thetas = lml_problem.theta_samples(B, seed=6)
    y0s = np.tile(lml_problem.U0, (B, 1))
    v, g, gy, st, _ = adjoint(thetas, y0s, data, dt, num_steps, save_every, "float64", 9)
    assert (st == 0).all()
    for b in (0, B - 1):
        v1, g1, gy1, _, _ = adjoint(thetas[b:b + 1], y0s[b:b + 1], data, dt, num_steps, save_every, "float64", 9)
        assert v[b] == v1[0] and np.array_equal(g[b], g1[0]) and np.array_equal(gy[b], gy1[0])


def test_lotka_volterra_adjoint_equals_forward_mode():
    """Second field (four parameters): Lotka--Volterra in float64, synthetic data."""
    from probdiffeq_gb300 import _native, ensemble

    cfg = ensemble.make_config(field="lotka_volterra", num_derivatives=3, ode_dim=2, ssm="isotropic",
                               strategy="fixedpoint", solver="none", precision="float64")
    rng = np.random.default_rng(7)
    B, dt, num_steps, save_every = 3, 0.05, 200, 20
    params = np.array([0.5, 0.05, 0.5, 0.05]) * np.exp(0.1 * rng.standard_normal((B, 4)))
    y0 = 20.0 + rng.uniform(-2, 2, (B, 2))
    data = 20.0 + 5.0 * rng.standard_normal((num_steps // save_every + 1, 2))
    std = torch.full((data.shape[0],), 0.5, **F64)
    p_t, y_t, d_t = torch.tensor(params, **F64), torch.tensor(y0, **F64), torch.tensor(data, **F64)
    fwd = _native.lml_fwd(cfg, p_t, y_t, d_t, std, t0=0.0, dt=dt, num_steps=num_steps, save_every=save_every)
    bwd = _native.lml_bwd(fwd)
    fm = _native.lml_fixed_grid(cfg, p_t, y_t, d_t, std, t0=0.0, dt=dt, num_steps=num_steps, save_every=save_every,
                                gradient=True)
    torch.cuda.synchronize()
    assert (fwd["status"] == 0).all() and (fm["status"] == 0).all()
    assert torch.allclose(fwd["lml"], fm["lml"], rtol=1e-12, atol=0)
    g, g_fm = bwd["grad"].cpu().numpy(), fm["grad"].cpu().numpy()
    for b in range(B):
        assert rel(g[b], g_fm[b]) <= 1e-9, (g[b], g_fm[b])


def test_torch_autograd_adjoint_mode():
    """autograd.lml(mode="adjoint"): loss.backward() fills params.grad and
    y0.grad through pdq_lml_bwd; params.grad equals the forward mode's."""
    from probdiffeq_gb300 import autograd

    dt, save_every = 0.01, 10
    num_steps, data = lml_problem.observations(t1=2.0, dt=dt, save_every=save_every)
    thetas = torch.tensor(lml_problem.theta_samples(3, seed=8), **F64)
    kw = dict(dt=dt, num_steps=num_steps, save_every=save_every)
    d_t, std = torch.tensor(data, **F64), torch.full((data.shape[0],), lml_problem.STD, **F64)
    p1 = thetas.clone().requires_grad_(True)
    y1 = torch.tensor(np.tile(lml_problem.U0, (3, 1)), **F64).requires_grad_(True)
    lml1, st1 = autograd.lml(p1, y1, d_t, std, mode="adjoint", **kw)
    (lml1 * torch.tensor([1.0, 2.0, 3.0], **F64)).sum().backward()
    p2 = thetas.clone().requires_grad_(True)
    lml2, _ = autograd.lml(p2, y1.detach(), d_t, std, mode="forward", **kw)
    (lml2 * torch.tensor([1.0, 2.0, 3.0], **F64)).sum().backward()
    assert (st1 == 0).all()
    assert torch.allclose(p1.grad, p2.grad, rtol=1e-9, atol=1e-9 * float(p2.grad.abs().max()))
    _, og, ogy = oracle_with_y0(thetas[1].cpu().numpy(), lml_problem.U0, data, dt, num_steps, save_every)
    assert rel(y1.grad[1].cpu().numpy(), 2.0 * ogy) <= 1e-6


def test_oracle_pins_forward_mode_reference_helper():
    """The helper shared with the forward-mode tests still agrees with the
    oracle used here (params only)."""
    dt, save_every = 0.01, 10
    num_steps, data = lml_problem.observations(t1=1.0, dt=dt, save_every=save_every)
    th = lml_problem.theta_samples(1, seed=9)[0]
    v1, g1 = oracle_lml(th, data, dt, num_steps, save_every)
    v2, g2, _ = oracle_with_y0(th, lml_problem.U0, data, dt, num_steps, save_every)
    assert v1 == v2 and np.allclose(g1, g2, rtol=1e-14, atol=0)
