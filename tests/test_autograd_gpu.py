"""The LML kernel behind torch.autograd (GPU).

``probdiffeq_gb300.autograd.lml`` must give the same value as the C ABI call,
route cotangents into the kernel's parameter gradient, and agree with central
finite differences of the float64 kernel within 1e-4 relative (the accuracy
bar for adjoint gradients).
"""

import numpy as np
import pytest
import torch

from tests import lml_problem

pytestmark = pytest.mark.gpu


def _inputs(B, t1=2.0):
    num_steps, data = lml_problem.observations(t1=t1, dt=0.01, save_every=10)
    f64 = dict(dtype=torch.float64, device="cuda")
    thetas = torch.tensor(lml_problem.theta_samples(B, seed=3), **f64)
    y0 = torch.tensor(np.tile(lml_problem.U0, (B, 1)), **f64)
    data = torch.tensor(data, **f64)
    std = torch.full((data.shape[0],), lml_problem.STD, **f64)
    return num_steps, thetas, y0, data, std


def test_backward_applies_the_cotangent_to_the_kernel_gradient():
    from probdiffeq_gb300 import _native, autograd, ensemble

    num_steps, thetas, y0, data, std = _inputs(4)
    params = thetas.clone().requires_grad_(True)
    val, status = autograd.lml(params, y0, data, std, dt=0.01, num_steps=num_steps, save_every=10)
    w = torch.tensor([1.0, -2.0, 0.5, 3.0], dtype=torch.float64, device="cuda")
    (val * w).sum().backward()
    cfg = ensemble.make_config(field="fitzhugh_nagumo", num_derivatives=3, ode_dim=2, strategy="fixedpoint",
                               solver="none", precision="float64")
    ref = _native.lml_fixed_grid(cfg, thetas, y0, data, std, t0=0.0, dt=0.01, num_steps=num_steps, save_every=10,
                                 average_pdfs=False, gradient=True)
    assert (status == 0).all()
    assert torch.allclose(val.detach(), ref["lml"], rtol=1e-12, atol=0.0)
    assert torch.allclose(params.grad, w[:, None] * ref["grad"], rtol=1e-12, atol=0.0)


def test_gradient_matches_central_finite_differences():
    from probdiffeq_gb300 import autograd

    num_steps, thetas, y0, data, std = _inputs(2)
    params = thetas.clone().requires_grad_(True)
    val, _ = autograd.lml(params, y0, data, std, dt=0.01, num_steps=num_steps, save_every=10)
    val.sum().backward()
    eps = 1e-6
    for k in range(3):
        e = torch.zeros_like(thetas)
        e[:, k] = eps
        up, _ = autograd.lml(thetas + e, y0, data, std, dt=0.01, num_steps=num_steps, save_every=10)
        dn, _ = autograd.lml(thetas - e, y0, data, std, dt=0.01, num_steps=num_steps, save_every=10)
        fd = (up - dn) / (2 * eps)
        err = (params.grad[:, k] - fd).abs() / params.grad.norm(dim=1)
        assert float(err.max()) < 1e-4, (k, params.grad[:, k], fd)


def test_no_gradient_requested_runs_the_value_only_launch():
    from probdiffeq_gb300 import autograd

    num_steps, thetas, y0, data, std = _inputs(3)
    with torch.no_grad():
        val, status = autograd.lml(thetas, y0, data, std, dt=0.01, num_steps=num_steps, save_every=10)
    assert (status == 0).all() and torch.isfinite(val).all()
    with pytest.raises(ValueError):
        autograd.lml(thetas, y0, data[:-1], std[:-1], dt=0.01, num_steps=num_steps, save_every=10)
