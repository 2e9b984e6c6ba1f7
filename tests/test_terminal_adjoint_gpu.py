"""The terminal-value adjoint on the GPU (``pdq_terminal_fwd`` / ``pdq_terminal_bwd``,
``autograd.terminal_values(mode="adjoint")``).

* float64: the record pass solves exactly as the plain kernel (bit for bit),
  and the adjoint gradient equals the forward-mode one (``mode="forward"``,
  the sensitivity kernel, whose means agree to 1e-12) to 1e-9 relative, for
  Lotka--Volterra (nu = 4) and FitzHugh--Nagumo (nu = 3), several
  checkpoint spacings, solver mle and none;
* against central finite differences of the terminal mean within 1e-4
  relative: the gradient holds the step sizes constant, while a perturbed
  adaptive solve takes other steps, so the differences are taken at
  rtol = atol = 1e-12 (where the step sequence moves the solution by
  ~1e-12 of its size) with a relative parameter step of 1e-3 (the
  step-sequence noise in the quotient is then ~1e-7, the truncation ~1e-6);
* float32 bulk: within 1e-2 of the float64 gradient (as the forward-mode
  sensitivities in float32);
* a capacity below the accepted steps: the wrapper reruns with the exact
  count; the C ABI alone reports PDQ_INSTANCE_RECORD_FULL (and NaN
  gradients) without touching the solution;
* configurations the adjoint does not cover are rejected before launch.
"""

import pytest
import torch

from probdiffeq_gb300 import _native, autograd, ensemble

pytestmark = pytest.mark.gpu

CASES = {
    "lotka_volterra": (torch.tensor([[0.5, 0.05, 0.5, 0.05], [0.55, 0.045, 0.48, 0.052], [0.45, 0.06, 0.52, 0.047]],
                                    dtype=torch.float64),
                       torch.tensor([[20.0, 20.0], [15.0, 25.0], [25.0, 15.0]], dtype=torch.float64), 5.0, 4),
    "fitzhugh_nagumo": (torch.tensor([[0.2, 0.2, 3.0], [0.25, 0.15, 2.8]], dtype=torch.float64),
                        torch.tensor([[-1.0, 1.0], [-0.8, 1.2]], dtype=torch.float64), 4.0, 3),
}


def rel(a, b):
    return float((a - b).abs().max() / b.abs().max().clamp_min(1e-300))


def grads(field, mode, solver="mle", precision="float64", **kw):
    params, y0, t1, nu = CASES[field]
    p = params.cuda().requires_grad_(True)
    y = y0.cuda().requires_grad_(True)
    w = torch.randn((params.shape[0], nu + 1, 2), generator=torch.Generator().manual_seed(1), dtype=torch.float64)
    mean, status = autograd.terminal_values(p, y, t0=0.0, t1=t1, field=field, num_derivatives=nu, solver=solver,
                                            precision=precision, mode=mode, **kw)
    (mean * w.cuda()).sum().backward()
    torch.cuda.synchronize()
    assert (status == 0).all()
    return mean.detach().cpu(), p.grad.cpu(), y.grad.cpu()


@pytest.mark.parametrize("field", ["lotka_volterra", "fitzhugh_nagumo"])
@pytest.mark.parametrize("solver", ["mle", "none"])
@pytest.mark.parametrize("checkpoint_every", [None, 1, 5])
def test_adjoint_equals_forward_mode(field, solver, checkpoint_every):
    m_f, gp_f, gy_f = grads(field, "forward", solver)
    m_a, gp_a, gy_a = grads(field, "adjoint", solver, checkpoint_every=checkpoint_every)
    params, y0, t1, nu = CASES[field]
    cfg = ensemble.make_config(field=field, num_derivatives=nu, ode_dim=2, solver=solver, precision="float64",
                               clip_dt=True)
    plain = ensemble.solve_ensemble(cfg, params=params, y0=y0, save_at=torch.tensor([0.0, t1], dtype=torch.float64),
                                    device="cuda:0")
    torch.cuda.synchronize()
    assert torch.equal(m_a, plain["u_mean"][:, 0].cpu())  # the record pass solves as the plain kernel
    assert rel(m_a, m_f) < 1e-12  # the forward-mode kernel's path (another QR ordering)
    assert rel(gp_a, gp_f) < 1e-9, rel(gp_a, gp_f)
    assert rel(gy_a, gy_f) < 1e-9, rel(gy_a, gy_f)


def test_adjoint_against_central_finite_differences():
    params, y0, t1, nu = CASES["lotka_volterra"]
    w = torch.randn((params.shape[0], nu + 1, 2), generator=torch.Generator().manual_seed(2), dtype=torch.float64)
    tol = dict(atol=1e-12, rtol=1e-12)
    p = params.cuda().requires_grad_(True)
    y = y0.cuda().requires_grad_(True)
    mean, status = autograd.terminal_values(p, y, t0=0.0, t1=t1, num_derivatives=nu, mode="adjoint", **tol)
    (mean * w.cuda()).sum().backward()
    assert (status == 0).all()

    def loss(pp, yy):
        m, st = autograd.terminal_values(pp.cuda(), yy.cuda(), t0=0.0, t1=t1, num_derivatives=nu, **tol)
        assert (st == 0).all()
        return (m.cpu() * w).sum(dim=(1, 2))

    for k in range(params.shape[1]):
        e = torch.zeros_like(params)
        e[:, k] = 1e-3 * params[:, k]
        fd = (loss(params + e, y0) - loss(params - e, y0)) / (2 * e[:, k])
        assert rel(p.grad[:, k].cpu(), fd) < 1e-4, (k, p.grad[:, k].cpu(), fd)
    for j in range(2):
        e = torch.zeros_like(y0)
        e[:, j] = 1e-3 * y0[:, j]
        fd = (loss(params, y0 + e) - loss(params, y0 - e)) / (2 * e[:, j])
        assert rel(y.grad[:, j].cpu(), fd) < 1e-4, (j, y.grad[:, j].cpu(), fd)


def test_adjoint_float32():
    _, gp64, gy64 = grads("lotka_volterra", "adjoint")
    _, gp32, gy32 = grads("lotka_volterra", "adjoint", precision="float32")
    assert rel(gp32, gp64) < 1e-2 and rel(gy32, gy64) < 1e-2


def test_capacity_too_small():
    params, y0, t1, nu = CASES["lotka_volterra"]
    _, gp, gy = grads("lotka_volterra", "adjoint")
    _, gp2, gy2 = grads("lotka_volterra", "adjoint", capacity=None)
    assert torch.equal(gp, gp2) and torch.equal(gy, gy2)
    # through the bindings with a fixed capacity below the accepted steps
    cfg = ensemble.make_config(field="lotka_volterra", num_derivatives=nu, ode_dim=2, solver="mle", precision="float64")
    B = params.shape[0]
    dev = dict(dtype=torch.float64, device="cuda")
    save_at = torch.tensor([0.0, t1], **dev).expand(B, 2).contiguous()
    dt0 = torch.full((B,), 0.1, **dev)
    pc, yc = params.to(**dev), y0.to(**dev)
    big = _native.terminal_fwd(cfg, save_at, pc, yc, dt0, capacity=4096)
    steps = big["num_steps"][:, 0].cpu()
    cap = int(steps.min()) - 1
    small = _native.terminal_fwd(cfg, save_at, pc, yc, dt0, capacity=cap)
    torch.cuda.synchronize()
    assert torch.equal(small["u_mean"], big["u_mean"])
    assert ((small["status"].cpu() == _native.INSTANCE_RECORD_FULL) == (steps > cap)).all()
    cot = torch.ones((B, nu + 1, 2), **dev)
    g_small, _ = _native.terminal_bwd(cfg, small, pc, yc, cot)
    g_big, _ = _native.terminal_bwd(cfg, big, pc, yc, cot)
    torch.cuda.synchronize()
    full = steps > cap
    assert torch.isnan(g_small.cpu()[full]).all()
    assert torch.isfinite(g_big.cpu()).all()


def test_unsupported_configurations_are_rejected():
    params, y0, t1, nu = CASES["lotka_volterra"]
    B = params.shape[0]
    dev = dict(dtype=torch.float64, device="cuda")
    save_at = torch.tensor([0.0, t1], **dev).expand(B, 2).contiguous()
    dt0 = torch.full((B,), 0.1, **dev)
    for kw in (dict(solver="dynamic"), dict(constraint="ts1"), dict(strategy="fixedpoint"), dict(error="state_std"),
               dict(clip_dt=False), dict(ssm="dense")):
        cfg = ensemble.make_config(**{**dict(field="lotka_volterra", num_derivatives=nu, ode_dim=2, solver="mle",
                                             precision="float64"), **kw})
        with pytest.raises(_native.NativeError):
            _native.terminal_fwd(cfg, save_at, params.to(**dev), y0.to(**dev), dt0, capacity=64)
