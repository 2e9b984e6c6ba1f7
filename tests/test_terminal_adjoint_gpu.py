"""The terminal-value adjoint on the GPU (``pdq_terminal_fwd`` / ``pdq_terminal_bwd``,
``autograd.terminal_values(mode="adjoint")``).

* float64: the record pass solves exactly as the plain kernel (bit for bit),
  and the adjoint gradient equals the forward-mode one (``mode="forward"``,
  the sensitivity kernel; its separate predict and update round differently,
  its means agree to 1e-8) to 1e-7 relative (the host runs of the same
  bodies, which share one QR, agree to 1e-10), for
  Lotka--Volterra (nu = 4) and FitzHugh--Nagumo (nu = 3), several
  checkpoint spacings, solver mle and none;
* against central finite differences of the terminal mean within 1e-4
  relative, on a frozen step sequence (the gradient holds the step sizes
  constant, as the reference's stop-gradient does);
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
    # the forward-mode kernel takes another QR ordering (a separate predict and
    # update), whose rounding moves its means by up to ~1e-9 over the horizon
    assert rel(m_a, m_f) < 1e-8, rel(m_a, m_f)
    assert rel(gp_a, gp_f) < 1e-7, (rel(gp_a, gp_f), rel(m_a, m_f))
    assert rel(gy_a, gy_f) < 1e-7, (rel(gy_a, gy_f), rel(m_a, m_f))


def test_adjoint_against_central_finite_differences():
    """On a frozen step sequence: with factor_min = factor_max = 1 and a
    tolerance every attempt meets, the adaptive solve takes exactly the
    steps dt0 (a fixed grid of 100 steps to t1, the last one clipped), so a
    perturbed solve takes the same steps and central differences measure the
    gradient the adjoint computes (on adaptive solves they would also pick
    up the step sizes' dependence on the parameters, which the reference's
    stop-gradient leaves out: several percent on these problems)."""
    params, y0, t1, nu = CASES["lotka_volterra"]
    B = params.shape[0]
    dev = dict(dtype=torch.float64, device="cuda")
    cfg = ensemble.make_config(field="lotka_volterra", num_derivatives=nu, ode_dim=2, solver="mle",
                               precision="float64", atol=1e3, rtol=1e3, factor_min=1.0, factor_max=1.0)
    save_at = torch.tensor([0.0, t1], **dev).expand(B, 2).contiguous()
    dt0 = torch.full((B,), 0.05, **dev)
    w = torch.randn((B, nu + 1, 2), generator=torch.Generator().manual_seed(2), dtype=torch.float64).to(**dev)

    def solve(pp, yy):
        out = _native.terminal_fwd(cfg, save_at, pp.to(**dev).contiguous(), yy.to(**dev).contiguous(), dt0)
        torch.cuda.synchronize()
        assert (out["status"] == 0).all() and (out["num_steps"][:, 0] == 100).all()
        return out

    base = solve(params, y0)
    gp, gy = _native.terminal_bwd(cfg, base, params.to(**dev), y0.to(**dev), w)
    torch.cuda.synchronize()

    def loss(pp, yy):
        return (solve(pp, yy)["u_mean"][:, 0] * w).sum(dim=(1, 2)).cpu()

    for k in range(params.shape[1]):
        e = torch.zeros_like(params)
        e[:, k] = 1e-6 * params[:, k]
        fd = (loss(params + e, y0) - loss(params - e, y0)) / (2 * e[:, k])
        assert rel(gp[:, k].cpu(), fd) < 1e-4, (k, gp[:, k].cpu(), fd)
    for j in range(2):
        e = torch.zeros_like(y0)
        e[:, j] = 1e-6 * y0[:, j]
        fd = (loss(params, y0 + e) - loss(params, y0 - e)) / (2 * e[:, j])
        assert rel(gy[:, j].cpu(), fd) < 1e-4, (j, gy[:, j].cpu(), fd)


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
