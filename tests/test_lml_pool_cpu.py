"""Host logic of the adjoint LML's workspace pool (no GPU: the three native
calls are replaced by a recording stand-in; the rest of the library is the
real one).

A workspace holds the shared covariance plan, which the device builds in
milliseconds on first use, followed by one forward call's residuals.  The
torch autograd path returns a workspace to the pool once its backward call
is enqueued (or at once when no gradient is needed), and the next forward
call on the same device, stream and size reuses it; a second backward
through a released forward call is refused.
"""

import ctypes
import types

import pytest
import torch


class _RecordingLib:
    def __init__(self, real, nbytes=4096):
        self._real = real
        self.nbytes = nbytes
        self.calls = []

    def __getattr__(self, name):
        return getattr(self._real, name)

    def pdq_lml_adjoint_workspace_size(self, cfg, B, num_steps, save_every, ckpt, out):
        ctypes.cast(out, ctypes.POINTER(ctypes.c_size_t))[0] = self.nbytes
        return 0

    def pdq_lml_fwd(self, cfg, args, ws, nbytes, stream):
        self.calls.append(("fwd", ws.value))
        return 0

    def pdq_lml_bwd(self, cfg, args, ws, nbytes, stream):
        self.calls.append(("bwd", ws.value))
        return 0


@pytest.fixture()
def fake(monkeypatch):
    from probdiffeq_gb300 import _native
    from probdiffeq_gb300 import build as native_build

    native_build.build()
    lib = _RecordingLib(_native.load())
    monkeypatch.setattr(_native, "load", lambda: lib)
    monkeypatch.setattr(_native, "_LML_ADJ_POOL", {})
    return lib


def _inputs(B=4):
    params = torch.full((B, 3), 0.2, dtype=torch.float64)
    y0 = torch.zeros((B, 2), dtype=torch.float64)
    data = torch.zeros((21, 2), dtype=torch.float64)
    std = torch.full((21,), 0.01, dtype=torch.float64)
    return params, y0, data, std


STREAM = types.SimpleNamespace(cuda_stream=0)
KW = dict(dt=0.01, num_steps=200, save_every=10, stream=STREAM)


def test_backward_returns_the_workspace_for_the_next_forward(fake):
    from probdiffeq_gb300 import autograd

    params, y0, data, std = _inputs()
    p1 = params.clone().requires_grad_(True)
    lml1, _ = autograd.lml(p1, y0, data, std, mode="adjoint", **KW)
    lml1.sum().backward()
    p2 = params.clone().requires_grad_(True)
    lml2, _ = autograd.lml(p2, y0, data, std, mode="adjoint", **KW)
    lml2.sum().backward()
    kinds = [k for k, _ in fake.calls]
    assert kinds == ["fwd", "bwd", "fwd", "bwd"]
    ws = [w for _, w in fake.calls]
    assert ws[0] == ws[1] == ws[2] == ws[3]  # one workspace, its plan reused
    assert p1.grad is not None and p1.grad.shape == params.shape


def test_forward_calls_in_flight_get_distinct_workspaces(fake):
    from probdiffeq_gb300 import autograd

    params, y0, data, std = _inputs()
    p = params.clone().requires_grad_(True)
    a, _ = autograd.lml(p, y0, data, std, mode="adjoint", **KW)
    b, _ = autograd.lml(p, y0, data, std, mode="adjoint", **KW)
    (a.sum() + b.sum()).backward()
    fwd_ws = [w for k, w in fake.calls if k == "fwd"]
    bwd_ws = [w for k, w in fake.calls if k == "bwd"]
    assert fwd_ws[0] != fwd_ws[1]
    assert sorted(bwd_ws) == sorted(fwd_ws)


def test_no_gradient_releases_at_once_and_double_backward_is_refused(fake):
    from probdiffeq_gb300 import _native, autograd, ensemble

    params, y0, data, std = _inputs()
    autograd.lml(params, y0, data, std, mode="adjoint", **KW)  # no grad needed
    autograd.lml(params, y0, data, std, mode="adjoint", **KW)
    ws = [w for _, w in fake.calls]
    assert ws[0] == ws[1]
    cfg = ensemble.make_config(field="fitzhugh_nagumo", num_derivatives=3, ode_dim=2, ssm="isotropic",
                               strategy="fixedpoint", solver="none", precision="float32")
    fwd = _native.lml_fwd(cfg, params, y0, data, std, t0=0.0, **KW)
    _native.lml_bwd(fwd, None, release=True)
    with pytest.raises(RuntimeError, match="released"):
        _native.lml_bwd(fwd, None)


def test_ivpsolve_lml_fixed_grid_adjoint_mode_plumbing(fake):
    """ivpsolve.lml_fixed_grid(gradient="adjoint") runs the forward and the
    backward call on one workspace, returns (lml, d/d params, status,
    d/d y0) and pools the workspace; an unknown mode is refused."""
    import numpy as np

    from probdiffeq_gb300 import _native, ivpsolve, probdiffeq

    thetas = torch.tensor([[0.2, 0.2, 3.0], [0.21, 0.19, 3.1]], dtype=torch.float64)
    y0 = torch.tensor(np.tile([-1.0, 1.0], (2, 1)), dtype=torch.float64)
    vf = probdiffeq.ode("fitzhugh_nagumo", thetas)
    tcoeffs, _ = probdiffeq.jetexpand_ode_padded_scan(num=3)(vf, (y0,))
    prior = probdiffeq.state_space_model_isotropic().prior_wiener_integrated(tcoeffs)
    data = np.zeros((21, 2))
    out = ivpsolve.lml_fixed_grid(prior, data, 0.01, dt=0.01, num_steps=200, save_every=10, gradient="adjoint",
                                  device="cpu", stream=STREAM)
    assert len(out) == 4
    lml, grad, status, grad_y0 = out
    assert lml.shape == (2,) and grad.shape == (2, 3) and status.shape == (2,) and grad_y0.shape == (2, 2)
    assert [k for k, _ in fake.calls] == ["fwd", "bwd"]
    assert fake.calls[0][1] == fake.calls[1][1]
    assert sum(len(v) for v in _native._LML_ADJ_POOL.values()) == 1
    with pytest.raises(ValueError, match="gradient must be"):
        ivpsolve.lml_fixed_grid(prior, data, 0.01, dt=0.01, num_steps=200, save_every=10, gradient="reverse",
                                device="cpu", stream=STREAM)
