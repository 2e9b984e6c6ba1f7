"""The autotuner on the GPU: every candidate launch shape runs and agrees
with the default mapping, the tuned choice is cached per batch class."""

import pytest
import torch

from probdiffeq_gb300 import _native, autotune, ensemble

pytestmark = pytest.mark.gpu

LV = torch.tensor([0.5, 0.05, 0.5, 0.05], dtype=torch.float64)


def lv_batch(B, seed=0):
    g = torch.Generator().manual_seed(seed)
    params = (LV * torch.exp(0.2 * torch.randn((B, 4), generator=g, dtype=torch.float64))).cuda()
    y0 = (10.0 + 20.0 * torch.rand((B, 2), generator=g, dtype=torch.float64)).cuda()
    return params, y0


def test_every_isotropic_candidate_matches_the_default_mapping():
    B = 200
    params, y0 = lv_batch(B)
    save_at = torch.tensor([[0.0, 10.0]], dtype=torch.float64, device="cuda").expand(B, 2).contiguous()
    dt0 = torch.full((B,), 0.1, dtype=torch.float64, device="cuda")
    cfg = ensemble.make_config(field="lotka_volterra", num_derivatives=4, ode_dim=2, solver="mle", precision="float64",
                               clip_dt=True)
    ref = _native.solve_adaptive(cfg, save_at, params, y0, dt0, True, _native.alloc_outputs(cfg, B, 2, True, "cuda"))
    torch.cuda.synchronize()
    best, times = autotune.tune(cfg, save_at, params, y0, dt0, True)
    assert set(times) == set(autotune.candidates(cfg)) and best in times
    for v, ipb in autotune.candidates(cfg):
        c = ensemble.make_config(field="lotka_volterra", num_derivatives=4, ode_dim=2, solver="mle",
                                 precision="float64", clip_dt=True, kernel_variant=v, instances_per_block=ipb)
        out = _native.solve_adaptive(c, save_at, params, y0, dt0, True, _native.alloc_outputs(c, B, 2, True, "cuda"))
        torch.cuda.synchronize()
        assert (out["status"] == 0).all()
        # the mappings differ in summation order, so an instance may take one step more or
        # less; the terminal values then differ at the level of the tolerance (1e-6)
        err = ((out["u_mean"] - ref["u_mean"]).abs() / ref["u_mean"].abs().clamp_min(1e-12)).max().item()
        assert err < 1e-5, ((v, ipb), err)
        assert (out["num_steps"] - ref["num_steps"]).abs().max().item() <= 1
        if ipb in (0, 64, 32) and v == 1:
            assert torch.equal(out["u_mean"], ref["u_mean"])  # launch shape alone changes nothing


def test_tuned_config_is_cached_and_used_by_solve_ensemble(monkeypatch):
    autotune.clear_cache()
    B = 300
    params, y0 = lv_batch(B, seed=1)
    cfg = ensemble.make_config(field="lotka_volterra", num_derivatives=4, ode_dim=2, solver="mle", clip_dt=True)
    calls = []
    real = autotune.tune
    monkeypatch.setattr(autotune, "tune", lambda *a, **k: calls.append(1) or real(*a, **k))
    for _ in range(3):
        out = ensemble.solve_ensemble(cfg, params=params, y0=y0, save_at=torch.tensor([0.0, 10.0]), autotune=True)
        torch.cuda.synchronize()
        assert (out["status"] == 0).all()
    assert len(calls) == 1


def test_dense_candidates_run():
    B = 6
    mu = torch.linspace(1.0, 2.0, B, dtype=torch.float64, device="cuda")[:, None]
    y0 = torch.tensor([[2.0, 0.0]], dtype=torch.float64, device="cuda").expand(B, 2).contiguous()
    save_at = torch.tensor([[0.0, 2.0]], dtype=torch.float64, device="cuda").expand(B, 2).contiguous()
    dt0 = torch.full((B,), 0.1, dtype=torch.float64, device="cuda")
    cfg = ensemble.make_config(field="van_der_pol", num_derivatives=3, ode_dim=2, ssm="dense", constraint="ts1",
                               precision="float64", atol=1e-5, rtol=1e-5, clip_dt=False)
    best, times = autotune.tune(cfg, save_at, mu, y0, dt0, True)
    assert set(times) == set(autotune.candidates(cfg))
