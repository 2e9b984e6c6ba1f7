"""The split isotropic filter (kernel_variant 4, ``iso_split_kernel``: a
covariance warp and a mean warp per 32 instances) on the GPU.

It runs the one-thread kernel's arithmetic with the work of an attempt dealt
to two warps, so its outputs equal the one-thread kernel's (kernel_variant 1)
bit for bit -- means, factors, output scales, times, steps, attempts and
statuses -- for the three built-in fields, float64 and float32 bulk, solver
none and mle, terminal values and save_at records, ragged batch sizes, at
the headline size (16384 Lotka--Volterra instances on [0, 50]) and for the
failure statuses.  Configurations it does not cover are rejected before
launch.
"""

import pytest
import torch

from probdiffeq_gb300 import _native, ensemble

pytestmark = pytest.mark.gpu

FIELDS = {
    "lotka_volterra": ([0.5, 0.05, 0.5, 0.05], [20.0, 20.0], 0.2, 10.0),
    "van_der_pol": ([3.0], [2.0, 0.0], 0.3, 2.0),
    "fitzhugh_nagumo": ([0.2, 0.2, 3.0], [-1.0, 1.0], 0.2, 0.5),
}


def batch(field, B, seed=0):
    p, y, sp, sy = FIELDS[field]
    g = torch.Generator().manual_seed(seed)
    params = torch.tensor(p, dtype=torch.float64) * torch.exp(sp * torch.randn((B, len(p)), generator=g,
                                                                                 dtype=torch.float64))
    z = torch.randn((B, 2), generator=g, dtype=torch.float64)
    base = torch.tensor(y, dtype=torch.float64)
    # Lotka--Volterra populations stay positive (log-normal); the others shift additively
    y0 = base * torch.exp(0.3 * z) if field == "lotka_volterra" else base + sy * z
    return params, y0


def solve(variant, field, params, y0, save_at, *, nu=4, solver="mle", precision="float32", terminal_only=True,
          rtol=1e-6, **kw):
    cfg = ensemble.make_config(field=field, num_derivatives=nu, ode_dim=2, solver=solver, precision=precision,
                               atol=rtol, rtol=rtol, clip_dt=True, kernel_variant=variant, **kw)
    out = ensemble.solve_ensemble(cfg, params=params, y0=y0, save_at=torch.tensor(save_at, dtype=torch.float64),
                                  terminal_only=terminal_only, device="cuda:0")
    torch.cuda.synchronize()
    return {k: v.cpu() for k, v in out.items()}


def assert_same(a, b):
    assert a.keys() == b.keys()
    for k in a:
        assert torch.equal(a[k].nan_to_num(12345.0), b[k].nan_to_num(12345.0)), k


@pytest.mark.parametrize("precision", ["float32", "float64"])
@pytest.mark.parametrize("solver", ["mle", "none"])
@pytest.mark.parametrize("field", list(FIELDS))
def test_split_equals_one_thread_terminal(field, solver, precision):
    params, y0 = batch(field, 100, seed=1)
    t1 = {"lotka_volterra": 30.0, "van_der_pol": 6.0, "fitzhugh_nagumo": 20.0}[field]
    one = solve("thread", field, params, y0, [0.0, t1], solver=solver, precision=precision, rtol=1e-5)
    split = solve("split", field, params, y0, [0.0, t1], solver=solver, precision=precision, rtol=1e-5)
    assert (one["status"] == 0).all()
    assert_same(split, one)


@pytest.mark.parametrize("precision", ["float32", "float64"])
@pytest.mark.parametrize("nu", [2, 3, 4, 5])
def test_split_equals_one_thread_save_at(nu, precision):
    """A repeated and a close pair of checkpoints.  With nu = 5 a step
    clipped to 1e-3 at a checkpoint leaves some of these instances without a
    finite error estimate (the oracle's float64 solve of instance 6 exceeds
    its attempt bound there too), so nu = 5 compares the statuses as well
    and asks most instances to finish."""
    params, y0 = batch("lotka_volterra", 70, seed=2)
    save_at = [0.0, 0.5, 0.5 + 1e-3, 3.0, 3.0, 7.25, 12.0]
    one = solve("thread", "lotka_volterra", params, y0, save_at, nu=nu, precision=precision, terminal_only=False,
                rtol=1e-5)
    split = solve("split", "lotka_volterra", params, y0, save_at, nu=nu, precision=precision, terminal_only=False,
                  rtol=1e-5)
    if nu < 5:
        assert (one["status"] == 0).all()
    else:
        assert (one["status"] == 0).sum() >= 50
    assert_same(split, one)


@pytest.mark.parametrize("B", [1, 31, 33, 97])
def test_split_ragged_batches(B):
    params, y0 = batch("lotka_volterra", B, seed=3)
    one = solve("thread", "lotka_volterra", params, y0, [0.0, 10.0], nu=3)
    split = solve("split", "lotka_volterra", params, y0, [0.0, 10.0], nu=3)
    assert_same(split, one)


def test_split_headline_size():
    """16384 instances of the benchmark's Lotka--Volterra distribution on [0, 50], nu = 4, MLE, rtol 1e-6."""
    import bench

    params, y0 = bench.lv_inputs(16384, seed=0)
    one = solve("thread", "lotka_volterra", params, y0, [0.0, 50.0])
    split = solve("split", "lotka_volterra", params, y0, [0.0, 50.0])
    assert (one["status"] == 0).all()
    assert_same(split, one)


def test_split_failure_statuses():
    params, y0 = batch("lotka_volterra", 40, seed=4)
    y0[5, 0] = float("nan")
    one = solve("thread", "lotka_volterra", params, y0, [0.0, 5.0], nu=2)
    split = solve("split", "lotka_volterra", params, y0, [0.0, 5.0], nu=2)
    assert int(split["status"][5]) == 3  # NONFINITE
    assert_same(split, one)
    one = solve("thread", "lotka_volterra", params, y0, [0.0, 50.0], nu=2, max_attempts=7)
    split = solve("split", "lotka_volterra", params, y0, [0.0, 50.0], nu=2, max_attempts=7)
    assert int(split["status"][0]) == 1 and int(split["num_attempts"][0]) == 7  # MAX_STEPS
    assert_same(split, one)


def test_split_rejects_what_it_does_not_cover():
    params, y0 = batch("lotka_volterra", 4)
    for kw in (dict(solver="dynamic"), dict(damp=1e-3), dict(constraint="ts1"), dict(error="state_std"),
               dict(strategy="fixedpoint"), dict(instances_per_block=32)):
        with pytest.raises(_native.NativeError):
            solve("split", "lotka_volterra", params, y0, [0.0, 1.0], **kw)
    with pytest.raises(_native.NativeError):
        cfg = ensemble.make_config(field="lotka_volterra", num_derivatives=4, ode_dim=2, clip_dt=False,
                                   kernel_variant="split")
        ensemble.solve_ensemble(cfg, params=params, y0=y0, save_at=torch.tensor([0.0, 1.0]), device="cuda:0")
