"""The headline configuration at its own size and horizon (GPU).

512 instances of the 16384-instance Lotka--Volterra benchmark distribution
(``probdiffeq_gb300.configs.lv_ensemble``, seed 0), t in [0, 50], IWP with
nu = 4, isotropic TS0, filter, MLE calibration, rtol = atol = 1e-6, terminal
values with clip_dt -- the benchmark's configuration, through the C ABI:

* float64 kernel vs the float64 C port of the reference algorithm
  (``oracle/port``): terminal u within 1e-9 relative (to the instance's
  largest component), accepted steps within +-1, the output scale within 1e-6.
* float32 kernel vs the exact solution (fixed-step RK4, h = 1e-3, which
  agrees with DOP853 at rtol 1e-13 to ~1e-12): its terminal error stays
  within 2x the float64 kernel's own error against the same solution, in the
  median and at the maximum over the instances, and its mean attempt count
  within 2 % of the float64 kernel's.  This is the "matched accuracy"
  condition: the float32 bulk arithmetic must not add error beyond the
  solver's own discretisation error at rtol 1e-6.
"""

import numpy as np
import pytest
import torch

from probdiffeq_gb300 import configs, ensemble

pytestmark = pytest.mark.gpu

B = 512


def _solve(precision, params, y0):
    cfg = ensemble.make_config(field="lotka_volterra", num_derivatives=4, ode_dim=2, solver="mle", precision=precision,
                               atol=1e-6, rtol=1e-6)
    out = ensemble.solve_ensemble(cfg, params=params, y0=y0, save_at=torch.tensor(configs.LV_T_SPAN), device="cuda:0")
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in out.items() if not k.startswith("_")}


def _rel(u, ref):
    return np.abs(u - ref).max(axis=1) / np.abs(ref).max(axis=1)


@pytest.fixture(scope="module")
def runs():
    params, y0 = configs.lv_ensemble(B, seed=0)
    return {
        "params": params, "y0": y0,
        "f64": _solve("float64", params, y0),
        "f32": _solve("float32", params, y0),
        "truth": configs.lv_truth(params.numpy(), y0.numpy()),
    }


def test_float64_kernel_matches_c_port_at_full_horizon(runs):
    from oracle.port import port

    ref = port.solve_iso_terminal("lotka_volterra", runs["params"].numpy(), runs["y0"].numpy(), 4, "mle", atol=1e-6,
                                  rtol=1e-6, t0=0.0, t1=50.0)
    out = runs["f64"]
    assert (out["status"] == 0).all()
    err = _rel(out["u_mean"][:, 0, 0], ref["mean"][:, 0])
    assert err.max() <= 1e-9, err.max()
    steps = out["num_steps"][:, 0].astype(np.int64)
    assert np.abs(steps - ref["num_steps"]).max() <= 1
    scale = out["output_scale"][:, 0]
    assert np.abs(scale - ref["output_scale"]).max() <= 1e-6 * np.abs(ref["output_scale"]).max()


def test_float32_kernel_has_float64_accuracy_at_full_horizon(runs):
    f32, f64, truth = runs["f32"], runs["f64"], runs["truth"]
    assert (f32["status"] == 0).all()
    e32 = _rel(f32["u_mean"][:, 0, 0], truth)
    e64 = _rel(f64["u_mean"][:, 0, 0], truth)
    assert np.median(e32) <= 2.0 * np.median(e64), (np.median(e32), np.median(e64))
    assert e32.max() <= 2.0 * e64.max(), (e32.max(), e64.max())
    a32 = f32["num_attempts"].astype(np.float64).mean()
    a64 = f64["num_attempts"].astype(np.float64).mean()
    assert abs(a32 - a64) <= 0.02 * a64, (a32, a64)
    assert np.isfinite(f32["u_chol"]).all() and (f32["output_scale"] > 0).all()
