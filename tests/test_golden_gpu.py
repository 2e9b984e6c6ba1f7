"""The CUDA kernels against the committed golden fixtures (``tests/golden``).

The fixtures hold seeded inputs and the oracle's float64 outputs (written by
``tests/golden/make_golden.py``; ``tests/test_golden_cpu.py`` checks that
the oracle still reproduces them), so these tests need no oracle run.
Float64 bulk, the tolerances of the live-oracle parity tests: the solution
row u within 1e-9 relative, every Taylor row and the covariance L L^T within
1e-6, accepted steps within +-1, the MLE output scale within 1e-6; LML
within 1e-9 and its gradients within 1e-6 of their norm.
"""

import math

import numpy as np
import pytest
import torch

from tests.golden import make_golden

pytestmark = pytest.mark.gpu

F64 = dict(dtype=torch.float64, device="cuda")


def rel_rows(g, o):
    return max(float(np.abs(g[i] - o[i]).max() / max(np.abs(o[i]).max(), 1e-300)) for i in range(o.shape[0]))


@pytest.mark.parametrize("run", ["mle_terminal", "dynamic_save_at"])
def test_lv_filter_matches_fixture(run):
    from probdiffeq_gb300 import ensemble

    gold = make_golden.load("lv_filter.json")
    r = gold[run]
    solver = "mle" if run == "mle_terminal" else "dynamic"
    terminal = run == "mle_terminal"
    cfg = ensemble.make_config(field="lotka_volterra", num_derivatives=4, ode_dim=2, solver=solver,
                               precision="float64", atol=r["atol"], rtol=r["rtol"], clip_dt=r["clip_dt"])
    out = ensemble.solve_ensemble(cfg, params=torch.tensor(gold["params"], dtype=torch.float64),
                                  y0=torch.tensor(gold["y0"], dtype=torch.float64),
                                  save_at=torch.tensor(r["save_at"], dtype=torch.float64), dt0=gold["dt0"],
                                  terminal_only=terminal)
    torch.cuda.synchronize()
    out = {k: v.cpu().numpy() for k, v in out.items() if not k.startswith("_")}
    assert (out["status"] == 0).all()
    points = [len(r["save_at"]) - 1] if terminal else list(range(len(r["save_at"])))
    for b, rec in enumerate(r["records"]):
        for k, s in enumerate(points):
            gm, gc = out["u_mean"][b, k], out["u_chol"][b, k]
            om, oc = np.array(rec["u_mean"][s]), np.array(rec["u_chol"][s])
            assert float(np.abs(gm[0] - om[0]).max() / np.abs(om[0]).max()) <= 1e-9, (b, s)
            assert rel_rows(gm, om) <= 1e-6, (b, s)
            cg, co = gc @ gc.T, oc @ oc.T
            assert float(np.abs(cg - co).max() / max(np.abs(co).max(), 1e-300)) <= 1e-6, (b, s)
            steps_o = 0 if s == 0 else rec["num_steps"][s - 1]
            assert abs(int(out["num_steps"][b, k]) - steps_o) <= 1, (b, s, int(out["num_steps"][b, k]), steps_o)
            assert abs(float(out["t"][b, k]) - r["save_at"][s]) < 1e-7
        if terminal:
            so, sg = rec["output_scale"][-1], float(out["output_scale"][b, 0])
            assert math.isfinite(sg) and abs(sg - so) <= 1e-6 * abs(so), (sg, so)


def test_fhn_lml_forward_mode_and_adjoint_match_fixture():
    from probdiffeq_gb300 import _native, ensemble

    gold = make_golden.load("fhn_lml.json")
    cfg = ensemble.make_config(field="fitzhugh_nagumo", num_derivatives=3, ode_dim=2, ssm="isotropic",
                               strategy="fixedpoint", solver="none", precision="float64")
    params, y0 = torch.tensor(gold["params"], **F64), torch.tensor(gold["y0"], **F64)
    data = torch.tensor(gold["data"], **F64)
    std = torch.full((data.shape[0],), gold["std"], **F64)
    kw = dict(t0=0.0, dt=gold["dt"], num_steps=gold["num_steps"], save_every=gold["save_every"])
    fm = _native.lml_fixed_grid(cfg, params, y0, data, std, gradient=True, **kw)
    fwd = _native.lml_fwd(cfg, params, y0, data, std, **kw)
    bwd = _native.lml_bwd(fwd, None, params_grad=True, y0_grad=True)
    torch.cuda.synchronize()
    assert (fm["status"] == 0).all() and (fwd["status"] == 0).all()
    for b in range(len(gold["lml"])):
        v, g, gy = gold["lml"][b], np.array(gold["grad"][b]), np.array(gold["grad_y0"][b])
        for lml in (float(fm["lml"][b]), float(fwd["lml"][b])):
            assert abs(lml - v) <= 1e-9 * abs(v), (lml, v)
        for grad in (fm["grad"][b].cpu().numpy(), bwd["grad"][b].cpu().numpy()):
            assert np.abs(grad - g).max() <= 1e-6 * np.linalg.norm(g), (grad, g)
        gyb = bwd["grad_y0"][b].cpu().numpy()
        assert np.abs(gyb - gy).max() <= 1e-6 * np.linalg.norm(gy), (gyb, gy)
