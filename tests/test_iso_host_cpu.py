"""The headline isotropic kernel's float64 body run on the CPU against the
golden fixtures.

``tests/hostsim/iso_host.cpp`` compiles ``iso_adaptive_kernel`` (one thread
per instance, Lotka--Volterra, the lean TS0 / error_residual_std
instantiation the library launches for the filter) with the host compiler
under AddressSanitizer and UBSan and runs every instance on buffers of the
library's sizes.  Its records are compared with ``tests/golden/lv_filter.json``
(the oracle's outputs) with the GPU parity tests' float64 tolerances: the
solution row within 1e-9, every row and L L^T within 1e-6, accepted steps
within +-1, the MLE output scale within 1e-6.  The same source compiled for
sm_103a is checked against the same fixtures by ``tests/test_golden_gpu.py``.
"""

import numpy as np
import pytest

from tests import hostsim
from tests.golden import make_golden

SOLVER = {"mle": 1, "dynamic": 2}


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    return hostsim.compile_harness("iso_host.cpp", tmp_path_factory.mktemp("hostsim") / "iso_host")


def q1_iwp(nu):
    n = nu + 1
    H = np.array([[1.0 / (2 * nu + 1 - i - j) for j in range(n)] for i in range(n)])
    return np.linalg.cholesky(H)


@pytest.mark.parametrize("run", ["mle_terminal", "dynamic_save_at"])
def test_host_iso_kernel_matches_golden_records(harness, tmp_path, run):
    gold = make_golden.load("lv_filter.json")
    r = gold[run]
    nu, n, d = gold["num_derivatives"], gold["num_derivatives"] + 1, 2
    params, y0 = np.array(gold["params"]), np.array(gold["y0"])
    B, S = params.shape[0], len(r["save_at"])
    terminal = run == "mle_terminal"
    solver = SOLVER["mle" if terminal else "dynamic"]
    head = [nu, B, S, solver, 0, int(r["clip_dt"]), int(terminal)]
    body = np.concatenate([[r["atol"], r["rtol"]], np.tile(r["save_at"], B), params.ravel(), y0.ravel(),
                           np.full(B, gold["dt0"]), q1_iwp(nu).ravel()])
    path = tmp_path / "input.txt"
    path.write_text(" ".join(str(v) for v in head) + " " + " ".join(repr(float(v)) for v in body))
    lines = hostsim.run_harness(harness, path)
    points = [S - 1] if terminal else list(range(S))
    per = 1 + len(points)
    assert len(lines) == B * per
    for b, rec in enumerate(r["records"]):
        status, attempts = (int(x) for x in lines[b * per].split())
        assert status == 0 and attempts > 0
        for k, s in enumerate(points):
            vals = [float(x) for x in lines[b * per + 1 + k].split()]
            t, steps, scale = vals[0], int(vals[1]), vals[2]
            gm = np.array(vals[3:3 + n * d]).reshape(n, d)
            gc = np.array(vals[3 + n * d:]).reshape(n, n)
            om, oc = np.array(rec["u_mean"][s]), np.array(rec["u_chol"][s])
            assert abs(t - r["save_at"][s]) < 1e-7
            assert float(np.abs(gm[0] - om[0]).max() / np.abs(om[0]).max()) <= 1e-9, (b, s)
            for i in range(n):
                assert float(np.abs(gm[i] - om[i]).max() / max(np.abs(om[i]).max(), 1e-300)) <= 1e-6, (b, s, i)
            cg, co = gc @ gc.T, oc @ oc.T
            assert float(np.abs(cg - co).max() / max(np.abs(co).max(), 1e-300)) <= 1e-6, (b, s)
            steps_o = 0 if s == 0 else rec["num_steps"][s - 1]
            assert abs(steps - steps_o) <= 1, (b, s, steps, steps_o)
            if terminal:
                so = rec["output_scale"][-1]
                assert abs(scale - so) <= 1e-6 * abs(so), (scale, so)
