"""The oracle against the committed golden fixtures (``tests/golden``).

The fixtures were written by ``tests/golden/make_golden.py`` from the
oracle; re-running it must reproduce them (float64, 1e-10 relative: only
the host's BLAS and libm may differ).  The GPU tests compare the CUDA
kernels with the same fixtures (``tests/test_golden_gpu.py``), so a change
in either side shows up against a fixed record.
"""

import numpy as np
import torch

from tests.golden import make_golden


def close(a, b, tol=1e-10):
    a, b = np.asarray(a, dtype=float), np.asarray(b, dtype=float)
    assert a.shape == b.shape, (a.shape, b.shape)
    scale = max(float(np.abs(b).max()), 1e-300)
    assert float(np.abs(a - b).max()) <= tol * scale, (a, b)


def test_iwp_fixture():
    gold = make_golden.load("iwp.json")
    now = make_golden.iwp_fixture()
    assert sorted(gold) == ["2", "3", "4"]
    for nu in gold:
        for key in ("A", "Q", "p", "p_inv"):
            close(now[nu][key], gold[nu][key], 1e-14)
        # A1 is flip(Pascal) and Q1 Q1^T = flip(Hilbert) (utilities.py:57-71)
        A, Q = np.array(gold[nu]["A"]), np.array(gold[nu]["Q"])
        n = A.shape[0]
        H = np.array([[1.0 / (2 * n - 1 - i - j) for j in range(n)] for i in range(n)])
        close(Q @ Q.T, H, 1e-14)
        assert np.allclose(np.triu(Q, 1), 0) and (np.diag(Q) >= 0).all()


def test_lv_filter_fixture():
    gold = make_golden.load("lv_filter.json")
    now = make_golden.lv_filter_fixture(torch.tensor(gold["params"]), torch.tensor(gold["y0"]))
    for run in ("mle_terminal", "dynamic_save_at"):
        for rg, rn in zip(gold[run]["records"], now[run]["records"]):
            assert rg["num_steps"] == rn["num_steps"]
            close(rn["u_mean"], rg["u_mean"])
            close(rn["u_chol"], rg["u_chol"])
            close(rn["output_scale"], rg["output_scale"])


def test_fhn_lml_fixture():
    gold = make_golden.load("fhn_lml.json")
    inputs = (gold["num_steps"], np.array(gold["data"]), np.array(gold["params"]), np.array(gold["y0"]))
    now = make_golden.fhn_lml_fixture(inputs)
    close(now["lml"], gold["lml"])
    close(now["grad"], gold["grad"], 1e-9)
    close(now["grad_y0"], gold["grad_y0"], 1e-9)


def test_vdp_dense_fixture():
    gold = make_golden.load("vdp_dense.json")
    now = make_golden.vdp_dense_fixture(gold["mu"])
    for rg, rn in zip(gold["records"], now["records"]):
        assert rg["num_steps"] == rn["num_steps"]
        close(rn["u_mean"], rg["u_mean"])
        close(rn["u_chol"], rg["u_chol"])


def test_lv_fixedpoint_fixture():
    gold = make_golden.load("lv_fixedpoint.json")
    now = make_golden.lv_fixedpoint_fixture(torch.tensor(gold["params"]), torch.tensor(gold["y0"]))
    for rg, rn in zip(gold["records"], now["records"]):
        assert rg["num_steps"] == rn["num_steps"]
        close(rn["u_mean"], rg["u_mean"])
        close(rn["u_chol"], rg["u_chol"])
        close(rn["output_scale"], rg["output_scale"])


def test_lv_sensitivities_fixture():
    gold = make_golden.load("lv_sensitivities.json")
    now = make_golden.lv_sensitivities_fixture(torch.tensor(gold["params"]), torch.tensor(gold["y0"]))
    for rg, rn in zip(gold["records"], now["records"]):
        assert rg["num_steps"] == rn["num_steps"]
        close(rn["u_mean"], rg["u_mean"])
        close(rn["d_params"], rg["d_params"], 1e-9)
        close(rn["d_y0"], rg["d_y0"], 1e-9)
