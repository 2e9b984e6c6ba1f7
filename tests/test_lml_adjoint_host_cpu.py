"""The LML kernels' float64 bodies run on the CPU against the oracle: the
adjoint pair and the forward-mode kernel.

``tests/hostsim`` compiles the kernel templates of ``lml_adjoint.cuh`` with
the host compiler (a stand-in for ``cuda_runtime.h`` turns the CUDA
qualifiers into no-ops) under AddressSanitizer and UBSan, and runs the plan
kernel's thread and every sample's value and adjoint pass one after another
on buffers of exactly the size the library computes.  This pins the adjoint
algebra and the residual layout without a GPU: value, d/d params and d/d y0
against the oracle's PyTorch reverse mode to 1e-10 relative, for sqrt(N),
single-step, ragged and whole-grid checkpoint spacings, averaged pdfs and
non-unit cotangents, for FitzHugh--Nagumo with nu = 3 and nu = 2 and for
Lotka--Volterra (four parameters).  The GPU tests check the same kernels
compiled for sm_103a.
"""

import numpy as np
import pytest

from tests import hostsim
from tests import lml_problem
from tests.lml_oracle import lml_value_and_grads



@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    return hostsim.compile_harness("lml_adjoint_host.cpp", tmp_path_factory.mktemp("hostsim") / "lml_adjoint_host")


def q1_iwp(nu):
    """Lower Cholesky factor of flip(Hilbert), (Q1 Q1^T)[i, j] = 1 / (2 nu + 1 - i - j)."""
    n = nu + 1
    H = np.array([[1.0 / (2 * nu + 1 - i - j) for j in range(n)] for i in range(n)])
    return np.linalg.cholesky(H)


def run(harness, tmp_path, thetas, y0s, data, dt, num_steps, save_every, ckpt, average, cot, field=0, nu=3,
        std=lml_problem.STD, precision=1):
    B = len(thetas)
    head = [precision, field, nu, B, num_steps, save_every, ckpt, int(average)]
    body = np.concatenate([np.ravel(thetas), np.ravel(y0s), np.ravel(data), np.full(data.shape[0], std),
                           np.asarray(cot, dtype=float), [dt], np.ravel(q1_iwp(nu))])
    path = tmp_path / "input.txt"
    path.write_text(" ".join(str(int(v)) for v in head) + " " + " ".join(repr(float(v)) for v in body))
    return np.array([[float(x) for x in line.split()] for line in hostsim.run_harness(harness, path)])


@pytest.mark.parametrize("t1,ckpt,average", [(2.0, 14, False), (2.0, 1, False), (2.0, 7, True), (2.0, 200, False),
                                             (20.0, 45, False)])
def test_host_adjoint_matches_oracle_reverse_mode(harness, tmp_path, t1, ckpt, average):
    dt, save_every = 0.01, 10
    num_steps, data = lml_problem.observations(t1=t1, dt=dt, save_every=save_every)
    thetas = lml_problem.theta_samples(3, seed=1)
    y0s = np.tile(lml_problem.U0, (3, 1)) + np.array([[0.0, 0.0], [0.1, -0.05], [-0.02, 0.03]])
    cot = [1.0, -0.5, 2.0]
    out = run(harness, tmp_path, thetas, y0s, data, dt, num_steps, save_every, ckpt, average, cot)
    assert out.shape == (3, 7)
    for b in range(3):
        v, g, gy = lml_value_and_grads(thetas[b], y0s[b], data, dt, num_steps, save_every, average_pdfs=average)
        assert out[b, 0] == 0
        assert abs(out[b, 1] - v) <= 1e-10 * abs(v), (out[b, 1], v)
        assert np.abs(out[b, 2:5] - cot[b] * g).max() <= 1e-10 * np.linalg.norm(cot[b] * g), (out[b, 2:5], g)
        assert np.abs(out[b, 5:7] - cot[b] * gy).max() <= 1e-10 * np.linalg.norm(cot[b] * gy), (out[b, 5:7], gy)


@pytest.mark.parametrize("field,nu", [("fitzhugh_nagumo", 2), ("lotka_volterra", 3)])
def test_host_adjoint_other_instantiations(harness, tmp_path, field, nu):
    """The library's other adjoint instantiations: FitzHugh--Nagumo with
    nu = 2, and Lotka--Volterra (four parameters) on seeded synthetic data."""
    rng = np.random.default_rng(3)
    if field == "fitzhugh_nagumo":
        dt, num_steps, save_every, std = 0.01, 200, 10, lml_problem.STD
        _, data = lml_problem.observations(t1=2.0, dt=dt, save_every=save_every)
        thetas = lml_problem.theta_samples(2, seed=4)
        y0s = np.tile(lml_problem.U0, (2, 1))
        code = 0
    else:
        dt, num_steps, save_every, std = 0.05, 200, 20, 0.5
        data = 20.0 + 5.0 * rng.standard_normal((num_steps // save_every + 1, 2))
        thetas = np.array([0.5, 0.05, 0.5, 0.05]) * np.exp(0.1 * rng.standard_normal((2, 4)))
        y0s = 20.0 + rng.uniform(-2, 2, (2, 2))
        code = 1
    cot = [1.0, -2.0]
    out = run(harness, tmp_path, thetas, y0s, data, dt, num_steps, save_every, 11, False, cot, field=code, nu=nu,
              std=std)
    P = thetas.shape[1]
    assert out.shape == (2, 2 + P + 2)
    for b in range(2):
        v, g, gy = lml_value_and_grads(thetas[b], y0s[b], data, dt, num_steps, save_every, field=field,
                                       num_derivatives=nu, std=std)
        assert out[b, 0] == 0
        assert abs(out[b, 1] - v) <= 1e-10 * abs(v), (out[b, 1], v)
        assert np.abs(out[b, 2:2 + P] - cot[b] * g).max() <= 1e-10 * np.linalg.norm(cot[b] * g), (out[b, 2:2 + P], g)
        assert np.abs(out[b, 2 + P:] - cot[b] * gy).max() <= 1e-10 * np.linalg.norm(cot[b] * gy), (out[b, 2 + P:], gy)


@pytest.fixture(scope="module")
def forward_harness(tmp_path_factory):
    return hostsim.compile_harness("lml_forward_host.cpp", tmp_path_factory.mktemp("hostsim") / "lml_forward_host")


@pytest.mark.parametrize("t1,average", [(2.0, False), (2.0, True), (20.0, False)])
def test_host_forward_mode_lml_matches_oracle(forward_harness, tmp_path, t1, average):
    """The forward-mode kernel (the LML benchmark's kernel, P tangent
    threads per sample) on the CPU: value and d/d params against the
    oracle's reverse mode to 1e-10, on the 2000-step benchmark grid too."""
    dt, save_every = 0.01, 10
    num_steps, data = lml_problem.observations(t1=t1, dt=dt, save_every=save_every)
    thetas = lml_problem.theta_samples(3, seed=1)
    y0s = np.tile(lml_problem.U0, (3, 1))
    head = [0, 3, 3, num_steps, save_every, int(average)]
    body = np.concatenate([thetas.ravel(), y0s.ravel(), np.ravel(data), np.full(data.shape[0], lml_problem.STD), [dt],
                           np.ravel(q1_iwp(3))])
    path = tmp_path / "input.txt"
    path.write_text(" ".join(str(int(v)) for v in head) + " " + " ".join(repr(float(v)) for v in body))
    out = np.array([[float(x) for x in line.split()] for line in hostsim.run_harness(forward_harness, path)])
    assert out.shape == (3, 5)
    for b in range(3):
        v, g, _ = lml_value_and_grads(thetas[b], y0s[b], data, dt, num_steps, save_every, average_pdfs=average)
        assert out[b, 0] == 0
        assert abs(out[b, 1] - v) <= 1e-10 * abs(v), (out[b, 1], v)
        assert np.abs(out[b, 2:5] - g).max() <= 1e-10 * np.linalg.norm(g), (out[b, 2:5], g)


def test_host_float32_adjoint_against_oracle(harness, tmp_path):
    """The float32 adjoint (float32 bulk; log-pdf sums and the parameter
    adjoint's totals in float64) on the 2000-step benchmark grid: value
    within 1e-3 and gradients within 5e-2 of the float64 oracle, the bounds
    of the GPU float32 tests."""
    dt, save_every = 0.01, 10
    num_steps, data = lml_problem.observations(t1=20.0, dt=dt, save_every=save_every)
    thetas = lml_problem.theta_samples(2, seed=1)
    y0s = np.tile(lml_problem.U0, (2, 1))
    out = run(harness, tmp_path, thetas, y0s, data, dt, num_steps, save_every, 45, False, [1.0, 1.0], precision=0)
    for b in range(2):
        v, g, gy = lml_value_and_grads(thetas[b], y0s[b], data, dt, num_steps, save_every)
        assert out[b, 0] == 0
        assert abs(out[b, 1] - v) <= 1e-3 * abs(v), (out[b, 1], v)
        assert np.abs(out[b, 2:5] - g).max() <= 5e-2 * np.linalg.norm(g), (out[b, 2:5], g)
        assert np.abs(out[b, 5:7] - gy).max() <= 5e-2 * np.linalg.norm(gy), (out[b, 5:7], gy)


def test_host_lml_kernels_with_concurrent_lanes(harness, forward_harness, tmp_path, monkeypatch):
    """Each block's 32 lanes as host threads, so the step tables are staged
    into shared memory by the whole warp between its barriers (as on the
    device) instead of by each lane alone: the records equal the one-lane
    runs bit for bit (the adjoint pair, and the forward-mode kernel with its
    P tangent lanes per sample)."""
    dt, save_every = 0.01, 10
    num_steps, data = lml_problem.observations(t1=2.0, dt=dt, save_every=save_every)
    thetas = lml_problem.theta_samples(5, seed=2)
    y0s = np.tile(lml_problem.U0, (5, 1))
    cot = [1.0, -0.5, 2.0, 0.25, -1.0]
    monkeypatch.delenv("PDQ_HOST_LML_WARPS", raising=False)
    one = run(harness, tmp_path, thetas, y0s, data, dt, num_steps, save_every, 14, False, cot)
    monkeypatch.setenv("PDQ_HOST_LML_WARPS", "1")
    lanes = run(harness, tmp_path, thetas, y0s, data, dt, num_steps, save_every, 14, False, cot)
    assert np.array_equal(one, lanes)

    head = [0, 3, 5, num_steps, save_every, 0]
    body = np.concatenate([thetas.ravel(), y0s.ravel(), np.ravel(data), np.full(data.shape[0], lml_problem.STD), [dt],
                           np.ravel(q1_iwp(3))])
    path = tmp_path / "forward.txt"
    path.write_text(" ".join(str(int(v)) for v in head) + " " + " ".join(repr(float(v)) for v in body))
    lanes_fwd = hostsim.run_harness(forward_harness, path)
    monkeypatch.delenv("PDQ_HOST_LML_WARPS")
    assert hostsim.run_harness(forward_harness, path) == lanes_fwd
