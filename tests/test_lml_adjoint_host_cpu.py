"""The adjoint LML kernels' float64 bodies run on the CPU against the oracle.

``tests/hostsim`` compiles the kernel templates of ``lml_adjoint.cuh`` with
the host compiler (a stand-in for ``cuda_runtime.h`` turns the CUDA
qualifiers into no-ops) under AddressSanitizer and UBSan, and runs the plan
kernel's thread and every sample's value and adjoint pass one after another
on buffers of exactly the size the library computes.  This pins the adjoint
algebra and the residual layout without a GPU: value, d/d params and d/d y0
against the oracle's PyTorch reverse mode to 1e-10 relative, for sqrt(N),
single-step, ragged and whole-grid checkpoint spacings, averaged pdfs and
non-unit cotangents.  The GPU tests check the same kernels compiled for
sm_103a.
"""

import os
import shutil
import subprocess

import numpy as np
import pytest

from tests import lml_problem
from tests.lml_oracle import lml_value_and_grads

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path_factory.mktemp("hostsim") / "lml_adjoint_host")
    cmd = [cxx, "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=all",
           "-I" + os.path.join(HERE, "hostsim"), "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "probdiffeq_gb300", "csrc"), os.path.join(HERE, "hostsim", "lml_adjoint_host.cpp"),
           "-o", exe]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0 and "sanitize" in res.stderr:
        cmd = [c for c in cmd if "sanitize" not in c]  # a toolchain without the sanitizer runtimes
        res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-4000:]
    return exe


def q1_iwp(nu):
    """Lower Cholesky factor of flip(Hilbert), (Q1 Q1^T)[i, j] = 1 / (2 nu + 1 - i - j)."""
    n = nu + 1
    H = np.array([[1.0 / (2 * nu + 1 - i - j) for j in range(n)] for i in range(n)])
    return np.linalg.cholesky(H)


def run(harness, tmp_path, thetas, y0s, data, dt, num_steps, save_every, ckpt, average, cot):
    B = len(thetas)
    head = [B, num_steps, save_every, ckpt, int(average)]
    body = np.concatenate([np.ravel(thetas), np.ravel(y0s), np.ravel(data), np.full(data.shape[0], lml_problem.STD),
                           np.asarray(cot, dtype=float), [dt], np.ravel(q1_iwp(3))])
    path = tmp_path / "input.txt"
    path.write_text(" ".join(str(int(v)) for v in head) + " " + " ".join(repr(float(v)) for v in body))
    res = subprocess.run([harness, str(path)], capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-4000:]
    return np.array([[float(x) for x in line.split()] for line in res.stdout.strip().splitlines()])


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
