"""The warp-cooperative kernels under ThreadSanitizer.

The host harnesses run each warp's lanes as host threads, with
``__syncwarp``, ``__any_sync``, the shuffles and the named barriers emulated
by mutex-guarded barriers (``tests/hostsim/cuda_runtime.h``), so a lane that
reads shared memory another lane writes without a barrier between them is a
data race ThreadSanitizer reports (and the harness exits non-zero).  Covered:
the dense lane-cooperative kernel (fixed-point smoother with MLE
calibration: the update's R_Y is read from the shared workspace that the
merge then overwrites), the structure-exploiting dense kernel on four, eight
and sixteen lanes, the isotropic split (covariance / mean warp) and
eight-lane kernels, and the LML kernels' warp-staged step tables.
"""

import os
import subprocess

import numpy as np
import pytest

from tests import hostsim


def q1_iwp(nu):
    n = nu + 1
    H = np.array([[1.0 / (2 * nu + 1 - i - j) for j in range(n)] for i in range(n)])
    return np.linalg.cholesky(H)


@pytest.fixture(scope="module")
def dense_tsan(tmp_path_factory):
    return hostsim.compile_harness("dense_host.cpp", tmp_path_factory.mktemp("tsan") / "dense_host_tsan",
                                   sanitize="thread")


@pytest.fixture(scope="module")
def iso_tsan(tmp_path_factory):
    return hostsim.compile_harness("iso_host.cpp", tmp_path_factory.mktemp("tsan") / "iso_host_tsan",
                                   sanitize="thread")


@pytest.mark.parametrize("kernel,lanes", [("coop", 1), ("struct", 4), ("struct", 8), ("struct", 16)])
@pytest.mark.parametrize("solver", [1, 2])
def test_dense_cooperative_kernels_have_no_races(dense_tsan, tmp_path, monkeypatch, kernel, lanes, solver):
    """Lotka--Volterra, nu = 2, TS1, the fixed-point smoother, 12 save points."""
    ts = np.linspace(0.0, 1.9, 12)
    head = [0, 2, 1, 1, len(ts), solver, 0, 0]
    body = np.concatenate([[0.1, 0.1], ts, [0.5, 0.05, 0.5, 0.05], [20.0, 20.0], [0.1], q1_iwp(2).ravel()])
    path = tmp_path / "input.txt"
    path.write_text(" ".join(str(v) for v in head) + " " + " ".join(repr(float(v)) for v in body))
    monkeypatch.setenv("PDQ_HOST_DENSE_KERNEL", kernel)
    monkeypatch.setenv("PDQ_HOST_DENSE_LANES", str(lanes))
    lines = hostsim.run_harness(dense_tsan, path)  # a reported race exits non-zero
    assert int(lines[0].split()[0]) == 0
    assert all(np.isfinite([float(x) for x in line.split()]).all() for line in lines[1:])


@pytest.mark.parametrize("mode", [6, 8, 9])
@pytest.mark.parametrize("precision", [1, 0])
def test_isotropic_cooperative_kernels_have_no_races(iso_tsan, tmp_path, mode, precision):
    """The split kernel (mode 6: one-lane warps; mode 9: as launched, two
    32-lane warps as 64 host threads) and the eight-lane kernel (mode 8): four of
    the benchmark's Lotka--Volterra instances, nu = 4, MLE, exact landings on
    4 save points."""
    import bench

    params, y0 = (x.numpy() for x in bench.lv_inputs(4, seed=3))
    B, save_at = 4, [0.0, 1.0, 1.0 + 1e-3, 7.5]
    head = [precision, mode, 4, B, len(save_at), 1, 0, 1, 0]
    body = np.concatenate([[1e-6, 1e-6], np.tile(save_at, B), params.ravel(), y0.ravel(), np.full(B, 0.1),
                           q1_iwp(4).ravel()])
    path = tmp_path / "input.txt"
    path.write_text(" ".join(str(v) for v in head) + " " + " ".join(repr(float(v)) for v in body))
    lines = hostsim.run_harness(iso_tsan, path)
    assert all(int(lines[b * (1 + len(save_at))].split()[0]) == 0 for b in range(B))


def test_thread_sanitizer_is_active(dense_tsan, tmp_path):
    """The harness really is a ThreadSanitizer build (else the tests above
    prove nothing): the sanitizer's runtime answers TSAN_OPTIONS=help=1."""
    empty = tmp_path / "empty.txt"
    empty.write_text("")
    res = subprocess.run([dense_tsan, str(empty)], capture_output=True, text=True, timeout=60,
                         env=dict(os.environ, TSAN_OPTIONS="help=1"))
    assert "ThreadSanitizer" in res.stderr or "tsan" in res.stderr.lower()


@pytest.fixture(scope="module")
def lml_tsan(tmp_path_factory):
    return hostsim.compile_harness("lml_adjoint_host.cpp", tmp_path_factory.mktemp("tsan") / "lml_adjoint_tsan",
                                   sanitize="thread")


def test_lml_adjoint_kernels_have_no_races(lml_tsan, tmp_path, monkeypatch):
    """The LML value and adjoint passes with each block's 32 lanes as
    threads: the warp stages every chunk of step tables into shared memory
    between two barriers while the lanes read the previous chunk."""
    from tests import lml_problem

    dt, save_every = 0.01, 10
    num_steps, data = lml_problem.observations(t1=1.0, dt=dt, save_every=save_every)
    thetas = lml_problem.theta_samples(3, seed=1)
    y0s = np.tile(lml_problem.U0, (3, 1))
    head = [1, 0, 3, 3, num_steps, save_every, 10, 0]
    body = np.concatenate([np.ravel(thetas), np.ravel(y0s), np.ravel(data), np.full(data.shape[0], lml_problem.STD),
                           [1.0, 1.0, 1.0], [dt], np.ravel(q1_iwp(3))])
    path = tmp_path / "input.txt"
    path.write_text(" ".join(str(int(v)) for v in head) + " " + " ".join(repr(float(v)) for v in body))
    monkeypatch.setenv("PDQ_HOST_LML_WARPS", "1")
    lines = hostsim.run_harness(lml_tsan, path)
    assert len(lines) == 3 and all(line.split()[0] == "0" for line in lines)
