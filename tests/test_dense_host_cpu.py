"""The dense kernels' float64 bodies run on the CPU against the golden fixture.

``tests/hostsim/dense_host.cpp`` compiles ``dense_adaptive_kernel`` (one
thread per instance; van der Pol, TS1 with the Jacobian on dual numbers, the
fixed-point smoother with its scratch of backward conditionals and the
backward pass) and ``dense_struct_kernel`` (the structure-exploiting QRs;
one lane per instance, its shared memory a host buffer; and with four,
eight and sixteen lanes, each block's 32 lanes as host threads) and
``dense_coop_kernel`` (eight lanes per instance as host threads, shuffles
emulated) with the host
compiler under AddressSanitizer and UBSan, and runs them on the inputs of
``tests/golden/vdp_dense.json`` (the oracle's
smoothed marginals at 8 save points reached by interpolation, mu = 1 and
3).  Tolerances of the GPU parity tests (float64): the solution within 1e-8,
every Taylor row and L L^T within 1e-5, accepted steps within +-1.
"""

import numpy as np
import pytest

from tests import hostsim
from tests.golden import make_golden


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    return hostsim.compile_harness("dense_host.cpp", tmp_path_factory.mktemp("hostsim") / "dense_host")


def q1_iwp(nu):
    n = nu + 1
    H = np.array([[1.0 / (2 * nu + 1 - i - j) for j in range(n)] for i in range(n)])
    return np.linalg.cholesky(H)


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


KERNELS = ["thread", "struct"]


@pytest.fixture(params=KERNELS)
def kernel(request, monkeypatch):
    monkeypatch.setenv("PDQ_HOST_DENSE_KERNEL", request.param)
    return request.param


# the lane-cooperative kernel too (its eight lanes as host threads with
# emulated shuffles: slower on the host, so on the short Lotka--Volterra runs)
@pytest.fixture(params=KERNELS + ["coop"])
def kernel_all(request, monkeypatch):
    monkeypatch.setenv("PDQ_HOST_DENSE_KERNEL", request.param)
    return request.param


def test_host_dense_fixed_point_kernel_matches_golden_records(harness, tmp_path, kernel):
    gold = make_golden.load("vdp_dense.json")
    mus = gold["mu"]
    B, S, d, N = len(mus), len(gold["save_at"][0]), 2, 8
    head = [1, 3, 1, B, S, 2, 0, 0]  # van der Pol, nu = 3, fixed point; solver_dynamic, control_integral, no clip_dt
    body = np.concatenate([[gold["atol"], gold["rtol"]], np.ravel(gold["save_at"]), mus,
                           np.tile(gold["y0"], B), np.full(B, gold["dt0"]), q1_iwp(3).ravel()])
    path = tmp_path / "input.txt"
    path.write_text(" ".join(str(v) for v in head) + " " + " ".join(repr(float(v)) for v in body))
    lines = hostsim.run_harness(harness, path)
    assert len(lines) == B * (1 + S)
    for b, rec in enumerate(gold["records"]):
        status, attempts = (int(x) for x in lines[b * (1 + S)].split())
        assert status == 0 and attempts > 0
        steps_o = [0] + rec["num_steps"]
        for s in range(S):
            vals = [float(x) for x in lines[b * (1 + S) + 1 + s].split()]
            t, steps = vals[0], int(vals[1])
            gm = np.array(vals[2:2 + N])
            gc = np.array(vals[2 + N:]).reshape(N, N)
            om, oc = np.array(rec["u_mean"][s]), np.array(rec["u_chol"][s])
            assert abs(t - gold["save_at"][b][s]) < 1e-7
            assert rel(gm[:d], om[:d]) <= 1e-8, (b, s)
            for i in range(N // d):
                assert rel(gm[i * d:(i + 1) * d], om[i * d:(i + 1) * d]) <= 1e-5, (b, s, i)
            assert rel(gc @ gc.T, oc @ oc.T) <= 1e-5, (b, s)
            assert abs(steps - steps_o[s]) <= 1, (b, s, steps, steps_o[s])


def _run_lv(harness, tmp_path, strategy, solver, save_at, tol):
    head = [0, 2, 1 if strategy == "smoother" else 0, 1, len(save_at), solver, 0, 0]
    body = np.concatenate([[tol, tol], save_at, [0.5, 0.05, 0.5, 0.05], [20.0, 20.0], [0.1], q1_iwp(2).ravel()])
    path = tmp_path / f"input_{len(save_at)}.txt"
    path.write_text(" ".join(str(v) for v in head) + " " + " ".join(repr(float(v)) for v in body))
    lines = hostsim.run_harness(harness, path)
    assert int(lines[0].split()[0]) == 0
    return [np.array([float(x) for x in line.split()[2:]]) for line in lines[1:]]


@pytest.mark.parametrize("solver", [0, 1, 2])
@pytest.mark.parametrize("strategy", ["filter", "smoother"])
def test_host_dense_kernel_behaviour_close_to_t1(harness, tmp_path, strategy, solver, kernel_all):
    """The reference's test_dense_output/test_behaviour_close_to_t1.py:58-94
    on the dense kernel: Lotka--Volterra, TS1, nu = 2, tol 1e-1, 30 save
    points up to the second-to-last point of the oracle's save-every-step
    grid; dropping the last save point leaves every other marginal unchanged
    (the reference's float64 allclose: atol sqrt(eps), rtol 10 sqrt(eps))."""
    import torch

    from oracle import problems, solvers, ssm

    S = ssm.DenseSSM()
    p = torch.tensor([0.5, 0.05, 0.5, 0.05], dtype=torch.float64)
    tc = problems.taylor_derivatives(problems.lotka_volterra, torch.tensor([20.0, 20.0], dtype=torch.float64), p, 2)
    c = S.constraint_ode_ts1(lambda u, t: problems.lotka_volterra(u[0], p),
                             lambda u, t: problems.jacobian(problems.lotka_volterra, u, p), 2)
    cls = {0: solvers.SolverPlain, 1: solvers.SolverMLE, 2: solvers.SolverDynamic}[solver]
    strat = solvers.StrategyFilter() if strategy == "filter" else solvers.StrategyFixedInterval()
    every = solvers.solve_adaptive_save_every_step(cls(strat, c), solvers.ErrorResidualStd(c),
                                                   S.prior_wiener_integrated(tc), 0.0, 2.0, 1e-1, 1e-1)
    ts = np.linspace(float(every.t[0]), float(every.t[-2]), 30)
    full = _run_lv(harness, tmp_path, strategy, solver, ts, 1e-1)
    cut = _run_lv(harness, tmp_path, strategy, solver, ts[:-1], 1e-1)
    assert len(full) == 30 and len(cut) == 29
    tol = np.sqrt(np.finfo(np.float64).eps)
    N = 6
    for a, b in zip(full[:-1], cut):
        ma, La = a[:N], a[N:].reshape(N, N)
        mb, Lb = b[:N], b[N:].reshape(N, N)
        assert np.allclose(ma, mb, atol=tol, rtol=10 * tol)
        assert np.allclose(La @ La.T, Lb @ Lb.T, atol=tol, rtol=10 * tol)


def test_host_dense_mu30_100_save_points_matches_fixture(harness, tmp_path, kernel):
    """The stiff configuration's solver at mu = 30 with 100 save points
    (``tests/golden/vdp_dense_mu30.json``: the oracle's 1.9e4 accepted steps
    in 3.2e4 attempts): the same attempt count, accepted steps within +-1 at
    every save point, the solution within 1e-8, rows and L L^T within 1e-5."""
    gold = make_golden.load("vdp_dense_mu30.json")
    rec = gold["records"][0]
    S, d, N = len(gold["save_at"][0]), 2, 8
    head = [1, 3, 1, 1, S, 2, 0, 0]
    body = np.concatenate([[gold["atol"], gold["rtol"]], np.ravel(gold["save_at"]), gold["mu"], gold["y0"],
                           [gold["dt0"]], q1_iwp(3).ravel()])
    path = tmp_path / "input_mu30.txt"
    path.write_text(" ".join(str(v) for v in head) + " " + " ".join(repr(float(v)) for v in body))
    lines = hostsim.run_harness(harness, path)
    status, attempts = (int(x) for x in lines[0].split())
    assert status == 0 and attempts == rec["num_attempts"]
    steps_o = [0] + rec["num_steps"]
    for s in range(S):
        vals = [float(x) for x in lines[1 + s].split()]
        gm, gc = np.array(vals[2:2 + N]), np.array(vals[2 + N:]).reshape(N, N)
        om, oc = np.array(rec["u_mean"][s]), np.array(rec["u_chol"][s])
        assert rel(gm[:d], om[:d]) <= 1e-8, s
        assert max(rel(gm[i * d:(i + 1) * d], om[i * d:(i + 1) * d]) for i in range(N // d)) <= 1e-5, s
        assert rel(gc @ gc.T, oc @ oc.T) <= 1e-5, s
        assert abs(int(vals[1]) - steps_o[s]) <= 1, s


def test_host_struct_kernel_lane_counts_agree(harness, tmp_path, monkeypatch):
    """The structure-exploiting kernel as launched with four, eight and
    sixteen lanes per instance (32 / L instances per block, the 32 lanes as
    host threads meeting at the warp's barriers, the slots of absent
    instances running the warp-uniform loop's dummy steps) gives the records
    of the one-lane run bit for bit: the lanes change which lane computes a
    column or row, not the order of any sum.  Van der Pol mu = 1, TS1, the
    fixed-point smoother, 8 save points by interpolation."""
    gold = make_golden.load("vdp_dense.json")
    mus = gold["mu"][:1]  # mu = 1 (the stiffer mu = 3 instance only lengthens the host run)
    B, S = len(mus), len(gold["save_at"][0])
    head = [1, 3, 1, B, S, 2, 0, 0]
    body = np.concatenate([[gold["atol"], gold["rtol"]], np.ravel(gold["save_at"][:B]), mus,
                           np.tile(gold["y0"], B), np.full(B, gold["dt0"]), q1_iwp(3).ravel()])
    path = tmp_path / "input.txt"
    path.write_text(" ".join(str(v) for v in head) + " " + " ".join(repr(float(v)) for v in body))
    monkeypatch.setenv("PDQ_HOST_DENSE_KERNEL", "struct")
    outs = {}
    for lanes in (1, 4, 8, 16):
        monkeypatch.setenv("PDQ_HOST_DENSE_LANES", str(lanes))
        outs[lanes] = hostsim.run_harness(harness, path)
    assert len(outs[1]) == B * (1 + S)
    assert all(int(outs[1][b * (1 + S)].split()[0]) == 0 for b in range(B))
    for lanes in (4, 8, 16):
        assert outs[lanes] == outs[1], lanes
