"""The isotropic kernel's float64 bodies run on the CPU against the golden
fixtures: the headline filter instantiation, the fixed-point smoother and
the forward-mode sensitivities.

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
    head = [1, 0, nu, B, S, solver, 0, int(r["clip_dt"]), int(terminal)]
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


def _run(harness, tmp_path, mode, gold, solver, clip_dt, terminal):
    nu = gold["num_derivatives"]
    params, y0 = np.array(gold["params"]), np.array(gold["y0"])
    B, S = params.shape[0], len(gold["save_at"])
    head = [1, mode, nu, B, S, solver, 0, int(clip_dt), int(terminal)]
    body = np.concatenate([[gold["atol"], gold["rtol"]], np.tile(gold["save_at"], B), params.ravel(), y0.ravel(),
                           np.full(B, gold["dt0"]), q1_iwp(nu).ravel()])
    path = tmp_path / "input.txt"
    path.write_text(" ".join(str(v) for v in head) + " " + " ".join(repr(float(v)) for v in body))
    lines = hostsim.run_harness(harness, path)
    assert len(lines) == B * (1 + (1 if terminal else S))
    return lines


def test_host_iso_fixed_point_smoother_matches_golden_records(harness, tmp_path):
    """Fixed-point smoother (scratch of backward conditionals, backward pass),
    solver_mle, clip_dt: smoothed marginals at every save point."""
    gold = make_golden.load("lv_fixedpoint.json")
    nu, n, d = gold["num_derivatives"], gold["num_derivatives"] + 1, 2
    S = len(gold["save_at"])
    lines = _run(harness, tmp_path, 1, gold, SOLVER["mle"], True, False)
    for b, rec in enumerate(gold["records"]):
        status, _ = (int(x) for x in lines[b * (1 + S)].split())
        assert status == 0
        for s in range(S):
            vals = [float(x) for x in lines[b * (1 + S) + 1 + s].split()]
            gm = np.array(vals[3:3 + n * d]).reshape(n, d)
            gc = np.array(vals[3 + n * d:]).reshape(n, n)
            om, oc = np.array(rec["u_mean"][s]), np.array(rec["u_chol"][s])
            assert float(np.abs(gm[0] - om[0]).max() / np.abs(om[0]).max()) <= 1e-9, (b, s)
            for i in range(n):
                assert float(np.abs(gm[i] - om[i]).max() / max(np.abs(om[i]).max(), 1e-300)) <= 1e-6, (b, s, i)
            cg, co = gc @ gc.T, oc @ oc.T
            assert float(np.abs(cg - co).max() / max(np.abs(co).max(), 1e-300)) <= 1e-6, (b, s)
            steps_o = 0 if s == 0 else rec["num_steps"][s - 1]
            assert abs(int(vals[1]) - steps_o) <= 1
        so = rec["output_scale"][-1]
        assert abs(vals[2] - so) <= 1e-6 * abs(so)


def test_host_iso_sensitivities_match_golden_reverse_mode(harness, tmp_path):
    """Forward-mode sensitivities (P + d threads per instance) against the
    oracle's reverse mode: 1e-9 (values) / 1e-8 (sensitivities) relative when
    the accepted-step counts agree, the solver tolerance (1e-6 / 1e-5)
    otherwise."""
    gold = make_golden.load("lv_sensitivities.json")
    nu, n, d, P = gold["num_derivatives"], gold["num_derivatives"] + 1, 2, 4
    S = len(gold["save_at"])
    lines = _run(harness, tmp_path, 2, gold, SOLVER["mle"], True, False)
    for b, rec in enumerate(gold["records"]):
        status, _ = (int(x) for x in lines[b * (1 + S)].split())
        assert status == 0
        for s in range(S):
            vals = np.array([float(x) for x in lines[b * (1 + S) + 1 + s].split()])
            o = 3
            gm = vals[o:o + n * d].reshape(n, d)
            o += n * d + n * n
            gp = vals[o:o + n * d * P].reshape(n, d, P)
            gy = vals[o + n * d * P:].reshape(n, d, d)
            om, op, oy = np.array(rec["u_mean"][s]), np.array(rec["d_params"][s]), np.array(rec["d_y0"][s])
            steps_o = 0 if s == 0 else rec["num_steps"][s - 1]
            same = int(vals[1]) == steps_o
            assert abs(int(vals[1]) - steps_o) <= 1
            tol_v, tol_g = (1e-9, 1e-8) if same else (1e-6, 1e-5)
            rel = lambda g, w: float(np.abs(g - w).max() / max(np.abs(w).max(), 1e-300))  # noqa: E731
            assert rel(gm, om) < tol_v, (b, s)
            assert rel(gp, op) < tol_g, (b, s, rel(gp, op))
            assert rel(gy, oy) < tol_g, (b, s, rel(gy, oy))


def test_host_iso_float32_kernel_against_golden_records(harness, tmp_path):
    """The float32 headline instantiation (bulk float32, time and
    accumulators in float pairs): the solution row within 1e-4 and u' within
    1e-2 of the float64 oracle, a valid covariance and output scale, accepted
    steps within 10 % (the float32 bounds of the GPU parity tests)."""
    gold = make_golden.load("lv_filter.json")
    r = gold["mle_terminal"]
    nu, n, d = gold["num_derivatives"], gold["num_derivatives"] + 1, 2
    params, y0 = np.array(gold["params"]), np.array(gold["y0"])
    B, S = params.shape[0], len(r["save_at"])
    head = [0, 0, nu, B, S, SOLVER["mle"], 0, 1, 1]
    body = np.concatenate([[r["atol"], r["rtol"]], np.tile(r["save_at"], B), params.ravel(), y0.ravel(),
                           np.full(B, gold["dt0"]), q1_iwp(nu).ravel()])
    path = tmp_path / "input.txt"
    path.write_text(" ".join(str(v) for v in head) + " " + " ".join(repr(float(v)) for v in body))
    lines = hostsim.run_harness(harness, path)
    assert len(lines) == 2 * B
    for b, rec in enumerate(r["records"]):
        status, _ = (int(x) for x in lines[2 * b].split())
        assert status == 0
        vals = [float(x) for x in lines[2 * b + 1].split()]
        gm = np.array(vals[3:3 + n * d]).reshape(n, d)
        gc = np.array(vals[3 + n * d:]).reshape(n, n)
        om = np.array(rec["u_mean"][-1])
        assert float(np.abs(gm[0] - om[0]).max() / np.abs(om[0]).max()) <= 1e-4, b
        assert float(np.abs(gm[1] - om[1]).max() / np.abs(om[1]).max()) <= 1e-2, b
        assert np.isfinite(gc).all() and (np.diag(gc @ gc.T) >= 0).all()
        assert np.isfinite(vals[2]) and vals[2] > 0
        steps_o = rec["num_steps"][-1]
        assert abs(int(vals[1]) - steps_o) <= max(1, int(np.ceil(0.1 * steps_o))), (int(vals[1]), steps_o)


@pytest.mark.parametrize("constraint", ["ts0", "ts1"])
def test_host_iso_error_state_std_matches_oracle(harness, tmp_path, constraint):
    """The general instantiation with error_state_std (solvers.py:999-1098),
    TS0 and TS1 (trace of the Jacobian along d), solver_mle, clip_dt, on two
    Lotka--Volterra instances of the golden inputs, against the oracle run
    here (float64 tolerances of the GPU parity tests)."""
    import torch

    from oracle import problems, solvers, ssm

    gold = make_golden.load("lv_fixedpoint.json")
    gold = dict(gold, save_at=[0.0, 8.0])
    nu, n, d = 3, 4, 2
    mode = 3 if constraint == "ts0" else 4
    lines = _run(harness, tmp_path, mode, gold, SOLVER["mle"], True, True)
    for b in range(2):
        p, y = torch.tensor(gold["params"][b]), torch.tensor(gold["y0"][b])
        fn = problems.FIELDS["lotka_volterra"]
        tc = problems.taylor_derivatives(fn, y, p, nu)
        S = ssm.IsoSSM()
        vf = lambda u, t, p=p: fn(u[0], p)  # noqa: E731
        c = S.constraint_ode_ts1(vf) if constraint == "ts1" else S.constraint_ode_ts0(vf)
        res = solvers.solve_adaptive_save_at(solvers.SolverMLE(solvers.StrategyFilter(), c), solvers.ErrorStateStd(c),
                                             S.prior_wiener_integrated(tc), gold["save_at"], 1e-5, 1e-5, clip_dt=True,
                                             dt0=0.1)
        status, _ = (int(x) for x in lines[2 * b].split())
        assert status == 0
        vals = [float(x) for x in lines[2 * b + 1].split()]
        gm = np.array(vals[3:3 + n * d]).reshape(n, d)
        gc = np.array(vals[3 + n * d:]).reshape(n, n)
        om, oc = res.u[-1].mean.numpy(), res.u[-1].cholesky.numpy()
        assert float(np.abs(gm[0] - om[0]).max() / np.abs(om[0]).max()) <= 1e-9
        for i in range(n):
            assert float(np.abs(gm[i] - om[i]).max() / max(np.abs(om[i]).max(), 1e-300)) <= 1e-6, i
        cg, co = gc @ gc.T, oc @ oc.T
        assert float(np.abs(cg - co).max() / max(np.abs(co).max(), 1e-300)) <= 1e-6
        assert abs(int(vals[1]) - res.num_steps[-1]) <= 1


@pytest.mark.parametrize("precision", [1, 0])
def test_host_headline_kernel_on_the_benchmark_distribution(harness, tmp_path, precision):
    """The headline configuration on its own input distribution (32 of the
    benchmark's Lotka--Volterra instances, t in [0, 50], nu = 4, MLE,
    rtol = atol = 1e-6, clip_dt) against the float64 C port of the reference
    algorithm (the CPU baseline): float64 -- terminal u within 1e-9 relative,
    accepted steps within +-1, the output scale within 1e-6; float32 bulk --
    u within 1e-3 relative (the full horizon accumulates the float32 rounding
    of every step) and accepted steps within 10 %."""
    import bench
    from oracle.port import port

    params, y0 = (x.numpy() for x in bench.lv_inputs(32, seed=0))
    ref = port.solve_iso_terminal("lotka_volterra", params, y0, 4, "mle", atol=1e-6, rtol=1e-6, t0=0.0, t1=50.0,
                                  threads=1)
    nu, n, d, B = 4, 5, 2, 32
    head = [precision, 0, nu, B, 2, SOLVER["mle"], 0, 1, 1]
    body = np.concatenate([[1e-6, 1e-6], np.tile([0.0, 50.0], B), params.ravel(), y0.ravel(), np.full(B, 0.1),
                           q1_iwp(nu).ravel()])
    path = tmp_path / "input.txt"
    path.write_text(" ".join(str(v) for v in head) + " " + " ".join(repr(float(v)) for v in body))
    lines = hostsim.run_harness(harness, path)
    assert len(lines) == 2 * B
    for b in range(B):
        status, _ = (int(x) for x in lines[2 * b].split())
        assert status == 0
        vals = [float(x) for x in lines[2 * b + 1].split()]
        u = np.array(vals[3:3 + n * d]).reshape(n, d)[0]
        ru = ref["mean"][b, 0]
        err = float(np.abs(u - ru).max() / np.abs(ru).max())
        steps, rsteps = int(vals[1]), int(ref["num_steps"][b])
        if precision == 1:
            assert err <= 1e-9 and abs(steps - rsteps) <= 1, (b, err, steps, rsteps)
            assert abs(vals[2] - ref["output_scale"][b]) <= 1e-6 * abs(ref["output_scale"][b])
        else:
            assert err <= 1e-3 and abs(steps - rsteps) <= max(1, int(0.1 * rsteps)), (b, err, steps, rsteps)


@pytest.mark.parametrize("precision", [1, 0])
@pytest.mark.parametrize("solver,terminal", [("mle", True), ("none", True), ("mle", False)])
def test_host_lean_and_split_kernels_equal_the_one_thread_kernel(harness, tmp_path, precision, solver, terminal):
    """The branch-light lean kernel (iso_lean_kernel) and the split filter
    (iso_split_kernel: a covariance warp and a mean warp, here with one lane
    per warp as two host threads meeting at the named barriers, and as
    launched with 32-lane warps as 64 host threads) run the arithmetic of
    iso_adaptive_kernel's lean instantiation, so their records are its own bit
    for bit: 16 of the benchmark's Lotka--Volterra instances, nu = 4,
    rtol = atol = 1e-6, exact landings, terminal values or 6 save points,
    float64 and float32 bulk."""
    import bench

    params, y0 = (x.numpy() for x in bench.lv_inputs(16, seed=3))
    nu, B = 4, 16
    save_at = [0.0, 50.0] if terminal else [0.0, 1.0, 1.0 + 1e-3, 7.5, 20.0, 30.0]
    codes = {"none": 0, "mle": 1}

    def run(mode):
        head = [precision, mode, nu, B, len(save_at), codes[solver], 0, 1, int(terminal)]
        body = np.concatenate([[1e-6, 1e-6], np.tile(save_at, B), params.ravel(), y0.ravel(), np.full(B, 0.1),
                               q1_iwp(nu).ravel()])
        path = tmp_path / f"input{mode}.txt"
        path.write_text(" ".join(str(v) for v in head) + " " + " ".join(repr(float(v)) for v in body))
        return hostsim.run_harness(harness, path)

    one, split, lean, split32 = run(0), run(6), run(7), run(9)
    assert len(one) == B * (1 + (1 if terminal else len(save_at)))
    assert split == one
    assert lean == one
    assert split32 == one  # as launched: two 32-lane warps, 16 of the 32 instance slots empty
    assert all(line.split()[0] == "0" for line in one[::1 + (1 if terminal else len(save_at))])


@pytest.mark.parametrize("nu", [3, 5])
def test_host_lean_and_split_kernels_equal_the_one_thread_kernel_with_failures(harness, tmp_path, nu):
    """The same equality where some instances fail: with nu = 5 a step
    clipped to 1e-3 at a checkpoint leaves some Lotka--Volterra instances
    without a finite error estimate (PDQ_INSTANCE_NONFINITE, NaN records);
    the three kernels report the same statuses, attempts and records."""
    import bench

    params, y0 = (x.numpy() for x in bench.lv_inputs(24, seed=5))
    y0 = y0 * 2.0
    B = 24
    save_at = [0.0, 0.5, 0.501, 3.0, 3.0, 7.25, 12.0]

    def run(mode):
        head = [1, mode, nu, B, len(save_at), 1, 0, 1, 0]
        body = np.concatenate([[1e-5, 1e-5], np.tile(save_at, B), params.ravel(), y0.ravel(), np.full(B, 0.1),
                               q1_iwp(nu).ravel()])
        path = tmp_path / f"input{mode}.txt"
        path.write_text(" ".join(str(v) for v in head) + " " + " ".join(repr(float(v)) for v in body))
        return hostsim.run_harness(harness, path)

    one, split, lean = run(0), run(6), run(7)
    assert split == one and lean == one
    statuses = [int(one[b * (1 + len(save_at))].split()[0]) for b in range(B)]
    assert statuses.count(0) >= B // 2
    if nu == 5:
        assert any(s != 0 for s in statuses)


@pytest.mark.parametrize("precision", [1, 0])
def test_host_eight_lane_kernel_matches_golden_records(harness, tmp_path, precision):
    """The eight-lane kernel (iso_warp_kernel: a group of eight lanes per
    instance exchanging reflectors and rotations by shuffles; here each
    warp's 32 lanes run as host threads with emulated shuffles) on the
    golden MLE terminal-value run: float64 within the GPU parity tests'
    tolerances of the oracle's records (solution 1e-9, rows and L L^T 1e-6,
    accepted steps +-1, output scale 1e-6); float32 bulk within 1e-4 of the
    solution and +-10 % of the steps."""
    gold = make_golden.load("lv_filter.json")
    r = gold["mle_terminal"]
    assert r["clip_dt"]
    nu, n, d = gold["num_derivatives"], gold["num_derivatives"] + 1, 2
    params, y0 = np.array(gold["params"]), np.array(gold["y0"])
    B, S = params.shape[0], len(r["save_at"])
    head = [precision, 8, nu, B, S, SOLVER["mle"], 0, 1, 1]
    body = np.concatenate([[r["atol"], r["rtol"]], np.tile(r["save_at"], B), params.ravel(), y0.ravel(),
                           np.full(B, gold["dt0"]), q1_iwp(nu).ravel()])
    path = tmp_path / "input.txt"
    path.write_text(" ".join(str(v) for v in head) + " " + " ".join(repr(float(v)) for v in body))
    lines = hostsim.run_harness(harness, path)
    assert len(lines) == 2 * B
    for b, rec in enumerate(r["records"]):
        status, attempts = (int(x) for x in lines[2 * b].split())
        assert status == 0 and attempts > 0
        vals = [float(x) for x in lines[2 * b + 1].split()]
        steps, scale = int(vals[1]), vals[2]
        gm = np.array(vals[3:3 + n * d]).reshape(n, d)
        gc = np.array(vals[3 + n * d:]).reshape(n, n)
        om, oc = np.array(rec["u_mean"][S - 1]), np.array(rec["u_chol"][S - 1])
        steps_o = rec["num_steps"][S - 2]
        err = float(np.abs(gm[0] - om[0]).max() / np.abs(om[0]).max())
        if precision == 1:
            assert err <= 1e-9, (b, err)
            for i in range(n):
                assert float(np.abs(gm[i] - om[i]).max() / max(np.abs(om[i]).max(), 1e-300)) <= 1e-6, (b, i)
            cg, co = gc @ gc.T, oc @ oc.T
            assert float(np.abs(cg - co).max() / max(np.abs(co).max(), 1e-300)) <= 1e-6, b
            assert abs(steps - steps_o) <= 1, (b, steps, steps_o)
            so = rec["output_scale"][-1]
            assert abs(scale - so) <= 1e-6 * abs(so), (scale, so)
        else:
            assert err <= 1e-4 and abs(steps - steps_o) <= max(1, int(0.1 * steps_o)), (b, err, steps, steps_o)
