"""The block-diagonal kernel's body runs on the CPU.

``tests/hostsim/bd_host.cpp`` compiles ``bd_adaptive_kernel`` (the Burgers
stencil, IWP nu = 3) with the host compiler and runs each instance's
thread-block cluster as host threads -- every block's 256 threads at once,
with ``__syncthreads``, the warps' shuffles and the cluster's barriers and
distributed shared memory emulated -- on buffers of exactly the library's
sizes, under AddressSanitizer and UBSan, and in a second build under
ThreadSanitizer.  Checked at d = 64 on t in [0, 0.05] (the GPU parity tests'
case): float64 against the oracle with their tolerances (solution 1e-8,
every row and L L^T 1e-5, the same step count) with one block and with a
cluster of four (the stencil's halo read from the neighbours' distributed
shared memory, the error norm summed over the blocks); the fixed-point
smoother's records against the oracle; no data race.
"""

import numpy as np
import pytest
import torch

from tests import hostsim

NU_VISC = 0.01


def burgers_ic(d, seed):
    g = np.random.default_rng(seed)
    x = np.arange(d) / d
    k = np.arange(1, 9)
    amp = g.normal(0.0, 1.0 / k)
    phase = g.uniform(0.0, 2 * np.pi, size=8)
    return (amp[:, None] * np.sin(2 * np.pi * k[:, None] * x[None, :] + phase[:, None])).sum(axis=0)


def q1_iwp(nu):
    n = nu + 1
    H = np.array([[1.0 / (2 * nu + 1 - i - j) for j in range(n)] for i in range(n)])
    return np.linalg.cholesky(H)


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    return hostsim.compile_harness("bd_host.cpp", tmp_path_factory.mktemp("hostsim") / "bd_host")


@pytest.fixture(scope="module")
def harness_tsan(tmp_path_factory):
    return hostsim.compile_harness("bd_host.cpp", tmp_path_factory.mktemp("tsan") / "bd_host_tsan", sanitize="thread")


def run(exe, tmp_path, u0, save_at, cluster, solver=2, precision=1, fp=0):
    d, S = len(u0), len(save_at)
    head = [precision, fp, 1, d, S, cluster, solver, 0]
    body = np.concatenate([[1e-4, 1e-4], save_at, [NU_VISC], u0, [0.1 * save_at[-1]], q1_iwp(3).ravel()])
    path = tmp_path / f"input_{cluster}_{fp}_{precision}.txt"
    path.write_text(" ".join(str(v) for v in head) + " " + " ".join(repr(float(v)) for v in body))
    lines = hostsim.run_harness(exe, path)
    assert len(lines) == 1 + S
    status, attempts = (int(x) for x in lines[0].split())
    recs = []
    for line in lines[1:]:
        v = np.array([float(x) for x in line.split()])
        recs.append(dict(t=v[0], steps=int(v[1]), mean=v[2:2 + 4 * d].reshape(d, 4),
                         chol=v[2 + 4 * d:].reshape(d, 4, 4)))
    return status, attempts, recs, lines


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def check(rec, o, steps_o, tol):
    om, oc = o.mean.numpy(), o.cholesky.numpy()
    assert rel(rec["mean"][:, 0], om[:, 0]) <= tol["u"]
    for i in range(4):
        assert rel(rec["mean"][:, i], om[:, i]) <= tol["rows"], i
    cg = rec["chol"] @ rec["chol"].transpose(0, 2, 1)
    co = oc @ oc.transpose(0, 2, 1)
    assert max(rel(cg[j], co[j]) for j in range(len(co))) <= tol["cov"]
    assert rec["steps"] == steps_o


@pytest.mark.parametrize("solver", ["dynamic", "mle"])
def test_host_bd_kernel_matches_oracle_with_one_and_four_blocks(harness, tmp_path, solver):
    from oracle import problems, solvers, ssm

    d, t1 = 64, 0.05
    u0 = burgers_ic(d, 1)
    code = {"dynamic": 2, "mle": 1}[solver]
    st1, att1, recs1, lines1 = run(harness, tmp_path, u0, [0.0, t1], 1, solver=code)
    st4, att4, recs4, lines4 = run(harness, tmp_path, u0, [0.0, t1], 4, solver=code)
    assert st1 == 0 and st4 == 0
    p = torch.tensor([NU_VISC], dtype=torch.float64)
    tc = problems.taylor_derivatives(problems.burgers, torch.tensor(u0), p, 3)
    S = ssm.BdSSM()
    c = S.constraint_ode_ts0(lambda u, t: problems.burgers(u[0], p))
    cls = {"dynamic": solvers.SolverDynamic, "mle": solvers.SolverMLE}[solver]
    res = solvers.solve_adaptive_terminal_values(cls(solvers.StrategyFilter(), c), solvers.ErrorResidualStd(c),
                                                 S.prior_wiener_integrated(tc), 0.0, t1, 1e-4, 1e-4, dt0=0.1 * t1)
    # one block, and a cluster of four (the stencil's halo read from the
    # neighbours' shared memory, the error norm summed over the blocks in
    # another order: the same tolerance, not the same bits)
    for recs in (recs1, recs4):
        check(recs[-1], res.u[-1], res.num_steps[-1], dict(u=1e-8, rows=1e-5, cov=1e-5))


def test_host_bd_fixed_point_smoother_matches_oracle(harness, tmp_path):
    from oracle import problems, solvers, ssm

    d, t1 = 64, 0.05
    save_at = np.linspace(0.0, t1, 5)
    u0 = burgers_ic(d, 3)
    st, att, recs, lines = run(harness, tmp_path, u0, save_at, 4, fp=1)
    assert st == 0
    p = torch.tensor([NU_VISC], dtype=torch.float64)
    tc = problems.taylor_derivatives(problems.burgers, torch.tensor(u0), p, 3)
    S = ssm.BdSSM()
    c = S.constraint_ode_ts0(lambda u, t: problems.burgers(u[0], p))
    res = solvers.solve_adaptive_save_at(solvers.SolverDynamic(solvers.StrategyFixedPoint(), c),
                                         solvers.ErrorResidualStd(c), S.prior_wiener_integrated(tc), save_at,
                                         1e-4, 1e-4, clip_dt=True, dt0=0.1 * t1)
    steps_o = [0] + list(res.num_steps)
    for s in range(len(save_at)):
        check(recs[s], res.u[s], steps_o[s], dict(u=1e-8, rows=1e-5, cov=1e-5))


@pytest.mark.parametrize("precision,fp", [(1, 0), (0, 0), (1, 1)])
def test_host_bd_kernel_has_no_races(harness_tsan, tmp_path, precision, fp):
    """A cluster of four blocks under ThreadSanitizer: the staged means read
    across blocks, the warps' and blocks' partial sums, the parity buffers."""
    d, t1 = 64, 0.02
    u0 = burgers_ic(d, 2)
    save_at = np.linspace(0.0, t1, 3) if fp else np.array([0.0, t1])
    st, _, recs, _ = run(harness_tsan, tmp_path, u0, save_at, 4, precision=precision, fp=fp)
    assert st == 0
    assert all(np.isfinite(r["mean"]).all() and np.isfinite(r["chol"]).all() for r in recs)
