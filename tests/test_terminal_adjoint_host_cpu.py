"""The terminal-value adjoint's float64 bodies run on the CPU.

``tests/hostsim/iso_host.cpp`` (mode 5) compiles the record pass
(``iso_adaptive_kernel`` with REC: the lean TS0 filter recording step sizes
and the state every C accepted steps) and the adjoint pass
(``iso_tv_bwd_kernel``) with the host compiler under AddressSanitizer and
UBSan and runs them on buffers of the library's sizes.  For a cotangent of
the terminal mean, the gradients with respect to the parameters and y0:

* equal the forward-mode sensitivities of the same kernel contracted with
  the cotangent (mode 2) to 1e-10 relative, for C = 1, C = 7 (segments of
  the recorded steps, the last one partial) and C = capacity (one segment);
* equal PyTorch reverse mode through the oracle's solve_adaptive_terminal_values
  (the step sizes held constant, as the reference's stop-gradient does) to
  1e-8 relative when the accepted-step counts agree;
* an instance with more accepted steps than the record holds reports
  PDQ_INSTANCE_RECORD_FULL and NaN gradients, its solution intact.
"""

import numpy as np
import pytest
import torch

from tests import hostsim

NU = 4
T1 = 5.0


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    return hostsim.compile_harness("iso_host.cpp", tmp_path_factory.mktemp("hostsim") / "iso_host")


def q1_iwp(nu):
    n = nu + 1
    H = np.array([[1.0 / (2 * nu + 1 - i - j) for j in range(n)] for i in range(n)])
    return np.linalg.cholesky(H)


def inputs():
    params = np.array([[0.5, 0.05, 0.5, 0.05], [0.55, 0.045, 0.48, 0.052], [0.45, 0.06, 0.52, 0.047]])
    y0 = np.array([[20.0, 20.0], [18.0, 22.0], [25.0, 15.0]])
    cot = np.random.default_rng(3).normal(size=(3, NU + 1, 2))
    return params, y0, cot


def run(harness, tmp_path, mode, params, y0, cot=None, capacity=0, ckpt=0, tol=1e-6):
    B = params.shape[0]
    head = [1, mode, NU, B, 2, 1, 0, 1, 1]  # float64, mode, nu, B, S = 2, solver_mle, integral, clip_dt, terminal
    body = [tol, tol] + [0.0, T1] * B + list(params.ravel()) + list(y0.ravel()) + [0.1] * B + list(q1_iwp(NU).ravel())
    if mode == 5:
        body += list(cot.ravel())
    tail = f" {capacity} {ckpt}" if mode == 5 else ""
    path = tmp_path / f"input_{mode}_{capacity}_{ckpt}.txt"
    path.write_text(" ".join(str(v) for v in head) + " " + " ".join(repr(float(v)) for v in body) + tail)
    lines = hostsim.run_harness(harness, path)
    assert len(lines) == 2 * B
    out = []
    n, d, P = NU + 1, 2, 4
    for b in range(B):
        status, _ = (int(x) for x in lines[2 * b].split())
        vals = np.array([float(x) for x in lines[2 * b + 1].split()])
        rec = {"status": status, "steps": int(vals[1]), "mean": vals[3:3 + n * d].reshape(n, d)}
        o = 3 + n * d + n * n
        if mode == 2:
            rec["d_params"] = vals[o:o + n * d * P].reshape(n, d, P)
            rec["d_y0"] = vals[o + n * d * P:o + n * d * P + n * d * d].reshape(n, d, d)
        if mode == 5:
            rec["grad_params"] = vals[o:o + P]
            rec["grad_y0"] = vals[o + P:o + P + d]
        out.append(rec)
    return out


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("ckpt", [1, 7, 4096])
def test_adjoint_equals_forward_mode(harness, tmp_path, ckpt):
    params, y0, cot = inputs()
    tan = run(harness, tmp_path, 2, params, y0)
    adj = run(harness, tmp_path, 5, params, y0, cot, capacity=4096, ckpt=ckpt)
    for b in range(params.shape[0]):
        assert tan[b]["status"] == 0 and adj[b]["status"] == 0
        assert adj[b]["steps"] == tan[b]["steps"]
        assert np.array_equal(adj[b]["mean"], tan[b]["mean"])  # the record pass solves as the plain kernel
        gp = np.einsum("ij,ijk->k", cot[b], tan[b]["d_params"])
        gy = np.einsum("ij,ijk->k", cot[b], tan[b]["d_y0"])
        assert rel(adj[b]["grad_params"], gp) < 1e-10, (b, adj[b]["grad_params"], gp)
        assert rel(adj[b]["grad_y0"], gy) < 1e-10, (b, adj[b]["grad_y0"], gy)


def test_adjoint_matches_oracle_reverse_mode(harness, tmp_path):
    from oracle import problems, solvers, ssm

    params, y0, cot = inputs()
    adj = run(harness, tmp_path, 5, params, y0, cot, capacity=4096, ckpt=16)
    for b in range(params.shape[0]):
        p = torch.tensor(params[b], dtype=torch.float64, requires_grad=True)
        y = torch.tensor(y0[b], dtype=torch.float64, requires_grad=True)
        tc = problems.taylor_derivatives(problems.lotka_volterra, y, p, NU)
        S = ssm.IsoSSM()
        c = S.constraint_ode_ts0(lambda u, t: problems.lotka_volterra(u[0], p))
        res = solvers.solve_adaptive_terminal_values(solvers.SolverMLE(solvers.StrategyFilter(), c),
                                                     solvers.ErrorResidualStd(c), S.prior_wiener_integrated(tc),
                                                     0.0, T1, 1e-6, 1e-6, dt0=0.1)
        loss = (res.u[-1].mean * torch.tensor(cot[b])).sum()
        gp, gy = torch.autograd.grad(loss, (p, y))
        assert abs(adj[b]["steps"] - res.num_steps[-1]) <= 1
        tol = 1e-8 if adj[b]["steps"] == res.num_steps[-1] else 1e-5
        assert rel(adj[b]["grad_params"], gp.numpy()) < tol, b
        assert rel(adj[b]["grad_y0"], gy.numpy()) < tol, b


def test_record_full_reports_and_keeps_the_solution(harness, tmp_path):
    params, y0, cot = inputs()
    full = run(harness, tmp_path, 5, params, y0, cot, capacity=4096, ckpt=8)
    cap = min(r["steps"] for r in full) - 1  # one instance at least overflows
    small = run(harness, tmp_path, 5, params, y0, cot, capacity=cap, ckpt=8)
    for b in range(params.shape[0]):
        assert np.array_equal(small[b]["mean"], full[b]["mean"])
        if full[b]["steps"] > cap:
            assert small[b]["status"] == 4  # PDQ_INSTANCE_RECORD_FULL
            assert np.isnan(small[b]["grad_params"]).all() and np.isnan(small[b]["grad_y0"]).all()
        else:
            assert small[b]["status"] == 0
            assert np.array_equal(small[b]["grad_params"], full[b]["grad_params"])
