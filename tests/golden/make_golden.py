"""Generate the golden fixtures in this directory from the oracle.

    python tests/golden/make_golden.py

The oracle (``oracle/``, the float64 CPU restatement of the reference, pinned
to the reference's own known-answer and equivalence tests) is run on small
seeded inputs; inputs and outputs are written as JSON.  The reference itself
is JAX code that cannot be installed in this environment, so these fixtures
come from the restatement.  ``tests/test_golden_cpu.py`` re-runs the oracle
against them; ``tests/test_golden_gpu.py`` checks the CUDA kernels against
them without running the oracle.

Fixtures:
  iwp.json         A1 = flip(Pascal), Q1 = lower sqrt of flip(Hilbert) for
                   nu = 2, 3, 4 and the Taylor preconditioner at dt = 1.234
                   (_probdiffeq/utilities.py:57-84)
  lv_filter.json   4 Lotka--Volterra instances, isotropic TS0, filter,
                   error_residual_std, integral control, nu = 4, dt0 = 0.1:
                   solver_mle terminal values at t1 = 5 with clip_dt, and
                   solver_dynamic at save_at (0, 0.7, 2, 3.3, 5) by
                   interpolation; means, Cholesky factors, output scales and
                   accepted steps
  lv_fixedpoint.json  2 Lotka--Volterra instances, isotropic TS0, fixed-point
                   smoother, solver_mle, clip_dt, nu = 3, 5 save points:
                   smoothed means, Cholesky factors, steps, output scale
  lv_sensitivities.json  2 Lotka--Volterra instances, isotropic TS0 filter,
                   solver_mle, clip_dt, nu = 3, 4 save points: means and
                   d u_mean / d params, d u_mean / d y0 (reverse mode)
  vdp_dense.json   van der Pol (mu = 1, 3), dense TS1, fixed-point smoother,
                   solver_dynamic, rtol = atol = 1e-5, 8 save points by
                   interpolation: smoothed means, Cholesky factors, steps
  vdp_dense_mu30.json  the stiff dense configuration's solver at mu = 30:
                   van der Pol, dense TS1, fixed-point smoother,
                   solver_dynamic, rtol = atol = 1e-5, 100 save points
                   linspace(0, 2 mu, 100) by interpolation: smoothed means,
                   Cholesky factors, accepted steps and the attempt count
                   (about 10 minutes of oracle time; not re-run by the CPU
                   tests)
  fhn_lml.json     FitzHugh--Nagumo LML on 200 steps of 0.01 with 21
                   observations (data included), 2 parameter samples with
                   perturbed initial values: lml, d lml / d params,
                   d lml / d y0 (PyTorch reverse mode through the oracle)
"""

import json
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

NOMINAL_LV = [0.5, 0.05, 0.5, 0.05]


def iwp_fixture():
    from oracle import ssm

    out = {}
    for nu in (2, 3, 4):
        A, Q = ssm.system_matrices_1d_iwp(nu)
        p, p_inv = ssm.preconditioner_taylor(nu)(1.234)
        out[str(nu)] = {"A": A.tolist(), "Q": Q.tolist(), "p": p.tolist(), "p_inv": p_inv.tolist(), "dt": 1.234}
    return out


def lv_inputs():
    g = torch.Generator().manual_seed(11)
    params = torch.tensor(NOMINAL_LV, dtype=torch.float64) * torch.exp(
        0.2 * torch.randn((4, 4), generator=g, dtype=torch.float64))
    y0 = 10.0 + 20.0 * torch.rand((4, 2), generator=g, dtype=torch.float64)
    return params, y0


def lv_filter_fixture(params=None, y0=None):
    """Two configurations, both with the isotropic TS0 filter and nu = 4:
    solver_mle, clip_dt, terminal values at t1 = 5 (rtol = atol = 1e-6); and
    solver_dynamic, save_at (0, 0.7, 2, 3.3, 5) reached by interpolation
    (no clip_dt, rtol = atol = 1e-5)."""
    from oracle import problems, solvers, ssm

    if params is None:
        params, y0 = lv_inputs()
    runs = {
        "mle_terminal": dict(cls=solvers.SolverMLE, save_at=[0.0, 5.0], tol=1e-6, clip_dt=True),
        "dynamic_save_at": dict(cls=solvers.SolverDynamic, save_at=[0.0, 0.7, 2.0, 3.3, 5.0], tol=1e-5, clip_dt=False),
    }
    out = {"params": params.tolist(), "y0": y0.tolist(), "num_derivatives": 4, "dt0": 0.1}
    for name, r in runs.items():
        records = []
        for b in range(params.shape[0]):
            tc = problems.taylor_derivatives(problems.lotka_volterra, y0[b], params[b], 4)
            S = ssm.IsoSSM()
            c = S.constraint_ode_ts0(lambda u, t, p=params[b]: problems.lotka_volterra(u[0], p))
            res = solvers.solve_adaptive_save_at(
                r["cls"](solvers.StrategyFilter(), c), solvers.ErrorResidualStd(c), S.prior_wiener_integrated(tc),
                r["save_at"], r["tol"], r["tol"], control=solvers.ControlIntegral(), clip_dt=r["clip_dt"], dt0=0.1,
            )
            records.append({
                "u_mean": [u.mean.tolist() for u in res.u],
                "u_chol": [u.cholesky.tolist() for u in res.u],
                "output_scale": [float(s) for s in res.output_scale],
                "num_steps": [int(s) for s in res.num_steps],
            })
        out[name] = {"save_at": r["save_at"], "rtol": r["tol"], "atol": r["tol"], "clip_dt": r["clip_dt"],
                     "records": records}
    return out


def lv_fixedpoint_fixture(params=None, y0=None):
    """Isotropic TS0 fixed-point smoother, solver_mle, clip_dt, nu = 3,
    rtol = atol = 1e-5, save_at (0, 1.3, 2, 3.7, 5), two Lotka--Volterra
    instances: smoothed means, Cholesky factors, steps, output scale."""
    from oracle import problems, solvers, ssm

    if params is None:
        params, y0 = lv_inputs()
        params, y0 = params[:2], y0[:2]
    save_at = [0.0, 1.3, 2.0, 3.7, 5.0]
    out = {"params": params.tolist(), "y0": y0.tolist(), "num_derivatives": 3, "save_at": save_at, "rtol": 1e-5,
           "atol": 1e-5, "dt0": 0.1, "records": []}
    for b in range(params.shape[0]):
        tc = problems.taylor_derivatives(problems.lotka_volterra, y0[b], params[b], 3)
        S = ssm.IsoSSM()
        c = S.constraint_ode_ts0(lambda u, t, p=params[b]: problems.lotka_volterra(u[0], p))
        res = solvers.solve_adaptive_save_at(solvers.SolverMLE(solvers.StrategyFixedPoint(), c),
                                             solvers.ErrorResidualStd(c), S.prior_wiener_integrated(tc), save_at,
                                             1e-5, 1e-5, clip_dt=True, dt0=0.1)
        out["records"].append({
            "u_mean": [u.mean.tolist() for u in res.u],
            "u_chol": [u.cholesky.tolist() for u in res.u],
            "output_scale": [float(s) for s in res.output_scale],
            "num_steps": [int(s) for s in res.num_steps],
        })
    return out


def lv_sensitivities_fixture(params=None, y0=None):
    """d u_mean / d params and d u_mean / d y0 of the isotropic TS0 filter
    (solver_mle, clip_dt, nu = 3, rtol = atol = 1e-6) at save_at
    linspace(0, 5, 4), two Lotka--Volterra instances: PyTorch reverse mode
    through the oracle, the step sizes held constant as in the reference."""
    from oracle import problems, solvers, ssm

    if params is None:
        params, y0 = lv_inputs()
        params, y0 = params[2:], y0[2:]
    save_at = [0.0, 5.0 / 3.0, 10.0 / 3.0, 5.0]
    out = {"params": params.tolist(), "y0": y0.tolist(), "num_derivatives": 3, "save_at": save_at, "rtol": 1e-6,
           "atol": 1e-6, "dt0": 0.1, "records": []}
    for b in range(params.shape[0]):
        p = params[b].clone().requires_grad_(True)
        y = y0[b].clone().requires_grad_(True)
        tc = problems.taylor_derivatives(problems.lotka_volterra, y, p, 3)
        S = ssm.IsoSSM()
        c = S.constraint_ode_ts0(lambda u, t: problems.lotka_volterra(u[0], p))
        res = solvers.solve_adaptive_save_at(solvers.SolverMLE(solvers.StrategyFilter(), c), solvers.ErrorResidualStd(c),
                                             S.prior_wiener_integrated(tc), save_at, 1e-6, 1e-6, clip_dt=True, dt0=0.1)
        rec = {"u_mean": [], "d_params": [], "d_y0": [], "num_steps": [int(s) for s in res.num_steps]}
        for u in res.u:
            m = u.mean
            jp = torch.zeros(m.shape + p.shape, dtype=torch.float64)
            jy = torch.zeros(m.shape + y.shape, dtype=torch.float64)
            for i in range(m.shape[0]):
                for j in range(m.shape[1]):
                    if not m[i, j].requires_grad:
                        continue
                    gp, gy = torch.autograd.grad(m[i, j], (p, y), retain_graph=True, allow_unused=True)
                    jp[i, j] = gp if gp is not None else 0.0
                    jy[i, j] = gy if gy is not None else 0.0
            rec["u_mean"].append(m.detach().tolist())
            rec["d_params"].append(jp.tolist())
            rec["d_y0"].append(jy.tolist())
        out["records"].append(rec)
    return out


def vdp_dense_mu30_fixture(mu=30.0, num_save=100):
    """One instance of the stiff dense configuration at mu = 30 with its 100
    save points (the oracle needs ~2e4 attempts)."""
    out = vdp_dense_fixture([mu], num_save=num_save)
    return out


def vdp_dense_fixture(mus=None, num_save=8):
    """Dense TS1 van der Pol (first order), fixed-point smoother, dynamic
    calibration, error_residual_std, integral control, nu = 3,
    rtol = atol = 1e-5, save_at = linspace(0, 2 mu, 8) reached by
    interpolation: smoothed means, Cholesky factors and accepted steps at the
    save points."""
    from oracle import problems, solvers, ssm

    mus = [1.0, 3.0] if mus is None else mus
    out = {"mu": list(mus), "y0": [2.0, 0.0], "num_derivatives": 3, "rtol": 1e-5, "atol": 1e-5, "dt0": 0.1,
           "save_at": [], "records": []}
    for mu in mus:
        save_at = np.linspace(0.0, 2.0 * mu, num_save)
        p = torch.tensor([mu], dtype=torch.float64)
        tc = problems.taylor_derivatives(problems.van_der_pol, torch.tensor([2.0, 0.0], dtype=torch.float64), p, 3)
        D = ssm.DenseSSM()
        c = D.constraint_ode_ts1(lambda u, t: problems.van_der_pol(u[0], p),
                                 lambda u, t: problems.jacobian(problems.van_der_pol, u, p), 2)
        res = solvers.solve_adaptive_save_at(solvers.SolverDynamic(solvers.StrategyFixedPoint(), c),
                                             solvers.ErrorResidualStd(c), D.prior_wiener_integrated(tc),
                                             save_at, 1e-5, 1e-5)
        out["save_at"].append(save_at.tolist())
        out["records"].append({
            "u_mean": [u.mean.tolist() for u in res.u],
            "u_chol": [u.cholesky.tolist() for u in res.u],
            "num_steps": [int(s) for s in res.num_steps],
            "num_attempts": int(res.num_attempts),
        })
    return out


def fhn_lml_fixture(inputs=None):
    from tests import lml_problem
    from tests.lml_oracle import lml_value_and_grads

    dt, save_every = 0.01, 10
    if inputs is None:
        num_steps, data = lml_problem.observations(t1=2.0, dt=dt, save_every=save_every)
        thetas = lml_problem.theta_samples(2, seed=12)
        y0s = np.tile(lml_problem.U0, (2, 1)) + np.array([[0.0, 0.0], [0.05, -0.02]])
    else:
        num_steps, data, thetas, y0s = inputs
    out = {"dt": dt, "num_steps": num_steps, "save_every": save_every, "std": lml_problem.STD,
           "data": np.asarray(data).tolist(), "params": np.asarray(thetas).tolist(), "y0": np.asarray(y0s).tolist(),
           "lml": [], "grad": [], "grad_y0": []}
    for b in range(len(thetas)):
        v, g, gy = lml_value_and_grads(np.asarray(thetas[b]), np.asarray(y0s[b]), np.asarray(data), dt, num_steps,
                                       save_every)
        out["lml"].append(v)
        out["grad"].append(g.tolist())
        out["grad_y0"].append(gy.tolist())
    return out


def load(name):
    with open(os.path.join(HERE, name)) as f:
        return json.load(f)


def main(names=None):
    """Writes every fixture, or only those named on the command line."""
    torch.set_default_dtype(torch.float64)
    for name, fn in (("iwp.json", iwp_fixture), ("lv_filter.json", lv_filter_fixture),
                     ("lv_fixedpoint.json", lv_fixedpoint_fixture), ("lv_sensitivities.json", lv_sensitivities_fixture),
                     ("vdp_dense.json", vdp_dense_fixture), ("vdp_dense_mu30.json", vdp_dense_mu30_fixture),
                     ("fhn_lml.json", fhn_lml_fixture)):
        if names and name not in names:
            continue
        with open(os.path.join(HERE, name), "w") as f:
            json.dump(fn(), f, indent=1)
        print("wrote", name)


if __name__ == "__main__":
    main(sys.argv[1:])
