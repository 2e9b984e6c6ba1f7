"""The log-marginal likelihood of a time series through the oracle, and its
gradient by PyTorch reverse mode (test infrastructure; also the CPU baseline
of the LML-gradient workload).

The reference's pipeline in float64 on the CPU: the fixed-point smoother on
a fixed grid with checkpoint resets at the observations
(_probdiffeq/estimators_and_losses.py:534-547), then loss_lml_timeseries
(estimators_and_losses.py:53-105, 180-218), with the reference's qr_r
derivative rule (Q held constant, probdiffeq/backend/linalg.py:13-37).
"""

import torch


def lml_value_and_grads(theta, y0, data, dt, num_steps, save_every, std, average_pdfs=False, field="fitzhugh_nagumo",
                        num_derivatives=3):
    """Returns (lml, d lml / d theta, d lml / d y0) as (float, ndarray, ndarray).

    ``field`` names a field of ``oracle.problems.FIELDS`` or is a callable
    f(u, params) written with ``oracle.problems.stack``."""
    from oracle import linalg, problems, solvers, ssm

    linalg.set_qr_derivative("reference")
    fn = field if callable(field) else problems.FIELDS[field]
    th = torch.tensor(theta, dtype=torch.float64, requires_grad=True)
    u0 = torch.tensor(y0, dtype=torch.float64, requires_grad=True)
    tc = problems.taylor_derivatives(fn, u0, th, num_derivatives)
    S = ssm.IsoSSM()
    prior = S.prior_wiener_integrated(tc)
    c = S.constraint_ode_ts0(lambda u, t: fn(u[0], th))
    solver = solvers.SolverPlain(solvers.StrategyFixedPoint(), c)
    _, post = solvers.solve_fixed_steps_save_at(solver, prior, 0.0, dt, num_steps, save_every)
    d = torch.tensor(data, dtype=torch.float64)
    lml = solvers.loss_lml_timeseries(list(d), post, std * torch.ones(d.shape[0]), average_pdfs=average_pdfs)
    g, gy = torch.autograd.grad(lml, (th, u0))
    return float(lml.detach()), g.numpy(), gy.numpy()
