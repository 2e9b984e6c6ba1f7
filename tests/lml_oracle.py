"""The oracle's LML for the FitzHugh--Nagumo configuration, differentiated by
PyTorch autograd with respect to the parameters and the initial values.

The oracle runs the reference's pipeline in float64 on the CPU (fixed-point
smoother on the fixed grid with checkpoint resets, loss_lml_timeseries) with
the reference's qr_r derivative rule (Q held constant,
probdiffeq/backend/linalg.py:13-37).
"""

import torch

from tests import lml_problem


def lml_value_and_grads(theta, y0, data, dt, num_steps, save_every, average_pdfs=False, field="fitzhugh_nagumo",
                        num_derivatives=3, std=lml_problem.STD):
    """Returns (lml, d lml / d theta, d lml / d y0) as (float, ndarray, ndarray)."""
    from oracle import linalg, problems, solvers, ssm

    linalg.set_qr_derivative("reference")
    fn = problems.FIELDS[field]
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
