"""loss_lml_terminal_values on GPU solutions (the reference's
test_lml_terminal_values.py pattern: solve, then the terminal-value LML of
data near the solution), compared with the oracle's loss of the oracle's
terminal marginal.  Float64 bulk: the marginal matches the oracle to 1e-9
(mean) / 1e-6 (covariance), so the loss to 1e-6 relative.
"""

import math

import pytest
import torch

from oracle import solvers
from probdiffeq_gb300 import ivpsolve, probdiffeq
from tests.test_api_gpu import LV, oracle_terminal

pytestmark = pytest.mark.gpu


def test_terminal_values_lml_of_a_batch_matches_oracle():
    y0 = torch.tensor([[20.0, 20.0], [15.0, 25.0], [30.0, 12.0]], dtype=torch.float64)
    vf = probdiffeq.ode("lotka_volterra", LV)
    tcoeffs, _ = probdiffeq.jetexpand_ode_padded_scan(num=4)(vf, (y0,), t=0.0)
    ssm_ = probdiffeq.state_space_model_isotropic()
    ts0 = ssm_.constraint_ode_ts0(vf)
    solver = probdiffeq.solver_mle(strategy=probdiffeq.strategy_filter(), constraint=ts0)
    error = probdiffeq.error_residual_std(constraint=ts0)
    sol = ivpsolve.solve_adaptive_terminal_values(solver, error, precision="float64")(
        ssm_.prior_wiener_integrated(tcoeffs), t0=0.0, t1=10.0, atol=1e-6, rtol=1e-6)
    torch.cuda.synchronize()
    assert (sol.status == 0).all()
    data = sol.u.mean[0] + 0.1  # (B, 1, d)
    std = torch.ones((3, 1), dtype=torch.float64, device=data.device)
    loss = probdiffeq.loss_lml_terminal_values()
    val = loss(data, marginals=sol.u, std=std)
    assert val.shape == (3, 1)
    for b in range(3):
        res = oracle_terminal(y0[b], 10.0, solvers.SolverMLE)
        want = float(solvers.loss_lml_terminal_values(data[b, 0].cpu(), res.u[-1], torch.tensor(1.0, dtype=torch.float64)))
        got = float(val[b, 0])
        assert math.isfinite(got) and abs(got - want) <= 1e-6 * abs(want), (got, want)
    with pytest.raises(ValueError, match="container differs"):
        loss(data, marginals=sol.u, std=std[..., None])
