"""``probdiffeq.loss_lml_terminal_values`` (estimators_and_losses.py:20-50)
against the oracle's restatement, for the three factorisations (CPU).

The loss observes coefficient ``tcoeff_index`` of a batch of marginals with
noise ``std`` and returns one log-pdf per instance; values and gradients
with respect to the marginal means equal the oracle's (which follows the
reference's ``to_derivative`` / ``marginalise`` / ``logpdf`` chain with
QR-based square roots) to 1e-12.  A std container of the wrong shape raises
the reference's ValueError (its test_lml_terminal_values.py checks the
message).
"""

import pytest
import torch

from oracle import solvers, ssm
from probdiffeq_gb300 import ivpsolve, probdiffeq

n, d, B = 5, 2, 3


def random_marginals(kind, seed=0):
    g = torch.Generator().manual_seed(seed)
    if kind == "isotropic":
        mean = torch.randn((B, 1, n, d), generator=g)
        chol = torch.tril(torch.randn((B, 1, n, n), generator=g))
    elif kind == "blockdiag":
        mean = torch.randn((B, 1, d, n), generator=g)
        chol = torch.tril(torch.randn((B, 1, d, n, n), generator=g))
    else:
        mean = torch.randn((B, 1, n * d), generator=g)
        chol = torch.tril(torch.randn((B, 1, n * d, n * d), generator=g))
    return mean, chol


def oracle_loss(kind, mean, chol, u, std, k):
    if kind == "isotropic":
        marg = ssm.IsoNormal(mean, chol)
    elif kind == "blockdiag":
        marg = ssm.BdNormal(mean, chol)
    else:
        marg = ssm.DenseNormal(mean, chol, d)
    return solvers.loss_lml_terminal_values(u, marg, std, tcoeff_index=k)


@pytest.mark.parametrize("k", [0, 1])
@pytest.mark.parametrize("kind", ["isotropic", "blockdiag", "dense"])
def test_values_and_mean_gradients_match_oracle(kind, k):
    mean, chol = random_marginals(kind)
    g = torch.Generator().manual_seed(1)
    u = torch.randn((B, 1, d), generator=g)
    std = (0.1 + torch.rand((B, 1), generator=g)) if kind == "isotropic" else (0.1 + torch.rand((B, 1, d), generator=g))
    m = mean.clone().requires_grad_(True)
    got = probdiffeq.loss_lml_terminal_values(tcoeff_index=k)(u, marginals=ivpsolve.Normal(m, chol, kind), std=std)
    assert got.shape == (B, 1)
    got.sum().backward()
    for b in range(B):
        mo = mean[b, 0].clone().requires_grad_(True)
        want = oracle_loss(kind, mo, chol[b, 0], u[b, 0], std[b, 0], k)
        (gm,) = torch.autograd.grad(want, mo)
        assert abs(float(got[b, 0].detach()) - float(want.detach())) <= 1e-12 * max(1.0, abs(float(want.detach())))
        assert torch.allclose(m.grad[b, 0], gm, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("kind", ["isotropic", "blockdiag", "dense"])
def test_std_container_of_the_wrong_shape_is_rejected(kind):
    mean, chol = random_marginals(kind)
    u = torch.zeros((B, 1, d))
    std = torch.ones((B, 1)) if kind == "isotropic" else torch.ones((B, 1, d))
    loss = probdiffeq.loss_lml_terminal_values()
    loss(u, marginals=ivpsolve.Normal(mean, chol, kind), std=std)
    with pytest.raises(ValueError, match="container differs"):
        loss(u, marginals=ivpsolve.Normal(mean, chol, kind), std=std[..., None])
