"""Posterior sampling of fixed-point smoother solutions (pdq_sample_markov, GPU).

* The kernel's recursion equals the oracle's restatement of the reference's
  MarkovSequence.sample (oracle/markov.py: estimators_and_losses.py:233-273
  with each factorisation's apply_flat / sample_flat) on the same
  conditionals and normal draws, for the isotropic, dense and block-diagonal
  factorisations (float64, 1e-10 of the largest sample entry: summation
  order only; 1e-9 block-diagonal).  Block-diagonal solutions run on the
  isotropic kernel as B * d one-dimensional instances.
* Samples reproduce the smoothed marginals: over 40000 samples the sample
  mean and std of every Taylor coefficient at every checkpoint match the
  solution's marginals (mean within 5 standard errors, std within 3 %).
"""

import numpy as np
import pytest
import torch

from probdiffeq_gb300 import _native, ensemble, markov

pytestmark = pytest.mark.gpu


def _solve(ssm, B=2, S=6):
    from tests.test_iso_gpu import lv_instances

    params, y0 = lv_instances(B, seed=11)
    save_at = torch.linspace(0.0, 4.0, S, dtype=torch.float64)
    cfg = ensemble.make_config(field="lotka_volterra", num_derivatives=3, ode_dim=2, ssm=ssm, strategy="fixedpoint",
                               solver="mle", precision="float64", atol=1e-4, rtol=1e-4, clip_dt=False)
    outs = _native.alloc_outputs(cfg, B, S, False, "cuda", posterior=True)
    out = ensemble.solve_ensemble(cfg, params=params, y0=y0, save_at=save_at, dt0=0.1, terminal_only=False, outputs=outs)
    torch.cuda.synchronize()
    assert (out["status"] == 0).all()
    return out


def _oracle_samples(out, z, ssm_kind, d=2):
    """The oracle's MarkovSequence.sample on the kernel's posterior and normals."""
    from oracle import markov as omarkov
    from oracle import ssm as ossm

    cpu = {k: v.cpu() for k, v in out.items() if torch.is_tensor(v)}
    z = z.cpu()
    B, K, S = z.shape[:3]
    res = torch.zeros((B, K, S) + tuple(cpu["u_mean"].shape[2:]), dtype=torch.float64)
    for b in range(B):
        if ssm_kind == "isotropic":
            Normal = lambda m, c: ossm.IsoNormal(m, c)  # noqa: E731
            Cond = ossm.IsoCond
        elif ssm_kind == "blockdiag":
            Normal = lambda m, c: ossm.BdNormal(m, c)  # noqa: E731
            Cond = ossm.BdCond
        else:
            Normal = lambda m, c: ossm.DenseNormal(m, c, d)  # noqa: E731
            Cond = ossm.DenseCond
        conds = [Cond(cpu["cond_A"][b, s], Normal(cpu["cond_noise_mean"][b, s], cpu["cond_noise_chol"][b, s]),
                      cpu["cond_to_latent"][b, s], cpu["cond_to_observed"][b, s]) for s in range(S - 1)]
        marginal = Normal(cpu["u_mean"][b, -1], cpu["u_chol"][b, -1])
        for k in range(K):
            smp = omarkov.sample_backward(marginal, conds, [z[b, k, s] for s in range(S)])
            for s in range(S):
                res[b, k, s] = smp[s]
    return res


def _solve_blockdiag(B=2):
    from tests.test_blockdiag_gpu import NU_VISC, burgers_ic

    d, S = 8, 5
    u0t = torch.as_tensor(np.asarray([burgers_ic(d, 20 + b) for b in range(B)]), dtype=torch.float64)
    save_at = torch.linspace(0.0, 0.02, S, dtype=torch.float64)
    cfg = ensemble.make_config(field="burgers", num_derivatives=3, ode_dim=d, ssm="blockdiag", strategy="fixedpoint",
                               solver="mle", precision="float64", atol=1e-4, rtol=1e-4, clip_dt=True)
    outs = _native.alloc_outputs(cfg, B, S, False, "cuda", posterior=True)
    out = ensemble.solve_ensemble(cfg, params=torch.full((B, 1), NU_VISC, dtype=torch.float64), y0=u0t,
                                  save_at=save_at, dt0=0.002, terminal_only=False, outputs=outs)
    torch.cuda.synchronize()
    assert (out["status"] == 0).all()
    return out


@pytest.mark.parametrize("ssm", ["isotropic", "dense", "blockdiag"])
def test_sampling_recursion_matches_the_oracle(ssm):
    out = _solve_blockdiag() if ssm == "blockdiag" else _solve(ssm)
    B, S = out["u_mean"].shape[:2]
    g = torch.Generator(device="cuda").manual_seed(0)
    if ssm == "blockdiag":
        zshape = (B, 5, S) + tuple(out["u_mean"].shape[2:])
    else:
        zshape = (B, 5, S, 4 if ssm == "isotropic" else 8)
    z = torch.randn(zshape, dtype=torch.float64, device="cuda", generator=g)
    smp = markov.sample(out, 5, normals=z, ode_dim=2)
    torch.cuda.synchronize()
    ref = _oracle_samples(out, z, ssm)
    err = float((smp.cpu() - ref).abs().max() / ref.abs().max())
    # summation order only; block-diagonal: the noise mean is scaled by
    # to_observed before the isotropic kernel adds it (one more rounding)
    assert err < (1e-9 if ssm == "blockdiag" else 1e-10), err


@pytest.mark.parametrize("ssm", ["isotropic", "dense", "blockdiag"])
def test_samples_reproduce_the_smoothed_marginals(ssm):
    out = _solve_blockdiag(B=1) if ssm == "blockdiag" else _solve(ssm, B=1)
    K = 40000
    g = torch.Generator(device="cuda").manual_seed(1)
    smp = markov.sample(out, K, generator=g, ode_dim=2)[0]  # (K, S, ...)
    mean = out["u_mean"][0]
    chol = out["u_chol"][0]
    cov = chol @ chol.transpose(-1, -2)
    sd = torch.sqrt(torch.diagonal(cov, dim1=-2, dim2=-1))  # (S, n) or (S, N)
    if ssm == "isotropic":
        sd = sd[:, :, None].expand_as(mean)
    emp_mean, emp_sd = smp.mean(0), smp.std(0)
    ok = sd > 1e-12
    z = ((emp_mean - mean).abs() / (sd / K**0.5))[ok]
    assert float(z.max()) < 5.0, float(z.max())
    assert float(((emp_sd - sd).abs() / sd)[ok].max()) < 0.03
