"""Posterior sampling of fixed-point smoother solutions (pdq_sample_markov, GPU).

* The kernel's recursion equals the reference's MarkovSequence.sample
  (estimators_and_losses.py:233-273 with apply_flat / sample_flat) restated
  in numpy on the same conditionals and normal draws (float64, 1e-10 of the
  largest sample entry: summation order only).
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


def _numpy_reference(out, z, ssm):
    mean, chol = out["u_mean"].cpu().numpy(), out["u_chol"].cpu().numpy()
    A, xi, X = (out[k].cpu().numpy() for k in ("cond_A", "cond_noise_mean", "cond_noise_chol"))
    tl, to = out["cond_to_latent"].cpu().numpy(), out["cond_to_observed"].cpu().numpy()
    z = z.cpu().numpy()
    B, K, S = z.shape[:3]
    res = np.zeros((B, K, S) + mean.shape[2:])
    for b in range(B):
        for k in range(K):
            if ssm == "isotropic":
                x = mean[b, -1] + (chol[b, -1] @ z[b, k, -1])[:, None]
            else:
                x = mean[b, -1] + chol[b, -1] @ z[b, k, -1]
            res[b, k, -1] = x
            for s in range(S - 2, -1, -1):
                if ssm == "isotropic":
                    m = (to[b, s][:, None] * A[b, s]) @ (tl[b, s][:, None] * x) + xi[b, s]
                    x = m + (np.abs(to[b, s])[:, None] * X[b, s] @ z[b, k, s])[:, None]
                else:
                    m = (to[b, s][:, None] * A[b, s]) @ (tl[b, s] * x) + xi[b, s]
                    x = m + (np.abs(to[b, s])[:, None] * X[b, s]) @ z[b, k, s]
                res[b, k, s] = x
    return res


@pytest.mark.parametrize("ssm", ["isotropic", "dense"])
def test_sampling_recursion_matches_the_reference_algorithm(ssm):
    out = _solve(ssm)
    B, S = out["u_mean"].shape[:2]
    N = 4 if ssm == "isotropic" else 8
    g = torch.Generator(device="cuda").manual_seed(0)
    z = torch.randn((B, 5, S, N), dtype=torch.float64, device="cuda", generator=g)
    smp = markov.sample(out, 5, normals=z, ode_dim=2)
    torch.cuda.synchronize()
    ref = _numpy_reference(out, z, ssm)
    err = np.abs(smp.cpu().numpy() - ref).max() / np.abs(ref).max()
    assert err < 1e-10, err  # summation order only


@pytest.mark.parametrize("ssm", ["isotropic", "dense"])
def test_samples_reproduce_the_smoothed_marginals(ssm):
    out = _solve(ssm, B=1)
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
