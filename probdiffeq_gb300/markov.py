"""Posterior samples of fixed-point smoother solutions (MarkovSequence.sample).

``sample(solution, num_samples)`` draws joint samples of the solution at all
checkpoints (estimators_and_losses.py:233-273): the last checkpoint from its
marginal, the earlier ones through the posterior's backward conditionals, on
the GPU (``pdq_sample_markov``).  The solution must come from a fixed-point
smoother solve with ``posterior=True`` (``ivpsolve.solve_adaptive_save_at`` or
``ensemble.solve_ensemble`` with ``_native.alloc_outputs(..., posterior=True)``).
"""

import torch

from . import _native

__all__ = ["sample"]


def sample(solution, num_samples, *, generator=None, normals=None, ode_dim=None):
    """Joint samples at the checkpoints: (B, K, S, n, d) isotropic, (B, K, S, n*d)
    dense, (B, K, S, d, n) block-diagonal.

    ``solution`` is an ``ivpsolve.Solution`` (its ``posterior`` dict holds the
    conditionals) or a dict of solve outputs (then give ``ode_dim`` for the
    dense factorisation).  ``normals`` (standard normal, (B, K, S, n)
    isotropic, (B, K, S, N) dense, (B, K, S, d, n) block-diagonal) may be
    given for reproducibility; otherwise they are drawn with ``generator``.
    """
    if isinstance(solution, dict):
        mean, chol, post = solution["u_mean"], solution["u_chol"], solution
        ssm = "blockdiag" if chol.ndim == 5 else ("isotropic" if mean.ndim == 4 else "dense")
    else:
        mean, chol, post, ssm = solution.u.mean_flat, solution.u.cholesky_flat, solution.posterior, solution.u.ssm
        ode_dim = ode_dim or getattr(solution, "ode_dim", None)
    if post is None or "cond_A" not in post:
        raise ValueError("sampling needs the posterior: solve with the fixed-point smoother and posterior=True")
    B, S = mean.shape[0], mean.shape[1]
    if post["cond_A"].shape[1] != S - 1:
        raise ValueError("the solution holds terminal values only; solve with terminal_only=False")
    if ssm == "blockdiag":
        return _sample_blockdiag(mean, chol, post, num_samples, generator, normals)
    if ssm == "isotropic":
        n, d = mean.shape[2], mean.shape[3]
        nu = n - 1
        zshape = (B, num_samples, S, n)
    else:
        N = mean.shape[2]
        if ode_dim is None:
            raise ValueError("give ode_dim for a dense solution")
        d = int(ode_dim)
        nu = N // d - 1
        zshape = (B, num_samples, S, N)
    if normals is None:
        normals = torch.randn(zshape, dtype=torch.float64, device=mean.device, generator=generator)
    elif tuple(normals.shape) != zshape:
        raise ValueError(f"normals must have shape {zshape}")
    last_mean = mean[:, -1].contiguous()
    last_chol = chol[:, -1].contiguous()
    return _native.sample_markov(ssm, nu, d, last_mean, last_chol, post, normals.contiguous())


def _sample_blockdiag(mean, chol, post, K, generator, normals):
    """Block-diagonal solutions through the isotropic kernel: dimension j of
    instance b is instance b * d + j of dimension 1 (the dimensions of a
    block-diagonal Markov sequence are independent, ssm_impl_blockdiag.py:334-347
    samples them with one key each).  The block-diagonal apply_flat scales
    the noise mean by to_observed (ssm_impl_blockdiag.py:19-26), the
    isotropic one adds it after the scaling (ssm_impl_isotropic.py:75-79),
    so the kernel gets the scaled noise mean."""
    B, S, d, n = mean.shape
    zshape = (B, K, S, d, n)
    if normals is None:
        normals = torch.randn(zshape, dtype=torch.float64, device=mean.device, generator=generator)
    elif tuple(normals.shape) != zshape:
        raise ValueError(f"normals must have shape {zshape}")

    def per_dim(x, tail):  # (B, T, d, *tail) -> (B * d, T, *tail)
        T = x.shape[1]
        return x.reshape(B, T, d, *tail).movedim(2, 1).reshape(B * d, T, *tail).contiguous()

    to = post["cond_to_observed"]
    iso_post = {
        "cond_A": per_dim(post["cond_A"], (n, n)),
        "cond_noise_mean": per_dim(post["cond_noise_mean"] * to, (n,)).unsqueeze(-1).contiguous(),
        "cond_noise_chol": per_dim(post["cond_noise_chol"], (n, n)),
        "cond_to_latent": per_dim(post["cond_to_latent"], (n,)),
        "cond_to_observed": per_dim(to, (n,)),
    }
    last_mean = mean[:, -1].reshape(B * d, n, 1).contiguous()
    last_chol = chol[:, -1].reshape(B * d, n, n).contiguous()
    z = normals.movedim(3, 1).reshape(B * d, K, S, n).contiguous()
    smp = _native.sample_markov("isotropic", n - 1, 1, last_mean, last_chol, iso_post, z)  # (B*d, K, S, n, 1)
    return smp.reshape(B, d, K, S, n).movedim(1, 3).contiguous()
