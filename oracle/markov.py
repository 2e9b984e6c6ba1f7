"""Posterior samples of a backward Markov sequence (test infrastructure).

MarkovSequence.sample (probdiffeq/_probdiffeq/estimators_and_losses.py:233-273)
with reverse=True, the smoother's posterior: the last point from its
marginal, then a reversed scan over the conditionals, each step taking
``cond.apply_flat(x)`` and drawing from it (sample_flat:
ssm_impl_isotropic.py:255-258, ssm_impl_blockdiag.py:343-350,
ssm_impl_dense.py:192-194).  The standard-normal draws are arguments (the
reference splits a PRNG key; here the same normals reach the kernel and this
restatement).
"""

import torch

from oracle import ssm


def sample_flat(normal, z):
    """One draw from ``normal`` with standard-normal base ``z``."""
    if isinstance(normal, ssm.IsoNormal):
        return normal.mean + (normal.cholesky @ z)[:, None]  # base (n,), shared by the d columns
    if isinstance(normal, ssm.BdNormal):
        return normal.mean + torch.einsum("dij,dj->di", normal.cholesky, z)  # base (d, n)
    return normal.mean + normal.cholesky @ z  # dense, base (N,)


def sample_backward(marginal, conds, normals):
    """Samples at points 0..S-1 of a reverse Markov sequence.

    marginal: the last point's normal; conds[s] maps the sample at point s + 1
    to the distribution at point s; normals[s]: the base draw at point s.
    Returns the list of samples in time order."""
    S = len(conds) + 1
    out = [None] * S
    x = sample_flat(marginal, normals[S - 1])
    out[S - 1] = x
    for s in range(S - 2, -1, -1):
        x = sample_flat(conds[s].apply_flat(x), normals[s])
        out[s] = x
    return out
