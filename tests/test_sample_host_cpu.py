"""The posterior-sampling kernels' bodies run on the CPU under
AddressSanitizer and UBSan (``tests/hostsim/sample_host.cpp``): on random
conditionals, marginals and normal draws in pdq_sample_markov's layouts,
the samples equal the oracle's restatement of MarkovSequence.sample
(``oracle/markov.py``: estimators_and_losses.py:233-273 with each
factorisation's apply_flat / sample_flat) to 1e-12, isotropic and dense."""

import numpy as np
import pytest
import torch

from tests import hostsim


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    return hostsim.compile_harness("sample_host.cpp", tmp_path_factory.mktemp("hostsim") / "sample_host")


@pytest.mark.parametrize("kind", ["isotropic", "dense"])
def test_host_sampling_matches_oracle(harness, tmp_path, kind):
    from oracle import markov as omarkov
    from oracle import ssm as ossm

    nu, d, S, B, K = 3, 2, 4, 3, 5
    n, N = nu + 1, (nu + 1) * d
    g = torch.Generator().manual_seed(7)
    iso = kind == "isotropic"
    mshape, cshape, vlen = ((n, d), (n, n), n) if iso else ((N,), (N, N), N)

    def lower(shape):
        return torch.tril(torch.randn(shape, generator=g, dtype=torch.float64))

    mm = torch.randn((B,) + mshape, generator=g, dtype=torch.float64)
    mc = lower((B,) + cshape)
    cA = torch.randn((B, S - 1) + cshape, generator=g, dtype=torch.float64)
    cxi = torch.randn((B, S - 1) + mshape, generator=g, dtype=torch.float64)
    cX = lower((B, S - 1) + cshape)
    ctl = torch.rand((B, S - 1, vlen), generator=g, dtype=torch.float64) + 0.5
    cto = torch.rand((B, S - 1, vlen), generator=g, dtype=torch.float64) + 0.5
    z = torch.randn((B, K, S, vlen), generator=g, dtype=torch.float64)
    head = [0 if iso else 2, nu, d, S, B, K]
    body = np.concatenate([x.numpy().ravel() for x in (mm, mc, cA, cxi, cX, ctl, cto, z)])
    path = tmp_path / "input.txt"
    path.write_text(" ".join(str(v) for v in head) + " " + " ".join(repr(float(v)) for v in body))
    lines = hostsim.run_harness(harness, path)
    assert len(lines) == B * K
    if iso:
        Normal = lambda m, c: ossm.IsoNormal(m, c)  # noqa: E731
        Cond = ossm.IsoCond
    else:
        Normal = lambda m, c: ossm.DenseNormal(m, c, d)  # noqa: E731
        Cond = ossm.DenseCond
    for b in range(B):
        conds = [Cond(cA[b, s], Normal(cxi[b, s], cX[b, s]), ctl[b, s], cto[b, s]) for s in range(S - 1)]
        marginal = Normal(mm[b], mc[b])
        for k in range(K):
            got = np.array([float(x) for x in lines[b * K + k].split()]).reshape((S,) + mshape)
            want = omarkov.sample_backward(marginal, conds, [z[b, k, s] for s in range(S)])
            for s in range(S):
                w = want[s].numpy()
                assert np.abs(got[s] - w).max() <= 1e-12 * max(np.abs(w).max(), 1.0), (b, k, s)
