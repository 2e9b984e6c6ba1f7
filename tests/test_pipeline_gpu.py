"""The streamed ensemble pipeline (probdiffeq_gb300.pipeline) on the GPU.

Batches submitted to the overlapped upload / solve / download pipeline --
with the solver launch eager or replayed from a captured CUDA graph --
give bit-identical outputs to one ``ensemble.solve_ensemble`` call per
batch; slots are reused with new inputs (a replayed graph reads them).
"""

import pytest
import torch

from probdiffeq_gb300 import ensemble, pipeline

pytestmark = pytest.mark.gpu

LV = torch.tensor([0.5, 0.05, 0.5, 0.05], dtype=torch.float64)


def batch(B, seed):
    g = torch.Generator().manual_seed(seed)
    params = LV * torch.exp(0.2 * torch.randn((B, 4), generator=g, dtype=torch.float64))
    y0 = 10.0 + 20.0 * torch.rand((B, 2), generator=g, dtype=torch.float64)
    return params, y0


@pytest.mark.parametrize("depth,graph", [(2, False), (2, True), (1, True), (3, True)])
def test_pipeline_matches_one_call_per_batch(depth, graph):
    B, t1 = 300, 10.0
    cfg = ensemble.make_config(field="lotka_volterra", num_derivatives=4, ode_dim=2, solver="mle", precision="float32",
                               atol=1e-6, rtol=1e-6, clip_dt=True)
    save_at = torch.tensor([0.0, t1], dtype=torch.float64)
    pipe = pipeline.EnsemblePipeline(cfg, B, 2, 4, terminal_only=True, depth=depth, graph=graph)
    batches = [batch(B, s) for s in range(5)]
    outs = [pipe.alloc_host_outputs() for _ in batches]
    for (params, y0), out in zip(batches, outs):
        pipe.submit(params.pin_memory(), y0.pin_memory(), save_at, 0.1, out)
    pipe.synchronize()
    for (params, y0), out in zip(batches, outs):
        ref = ensemble.solve_ensemble(cfg, params=params, y0=y0, save_at=save_at, dt0=0.1, terminal_only=True)
        torch.cuda.synchronize()
        for k in pipe.output_names():
            assert torch.equal(out[k], ref[k].cpu()), k
        assert (out["status"] == 0).all()
    assert graph == all(s["cuda_graph"] is not None for s in pipe.slots)
