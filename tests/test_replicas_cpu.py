"""Multi-process (world size 2, gloo on CPU) tests of the replica sharding.

Instances are independent, so N GPUs run N shards with no collective on the
data path; these tests cover the host logic around that: the contiguous
balanced split, the max-over-ranks timing reduction and the all-gather of
ragged shards, with a stand-in solve that runs on the CPU.
"""

import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from probdiffeq_gb300 import replicas


def test_shard_is_a_contiguous_balanced_partition():
    for B in (0, 1, 7, 8, 16384, 16385):
        for world in (1, 2, 3, 8):
            parts = [replicas.shard(B, world, r) for r in range(world)]
            assert parts[0].start == 0 and parts[-1].stop == B
            assert all(a.stop == b.start for a, b in zip(parts, parts[1:]))
            sizes = [p.stop - p.start for p in parts]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        replicas.shard(4, 2, 2)


def test_without_process_group_everything_is_local():
    params, y0 = torch.randn(5, 3), torch.randn(5, 2)
    out = replicas.solve_sharded(lambda params, y0: {"u": y0 * 2, "s": params.sum(1)}, params, y0)
    assert torch.equal(out["u"], y0 * 2)
    assert replicas.max_over_ranks(1.5) == 1.5


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, B, results):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        g = torch.Generator().manual_seed(0)
        params, y0 = torch.randn(B, 4, generator=g, dtype=torch.float64), torch.randn(B, 2, generator=g, dtype=torch.float64)

        def fake_solve(params, y0, scale):
            # per-instance work that depends only on the instance's own row
            return {
                "u_mean": y0 * scale + params[:, :2],
                "num_steps": (params.abs().sum(1) * 100).to(torch.int32),
                "status": torch.zeros(y0.shape[0], dtype=torch.int32),
                "_workspace": torch.empty(3),
            }

        full = replicas.solve_sharded(fake_solve, params, y0, scale=3.0)
        local = replicas.solve_sharded(fake_solve, params, y0, scale=3.0, gather=False)
        t = replicas.max_over_ranks(float(rank + 1) * 0.25)
        ref = fake_solve(params, y0, 3.0)
        results[rank] = {
            "full_ok": all(torch.equal(full[k], ref[k]) for k in ("u_mean", "num_steps", "status")),
            "no_private_keys": "_workspace" not in full,
            "local_rows": local["u_mean"].shape[0],
            "max_time": t,
        }
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("B", [8, 7, 1])
def test_two_rank_gloo_sharded_solve_gathers_the_whole_batch(B):
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    results = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, B, results)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    rows = [results[r]["local_rows"] for r in range(2)]
    assert sum(rows) == B and rows == [replicas.shard(B, 2, r).stop - replicas.shard(B, 2, r).start for r in range(2)]
    for r in range(2):
        assert results[r]["full_ok"] and results[r]["no_private_keys"]
        assert results[r]["max_time"] == 0.5
