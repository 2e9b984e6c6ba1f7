"""Independent instances across GPUs: one process per GPU, no data-path collective.

IVP instances are independent (the reference's ``jax.vmap`` axis), so a batch
shards contiguously over ranks and every rank solves its shard alone.  The
only exchanges are at the end: the maximum of the per-rank timings (the
slowest rank bounds the job) and, when the caller wants the whole batch on
every rank, an all-gather of the per-instance outputs.

Works with any ``torch.distributed`` backend (NCCL on GPUs, gloo on CPU for
the tests).
"""

import torch
import torch.distributed as dist

__all__ = ["shard", "max_over_ranks", "gather_instances", "solve_sharded"]


def shard(num_instances, world_size, rank):
    """Contiguous, balanced slice of the instances owned by ``rank``.

    The first ``num_instances % world_size`` ranks hold one extra instance.
    """
    if world_size < 1 or not 0 <= rank < world_size:
        raise ValueError(f"rank {rank} outside world of size {world_size}")
    base, extra = divmod(int(num_instances), int(world_size))
    start = rank * base + min(rank, extra)
    return slice(start, start + base + (1 if rank < extra else 0))


def _collective_device(group):
    backend = dist.get_backend(group)
    return torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")


def max_over_ranks(value, group=None):
    """Maximum of a Python float over the ranks of ``group`` (identity without a process group)."""
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=_collective_device(group))
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def gather_instances(local, num_instances, group=None):
    """All-gather per-instance outputs (leading axis = instances) into the full batch.

    ``local`` maps names to tensors holding this rank's shard; shards may be
    ragged (they are padded to the largest shard for the collective).
    Returns the same names with all ``num_instances`` rows, in instance order.
    """
    if not (dist.is_available() and dist.is_initialized()):
        return dict(local)
    world = dist.get_world_size(group)
    sizes = [shard(num_instances, world, r) for r in range(world)]
    width = max(s.stop - s.start for s in sizes)
    dev = _collective_device(group)
    out = {}
    for name in sorted(local):
        x = local[name]
        pad = torch.zeros((width,) + tuple(x.shape[1:]), dtype=x.dtype, device=dev)
        pad[: x.shape[0]] = x.to(dev)
        parts = [torch.empty_like(pad) for _ in range(world)]
        dist.all_gather(parts, pad, group=group)
        out[name] = torch.cat([p[: s.stop - s.start] for p, s in zip(parts, sizes)]).to(x.device)
    return out


def solve_sharded(solve, params, y0, *, group=None, gather=True, **kwargs):
    """Solve this rank's contiguous shard with ``solve(params=..., y0=..., **kwargs)``.

    ``solve`` is ``ensemble.solve_ensemble`` (with its config bound) or any
    callable returning a dict of per-instance tensors.  With ``gather`` the
    full batch's outputs are returned on every rank, else the local shard's.
    """
    B = y0.shape[0]
    world = dist.get_world_size(group) if dist.is_available() and dist.is_initialized() else 1
    rank = dist.get_rank(group) if world > 1 else 0
    sl = shard(B, world, rank)
    local = solve(params=params[sl], y0=y0[sl], **kwargs)
    local = {k: v for k, v in local.items() if not k.startswith("_") and v is not None and v.shape[:1] == (sl.stop - sl.start,)}
    return gather_instances(local, B, group) if gather and world > 1 else local
