"""Autotuner for the instance-to-thread mapping and the instances per CTA.

Which mapping is fastest depends on the batch: one thread per instance
wins when the batch leaves the GPU latency-bound (a few warps per scheduler),
eight lanes per instance can win on small batches of long solves, and the
instances per CTA decide how the warps spread over the 152 SMs.  ``tune``
times every applicable candidate on (a leading sample of) the caller's own
batch -- one untimed launch, then ``repeats`` launches timed with CUDA events
on the launching stream -- and keeps the fastest.  ``tuned_config`` caches
the choice per (configuration, batch-size class, checkpoint count, device),
so a stream of equal batches is tuned once.
"""

import copy
import threading

import torch

from . import _native

__all__ = ["candidates", "tune", "tuned_config", "cache_key", "clear_cache"]

# (kernel_variant, instances_per_block), see include/pdq.h
_ISO_THREAD = [(1, 64), (1, 32)]
_ISO_LANES = [(2, 32), (2, 16), (3, 32)]
_ISO_SPLIT = [(4, 0)]
_DENSE_THREAD = [(1, 32), (1, 16)]
_DENSE_LANES = [(3, 0), (4, 0), (5, 0), (2, 4), (2, 2)]

_cache = {}
_lock = threading.Lock()


def candidates(cfg):
    """The (kernel_variant, instances_per_block) pairs the ABI accepts for ``cfg``."""
    if cfg.ssm == _native.SSM["isotropic"]:
        lanes_ok = (cfg.clip_dt and cfg.constraint == _native.CONSTRAINT["ts0"]
                    and cfg.error == _native.ERROR["residual_std"] and cfg.strategy == _native.STRATEGY["filter"]
                    and cfg.field < _native.FIELD_USER_BASE)
        split_ok = (lanes_ok and cfg.damp == 0.0 and cfg.solver != _native.SOLVER["dynamic"])
        return _ISO_THREAD + (_ISO_LANES if lanes_ok else []) + (_ISO_SPLIT if split_ok else [])
    if cfg.ssm == _native.SSM["dense"]:
        lanes_ok = cfg.error == _native.ERROR["residual_std"] and cfg.field < _native.FIELD_USER_BASE
        return _DENSE_THREAD + (_DENSE_LANES if lanes_ok else [])
    return [(0, 0)]


def cache_key(cfg, B, S, terminal_only, device):
    """Everything but the mapping, the batch size rounded up to a power of two, and the device."""
    fields = tuple((name, getattr(cfg, name)) for name, _ in cfg._fields_
                   if name not in ("kernel_variant", "instances_per_block"))
    size_class = 1 << max(0, int(B) - 1).bit_length()
    dev = torch.device(device)
    name = torch.cuda.get_device_name(dev) if dev.type == "cuda" else str(dev)
    return fields, size_class, int(S), bool(terminal_only), name


def clear_cache():
    with _lock:
        _cache.clear()


def _with(cfg, variant, ipb):
    c = copy.copy(cfg)
    c.kernel_variant, c.instances_per_block = variant, ipb
    return c


def tune(cfg, save_at, params, y0, dt0, terminal_only, *, sample=None, repeats=1, stream=None):
    """Time each candidate on device tensors (B, ...) -- the first ``sample``
    instances when given -- and return ((kernel_variant, instances_per_block),
    {candidate: milliseconds})."""
    if sample is not None and sample < y0.shape[0]:
        save_at, params, y0, dt0 = save_at[:sample], params[:sample], y0[:sample], dt0[:sample]
    B, S = y0.shape[0], save_at.shape[1]
    stream = torch.cuda.current_stream(y0.device) if stream is None else stream
    outputs = _native.alloc_outputs(cfg, B, S, terminal_only, y0.device)
    ws_bytes = _native.workspace_size(cfg, B, S)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=y0.device) if ws_bytes else None
    times = {}
    for cand in candidates(cfg):
        c = _with(cfg, *cand)
        run = lambda: _native.solve_adaptive(c, save_at, params, y0, dt0, terminal_only, outputs, stream=stream,  # noqa: E731
                                             workspace=ws)
        run()
        best = float("inf")
        for _ in range(repeats):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            run()
            e1.record(stream)
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        times[cand] = best
    return min(times, key=times.get), times


def tuned_config(cfg, save_at, params, y0, dt0, terminal_only, *, sample=None, repeats=1, stream=None):
    """``cfg`` with the cached (or freshly tuned) mapping for this batch."""
    key = cache_key(cfg, y0.shape[0], save_at.shape[1], terminal_only, y0.device)
    with _lock:
        hit = _cache.get(key)
    if hit is None:
        hit, _ = tune(cfg, save_at, params, y0, dt0, terminal_only, sample=sample, repeats=repeats, stream=stream)
        with _lock:
            _cache[key] = hit
    return _with(cfg, *hit)
