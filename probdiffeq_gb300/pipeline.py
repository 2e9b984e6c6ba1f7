"""Streamed ensemble solves: host<->device copies overlapped with the solver.

A stream of batches of B instances each goes through ``depth`` slots of
device buffers.  Batch k's inputs are uploaded on the upload stream while
batch k-1 is solved on the compute stream and batch k-2's outputs are
downloaded on the download stream; per slot, events order the three
streams (a slot's inputs are overwritten only after the solve that read them,
its outputs only after they were downloaded).  With ``graph=True`` each
slot's ``pdq_solve_adaptive`` launch is captured once into a CUDA graph and
replayed afterwards: the solve path neither allocates nor synchronises, so
it is capture-safe once its first (eager) launch has prepared the kernel.

The reference has no counterpart: its ``jax.vmap``-ed solve is one
synchronous XLA call per batch.
"""

import torch

from . import _native

__all__ = ["EnsemblePipeline"]


class EnsemblePipeline:
    """Double-buffered (``depth`` >= 2) ensemble solves on three CUDA streams.

    ``cfg`` is a ``pdq_config`` (``ensemble.make_config``); every batch has
    ``num_instances`` instances, ``num_save_at`` checkpoints and
    ``num_params`` field parameters.  ``submit`` takes host tensors (pinned
    for asynchronous copies) and fills the host tensors of ``out`` (a dict
    keyed like ``output_names()``) asynchronously; it returns the CUDA event
    after which ``out`` is complete and the inputs may be reused.
    """

    def __init__(self, cfg, num_instances, num_save_at, num_params, *, terminal_only=True, device="cuda", depth=2,
                 graph=False):
        if depth < 1:
            raise ValueError("depth must be >= 1")
        self.cfg = cfg
        self.B, self.S, self.P = int(num_instances), int(num_save_at), int(num_params)
        self.terminal_only = terminal_only
        self.device = torch.device(device)
        self.graph = graph
        self.streams = {k: torch.cuda.Stream(self.device) for k in ("upload", "compute", "download")}
        d = cfg.ode_dim
        ws_bytes = _native.workspace_size(cfg, self.B, self.S)
        f64 = dict(dtype=torch.float64, device=self.device)
        self.slots = []
        for _ in range(depth):
            self.slots.append({
                "params": torch.empty((self.B, self.P), **f64),
                "y0": torch.empty((self.B, d), **f64),
                "save_at": torch.empty((self.B, self.S), **f64),
                "dt0": torch.empty((self.B,), **f64),
                "outputs": _native.alloc_outputs(cfg, self.B, self.S, terminal_only, self.device),
                "workspace": torch.empty(ws_bytes, dtype=torch.uint8, device=self.device) if ws_bytes else None,
                "uploaded": torch.cuda.Event(),
                "solved": torch.cuda.Event(),
                "downloaded": torch.cuda.Event(),
                "cuda_graph": None,
                "used": False,
            })
        self.k = 0

    def output_names(self):
        return [k for k in self.slots[0]["outputs"] if not k.startswith("_")]

    def alloc_host_outputs(self, pin_memory=True):
        """Host tensors for ``submit``'s ``out`` (pinned by default)."""
        return {k: torch.empty(v.shape, dtype=v.dtype, pin_memory=pin_memory)
                for k, v in self.slots[0]["outputs"].items() if not k.startswith("_")}

    def _solve(self, slot):
        if slot["cuda_graph"] is not None:
            slot["cuda_graph"].replay()
            return
        args = (self.cfg, slot["save_at"], slot["params"], slot["y0"], slot["dt0"], self.terminal_only, slot["outputs"])
        _native.solve_adaptive(*args, workspace=slot["workspace"])
        if self.graph:
            # the eager launch above prepared the kernel (stack limit, attributes); capture the next ones
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                _native.solve_adaptive(*args, workspace=slot["workspace"])
            slot["cuda_graph"] = g

    def submit(self, params, y0, save_at, dt0, out):
        """Enqueue one batch; returns the event that completes ``out``."""
        slot = self.slots[self.k % len(self.slots)]
        up, comp, down = self.streams["upload"], self.streams["compute"], self.streams["download"]
        if slot["used"]:
            up.wait_event(slot["solved"])  # the previous batch of this slot has read its inputs
        with torch.cuda.stream(up):
            for name, src in (("params", params), ("y0", y0), ("save_at", save_at), ("dt0", dt0)):
                src = torch.as_tensor(src, dtype=torch.float64)
                slot[name].copy_(src.expand(slot[name].shape), non_blocking=True)
            slot["uploaded"].record(up)
        comp.wait_event(slot["uploaded"])
        if slot["used"]:
            comp.wait_event(slot["downloaded"])  # the previous batch's outputs have left the slot
        with torch.cuda.stream(comp):
            self._solve(slot)
            slot["solved"].record(comp)
        down.wait_event(slot["solved"])
        with torch.cuda.stream(down):
            for k in self.output_names():
                out[k].copy_(slot["outputs"][k], non_blocking=True)
            slot["downloaded"].record(down)
        slot["used"] = True
        self.k += 1
        return slot["downloaded"]

    def synchronize(self):
        for s in self.streams.values():
            s.synchronize()
