"""Benchmark: ensemble IVP solves/s on one GB300 (or N replicas).

Workload (the configuration the headline metric is quoted on): 16384
Lotka--Volterra instances, each of (a, b, c, d) = nominal * exp(0.2 z),
z ~ N(0, 1), y0 ~ U[10, 30]^2 (seed 0; rank r uses seed r), t in [0, 50],
IWP prior with 4 derivatives (Taylor-mode initial derivatives on device),
isotropic TS0, filter, MLE calibration, error_residual_std, integral
control, terminal values with clip_dt, rtol = atol = 1e-6, dt0 = 0.1.
Bulk arithmetic float32; time, calibration and error-norm sums float64.

A "step" is one full ensemble solve.  ``value`` times the native solve on
device-resident inputs (CUDA events on the launching stream, an L2 flush
between steps outside the events); ``e2e`` times the public API
(``probdiffeq_gb300.ensemble.solve_ensemble``) from pinned host inputs to
pinned host outputs, copies included.

``--impl reference`` times the CPU restatement of the reference's algorithm
(the C port in ``oracle/port``, float64, all host cores) on the same
workload; the reference itself is JAX code and JAX is not installed.
"""

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ensemble IVP solves/s at matched rtol (batched FP32 vs plain FP64); LML grads/s"
UNIT = "solves/s"
WORKLOAD = {
    "workload": "lotka_volterra_ensemble",
    "instances": 16384,
    "ode": "lotka_volterra d=2",
    "t_span": [0.0, 50.0],
    "num_derivatives": 4,
    "ssm": "isotropic",
    "constraint": "ts0",
    "strategy": "filter",
    "solver": "mle",
    "error": "residual_std",
    "control": "integral",
    "rtol": 1e-6,
    "atol": 1e-6,
    "dt0": 0.1,
    "output": "terminal values (clip_dt)",
    "l2": "flushed between timed steps (256 MiB write)",
}


def lv_inputs(B, seed):
    import torch

    g = torch.Generator().manual_seed(seed)
    nominal = torch.tensor([0.5, 0.05, 0.5, 0.05], dtype=torch.float64)
    params = nominal * torch.exp(0.2 * torch.randn((B, 4), generator=g, dtype=torch.float64))
    y0 = 10.0 + 20.0 * torch.rand((B, 2), generator=g, dtype=torch.float64)
    return params, y0


def flops_per_attempt(n, d):
    """Algorithmic FLOPs of one isotropic MLE attempt (reference algorithm).

    Dense matmuls count 2mnk, a Householder R-only QR of m x n costs
    2mn^2 - (2/3)n^3: A (pinv L) 2n^3; predict QR of 2n x n (10/3)n^3;
    revert QR of (n+1)^2 (4/3)(n+1)^3; the mean propagation and update 4n^2 d;
    vector field, residual, gain and error norm ~15 n d.
    """
    return 2 * n**3 + (10.0 / 3.0) * n**3 + (4.0 / 3.0) * (n + 1) ** 3 + 4 * n * n * d + 15 * n * d


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = (
        "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
        "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
        "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"
    )

    def __init__(self, index):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._thread = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(
                    ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits"],
                    capture_output=True, text=True, timeout=5,
                ).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                return
            self._stop.wait(0.2)

    def __enter__(self):
        self._thread = threading.Thread(target=self._run, daemon=True)
        self._thread.start()
        return self

    def __exit__(self, *exc):
        self._stop.set()
        if self._thread:
            self._thread.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if len(s) > 5 + i and s[5 + i] == "Active"})
        return {
            "sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": max(mx) if mx else None,
            "reasons": reasons,
            "samples": len(self.samples),
        }


def measured_fp32_peak(torch, _native, device):
    """FP32 FMA throughput of this GPU from the probe kernel (TFLOP/s), best of 3."""
    lib = _native.load()
    sms = lib.pdq_probe_sm_count()
    blocks, threads, iters = sms * 8, 256, 1 << 16
    out = torch.empty(blocks * threads, dtype=torch.float32, device=device)
    stream = torch.cuda.current_stream()
    best = 0.0
    for _ in range(4):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        assert lib.pdq_probe_fp32_fma(out.data_ptr(), iters, blocks, threads, stream.cuda_stream) == 0
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        best = max(best, blocks * threads * iters * 16 / (ms * 1e-3) / 1e12)
    return best, sms


def cpu_baseline(seconds_budget=20.0, impl_steps=None):
    """Time the C port of the oracle on host cores; returns a dict."""
    from oracle.port import port

    cores = os.cpu_count() or 1
    params, y0 = lv_inputs(WORKLOAD["instances"], 0)
    # calibrate the sample size to the time budget
    n = cores
    t = port.time_lv_ensemble(params[:n], y0[:n], threads=cores)
    per = t / n
    sample = int(max(cores, min(WORKLOAD["instances"], seconds_budget / max(per, 1e-9))))
    t = port.time_lv_ensemble(params[:sample], y0[:sample], threads=cores)
    return {
        "value": sample / t,
        "unit": UNIT,
        "cores": cores,
        "kind": "port",
        "sample": f"first {sample} of the {WORKLOAD['instances']} instances, float64 C port of the reference algorithm, {cores} threads",
        "seconds": t,
    }


def run_ours(args):
    import torch
    import torch.distributed as dist

    from probdiffeq_gb300 import _native, ensemble
    from probdiffeq_gb300 import build as native_build

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    native_build.build()
    device = torch.device(f"cuda:{local}")
    torch.cuda.set_device(device)

    B = args.instances
    WORKLOAD["instances"] = B
    params, y0 = lv_inputs(B, seed=rank)
    t0, t1 = WORKLOAD["t_span"]
    save_at = torch.tensor([t0, t1], dtype=torch.float64)
    cfg = ensemble.make_config(
        field="lotka_volterra", num_derivatives=4, ode_dim=2, solver="mle", precision="float32",
        atol=WORKLOAD["atol"], rtol=WORKLOAD["rtol"], clip_dt=True,
    )
    cfg64 = ensemble.make_config(
        field="lotka_volterra", num_derivatives=4, ode_dim=2, solver="mle", precision="float64",
        atol=WORKLOAD["atol"], rtol=WORKLOAD["rtol"], clip_dt=True,
    )
    stream = torch.cuda.current_stream()
    d_params, d_y0 = params.to(device), y0.to(device)
    d_save = save_at.expand(B, 2).contiguous().to(device)
    d_dt0 = torch.full((B,), WORKLOAD["dt0"], dtype=torch.float64, device=device)
    outs = _native.alloc_outputs(cfg, B, 2, True, device)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=device)

    def device_step(c):
        _native.solve_adaptive(c, d_save, d_params, d_y0, d_dt0, True, outs, stream=stream)

    def timed_steps(c, K, W):
        for _ in range(W):
            device_step(c)
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        total = 0.0
        for _ in range(K):
            flush.fill_(1.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            device_step(c)
            e1.record(stream)
            e1.synchronize()
            total += e0.elapsed_time(e1)
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        return total / 1e3

    # ---- autotune the instance-to-lane mapping on this workload ----
    def tune(base_precision, variants):
        times = {}
        for v in variants:
            c = ensemble.make_config(
                field="lotka_volterra", num_derivatives=4, ode_dim=2, solver="mle", precision=base_precision,
                atol=WORKLOAD["atol"], rtol=WORKLOAD["rtol"], clip_dt=True, kernel_variant=v,
            )
            device_step(c)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            device_step(c)
            e1.record(stream)
            e1.synchronize()
            times[v] = e0.elapsed_time(e1)
        best = min(times, key=times.get)
        return best, times

    names = {1: "thread per instance", 2: "8 lanes per instance, <=128 regs", 3: "8 lanes per instance, <=85 regs"}
    best32, tune32 = tune("float32", [1, 2, 3])
    best64, tune64 = tune("float64", [1, 2, 3])
    cfg.kernel_variant = best32
    cfg64.kernel_variant = best64

    # ---- value: device-resident inputs, FP32 bulk ----
    with ClockSampler(local) as clk:
        t_dev = timed_steps(cfg, args.steps, args.warmup)
    attempts = outs["num_attempts"].to(torch.float64).sum().item()
    steps_acc = outs["num_steps"].to(torch.float64).sum().item()
    status_ok = bool((outs["status"] == 0).all().item())
    mean32 = outs["u_mean"][:, 0].clone()
    max_attempts_inst = int(outs["num_attempts"].max().item())

    # ---- FP64 bulk (the plain per-instance float64 kernel, batched) ----
    t_dev64 = timed_steps(cfg64, max(1, args.steps // 2), 1)
    mean64 = outs["u_mean"][:, 0].clone()
    attempts64 = outs["num_attempts"].to(torch.float64).sum().item()
    k64 = max(1, args.steps // 2)
    rel_f32_f64 = ((mean32[:, 0] - mean64[:, 0]).abs() / mean64[:, 0].abs()).max().item()

    # ---- e2e through the public API, pinned host buffers, copies inside ----
    h_params, h_y0 = params.pin_memory(), y0.pin_memory()
    h_save = save_at.expand(B, 2).contiguous().pin_memory()
    h_dt0 = torch.full((B,), WORKLOAD["dt0"], dtype=torch.float64).pin_memory()
    h_out = {k: torch.empty(v.shape, dtype=v.dtype).pin_memory() for k, v in outs.items()}
    h2d = sum(t.numel() * t.element_size() for t in (h_params, h_y0, h_save, h_dt0))
    d2h = sum(t.numel() * t.element_size() for t in h_out.values())

    def e2e_step():
        o = ensemble.solve_ensemble(cfg, params=h_params, y0=h_y0, save_at=h_save, dt0=h_dt0, terminal_only=True, device=device, stream=stream)
        for k, v in o.items():
            h_out[k].copy_(v, non_blocking=True)

    for _ in range(args.warmup):
        e2e_step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    t_e2e = 0.0
    for _ in range(args.steps):
        flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        e2e_step()
        e1.record(stream)
        e1.synchronize()
        t_e2e += e0.elapsed_time(e1) / 1e3
    torch.cuda.synchronize()

    if world > 1:
        tt = torch.tensor([t_dev, t_e2e, t_dev64], dtype=torch.float64, device=device)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_dev, t_e2e, t_dev64 = tt.tolist()

    peak, sms = measured_fp32_peak(torch, _native, device)
    n, d = 5, 2
    fpa = flops_per_attempt(n, d)
    achieved = attempts * fpa / (t_dev / args.steps) / 1e12

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return
    result = {
        "metric": METRIC,
        "value": world * B * args.steps / t_dev,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * t_dev / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 bulk + f64 time/calibration/error-norm accumulators",
        "data": "synthetic (seeded Lotka-Volterra ensemble)",
        "config": dict(WORKLOAD, parallelism=f"replicas x{world}" if world > 1 else "single GPU"),
        "e2e": {
            "value": world * B * args.steps / t_e2e,
            "unit": UNIT,
            "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h,
        },
        "gpu_launches": args.steps,
        "autotune": {
            "float32": {names[k]: v for k, v in tune32.items()},
            "float64": {names[k]: v for k, v in tune64.items()},
            "unit": "ms per ensemble solve (one timed solve after one warm-up)",
            "chosen": {"float32": names[best32], "float64": names[best64]},
        },
        "roofline": {
            "bound": "fp32",
            "achieved": achieved,
            "peak": peak,
            "unit": "TFLOP/s",
            "frac": achieved / peak,
            "traffic": None,
            "peak_source": f"measured FP32 FMA probe on this GPU ({sms} SMs); MEASURED_PEAKS.json lists only HBM and bf16",
            "flops_per_attempt": fpa,
            "attempts_per_step": attempts,
        },
        "fp64": {
            "value": world * B * k64 / t_dev64,
            "unit": UNIT,
            "ms_per_step": 1e3 * t_dev64 / k64,
            "attempts_per_step": attempts64,
            "fp32_speedup": (B * args.steps / t_dev) / (B * k64 / t_dev64),
            "max_rel_terminal_diff_f32_vs_f64": rel_f32_f64,
        },
        "stats": {
            "accepted_steps_mean": steps_acc / B,
            "attempts_mean": attempts / B,
            "attempts_max": max_attempts_inst,
            "all_status_ok": status_ok,
        },
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline:
        try:
            result["cpu_baseline"] = cpu_baseline(args.cpu_seconds)
        except Exception as e:  # the port is test infrastructure; report why it is missing
            result["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port", "sample": f"unavailable: {e}"}
    print(json.dumps(result))
    if world > 1:
        dist.destroy_process_group()


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    vals = []
    cb = None
    for i in range(args.warmup + args.steps):
        cb = cpu_baseline(args.cpu_seconds / max(1, args.steps))
        if i >= args.warmup:
            vals.append(cb["value"])
    value = statistics.mean(vals)
    result = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * WORKLOAD["instances"] / value,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded Lotka-Volterra ensemble)",
        "config": dict(WORKLOAD, parallelism="host CPU"),
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cb["cores"], "kind": cb["kind"], "sample": cb["sample"]},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(result))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--instances", type=int, default=WORKLOAD["instances"], help="ensemble size (16384 is the headline workload)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
