"""Benchmark: ensemble IVP solves/s on one GB300 (or N replicas).

Headline workload (``--workload lv_ensemble``, the default): 16384
Lotka--Volterra instances, each of (a, b, c, d) = nominal * exp(0.2 z),
z ~ N(0, 1), y0 ~ U[10, 30]^2 (seed 0; rank r uses seed r), t in [0, 50],
IWP prior with 4 derivatives (Taylor-mode initial derivatives on device),
isotropic TS0, filter, MLE calibration, error_residual_std, integral
control, terminal values with clip_dt, rtol = atol = 1e-6, dt0 = 0.1.
Bulk arithmetic float32; time, calibration and error-norm sums in float
pairs (48-bit significand).

A "step" is one full ensemble solve.  ``value`` times the native solve on
device-resident inputs (CUDA events on the launching stream, an L2 flush
between steps outside the events); ``e2e`` times the public API
(``probdiffeq_gb300.ensemble.solve_ensemble``) from pinned host inputs to
pinned host outputs, copies included.  The same line carries the float64
batch, the single-instance latencies (the plain per-instance method), the
LML-gradient throughput, the block-diagonal Burgers configuration (64
instances, d = 4096, t in [0, 1], float32, one solve) and the stiff dense
van der Pol configuration (4096 instances, mu <= 1000, 100 save points,
float32, one solve; float64 against float32 on mu <= 10) under
``secondary``.

Other workloads, one JSON line each (``--workload``):
  lv_single          one LV instance, dynamic calibration, float64 and float32
  fhn_lml            LML + gradient for 1024 FitzHugh--Nagumo parameter samples
                     (forward-mode kernel, and the adjoint pdq_lml_fwd + pdq_lml_bwd)
  vdp_dense          4096 stiff van der Pol instances, dense TS1, fixed-point
                     smoother, 100 checkpoints (minutes per solve at mu <= 1000)
  burgers_blockdiag  64 viscous Burgers instances, d = 4096, blockdiag TS0

``--impl reference`` times the CPU restatement of the reference's algorithm
(the C port in ``oracle/port``, float64, all host cores) on the headline
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
PROFILE_SUMMARY = os.path.join(ROOT, "profiles", "iso_lean_kernel_lv16384.md")


def lv_inputs(B, seed):
    from probdiffeq_gb300 import configs

    return configs.lv_ensemble(B, seed)


def flops_per_attempt(n, d):
    """Algorithmic FLOPs of one isotropic MLE attempt (reference algorithm).

    Dense matmuls count 2mnk, a Householder R-only QR of m x n costs
    2mn^2 - (2/3)n^3: A (pinv L) 2n^3; predict QR of 2n x n (10/3)n^3;
    revert QR of (n+1)^2 (4/3)(n+1)^3; the mean propagation and update 4n^2 d;
    vector field, residual, gain and error norm ~15 n d.
    """
    return 2 * n**3 + (10.0 / 3.0) * n**3 + (4.0 / 3.0) * (n + 1) ** 3 + 4 * n * n * d + 15 * n * d


def profiled_dram_bytes(path=PROFILE_SUMMARY):
    """DRAM bytes per launch of the headline kernel from the committed ncu summary, or None."""
    try:
        with open(path) as f:
            for line in f:
                if line.startswith("dram_bytes_per_launch:"):
                    return int(line.split(":", 1)[1].strip().split()[0])
    except OSError:
        return None
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the measurements run."""

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
    """FP32 FMA throughput of this GPU from the probe kernel (TFLOP/s), best of 4."""
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


def cpu_baseline(seconds_budget=15.0):
    """Time the C port of the oracle on all host cores over whole ensemble passes."""
    from oracle.port import port

    cores = os.cpu_count() or 1
    params, y0 = lv_inputs(WORKLOAD["instances"], 0)
    B = WORKLOAD["instances"]
    passes, total = 0, 0.0
    while passes == 0 or total < seconds_budget * 0.5:
        total += port.time_lv_ensemble(params, y0, threads=cores)
        passes += 1
        if total * (passes + 1) / passes > seconds_budget:
            break
    return {
        "value": passes * B / total,
        "unit": UNIT,
        "cores": cores,
        "kind": "port",
        "sample": f"{passes} pass(es) over all {B} instances, float64 C port of the reference algorithm, {cores} threads",
        "seconds": total,
    }


def timed_pipeline(torch, pipe, submit, K, W, world=1, dist=None):
    """W untimed batches, then K batches enqueued back to back on the
    pipeline's streams; one CUDA-event pair from the first upload to the
    last download; returns seconds."""
    for k in range(W):
        submit(k)
    pipe.synchronize()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(pipe.streams["upload"])
    for k in range(K):
        submit(W + k)
    e1.record(pipe.streams["download"])
    e1.synchronize()
    pipe.synchronize()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    return e0.elapsed_time(e1) / 1e3


def timed_region(torch, stream, fn, K, W, flush=None, world=1, dist=None):
    """W untimed calls, then K calls each bracketed by CUDA events; returns seconds."""
    for _ in range(W):
        fn()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    total = 0.0
    for _ in range(K):
        if flush is not None:
            flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        total += e0.elapsed_time(e1)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    return total / 1e3


# ---------------------------------------------------------------------------
# secondary measurements (single instance, LML gradients)
# ---------------------------------------------------------------------------


def accuracy_vs_exact(params, y0, mean32, mean64, subset=1024):
    """Terminal-value error of the float32 and float64 solves against the
    exact solution (fixed-step RK4 at h = 1e-3, ~1e-12 relative) on the first
    ``subset`` instances: the matched-accuracy check of the float32 bulk."""
    from probdiffeq_gb300 import configs

    k = min(subset, params.shape[0])
    truth = configs.lv_truth(params[:k].numpy(), y0[:k].numpy())
    out = {"subset": k, "exact": "fixed-step RK4, h = 1e-3 (probdiffeq_gb300.configs.lv_truth)",
           "error": "max_j |u_j - u_exact_j| / max_j |u_exact_j| per instance"}
    for name, m in (("float32", mean32), ("float64", mean64)):
        u = m[:k, 0].numpy()
        err = abs(u - truth).max(axis=1) / abs(truth).max(axis=1)
        out[name] = {"median": float(sorted(err)[k // 2]), "max": float(err.max())}
    out["f32_over_f64"] = {key: out["float32"][key] / out["float64"][key] for key in ("median", "max")}
    return out


def single_instance(torch, _native, ensemble, device, reps=3):
    """One LV instance (nominal parameters, y0 = (20, 20)), dynamic calibration,
    terminal values on [0, 50], rtol = atol = 1e-6: latency per solve."""
    out = {}
    stream = torch.cuda.current_stream()
    for prec in ("float64", "float32"):
        cfg = ensemble.make_config(field="lotka_volterra", num_derivatives=4, ode_dim=2, solver="dynamic",
                                   precision=prec, atol=1e-6, rtol=1e-6, clip_dt=True)
        p = torch.tensor([[0.5, 0.05, 0.5, 0.05]], dtype=torch.float64, device=device)
        y0 = torch.tensor([[20.0, 20.0]], dtype=torch.float64, device=device)
        sa = torch.tensor([[0.0, 50.0]], dtype=torch.float64, device=device)
        dt0 = torch.full((1,), 0.1, dtype=torch.float64, device=device)
        outs = _native.alloc_outputs(cfg, 1, 2, True, device)
        t = timed_region(torch, stream, lambda: _native.solve_adaptive(cfg, sa, p, y0, dt0, True, outs, stream=stream),
                         reps, 3)
        out[prec] = {
            "ms_per_solve": 1e3 * t / reps,
            "attempts": int(outs["num_attempts"][0]),
            "accepted_steps": int(outs["num_steps"][0, 0]),
            "status": int(outs["status"][0]),
        }
    return out


def single_instance_cpu_baseline(reps=20):
    """The plain single-instance method on the CPU (the configuration's own
    statement: one LV instance, float64 on the CPU): the float64 C port of the
    reference algorithm (dynamic calibration, terminal values on [0, 50]), one
    thread, the mean over ``reps`` solves."""
    import time

    from oracle.port import port

    params, y0 = [[0.5, 0.05, 0.5, 0.05]], [[20.0, 20.0]]
    port.solve_iso_terminal("lotka_volterra", params, y0, 4, "dynamic", threads=1)  # load, warm
    t = time.perf_counter()
    for _ in range(reps):
        out = port.solve_iso_terminal("lotka_volterra", params, y0, 4, "dynamic", threads=1)
    sec = (time.perf_counter() - t) / reps
    return {"value": 1e3 * sec, "unit": "ms per solve", "cores": 1, "kind": "port",
            "sample": f"{reps} solves of the one instance, float64 C port of the reference algorithm, one thread "
                      f"({int(out['num_attempts'][0])} attempts)"}


LML_FLOPS_PER_GRADIENT = None  # set in lml_gradients from the workload sizes


def lml_gradients(torch, _native, ensemble, device, precisions=("float32", "float64"), reps=3, B=1024):
    """LML of 200 FitzHugh--Nagumo observations and its gradient w.r.t. (a, b, c)
    for B parameter samples (fixed grid of 2000 steps on [0, 20], IWP nu = 3,
    isotropic TS0, fixed-point smoother checkpoints at the observations)."""
    import numpy as np

    from probdiffeq_gb300 import configs

    num_steps, data_np = configs.fhn_observations()
    thetas = torch.tensor(configs.fhn_theta_samples(B), dtype=torch.float64, device=device)
    y0 = torch.tensor(np.tile(configs.FHN_U0, (B, 1)), dtype=torch.float64, device=device)
    data = torch.tensor(data_np, dtype=torch.float64, device=device)
    std = torch.full((data.shape[0],), configs.FHN_STD, dtype=torch.float64, device=device)
    stream = torch.cuda.current_stream()
    res = {}
    for prec in precisions:
        cfg = ensemble.make_config(field="fitzhugh_nagumo", num_derivatives=3, ode_dim=2, strategy="fixedpoint",
                                   solver="none", precision=prec)
        holder = {}

        def call():
            holder.update(_native.lml_fixed_grid(cfg, thetas, y0, data, std, t0=0.0, dt=0.01, num_steps=num_steps,
                                                 save_every=10, average_pdfs=False, gradient=True, stream=stream,
                                                 workspace=holder.get("_workspace"), outputs=holder.get("out")))
            holder["out"] = {k: holder[k] for k in ("lml", "grad", "status")}

        t = timed_region(torch, stream, call, reps, 3)
        res[prec] = {
            "grads_per_s": B * reps / t,
            "ms_per_batch": 1e3 * t / reps,
            "all_status_ok": bool((holder["status"] == 0).all().item()),
        }
        # reverse mode: pdq_lml_fwd (value, sqrt(N) checkpoints) then pdq_lml_bwd (adjoint pass)
        adj = {}

        def fwd_call():
            adj["fwd"] = _native.lml_fwd(cfg, thetas, y0, data, std, t0=0.0, dt=0.01, num_steps=num_steps,
                                         save_every=10, stream=stream, workspace=adj.get("ws"),
                                         outputs=adj.get("fwd_out"))
            adj["ws"] = adj["fwd"]["_workspace"]
            adj["fwd_out"] = {k: adj["fwd"][k] for k in ("lml", "status")}

        def bwd_call():
            adj["bwd"] = _native.lml_bwd(adj["fwd"], None, outputs=adj.get("bwd"))

        t_fwd = timed_region(torch, stream, fwd_call, reps, 3)
        t_bwd = timed_region(torch, stream, bwd_call, reps, 3)
        g_fm, g_adj = holder["grad"], adj["bwd"]["grad"]
        # cold call: a fresh workspace, so the shared covariance plan is built
        # inside the timed call (lml_plan_kernel) before the adjoint pair runs
        cold = {}

        def cold_call():
            cold["fwd"] = _native.lml_fwd(cfg, thetas, y0, data, std, t0=0.0, dt=0.01, num_steps=num_steps,
                                          save_every=10, stream=stream)
            cold["bwd"] = _native.lml_bwd(cold["fwd"], None)

        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        cold_call()
        e1.record(stream)
        e1.synchronize()
        t_cold = e0.elapsed_time(e1) / 1e3
        res[prec]["adjoint"] = {
            "grads_per_s": B * reps / (t_fwd + t_bwd),
            "ms_fwd": 1e3 * t_fwd / reps,
            "ms_bwd": 1e3 * t_bwd / reps,
            "cold_grads_per_s": B / t_cold,
            "cold_ms": 1e3 * t_cold,
            "cold": "first call on a fresh workspace: allocation, the covariance plan (parameter-independent, "
                    "reused by every later call on the same grid, step and noise) and the adjoint pair",
            "checkpoint_every": int(round(num_steps ** 0.5)),
            "max_rel_diff_vs_forward_mode": float(((g_adj - g_fm).abs().amax(1) / g_fm.norm(dim=1)).max()),
        }
        res[prec]["forward_mode"] = {k: res[prec].pop(k) for k in ("grads_per_s", "ms_per_batch")}
        res[prec]["all_status_ok"] = res[prec]["all_status_ok"] and bool((adj["fwd"]["status"] == 0).all().item())
    res["config"] = {"samples": B, "num_steps": num_steps, "observations": int(data.shape[0]), "num_derivatives": 3,
                     "primary": "adjoint (pdq_lml_fwd + pdq_lml_bwd, sqrt(N) checkpoints), plan reused"}
    return res


def lml_cpu_baseline(samples=2):
    """The oracle's LML gradient (PyTorch float64 reverse mode through the CPU
    restatement of the reference) on a few of the workload's parameter
    samples, one process."""
    import time

    import torch

    from oracle import lml as oracle_lml
    from probdiffeq_gb300 import configs

    num_steps, data = configs.fhn_observations()
    thetas = configs.fhn_theta_samples(samples)
    threads = torch.get_num_threads()
    t = time.perf_counter()
    for th in thetas:
        oracle_lml.lml_value_and_grads(th, configs.FHN_U0, data, 0.01, num_steps, 10, configs.FHN_STD)
    dt = time.perf_counter() - t
    return {"value": samples / dt, "unit": "grads/s", "cores": threads, "kind": "port",
            "sample": f"{samples} parameter samples of the 1024, oracle (PyTorch float64 reverse mode through the "
                      f"CPU restatement), one process, {threads} torch threads", "seconds": dt}


def measured_peaks():
    """The measured peaks of this GPU pool (HBM copy GB/s, bf16 TF/s), or {}."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def measured_l2_copy_gbs(torch, device, sizes_mib=(16, 24, 32), reps=200):
    """Copy bandwidth of an L2-resident buffer pair (read + write bytes), the
    best over a few sizes that fit the L2 twice over, CUDA events over
    ``reps`` back-to-back copies: the ceiling of a kernel whose working set
    stays in L2."""
    best = 0.0
    for mib in sizes_mib:
        a = torch.ones(mib * 1024 * 1024 // 4, dtype=torch.float32, device=device)
        b = torch.empty_like(a)
        for _ in range(10):
            b.copy_(a)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            b.copy_(a)
        e1.record()
        e1.synchronize()
        best = max(best, 2 * a.numel() * 4 * reps / (e0.elapsed_time(e1) / 1e3) / 1e9)
        del a, b
    return best


# Algorithmic bytes per attempt and dimension of the block-diagonal solver, the
# configuration's work model: read and write m (n) and L (n^2) in float32, one f
# value (n = 4: 164 B; the kernel stores L packed, 2 x 14 floats + f = 116 B)
BURGERS_BYTES_PER_DIM = 2 * (4 + 16) * 4 + 4
BURGERS_STORED_BYTES_PER_DIM = 2 * 14 * 4 + 4


def oracle_burgers_attempt_seconds(d_small=64, t1=0.05):
    """Seconds per attempt of the oracle's block-diagonal Burgers solve
    (PyTorch float64, per-dimension loop) at d = d_small, measured over the
    solve on [0, t1] after the Taylor-mode start."""
    import time

    import torch

    from oracle import problems, solvers, ssm
    from probdiffeq_gb300 import configs

    threads = torch.get_num_threads()
    torch.set_num_threads(1)  # d = 64 tensors: one thread is the fastest setting
    try:
        p = torch.tensor([0.01], dtype=torch.float64)
        u0 = torch.tensor(configs.burgers_u0(1, d_small)[0])
        tc = problems.taylor_derivatives(problems.burgers, u0, p, 3)
        S = ssm.BdSSM()
        c = S.constraint_ode_ts0(lambda u, t: problems.burgers(u[0], p))
        t = time.perf_counter()
        res = solvers.solve_adaptive_terminal_values(solvers.SolverDynamic(solvers.StrategyFilter(), c),
                                                     solvers.ErrorResidualStd(c), S.prior_wiener_integrated(tc), 0.0,
                                                     t1, 1e-4, 1e-4, dt0=0.1 * t1)
        sec = (time.perf_counter() - t) / res.num_attempts
    finally:
        torch.set_num_threads(threads)
    return sec, res.num_attempts, 1


def burgers_blockdiag_secondary(torch, _native, ensemble, device, t1=1.0, cpu=True):
    """The high-dimensional block-diagonal configuration: 64 viscous Burgers
    instances (nu = 0.01), periodic grid of d = 4096, t in [0, t1], IWP nu = 3,
    TS0 blockdiag filter, dynamic calibration, rtol = atol = 1e-4, float32.

    One solve (seconds long) after a warm-up on a short horizon: the initial
    values are copied from pinned host memory, the solver runs, the terminal
    means are copied back to pinned host memory, all on one stream; CUDA
    events bracket the solver launch (``value``) and the whole step (``e2e``).
    The per-instance state (2 x 14 floats per dimension, 14.7 MB per buffer)
    stays in L2, so the roofline is taken against the measured L2 copy
    bandwidth and, for reference, the measured HBM copy bandwidth."""
    from probdiffeq_gb300 import configs

    B, d = 64, 4096
    stream = torch.cuda.current_stream()
    h_u0 = torch.tensor(configs.burgers_u0(B, d), dtype=torch.float64).pin_memory()
    h_prm = torch.full((B, 1), 0.01, dtype=torch.float64).pin_memory()
    d_u0 = torch.empty(h_u0.shape, dtype=torch.float64, device=device)
    d_prm = torch.empty(h_prm.shape, dtype=torch.float64, device=device)
    cfg = ensemble.make_config(field="burgers", num_derivatives=3, ode_dim=d, ssm="blockdiag", solver="dynamic",
                               precision="float32", atol=1e-4, rtol=1e-4, clip_dt=True, max_attempts=1 << 26)
    outs = _native.alloc_outputs(cfg, B, 2, True, device)
    h_mean = torch.empty(tuple(outs["u_mean"].shape), dtype=outs["u_mean"].dtype).pin_memory()

    def span(t_end):
        sa = torch.tensor([0.0, t_end], dtype=torch.float64, device=device).expand(B, 2).contiguous()
        return sa, torch.full((B,), 0.1 * t_end, dtype=torch.float64, device=device)

    sa_w, dt0_w = span(1e-4)
    sa, dt0 = span(t1)
    d_u0.copy_(h_u0)
    d_prm.copy_(h_prm)
    _native.solve_adaptive(cfg, sa_w, d_prm, d_u0, dt0_w, True, outs, stream=stream)  # warm-up
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    ev[0].record(stream)
    d_u0.copy_(h_u0, non_blocking=True)
    d_prm.copy_(h_prm, non_blocking=True)
    ev[1].record(stream)
    _native.solve_adaptive(cfg, sa, d_prm, d_u0, dt0, True, outs, stream=stream)
    ev[2].record(stream)
    h_mean.copy_(outs["u_mean"], non_blocking=True)
    ev[3].record(stream)
    ev[3].synchronize()
    t_kernel = ev[1].elapsed_time(ev[2]) / 1e3
    t_e2e = ev[0].elapsed_time(ev[3]) / 1e3
    attempts = outs["num_attempts"].to(torch.float64)
    status_ok = int((outs["status"] == 0).sum())
    finite = bool(torch.isfinite(h_mean).all())
    bytes_alg = float(attempts.sum()) * d * BURGERS_BYTES_PER_DIM
    achieved = bytes_alg / t_kernel / 1e9
    stored = float(attempts.sum()) * d * BURGERS_STORED_BYTES_PER_DIM / t_kernel / 1e9
    l2 = measured_l2_copy_gbs(torch, device)
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs")
    hbm_src = "MEASURED_PEAKS.json hbm_gbs (STREAM-style copy)"
    if not hbm:
        hbm, hbm_src = 6800.0, "fallback 6.8 TB/s (no measured peak file)"
    out = {
        "config": {"workload": "burgers_blockdiag", "instances": B, "d": d, "nu_visc": 0.01, "t_span": [0.0, t1],
                   "num_derivatives": 3, "ssm": "blockdiag", "constraint": "ts0", "strategy": "filter",
                   "solver": "dynamic", "rtol": 1e-4, "atol": 1e-4, "output": "terminal values (clip_dt)",
                   "precision": "float32", "steps": 1, "warmup": "one solve on [0, 1e-4]",
                   "l2": "state L2-resident by design; not flushed"},
        "value": B / t_kernel, "unit": "solves/s", "ms_per_step": 1e3 * t_kernel,
        "e2e": {"value": B / t_e2e, "unit": "solves/s", "h2d_bytes_per_step": h_u0.numel() * 8 + h_prm.numel() * 8,
                "d2h_bytes_per_step": h_mean.numel() * h_mean.element_size()},
        "stats": {"attempts_max": int(attempts.max()), "attempts_mean": float(attempts.mean()),
                  "us_per_attempt_slowest": 1e6 * t_kernel / float(attempts.max()), "status_ok": status_ok,
                  "terminal_means_finite": finite},
        "roofline": {"bound": "hbm", "achieved": achieved, "unit": "GB/s", "peak": hbm, "frac": achieved / hbm,
                     "peak_source": hbm_src,
                     "bytes_per_attempt_dimension": BURGERS_BYTES_PER_DIM,
                     "l2_peak": l2, "frac_of_l2": achieved / l2,
                     "l2_peak_source": "measured L2-resident copy (best of 2 x 16 / 24 / 32 MiB, read + write bytes)",
                     "stored_bytes_gbs": stored,
                     "note": "algorithmic bytes = sum over instances of attempts x d x (2 (n + n^2) 4 B + 4 B), "
                             "averaged over the launch, in which instances finish at different times; the state "
                             "(2 x 14.7 MB) stays L2-resident, DRAM sees only inputs and outputs"},
        "gpu_launches": 1,
    }
    if cpu:
        sec, n_att, threads = oracle_burgers_attempt_seconds()
        per_attempt = sec * d / 64
        out["cpu_baseline"] = {
            "value": 1.0 / (per_attempt * float(attempts.mean())), "unit": "solves/s", "cores": threads, "kind": "port",
            "sample": f"oracle (PyTorch float64 CPU restatement, per-dimension loop) at d = 64 over t in [0, 0.05] "
                      f"({n_att} attempts, {1e3 * sec:.1f} ms each), scaled x64 to d = 4096 and multiplied by this "
                      f"run's mean attempts per instance; one process, {threads} torch threads",
        }
    return out


def dense_flops_per_attempt(N=8, d=2):
    """Algorithmic FLOP per attempt of the dense TS1 fixed-point solver, the
    convention of the configuration's work model (matmuls dense 2mnk,
    Householder R-only QR of m x n 2mn^2 - (2/3)n^3): predict 2N^3 + (10/3)N^3,
    update (revert) (4/3)(N+d)^3, merge 2N^3 + (10/3)N^3, TS1 2dN."""
    return 2 * N**3 + 10 / 3 * N**3 + 4 / 3 * (N + d) ** 3 + 2 * N**3 + 10 / 3 * N**3 + 2 * d * N


VDP_FLOPS_PER_ATTEMPT = dense_flops_per_attempt()


def oracle_vdp_attempt_seconds(mu=3.0):
    """Seconds per attempt of the oracle's dense TS1 fixed-point solve of van
    der Pol (PyTorch float64, one thread) at ``mu`` with 100 save points."""
    import time

    import numpy as np
    import torch

    from oracle import problems, solvers, ssm

    threads = torch.get_num_threads()
    torch.set_num_threads(1)
    try:
        p = torch.tensor([mu], dtype=torch.float64)
        tc = problems.taylor_derivatives(problems.van_der_pol, torch.tensor([2.0, 0.0], dtype=torch.float64), p, 3)
        S = ssm.DenseSSM()
        c = S.constraint_ode_ts1(lambda u, t: problems.van_der_pol(u[0], p),
                                 lambda u, t: problems.jacobian(problems.van_der_pol, u, p), 2)
        t = time.perf_counter()
        res = solvers.solve_adaptive_save_at(solvers.SolverDynamic(solvers.StrategyFixedPoint(), c),
                                             solvers.ErrorResidualStd(c), S.prior_wiener_integrated(tc),
                                             np.linspace(0.0, 2.0 * mu, 100), 1e-5, 1e-5)
        sec = (time.perf_counter() - t) / res.num_attempts
    finally:
        torch.set_num_threads(threads)
    return sec, res.num_attempts


def vdp_dense_secondary(torch, _native, ensemble, device, mu_max=1000.0, cpu=True):
    """The stiff dense configuration: 4096 van der Pol instances, mu ~
    log-uniform [1, mu_max], y0 = (2, 0), t in [0, 2 mu] with 100 save points,
    IWP nu = 3, dense TS1, fixed-point smoother, dynamic calibration,
    rtol = atol = 1e-5; float32, the structure-exploiting kernel.

    One solve (about a minute at mu_max = 1000: the slowest instance takes
    3.1 M attempts) after a warm-up on mu <= 2: inputs copied from pinned host
    memory, the solver, the 100 smoothed marginals and the posterior's
    backward conditionals copied back to pinned host memory, CUDA events
    around the solver (``value``) and the whole step (``e2e``).  The float64
    batch and a float32 one for the ratio run on mu <= 10 (a float64 solve to
    mu = 1000 takes about ten minutes: GB300's FP64 pipe)."""
    from probdiffeq_gb300 import configs

    B, S = 4096, 100
    stream = torch.cuda.current_stream()

    # sixteen lanes per instance: the batch time is the stiffest instances' attempts run back to
    # back on an otherwise idle GPU, where the most lanes per attempt give the shortest chain
    def cfg_of(precision):
        return ensemble.make_config(field="van_der_pol", num_derivatives=3, ode_dim=2, ssm="dense", constraint="ts1",
                                    strategy="fixedpoint", solver="dynamic", precision=precision, atol=1e-5,
                                    rtol=1e-5, clip_dt=False, max_attempts=1 << 24, kernel_variant=5)

    def inputs(mu_hi):
        mu, save_at, y0 = configs.vdp_dense(B, mu_hi)
        return (mu[:, None].contiguous().pin_memory(), save_at.pin_memory(), y0.pin_memory(),
                torch.full((B,), 0.1, dtype=torch.float64).pin_memory())

    def solve(cfg, host, outs):
        dev = [x.to(device, non_blocking=True) for x in host]
        _native.solve_adaptive(cfg, dev[1], dev[0], dev[2], dev[3], False, outs, stream=stream)
        return dev

    cfg32 = cfg_of("float32")
    outs = _native.alloc_outputs(cfg32, B, S, False, device, posterior=True)
    solve(cfg32, inputs(2.0), outs)  # warm-up (module load, first touch)
    torch.cuda.synchronize()
    host = inputs(mu_max)
    h_out = {k: torch.empty(tuple(v.shape), dtype=v.dtype).pin_memory() for k, v in outs.items()
             if isinstance(v, torch.Tensor) and not k.startswith("_")}
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    ev[0].record(stream)
    dev = [x.to(device, non_blocking=True) for x in host]
    ev[1].record(stream)
    _native.solve_adaptive(cfg32, dev[1], dev[0], dev[2], dev[3], False, outs, stream=stream)
    ev[2].record(stream)
    for k, v in h_out.items():
        v.copy_(outs[k], non_blocking=True)
    ev[3].record(stream)
    ev[3].synchronize()
    t_kernel = ev[1].elapsed_time(ev[2]) / 1e3
    t_e2e = ev[0].elapsed_time(ev[3]) / 1e3
    attempts = outs["num_attempts"].to(torch.float64)
    steps = outs["num_steps"][:, -1].to(torch.float64)
    status_ok = int((outs["status"] == 0).sum())
    flops = float(attempts.sum()) * VDP_FLOPS_PER_ATTEMPT
    achieved = flops / t_kernel / 1e12
    peak, sms = measured_fp32_peak(torch, _native, device)
    out = {
        "config": {"workload": "van_der_pol_dense", "instances": B, "mu": f"log-uniform [1, {mu_max}]",
                   "t_span": "[0, 2 mu]", "save_at": S, "num_derivatives": 3, "ssm": "dense", "constraint": "ts1",
                   "strategy": "fixedpoint", "solver": "dynamic", "rtol": 1e-5, "atol": 1e-5, "precision": "float32",
                   "kernel": "structure-exploiting QRs, 16 lanes per instance", "steps": 1,
                   "warmup": "one solve with mu <= 2"},
        "value": B / t_kernel, "unit": "solves/s", "ms_per_step": 1e3 * t_kernel,
        "e2e": {"value": B / t_e2e, "unit": "solves/s",
                "h2d_bytes_per_step": sum(x.numel() * x.element_size() for x in host),
                "d2h_bytes_per_step": sum(v.numel() * v.element_size() for v in h_out.values())},
        "stats": {"attempts_max": int(attempts.max()), "attempts_mean": float(attempts.mean()),
                  "accepted_steps_max": int(steps.max()), "accepted_steps_mean": float(steps.mean()),
                  "us_per_attempt_slowest": 1e6 * t_kernel / float(attempts.max()), "status_ok": status_ok},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                     "flops_per_attempt": VDP_FLOPS_PER_ATTEMPT,
                     "peak_source": f"measured FP32 FMA probe on this GPU ({sms} SMs)",
                     "note": f"latency-bound: the batch time is the slowest instance's {attempts.max() / 1e6:.2f} M "
                             "attempts, each a chain of dependent reflectors on sixteen lanes; most SMs are idle "
                             "for most of it"},
        "gpu_launches": 1,
    }
    # float64 and float32 on mu <= 10 (the float64 batch to mu = 1000 does not fit the run's time)
    small = inputs(10.0)
    res = {}
    for precision in ("float32", "float64"):
        c = cfg_of(precision)
        o = _native.alloc_outputs(c, B, S, False, device, posterior=True)
        solve(c, small, o)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        d = [x.to(device) for x in small]
        torch.cuda.synchronize()
        e0.record(stream)
        _native.solve_adaptive(c, d[1], d[0], d[2], d[3], False, o, stream=stream)
        e1.record(stream)
        e1.synchronize()
        t = e0.elapsed_time(e1) / 1e3
        res[precision] = {"solves_per_s": B / t, "ms_per_step": 1e3 * t, "attempts_max": int(o["num_attempts"].max()),
                          "status_ok": int((o["status"] == 0).sum())}
    res["fp32_speedup"] = res["float32"]["solves_per_s"] / res["float64"]["solves_per_s"]
    out["mu_le_10"] = res
    if cpu:
        sec, n_att = oracle_vdp_attempt_seconds()
        out["cpu_baseline"] = {
            "value": 1.0 / (sec * float(attempts.mean())), "unit": "solves/s", "cores": 1, "kind": "port",
            "sample": f"oracle (PyTorch float64 CPU restatement) at mu = 3 with 100 save points ({n_att} attempts, "
                      f"{1e3 * sec:.1f} ms each), multiplied by this run's mean attempts per instance; one process, "
                      "one torch thread",
        }
    return out


# ---------------------------------------------------------------------------
# the headline workload
# ---------------------------------------------------------------------------


def run_lv_ensemble(args):
    import torch
    import torch.distributed as dist

    from probdiffeq_gb300 import _native, autotune, ensemble, pipeline, replicas
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

    def config(precision, variant=0, ipb=0):
        return ensemble.make_config(
            field="lotka_volterra", num_derivatives=4, ode_dim=2, solver="mle", precision=precision,
            atol=WORKLOAD["atol"], rtol=WORKLOAD["rtol"], clip_dt=True, kernel_variant=variant,
            instances_per_block=ipb,
        )

    stream = torch.cuda.current_stream()
    d_params, d_y0 = params.to(device), y0.to(device)
    d_save = save_at.expand(B, 2).contiguous().to(device)
    d_dt0 = torch.full((B,), WORKLOAD["dt0"], dtype=torch.float64, device=device)
    outs = _native.alloc_outputs(config("float32"), B, 2, True, device)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=device)

    def device_step(c):
        _native.solve_adaptive(c, d_save, d_params, d_y0, d_dt0, True, outs, stream=stream)

    names = {1: "thread per instance", 2: "8 lanes per instance, <=128 regs", 3: "8 lanes per instance, <=85 regs",
             4: "a covariance warp and a mean warp per 32 instances"}

    def label(cand):
        return f"{names[cand[0]]}, {cand[1] or 'default'} instances per CTA"

    clk = ClockSampler(local)
    clk.__enter__()
    try:
        # ---- the library autotuner picks the mapping and instances per CTA on this batch ----
        def tune(precision):
            return autotune.tune(config(precision), d_save, d_params, d_y0, d_dt0, True, stream=stream)

        fixed = {"thread": 1, "lanes": 2, "lanes_compact": 3, "split": 4}.get(args.variant)
        if fixed is None:
            best32, tune32 = tune("float32")
            best64, tune64 = tune("float64")
        else:
            best32 = best64 = (fixed, 0)
            tune32, tune64 = {}, {}
        cfg, cfg64 = config("float32", *best32), config("float64", *best64)

        # ---- value: device-resident inputs, FP32 bulk ----
        t_dev = timed_region(torch, stream, lambda: device_step(cfg), args.steps, args.warmup, flush, world, dist)
        attempts = outs["num_attempts"].to(torch.float64).sum().item()
        steps_acc = outs["num_steps"].to(torch.float64).sum().item()
        status_ok = bool((outs["status"] == 0).all().item())
        mean32 = outs["u_mean"][:, 0].clone()
        max_attempts_inst = int(outs["num_attempts"].max().item())

        # ---- FP64 bulk (the same kernel in float64, batched) ----
        k64 = max(3, args.steps // 20)
        t_dev64 = timed_region(torch, stream, lambda: device_step(cfg64), k64, 1, flush, world, dist)
        mean64 = outs["u_mean"][:, 0].clone()
        attempts64 = outs["num_attempts"].to(torch.float64).sum().item()
        # the plain float64 kernel (one thread per instance), when the autotuner chose another mapping
        cfg64_thread = config("float64", 1, 0)
        t_dev64_thread = (t_dev64 if best64[0] == 1 else
                          timed_region(torch, stream, lambda: device_step(cfg64_thread), k64, 1, flush, world, dist))
        # terminal u: float32 vs float64 relative to each instance's largest component
        rel = ((mean32[:, 0] - mean64[:, 0]).abs().amax(dim=1) / mean64[:, 0].abs().amax(dim=1)).cpu()
        rel_f32_f64 = {"median": rel.median().item(), "max": rel.max().item()}

        # ---- e2e through the public API: pinned host inputs -> solve -> pinned host outputs every step,
        # uploads / solves / downloads of consecutive batches overlapped on three streams ----
        h_params, h_y0 = params.pin_memory(), y0.pin_memory()
        h_save = save_at.expand(B, 2).contiguous().pin_memory()
        h_dt0 = torch.full((B,), WORKLOAD["dt0"], dtype=torch.float64).pin_memory()
        pipe = pipeline.EnsemblePipeline(cfg, B, 2, params.shape[1], terminal_only=True, device=device, depth=2,
                                         graph=not args.no_graph)
        h_outs = [pipe.alloc_host_outputs() for _ in range(2)]
        h2d = sum(t.numel() * t.element_size() for t in (h_params, h_y0, h_save, h_dt0))
        d2h = sum(t.numel() * t.element_size() for t in h_outs[0].values())

        def e2e_submit(k):
            with torch.cuda.stream(pipe.streams["upload"]):
                flush.fill_(1.0)  # evict L2 before this batch's upload
            pipe.submit(h_params, h_y0, h_save, h_dt0, h_outs[k % 2])

        t_e2e = timed_pipeline(torch, pipe, e2e_submit, args.steps, args.warmup, world, dist)
        e2e_ok = all(bool((h["status"] == 0).all()) for h in h_outs) and torch.equal(h_outs[0]["u_mean"][:, 0], mean32.cpu())

        # ---- secondary: the plain per-instance method and LML gradients ----
        secondary = None
        if not args.no_secondary:
            secondary = {
                "single_instance_lv_dynamic": single_instance(torch, _native, ensemble, device),
                "lml_gradients_fhn": lml_gradients(torch, _native, ensemble, device),
            }
            if not args.no_cpu_baseline:
                secondary["lml_gradients_fhn"]["cpu_baseline"] = lml_cpu_baseline()
                secondary["single_instance_lv_dynamic"]["cpu_baseline"] = single_instance_cpu_baseline()
            if args.burgers_t1 > 0 and world == 1:
                secondary["burgers_blockdiag"] = burgers_blockdiag_secondary(
                    torch, _native, ensemble, device, t1=args.burgers_t1, cpu=not args.no_cpu_baseline)
            if args.vdp_mu_max > 0 and world == 1:
                secondary["vdp_dense"] = vdp_dense_secondary(torch, _native, ensemble, device, mu_max=args.vdp_mu_max,
                                                             cpu=not args.no_cpu_baseline)
    finally:
        clk.__exit__(None, None, None)

    # the slowest replica bounds the job (no collective on the data path)
    t_dev, t_e2e, t_dev64 = (replicas.max_over_ranks(x) for x in (t_dev, t_e2e, t_dev64))

    peak, sms = measured_fp32_peak(torch, _native, device)
    n, d = 5, 2
    fpa = flops_per_attempt(n, d)
    achieved = attempts * fpa / (t_dev / args.steps) / 1e12

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return
    value = world * B * args.steps / t_dev
    result = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * t_dev / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 bulk + float-pair (48-bit) time/calibration/error-norm accumulators",
        "data": "synthetic (seeded Lotka-Volterra ensemble)",
        "config": dict(WORKLOAD, parallelism=f"replicas x{world}" if world > 1 else "single GPU"),
        "e2e": {
            "value": world * B * args.steps / t_e2e,
            "unit": UNIT,
            "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h,
            "path": "probdiffeq_gb300.pipeline.EnsemblePipeline: 2 slots, upload / compute / download streams"
                    + ("" if args.no_graph else ", solver launch replayed from a CUDA graph"),
            "l2": "flushed (256 MiB write) on the upload stream before each batch's upload",
            "outputs_match_device_run": e2e_ok,
        },
        "gpu_launches": args.steps,
        "autotune": {
            "float32": {label(k): v for k, v in tune32.items()},
            "float64": {label(k): v for k, v in tune64.items()},
            "unit": "ms per ensemble solve (probdiffeq_gb300.autotune: one timed solve after one warm-up)",
            "chosen": {"float32": label(best32), "float64": label(best64)},
        },
        "roofline": {
            "bound": "fp32",
            "achieved": achieved,
            "peak": peak,
            "unit": "TFLOP/s",
            "frac": achieved / peak,
            "traffic": profiled_dram_bytes(),
            "peak_source": f"measured FP32 FMA probe on this GPU ({sms} SMs); MEASURED_PEAKS.json lists only HBM and bf16",
            "flops_per_attempt": fpa,
            "attempts_per_step": attempts,
            "note": "latency-bound: 16384 one-thread instances fill < 1 warp per SM sub-partition",
        },
        "fp64": {
            "value": world * B * k64 / t_dev64,
            "unit": UNIT,
            "ms_per_step": 1e3 * t_dev64 / k64,
            "attempts_per_step": attempts64,
            "fp32_speedup": value / (world * B * k64 / t_dev64),
            "mapping": label(best64),
            "thread_per_instance": {"ms_per_step": 1e3 * t_dev64_thread / k64,
                                    "fp32_speedup": value / (world * B * k64 / t_dev64_thread)},
            "rel_terminal_diff_f32_vs_f64": rel_f32_f64,
        },
        "stats": {
            "accepted_steps_mean": steps_acc / B,
            "attempts_mean": attempts / B,
            "attempts_max": max_attempts_inst,
            "all_status_ok": status_ok,
        },
        "clocks": clk.summary(),
    }
    result["accuracy"] = accuracy_vs_exact(params, y0, mean32.cpu(), mean64.cpu())
    if secondary is not None:
        result["secondary"] = secondary
    if not args.no_cpu_baseline:
        try:
            result["cpu_baseline"] = cpu_baseline(args.cpu_seconds)
        except Exception as e:  # the port is test infrastructure; report why it is missing
            result["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                                      "sample": f"unavailable: {e}"}
    print(json.dumps(result))
    if world > 1:
        dist.destroy_process_group()


# ---------------------------------------------------------------------------
# the other workloads (one line each)
# ---------------------------------------------------------------------------


def base_line(metric, value, unit, args, ms, higher, dtype, config, **extra):
    line = {
        "metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": higher, "scaling": "weak", "vs_baseline": None, "dtype": dtype,
        "data": "synthetic", "config": config,
    }
    line.update(extra)
    return line


def run_lv_single(args):
    import torch

    from probdiffeq_gb300 import _native, ensemble
    from probdiffeq_gb300 import build as native_build

    native_build.build()
    device = torch.device("cuda:0")
    with ClockSampler(0) as clk:
        r = single_instance(torch, _native, ensemble, device, reps=args.steps)
    cfg = {"workload": "lotka_volterra_single", "instances": 1, "params": [0.5, 0.05, 0.5, 0.05], "y0": [20.0, 20.0],
           "t_span": [0.0, 50.0], "num_derivatives": 4, "solver": "dynamic", "rtol": 1e-6, "atol": 1e-6}
    cpu = None if args.no_cpu_baseline else single_instance_cpu_baseline()
    print(json.dumps(base_line("single-instance solve latency (float64)", r["float64"]["ms_per_solve"], "ms", args,
                               r["float64"]["ms_per_solve"], False, "f64", cfg, float32=r["float32"],
                               cpu_baseline=cpu, gpu_launches=args.steps, clocks=clk.summary())))


def run_fhn_lml(args):
    import torch

    from probdiffeq_gb300 import _native, ensemble
    from probdiffeq_gb300 import build as native_build

    native_build.build()
    device = torch.device("cuda:0")
    with ClockSampler(0) as clk:
        r = lml_gradients(torch, _native, ensemble, device, reps=args.steps)
    adj = r["float32"]["adjoint"]
    cpu = None if args.no_cpu_baseline else lml_cpu_baseline()
    print(json.dumps(base_line("LML grads/s", adj["grads_per_s"], "grads/s", args, adj["ms_fwd"] + adj["ms_bwd"],
                               True, "f32 bulk + f64 log-pdf sum", dict(r["config"], workload="fitzhugh_nagumo_lml"),
                               float32=r["float32"], float64=r["float64"], cpu_baseline=cpu,
                               gpu_launches=4 * args.steps,  # plan check + value pass, plan check + adjoint pass
                               clocks=clk.summary())))


def run_vdp_dense(args):
    import torch

    from probdiffeq_gb300 import _native, ensemble
    from probdiffeq_gb300 import build as native_build

    native_build.build()
    device = torch.device("cuda:0")
    B = args.instances if args.instances != WORKLOAD["instances"] else 4096
    from probdiffeq_gb300 import configs

    mu, save_at, y0 = configs.vdp_dense(B, args.mu_max)
    save_at, y0 = save_at.to(device), y0.to(device)
    prm = mu[:, None].contiguous().to(device)
    dt0 = torch.full((B,), 0.1, dtype=torch.float64, device=device)
    stream = torch.cuda.current_stream()
    res = {}
    with ClockSampler(0) as clk:
        for prec in args.precisions.split(","):
            cfg = ensemble.make_config(field="van_der_pol", num_derivatives=3, ode_dim=2, ssm="dense", constraint="ts1",
                                       strategy="fixedpoint", solver="dynamic", precision=prec, atol=1e-5, rtol=1e-5,
                                       clip_dt=False, max_attempts=1 << 24,
                                       kernel_variant={"lanes": 2, "thread": 1, "struct": 3, "struct8": 4}.get(
                                           args.variant, 5))
            outs = _native.alloc_outputs(cfg, B, 100, False, device, posterior=True)
            t = timed_region(torch, stream, lambda: _native.solve_adaptive(cfg, save_at, prm, y0, dt0, False, outs,
                                                                             stream=stream), args.steps, args.warmup)
            steps = outs["num_steps"][:, -1].to(torch.float64)
            res[prec] = {"solves_per_s": B * args.steps / t, "ms_per_step": 1e3 * t / args.steps,
                         "accepted_steps_max": int(steps.max()), "accepted_steps_mean": float(steps.mean()),
                         "attempts_max": int(outs["num_attempts"].max()),
                         "status_ok": int((outs["status"] == 0).sum())}
    first = args.precisions.split(",")[0]
    cfg = {"workload": "van_der_pol_dense", "instances": B, "mu": f"log-uniform [1, {args.mu_max}]", "t_span": "[0, 2 mu]",
           "num_derivatives": 3, "ssm": "dense", "constraint": "ts1", "strategy": "fixedpoint", "solver": "dynamic",
           "save_at": 100, "rtol": 1e-5, "atol": 1e-5,
           "mapping": {"lanes": "8 lanes per instance", "thread": "thread per instance",
                       "struct": "structure-exploiting QRs, 4 lanes per instance",
                       "struct8": "structure-exploiting QRs, 8 lanes per instance"}.get(
               args.variant, "structure-exploiting QRs, 16 lanes per instance")}
    print(json.dumps(base_line("ensemble IVP solves/s", res[first]["solves_per_s"], "solves/s", args,
                               res[first]["ms_per_step"], True, first, cfg, by_precision=res, gpu_launches=args.steps,
                               clocks=clk.summary())))


def run_burgers_blockdiag(args):
    import numpy as np
    import torch

    from probdiffeq_gb300 import _native, ensemble
    from probdiffeq_gb300 import build as native_build

    native_build.build()
    device = torch.device("cuda:0")
    B, d = 64, 4096
    from probdiffeq_gb300 import configs

    u0 = torch.tensor(configs.burgers_u0(B, d), dtype=torch.float64, device=device)
    t1 = args.t1
    prm = torch.full((B, 1), 0.01, dtype=torch.float64, device=device)
    sa = torch.tensor([0.0, t1], dtype=torch.float64, device=device).expand(B, 2).contiguous()
    dt0 = torch.full((B,), 0.1 * t1, dtype=torch.float64, device=device)
    stream = torch.cuda.current_stream()
    res = {}
    with ClockSampler(0) as clk:
        for prec in args.precisions.split(","):
            cfg = ensemble.make_config(field="burgers", num_derivatives=3, ode_dim=d, ssm="blockdiag", solver="dynamic",
                                       precision=prec, atol=1e-4, rtol=1e-4, clip_dt=True, max_attempts=1 << 26,
                                       constraint=args.constraint or "ts0")
            outs = _native.alloc_outputs(cfg, B, 2, True, device)
            t = timed_region(torch, stream, lambda: _native.solve_adaptive(cfg, sa, prm, u0, dt0, True, outs,
                                                                             stream=stream), args.steps, args.warmup)
            attempts = outs["num_attempts"].to(torch.float64)
            res[prec] = {"solves_per_s": B * args.steps / t, "ms_per_step": 1e3 * t / args.steps,
                         "attempts_max": int(attempts.max()), "attempts_mean": float(attempts.mean()),
                         "us_per_attempt_slowest": 1e6 * (t / args.steps) / float(attempts.max()),
                         "status_ok": int((outs["status"] == 0).sum())}
    first = args.precisions.split(",")[0]
    cfg = {"workload": "burgers_blockdiag", "instances": B, "d": d, "nu_visc": 0.01, "t_span": [0.0, t1],
           "num_derivatives": 3, "ssm": "blockdiag", "constraint": args.constraint or "ts0", "solver": "dynamic",
           "rtol": 1e-4, "atol": 1e-4}
    print(json.dumps(base_line("ensemble IVP solves/s", res[first]["solves_per_s"], "solves/s", args,
                               res[first]["ms_per_step"], True, first, cfg, by_precision=res, gpu_launches=args.steps,
                               clocks=clk.summary())))


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    vals = []
    cb = None
    for i in range(args.warmup + args.steps):
        cb = cpu_baseline(args.cpu_seconds / max(1, args.steps + args.warmup))
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
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="lv_ensemble",
                    choices=["lv_ensemble", "lv_single", "fhn_lml", "vdp_dense", "burgers_blockdiag"])
    ap.add_argument("--variant", default="auto", choices=["auto", "thread", "lanes", "lanes_compact", "split", "struct",
                                                              "struct8", "struct16"],
                    help="lv_ensemble: instance-to-lane mapping (auto = time the autotuner's candidates and keep "
                         "the fastest)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-graph", action="store_true", help="e2e: launch the solver eagerly instead of from CUDA graphs")
    ap.add_argument("--no-secondary", action="store_true",
                    help="skip the single-instance, LML and block-diagonal Burgers measurements")
    ap.add_argument("--burgers-t1", type=float, default=1.0,
                    help="lv_ensemble: horizon of the block-diagonal Burgers secondary (0 skips it)")
    ap.add_argument("--vdp-mu-max", type=float, default=1000.0,
                    help="lv_ensemble: mu range of the stiff dense van der Pol secondary (0 skips it)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--instances", type=int, default=WORKLOAD["instances"], help="ensemble size (16384 is the headline workload)")
    ap.add_argument("--mu-max", type=float, default=1000.0, help="vdp_dense: mu ~ log-uniform [1, mu_max]")
    ap.add_argument("--t1", type=float, default=1.0, help="burgers_blockdiag: end time")
    ap.add_argument("--precisions", default="float32,float64", help="vdp_dense / burgers_blockdiag precisions")
    ap.add_argument("--constraint", default=None, choices=["ts0", "ts1"],
                    help="burgers_blockdiag: linearisation (ts0 is the configuration's; ts1 uses the Jacobian diagonal)")
    args = ap.parse_args()
    if args.impl == "reference":
        args.warmup = max(args.warmup, 1)
        run_reference(args)
        return
    if args.workload == "lv_ensemble":
        args.warmup = max(args.warmup, 3)
        run_lv_ensemble(args)
    elif args.workload == "lv_single":
        run_lv_single(args)
    elif args.workload == "fhn_lml":
        run_fhn_lml(args)
    elif args.workload == "vdp_dense":
        run_vdp_dense(args)
    else:
        run_burgers_blockdiag(args)


if __name__ == "__main__":
    main()
