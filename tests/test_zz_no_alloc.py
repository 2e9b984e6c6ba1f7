"""The allocation-free LML entry point (pdq_lml_fixed_grid_static).

It serves callers that cannot allocate device memory (plugin hosts that pass
only input/output buffers, loops whose allocation policy forbids it): its
scratch is an array inside the library.  Called through the C ABI, twice in a row, it must reproduce the
allocating entry point pdq_lml_fixed_grid within the LML tests' float64
tolerance (value 1e-9 relative, gradient 1e-6 relative to its norm).  This
file is collected last so a run that stops at the first failure has run
every other test first.
"""

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _args(_native, B, thetas, y0, data, std, out_lml, out_grad, out_status, num_steps, save_every):
    a = _native.PdqLmlArgs()
    a.num_instances, a.num_steps, a.save_every = B, num_steps, save_every
    a.average_pdfs, a.with_gradient = 0, 1
    a.t0, a.dt = 0.0, 0.01
    a.params, a.y0, a.data, a.std = (ctypes.c_void_p(x.data_ptr()) for x in (thetas, y0, data, std))
    a.lml, a.grad, a.status = (ctypes.c_void_p(x.data_ptr()) for x in (out_lml, out_grad, out_status))
    return a


def test_static_scratch_entry_point_matches_allocating_entry_point():
    from probdiffeq_gb300 import _native, ensemble
    from probdiffeq_gb300 import build as native_build
    from tests import lml_problem

    native_build.build()
    lib = _native.load()
    num_steps, data_np = lml_problem.observations(t1=2.0)
    B = 8
    f64 = dict(dtype=torch.float64, device="cuda")
    thetas = torch.tensor(lml_problem.theta_samples(B, seed=7), **f64)
    y0 = torch.tensor(np.tile(lml_problem.U0, (B, 1)), **f64)
    data = torch.tensor(data_np, **f64)
    std = torch.full((data.shape[0],), lml_problem.STD, **f64)
    cfg = ensemble.make_config(field="fitzhugh_nagumo", num_derivatives=3, ode_dim=2, ssm="isotropic",
                               strategy="fixedpoint", solver="none", precision="float64")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    # the allocating entry point, with a caller-allocated workspace
    need = ctypes.c_size_t(0)
    assert lib.pdq_lml_workspace_size(ctypes.byref(cfg), B, num_steps, 10, ctypes.byref(need)) == 0
    ws = torch.empty(need.value, dtype=torch.uint8, device="cuda")
    ref = [torch.empty(B, **f64), torch.empty((B, 3), **f64), torch.empty(B, dtype=torch.int32, device="cuda")]
    a = _args(_native, B, thetas, y0, data, std, *ref, num_steps, 10)
    assert lib.pdq_lml_fixed_grid(ctypes.byref(cfg), ctypes.byref(a), ctypes.c_void_p(ws.data_ptr()), need, stream) == 0
    torch.cuda.synchronize()
    assert (ref[2] == 0).all()

    # the allocation-free entry point, twice in a row (the array keeps the last call's contents)
    for _ in range(2):
        out = [torch.full((B,), float("nan"), **f64), torch.full((B, 3), float("nan"), **f64),
               torch.full((B,), -1, dtype=torch.int32, device="cuda")]
        a = _args(_native, B, thetas, y0, data, std, *out, num_steps, 10)
        assert lib.pdq_lml_fixed_grid_static(ctypes.byref(cfg), ctypes.byref(a), stream) == 0
        torch.cuda.synchronize()
        assert (out[2] == 0).all()
        assert torch.allclose(out[0], ref[0], rtol=1e-9, atol=0.0)
        gerr = (out[1] - ref[1]).abs().max(dim=1).values / ref[1].norm(dim=1)
        assert float(gerr.max()) <= 1e-6

    # a call whose plan key differs from the one the array holds (another
    # noise std, another grid length) must rebuild the plan, not reuse it
    for std_k, steps_k in ((2.0 * std, num_steps), (std[: (num_steps // 2) // 10 + 1], num_steps // 2)):
        data_k = data[: std_k.shape[0]].contiguous()
        need_k = ctypes.c_size_t(0)
        assert lib.pdq_lml_workspace_size(ctypes.byref(cfg), B, steps_k, 10, ctypes.byref(need_k)) == 0
        ws_k = torch.zeros(need_k.value, dtype=torch.uint8, device="cuda")
        ref_k = [torch.empty(B, **f64), torch.empty((B, 3), **f64), torch.empty(B, dtype=torch.int32, device="cuda")]
        a = _args(_native, B, thetas, y0, data_k, std_k, *ref_k, steps_k, 10)
        assert lib.pdq_lml_fixed_grid(ctypes.byref(cfg), ctypes.byref(a), ctypes.c_void_p(ws_k.data_ptr()), need_k,
                                      stream) == 0
        out = [torch.full((B,), float("nan"), **f64), torch.full((B, 3), float("nan"), **f64),
               torch.full((B,), -1, dtype=torch.int32, device="cuda")]
        a = _args(_native, B, thetas, y0, data_k, std_k, *out, steps_k, 10)
        assert lib.pdq_lml_fixed_grid_static(ctypes.byref(cfg), ctypes.byref(a), stream) == 0
        torch.cuda.synchronize()
        assert (ref_k[2] == 0).all() and (out[2] == 0).all()
        assert torch.allclose(out[0], ref_k[0], rtol=1e-9, atol=0.0)
        assert not torch.allclose(out[0], ref[0], rtol=1e-6, atol=0.0)  # a different problem, a different LML
        gerr = (out[1] - ref_k[1]).abs().max(dim=1).values / ref_k[1].norm(dim=1)
        assert float(gerr.max()) <= 1e-6


def test_static_scratch_rejects_problems_beyond_its_size():
    from probdiffeq_gb300 import _native, ensemble
    from probdiffeq_gb300 import build as native_build

    native_build.build()
    lib = _native.load()
    cfg = ensemble.make_config(field="fitzhugh_nagumo", num_derivatives=3, ode_dim=2, ssm="isotropic",
                               strategy="fixedpoint", solver="none", precision="float64")
    B, num_steps = 4096, 2000  # far more scratch than the 32 MiB array holds
    need = ctypes.c_size_t(0)
    assert lib.pdq_lml_workspace_size(ctypes.byref(cfg), B, num_steps, 10, ctypes.byref(need)) == 0
    assert need.value > 32 * 1024 * 1024
    a = _native.PdqLmlArgs()
    a.num_instances, a.num_steps, a.save_every, a.dt = B, num_steps, 10, 0.01
    st = lib.pdq_lml_fixed_grid_static(ctypes.byref(cfg), ctypes.byref(a), None)
    assert st == 6 and _native.status_string(st) == "problem exceeds the library's static scratch array"
