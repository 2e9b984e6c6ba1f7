"""Host-side checks of the C ABI (no GPU needed; no compute calls).

The library must load, export every function ``include/*.h`` declares, and
reject malformed configurations before any launch.
"""

import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from probdiffeq_gb300 import _native
    from probdiffeq_gb300 import build as native_build

    native_build.build()
    return _native.load()


def declared_functions():
    names = set()
    for header in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(header).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(pdq_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert "pdq_solve_adaptive" in names
    for name in names:
        assert hasattr(lib, name), name


def test_abi_version_and_status_strings(lib):
    from probdiffeq_gb300 import _native

    assert lib.pdq_abi_version() == _native.ABI_VERSION
    assert _native.status_string(0) == "success"
    assert _native.status_string(2) == "unsupported configuration"


def test_config_default_matches_reference_defaults(lib):
    from probdiffeq_gb300 import _native

    cfg = _native.config_default("isotropic", "lotka_volterra", 4, 2)
    # control_integral defaults (controllers.py:66-84), solve(...) defaults (solvers_via_adaptive_steps.py:35)
    assert (cfg.safety, cfg.factor_min, cfg.factor_max) == (0.95, 0.2, 10.0)
    assert (cfg.exponent_integral, cfg.exponent_proportional) == (0.3, 0.4)
    assert cfg.eps == 1e-8 and cfg.damp == 0.0 and cfg.clip_dt == 1


def test_malformed_configs_are_rejected_before_launch(lib):
    from probdiffeq_gb300 import _native, ensemble

    bad = []
    cfg = ensemble.make_config(field="lotka_volterra", num_derivatives=4, ode_dim=3)  # LV has d = 2
    bad.append(cfg)
    cfg = ensemble.make_config(field="lotka_volterra", num_derivatives=9, ode_dim=2)
    bad.append(cfg)
    cfg = ensemble.make_config(field="lotka_volterra", num_derivatives=4, ode_dim=2)
    cfg.abi_version = 999
    bad.append(cfg)
    cfg = ensemble.make_config(field="lotka_volterra", num_derivatives=4, ode_dim=2, atol=0.0, rtol=0.0)
    bad.append(cfg)
    cfg = ensemble.make_config(field="lotka_volterra", num_derivatives=4, ode_dim=2, instances_per_block=48)
    bad.append(cfg)
    cfg = ensemble.make_config(field="lotka_volterra", num_derivatives=4, ode_dim=2)
    cfg.reserved0 = 1
    bad.append(cfg)
    for cfg in bad:
        ws = ctypes.c_size_t(0)
        st = lib.pdq_workspace_size(ctypes.byref(cfg), 4, 2, ctypes.byref(ws))
        assert st != 0
        args = _native.PdqAdaptiveArgs()
        args.num_instances = 4
        args.num_save_at = 2
        st = lib.pdq_solve_adaptive(ctypes.byref(cfg), ctypes.byref(args), None, 0, None)
        assert st != 0


def test_missing_buffers_are_rejected(lib):
    from probdiffeq_gb300 import _native, ensemble

    cfg = ensemble.make_config(field="lotka_volterra", num_derivatives=4, ode_dim=2)
    args = _native.PdqAdaptiveArgs()
    args.num_instances = 4
    args.num_save_at = 2
    assert lib.pdq_solve_adaptive(ctypes.byref(cfg), ctypes.byref(args), None, 0, None) == 1
    args.num_save_at = 1
    assert lib.pdq_solve_adaptive(ctypes.byref(cfg), ctypes.byref(args), None, 0, None) == 1


def test_offgrid_arguments_are_checked_before_launch(lib):
    """pdq_offgrid_marginals: the fixed-point smoother is unsupported (the
    reference raises NotImplementedError, solvers.py:163-164); missing
    buffers are rejected; an empty query set launches nothing."""
    from probdiffeq_gb300 import _native

    a = _native.PdqOffgridArgs()
    a.ssm, a.strategy, a.num_derivatives, a.ode_dim = 0, 1, 2, 2
    a.num_instances, a.num_points, a.num_queries = 2, 5, 3
    assert lib.pdq_offgrid_marginals(None, None) == 1
    assert lib.pdq_offgrid_marginals(ctypes.byref(a), None) == 2  # fixed-point: unsupported
    a.strategy = 2
    assert lib.pdq_offgrid_marginals(ctypes.byref(a), None) == 1  # buffers missing
    a.ssm = 1
    assert lib.pdq_offgrid_marginals(ctypes.byref(a), None) == 2  # block-diagonal: not native
    a.ssm, a.num_queries = 2, 0
    assert lib.pdq_offgrid_marginals(ctypes.byref(a), None) == 0


def test_lml_adjoint_arguments_are_checked_before_launch(lib):
    """pdq_lml_adjoint_workspace_size / pdq_lml_fwd / pdq_lml_bwd reject bad
    checkpoint spacings, missing buffers, a missing or misaligned workspace
    and a non-zero reserved field before any CUDA call; an empty batch
    launches nothing."""
    from probdiffeq_gb300 import _native, ensemble

    cfg = ensemble.make_config(field="fitzhugh_nagumo", num_derivatives=3, ode_dim=2, ssm="isotropic",
                               strategy="fixedpoint", solver="none", precision="float32")
    nb = ctypes.c_size_t(0)
    assert lib.pdq_lml_adjoint_workspace_size(ctypes.byref(cfg), 8, 2000, 10, 0, ctypes.byref(nb)) == 0
    # plan + 8 samples x (45 states + 200 offsets) x 8 + 201 x 2 innovations + 45 x 2 predicted u, float32
    per_sample = (45 * 8 + 200 * 8 + 201 * 2 + 45 * 2) * 4
    assert nb.value - 8 * per_sample > 0 and (nb.value - 8 * per_sample) % 256 == 0
    small = ctypes.c_size_t(0)
    assert lib.pdq_lml_adjoint_workspace_size(ctypes.byref(cfg), 8, 2000, 10, 2000, ctypes.byref(small)) == 0
    assert small.value > 0
    assert lib.pdq_lml_adjoint_workspace_size(ctypes.byref(cfg), 8, 2000, 10, -1, ctypes.byref(nb)) == 1
    assert lib.pdq_lml_adjoint_workspace_size(ctypes.byref(cfg), 8, 2000, 10, 2001, ctypes.byref(nb)) == 1
    assert lib.pdq_lml_adjoint_workspace_size(ctypes.byref(cfg), 8, 2000, 7, 0, ctypes.byref(nb)) == 1
    bad = ensemble.make_config(field="van_der_pol", num_derivatives=3, ode_dim=2, ssm="isotropic",
                               strategy="fixedpoint", solver="none", precision="float64")
    assert lib.pdq_lml_adjoint_workspace_size(ctypes.byref(bad), 8, 2000, 10, 0, ctypes.byref(nb)) == 2

    a = _native.PdqLmlAdjointArgs()
    a.lml.num_instances, a.lml.num_steps, a.lml.save_every, a.lml.dt = 8, 2000, 10, 0.01
    assert lib.pdq_lml_fwd(ctypes.byref(cfg), None, None, 0, None) == 1
    assert lib.pdq_lml_fwd(ctypes.byref(cfg), ctypes.byref(a), None, 0, None) == 1  # buffers missing
    fake = ctypes.c_void_p(4096)  # never dereferenced: the checks fail first
    for name in ("params", "y0", "data", "std", "lml", "status"):
        setattr(a.lml, name, fake)
    assert lib.pdq_lml_fwd(ctypes.byref(cfg), ctypes.byref(a), None, 0, None) == 4  # no workspace
    big = ctypes.c_size_t(1 << 40)
    assert lib.pdq_lml_fwd(ctypes.byref(cfg), ctypes.byref(a), ctypes.c_void_p(4096 + 8), big, None) == 4  # misaligned
    assert lib.pdq_lml_bwd(ctypes.byref(cfg), ctypes.byref(a), fake, big, None) == 1  # no gradient output
    a.reserved0 = 1
    assert lib.pdq_lml_fwd(ctypes.byref(cfg), ctypes.byref(a), fake, big, None) == 1
    a.reserved0 = 0
    a.checkpoint_every = 2001
    assert lib.pdq_lml_fwd(ctypes.byref(cfg), ctypes.byref(a), fake, big, None) == 1
    a.checkpoint_every = 0
    a.lml.num_instances = 0
    assert lib.pdq_lml_fwd(ctypes.byref(cfg), ctypes.byref(a), None, 0, None) == 0
    assert lib.pdq_lml_bwd(ctypes.byref(cfg), ctypes.byref(a), None, 0, None) == 0


def test_sample_markov_arguments_are_checked_before_launch(lib):
    """pdq_sample_markov: negative or empty sizes, factorisations without a
    native sampler and missing buffers are rejected before any launch; an
    empty batch launches nothing."""
    from probdiffeq_gb300 import _native

    assert lib.pdq_sample_markov(None, None) == 1
    a = _native.PdqSampleArgs()
    a.ssm, a.num_derivatives, a.ode_dim, a.num_points = 0, 2, 2, 5
    a.num_instances, a.num_samples = 2, 3
    assert lib.pdq_sample_markov(ctypes.byref(a), None) == 1  # buffers missing
    a.num_samples = -1
    assert lib.pdq_sample_markov(ctypes.byref(a), None) == 1
    a.num_samples, a.num_points = 3, 0
    assert lib.pdq_sample_markov(ctypes.byref(a), None) == 1
    a.num_points, a.ssm = 5, 1
    assert lib.pdq_sample_markov(ctypes.byref(a), None) == 2  # block-diagonal: no native sampler
    a.ssm, a.num_derivatives = 0, 9
    assert lib.pdq_sample_markov(ctypes.byref(a), None) == 2  # n beyond the isotropic kernel's bound
    a.ssm, a.num_derivatives, a.ode_dim = 2, 3, 20
    assert lib.pdq_sample_markov(ctypes.byref(a), None) == 2  # N = 80 beyond the dense bound
    a.ode_dim, a.num_instances = 2, 0
    assert lib.pdq_sample_markov(ctypes.byref(a), None) == 0
