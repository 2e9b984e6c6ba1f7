"""The XLA FFI handlers (``probdiffeq_gb300/jax_ffi``).

jaxlib is not installed on the build machine or the GPU machine, so the
handler library is never compiled here: these tests check that its build
step is skipped cleanly without jaxlib's headers, that the Python module
imports without jax, and that every handler calls the C ABI entry point it
wraps with that entry point's argument struct.  The end-to-end test runs only
where jax is importable.
"""

import os
import re

import pytest

from probdiffeq_gb300 import build

SRC = os.path.join(os.path.dirname(build.__file__), "jax_ffi", "ffi_pdq.cc")
HANDLERS = {
    "PdqSolveAdaptive": "pdq_solve_adaptive",
    "PdqLmlFwd": "pdq_lml_fwd",
    "PdqLmlBwd": "pdq_lml_bwd",
    "PdqTerminalFwd": "pdq_terminal_fwd",
    "PdqTerminalBwd": "pdq_terminal_bwd",
}


def test_build_is_skipped_without_jaxlib_headers():
    if build.jax_ffi_include_dir() is not None:
        pytest.skip("jaxlib headers present: the handler library builds")
    assert build.build_jax_ffi() is None


def test_module_imports_without_jax():
    import probdiffeq_gb300.jax_ffi as jf

    assert set(jf._TARGETS) == set(HANDLERS)


def test_each_handler_binds_its_entry_point():
    src = open(SRC).read()
    header = open(os.path.join(build.INCLUDE, "pdq.h")).read()
    for handler, entry in HANDLERS.items():
        m = re.search(r"XLA_FFI_DEFINE_HANDLER_SYMBOL\(" + handler + r",\s*(\w+),", src)
        assert m, handler
        impl = m.group(1)
        body = src[src.index("ffi::Error " + impl + "("):]
        body = body[:body.index("\n}\n")]
        assert entry + "(" in body, (handler, entry)
        assert entry + "(" in header, entry


@pytest.mark.gpu
def test_terminal_values_through_jax():
    jax = pytest.importorskip("jax")
    if build.jax_ffi_include_dir() is None:
        pytest.skip("jaxlib headers not found")
    import jax.numpy as jnp
    import numpy as np

    import probdiffeq_gb300.jax_ffi as jf
    from probdiffeq_gb300 import ensemble

    jax.config.update("jax_enable_x64", True)
    cfg = ensemble.make_config(field="lotka_volterra", num_derivatives=4, ode_dim=2, solver="mle", precision="float64")
    p = jnp.asarray([[0.5, 0.05, 0.5, 0.05]])
    y = jnp.asarray([[20.0, 20.0]])
    g = jax.grad(lambda pp: jf.terminal_values(cfg, pp, y, 0.0, 5.0).sum())(p)
    assert np.isfinite(np.asarray(g)).all()
