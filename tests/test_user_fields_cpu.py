"""Run-time compiled vector fields (pdq_register_field): compilation and diagnostics (CPU).

NVRTC compiles without a device, so registration -- which compiles one
variant of the isotropic solver with the field -- is tested here; solving
with the registered fields is in test_user_fields_gpu.py.
"""

import pytest

from probdiffeq_gb300 import _native, probdiffeq
from tests import user_fields


def test_registering_a_field_compiles_it_and_returns_a_user_id():
    fid = _native.register_field("cpu_test_brusselator", user_fields.BRUSSELATOR, 2, 2)
    assert fid >= 1000
    assert _native.FIELD["cpu_test_brusselator"] == fid
    fid2 = _native.register_field("cpu_test_lorenz", user_fields.LORENZ, 3, 3)
    assert fid2 == fid + 1 or fid2 > fid


def test_compiler_errors_come_back_with_the_log():
    with pytest.raises(_native.NativeError) as err:
        _native.register_field("cpu_test_broken", user_fields.BROKEN, 2, 1)
    assert err.value.status == 7
    assert "no_such_symbol" in str(err.value)
    assert _native.status_string(7) == "run-time compilation of the vector field failed"


def test_invalid_arguments_are_rejected_before_compiling():
    with pytest.raises(_native.NativeError) as err:
        _native.register_field("cpu_test_empty", "", 2, 1)
    assert err.value.status == 1


def test_api_registration_makes_the_name_usable():
    probdiffeq.register_field("cpu_test_api_brusselator", user_fields.BRUSSELATOR, dim=2, num_params=2)
    vf = probdiffeq.ode("cpu_test_api_brusselator", [1.0, 3.0])
    assert vf.name == "cpu_test_api_brusselator"
    with pytest.raises(ValueError):
        probdiffeq.ode("cpu_test_api_brusselator", [1.0, 3.0, 4.0])
    with pytest.raises(ValueError):
        probdiffeq.register_field("lotka_volterra", user_fields.LOTKA_VOLTERRA, dim=2, num_params=4)


def test_registering_a_stencil_compiles_the_block_diagonal_kernel():
    """A block-diagonal stencil (struct Stencil) compiles with the cluster
    kernel; a configuration of another factorisation rejects its id."""
    from probdiffeq_gb300 import ensemble

    fid = _native.register_stencil("cpu_test_allen_cahn", user_fields.ALLEN_CAHN_STENCIL, 1)
    assert fid >= 1000
    cfg = ensemble.make_config(field="cpu_test_allen_cahn", num_derivatives=3, ode_dim=64, ssm="blockdiag")
    assert cfg.field == fid
    with pytest.raises(_native.NativeError):  # a Field source is not a stencil
        _native.register_stencil("cpu_test_stencil_broken", user_fields.BRUSSELATOR, 2)
