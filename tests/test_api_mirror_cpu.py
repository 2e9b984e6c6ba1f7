"""Constructors of the drop-in namespace that need no GPU (CPU).

The IWP utilities equal the oracle's (the golden fixture, itself pinned to
the reference's closed forms); the default error normalisation and the
prior-mean Taylor point are accepted explicitly and lower to the same native
configuration as their defaults; the non-native alternatives raise
NotImplementedError before anything runs; the other Taylor-mode
constructors describe the same exact coefficients.
"""

import pytest
import torch

from probdiffeq_gb300 import probdiffeq
from tests.golden import make_golden


@pytest.mark.parametrize("nu", [2, 3, 4])
def test_iwp_utilities_match_the_golden_matrices(nu):
    gold = make_golden.load("iwp.json")[str(nu)]
    A, Q = probdiffeq.system_matrices_1d_iwp(nu)
    p, p_inv = probdiffeq.preconditioner_taylor(nu)(gold["dt"])
    for got, want in ((A, gold["A"]), (Q, gold["Q"]), (p, gold["p"]), (p_inv, gold["p_inv"])):
        want = torch.tensor(want, dtype=torch.float64)
        assert torch.allclose(got, want, rtol=1e-14, atol=1e-15), (got, want)


def _lowered(error=None, taylor_point=None):
    from probdiffeq_gb300 import _native
    from probdiffeq_gb300 import build as native_build

    native_build.build()
    _native.load()
    vf = probdiffeq.ode("lotka_volterra", torch.tensor([0.5, 0.05, 0.5, 0.05], dtype=torch.float64))
    ssm = probdiffeq.state_space_model_isotropic()
    c = ssm.constraint_ode_ts1(vf, taylor_point=taylor_point)
    solver = probdiffeq.solver_mle(strategy=probdiffeq.strategy_filter(), constraint=c)
    err = probdiffeq.error_residual_std(constraint=c) if error is None else error(c)
    cfg = probdiffeq.lower(solver, err, None, num_derivatives=4, y0=torch.zeros(2, dtype=torch.float64),
                           precision="float64", atol=1e-6, rtol=1e-6, clip_dt=True, eps=1e-8, damp=0.0)
    return bytes(cfg)


def test_explicit_defaults_lower_to_the_default_configuration():
    default = _lowered()
    explicit = _lowered(
        error=lambda c: probdiffeq.error_residual_std(constraint=c, error_norm=probdiffeq.error_norm_scale_then_rms()),
        taylor_point=probdiffeq.taylor_point_prior(),
    )
    assert explicit == default
    state = probdiffeq.error_state_std(constraint=probdiffeq.state_space_model_dense().constraint_ode_ts0(
        probdiffeq.ode("lotka_volterra", torch.ones(4))), error_norm=probdiffeq.error_norm_scale_then_rms())
    assert state.error_norm is not None


def test_non_native_alternatives_are_refused_before_running():
    vf = probdiffeq.ode("lotka_volterra", torch.ones(4))
    ssm = probdiffeq.state_space_model_isotropic()
    c = ssm.constraint_ode_ts0(vf)
    with pytest.raises(NotImplementedError):
        probdiffeq.error_residual_std(constraint=c, error_norm=probdiffeq.error_norm_rms_then_scale())
    with pytest.raises(NotImplementedError):
        probdiffeq.error_residual_std(constraint=c, error_norm=probdiffeq.error_norm_scale_then_rms(norm_order=1))
    with pytest.raises(NotImplementedError):
        probdiffeq.error_state_std(constraint=c, error_norm=probdiffeq.error_norm_rms_then_scale())
    with pytest.raises(NotImplementedError):
        ssm.constraint_ode_ts1(vf, taylor_point=probdiffeq.taylor_point_maximum_a_posteriori())


def test_taylor_mode_constructors_describe_the_same_coefficients():
    vf = probdiffeq.ode("lotka_volterra", torch.ones(4))
    y0 = torch.tensor([20.0, 20.0], dtype=torch.float64)
    a, _ = probdiffeq.jetexpand_ode_padded_scan(num=4)(vf, (y0,))
    b, _ = probdiffeq.jetexpand_ode_via_jvp(num=4)(vf, (y0,))
    c, _ = probdiffeq.jetexpand_ode_doubling_unroll(num_doublings=2)(vf, (y0,))
    assert len(a) == len(b) == 5 and len(c) == 4
    assert torch.equal(a.y0, b.y0) and b.field is vf
    with pytest.raises(ValueError):
        probdiffeq.jetexpand_ode_doubling_unroll(num_doublings=0)


def test_reference_type_names():
    """The reference's public type names (solvers.py:35, 72; ssm_impl_api.py:300)
    name the mirror's types, so annotations and isinstance checks carry over."""
    from probdiffeq_gb300 import ivpsolve, probdiffeq

    assert probdiffeq.ProbabilisticSolution is ivpsolve.Solution
    ts0 = probdiffeq.state_space_model_isotropic().constraint_ode_ts0(
        probdiffeq.ode("lotka_volterra", [0.5, 0.05, 0.5, 0.05]))
    assert isinstance(probdiffeq.solver_mle(strategy=probdiffeq.strategy_filter(), constraint=ts0),
                      probdiffeq.ProbabilisticSolver)
    for ssm in (probdiffeq.state_space_model_isotropic(), probdiffeq.state_space_model_blockdiag(),
                probdiffeq.state_space_model_dense()):
        assert isinstance(ssm, probdiffeq.StateSpaceModel)
    with pytest.raises(AttributeError):
        probdiffeq.no_such_name
