"""Host logic of the autotuner (no GPU): candidate sets and cache keys."""

import pytest

from probdiffeq_gb300 import autotune, ensemble


@pytest.fixture(autouse=True, scope="module")
def library():
    from probdiffeq_gb300 import build as native_build

    native_build.build()  # make_config fills the defaults through the C ABI


def test_candidates_follow_the_abi_rules():
    """The eight-lane isotropic mapping only for TS0 filters with exact landings
    and error_residual_std (include/pdq.h kernel_variant), the split one
    (covariance and mean warps) also not with damping or the dynamic solver;
    dense lanes not with error_state_std; block-diagonal has one launch shape."""
    iso = ensemble.make_config(field="lotka_volterra", num_derivatives=4, ode_dim=2, clip_dt=True)
    assert (2, 32) in autotune.candidates(iso) and (1, 64) in autotune.candidates(iso)
    mle = dict(field="lotka_volterra", num_derivatives=4, ode_dim=2, clip_dt=True, solver="mle")
    assert (4, 0) in autotune.candidates(ensemble.make_config(**mle))
    for kw in (dict(solver="dynamic"), dict(damp=1e-3)):
        c = ensemble.make_config(**{**mle, **kw})
        assert (4, 0) not in autotune.candidates(c) and (2, 32) in autotune.candidates(c), kw
    for kw in (dict(clip_dt=False), dict(constraint="ts1"), dict(error="state_std"), dict(strategy="fixedpoint")):
        c = ensemble.make_config(field="lotka_volterra", num_derivatives=4, ode_dim=2, **{"clip_dt": True, **kw})
        assert all(v == 1 for v, _ in autotune.candidates(c)), kw
    dense = ensemble.make_config(field="van_der_pol", num_derivatives=3, ode_dim=2, ssm="dense", constraint="ts1")
    assert (2, 4) in autotune.candidates(dense) and (3, 0) in autotune.candidates(dense)
    dense_se = ensemble.make_config(field="van_der_pol", num_derivatives=3, ode_dim=2, ssm="dense", error="state_std")
    assert all(v == 1 for v, _ in autotune.candidates(dense_se))
    bd = ensemble.make_config(field="burgers", num_derivatives=3, ode_dim=64, ssm="blockdiag")
    assert autotune.candidates(bd) == [(0, 0)]
    for v, ipb in autotune.candidates(iso) + autotune.candidates(dense):
        assert ipb in (2, 4, 8, 16, 32, 64) or (v, ipb) in ((3, 0), (4, 0), (5, 0))


def test_cache_key_ignores_the_mapping_and_buckets_batch_sizes():
    a = ensemble.make_config(field="lotka_volterra", num_derivatives=4, ode_dim=2)
    b = ensemble.make_config(field="lotka_volterra", num_derivatives=4, ode_dim=2, kernel_variant=2, instances_per_block=16)
    assert autotune.cache_key(a, 16384, 2, True, "cpu") == autotune.cache_key(b, 16384, 2, True, "cpu")
    assert autotune.cache_key(a, 9000, 2, True, "cpu") == autotune.cache_key(a, 16384, 2, True, "cpu")
    assert autotune.cache_key(a, 8192, 2, True, "cpu") != autotune.cache_key(a, 8193, 2, True, "cpu")
    c = ensemble.make_config(field="lotka_volterra", num_derivatives=4, ode_dim=2, precision="float64")
    assert autotune.cache_key(a, 100, 2, True, "cpu") != autotune.cache_key(c, 100, 2, True, "cpu")
    assert autotune.cache_key(a, 100, 2, True, "cpu") != autotune.cache_key(a, 100, 3, True, "cpu")


def test_kernel_variant_names_follow_the_state_space_model():
    """Names of the mappings (include/pdq.h kernel_variant) per factorisation:
    "split" is the isotropic covariance / mean warp pair, "struct8" the dense
    structure-exploiting kernel on eight lanes; a name of the other
    factorisation is rejected before any call."""
    iso = ensemble.make_config(field="lotka_volterra", num_derivatives=4, ode_dim=2, kernel_variant="split")
    assert iso.kernel_variant == 4
    dense = ensemble.make_config(field="van_der_pol", num_derivatives=3, ode_dim=2, ssm="dense",
                                 kernel_variant="struct16")
    assert dense.kernel_variant == 5
    assert ensemble.make_config(field="van_der_pol", num_derivatives=3, ode_dim=2, ssm="dense",
                                kernel_variant=4).kernel_variant == 4
    with pytest.raises(ValueError):
        ensemble.make_config(field="van_der_pol", num_derivatives=3, ode_dim=2, ssm="dense", kernel_variant="split")
    with pytest.raises(ValueError):
        ensemble.make_config(field="lotka_volterra", num_derivatives=4, ode_dim=2, kernel_variant="struct8")
