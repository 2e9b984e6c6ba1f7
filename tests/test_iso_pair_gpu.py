"""The warp-specialised isotropic filter (kernel_variant 4: a covariance warp
and a control warp per 32 instances, iso_pair.cuh) against the one-thread
kernel and the oracle (GPU).

Both mappings run the same algorithm, but the compiler rounds them
differently (FMA contraction and evaluation order differ between the two
kernels), so their records agree to rounding as the parity tests measure
it: float64 -- u within 1e-9, every Taylor row and L L^T within 1e-6,
accepted steps and attempts within one; float32 -- u within 1e-5, u' within
1e-3, L L^T within 1e-2 (the float32 covariance of u sits at the rounding
floor), step and attempt counts within 2 %.  The configurations cover what
the variant accepts: MLE, dynamic and uncalibrated solvers, integral and PI
control, terminal values (clip_dt) and save_at by interpolation, the three
built-in fields, and ragged batch sizes (a CTA holds 32 instances).  The
float64 records also meet the oracle at the parity tests' tolerances.
"""

import pytest
import torch

from tests.test_iso_gpu import compare_record, gpu_solve, lv_instances, oracle_solve, tolerances

pytestmark = pytest.mark.gpu


def _rel_rows(g, o):
    return max(float((g[..., i, :] - o[..., i, :]).abs().max() / o[..., i, :].abs().max().clamp_min(1e-300))
               for i in range(o.shape[-2]))


def _compare(a, b, precision):
    f64 = precision == "float64"
    assert torch.equal(a["status"], b["status"])
    ok = a["status"] == 0
    ua, ub = a["u_mean"][ok], b["u_mean"][ok]
    assert float((ua[..., 0, :] - ub[..., 0, :]).abs().max() / ub[..., 0, :].abs().max()) <= (1e-9 if f64 else 1e-5)
    if f64:
        assert _rel_rows(ua, ub) <= 1e-6
    else:
        assert float((ua[..., 1, :] - ub[..., 1, :]).abs().max() / ub[..., 1, :].abs().max()) <= 1e-3
    ca = a["u_chol"][ok] @ a["u_chol"][ok].transpose(-1, -2)
    cb = b["u_chol"][ok] @ b["u_chol"][ok].transpose(-1, -2)
    assert float((ca - cb).abs().max() / cb.abs().max()) <= (1e-6 if f64 else 1e-2)
    for key in ("num_steps", "num_attempts"):
        d = (a[key] - b[key]).abs()
        allowed = torch.ones_like(d) if f64 else torch.clamp((0.02 * b[key].abs()).ceil().to(d.dtype), min=1)
        assert bool((d <= allowed).all()), key
    sa, sb = a["output_scale"][ok], b["output_scale"][ok]
    assert float((sa - sb).abs().max() / sb.abs().max()) <= (1e-6 if f64 else 1e-2)


@pytest.mark.parametrize("precision", ["float64", "float32"])
@pytest.mark.parametrize("solver", ["mle", "dynamic", "none"])
def test_pair_equals_thread_terminal_values(solver, precision):
    params, y0 = lv_instances(70, seed=3)
    args = ("lotka_volterra", params, y0, 4, solver, [0.0, 20.0], 1e-6, 1e-6, True, precision, True)
    _compare(gpu_solve(*args, variant="pair"), gpu_solve(*args, variant="thread"), precision)


@pytest.mark.parametrize("precision", ["float64", "float32"])
@pytest.mark.parametrize("control", ["integral", "proportional_integral"])
def test_pair_equals_thread_save_at_interpolation(control, precision):
    params, y0 = lv_instances(33, seed=4)
    save_at = [0.0, 0.7, 1.9, 2.0, 5.5, 9.0]
    args = ("lotka_volterra", params, y0, 4, "dynamic", save_at, 1e-5, 1e-5, False, precision, False)
    _compare(gpu_solve(*args, control=control, variant="pair"), gpu_solve(*args, control=control, variant="thread"),
             precision)


@pytest.mark.parametrize("field, nu", [("van_der_pol", 3), ("fitzhugh_nagumo", 3), ("lotka_volterra", 2)])
def test_pair_equals_thread_other_fields(field, nu):
    B = 7
    if field == "van_der_pol":
        params, y0 = torch.full((B, 1), 2.0, dtype=torch.float64), torch.tensor([[2.0, 0.0]]).repeat(B, 1)
    elif field == "fitzhugh_nagumo":
        params = torch.tensor([[0.2, 0.2, 3.0]], dtype=torch.float64).repeat(B, 1)
        y0 = torch.tensor([[-1.0, 1.0]], dtype=torch.float64).repeat(B, 1) + 0.01 * torch.arange(B)[:, None]
    else:
        params, y0 = lv_instances(B, seed=5)
    args = (field, params, y0, nu, "mle", [0.0, 3.0, 6.0], 1e-6, 1e-6, True, "float64", False)
    _compare(gpu_solve(*args, variant="pair"), gpu_solve(*args, variant="thread"), "float64")


@pytest.mark.parametrize("B", [1, 31, 32, 33, 130])
def test_pair_ragged_batches_match_the_oracle(B):
    params, y0 = lv_instances(B, seed=6)
    out = gpu_solve("lotka_volterra", params, y0, 4, "mle", [0.0, 10.0], 1e-6, 1e-6, True, "float64", True,
                    variant="pair")
    assert (out["status"] == 0).all()
    for b in sorted({0, B // 2, B - 1}):
        res = oracle_solve("lotka_volterra", params[b], y0[b], 4, "mle", [0.0, 10.0], 1e-6, 1e-6, True)
        o = res.u[-1]
        compare_record(out["u_mean"][b, 0], out["u_chol"][b, 0], o.mean, o.cholesky, out["num_steps"][b, 0],
                       res.num_steps[-1], tolerances("float64"))
        assert abs(float(out["output_scale"][b, 0]) - float(res.output_scale[-1])) <= 1e-6 * float(res.output_scale[-1])


def test_pair_rejects_what_it_does_not_implement():
    from probdiffeq_gb300 import _native, ensemble

    params, y0 = lv_instances(4, seed=7)
    for kw in (dict(error="state_std"), dict(damp=1e-3), dict(constraint="ts1")):
        cfg = ensemble.make_config(field="lotka_volterra", num_derivatives=4, ode_dim=2, solver="mle",
                                   kernel_variant="pair", **kw)
        with pytest.raises(_native.NativeError):
            ensemble.solve_ensemble(cfg, params=params, y0=y0, save_at=torch.tensor([0.0, 1.0]))
