"""Constructors of the probabilistic solver, mirroring ``probdiffeq.probdiffeq``.

Same names and keyword signatures as the reference's public namespace
(``probdiffeq/probdiffeq.py:6-17``): state-space-model factories, priors,
constraints, strategies, solvers, error estimators, Taylor-mode
initialisation and the LML loss.  The objects are descriptions; solving
happens in one native call (``probdiffeq_gb300.ivpsolve``), so the shapes of
a batch of instances (the reference's ``jax.vmap`` axis) are the leading axis
of ``y0`` and of the vector-field parameters.

Vector fields are registered device functors (``ode("lotka_volterra",
params)``) rather than Python callables: the whole solve runs on the GPU.
"""

import dataclasses
from typing import Any, Optional

import torch

from . import _native

__all__ = [
    "ode",
    "register_field",
    "Field",
    "jetexpand_ode_padded_scan",
    "jetexpand_ode_unroll",
    "jetexpand_ode_via_jvp",
    "jetexpand_ode_doubling_unroll",
    "taylor_point_prior",
    "taylor_point_maximum_a_posteriori",
    "error_norm_scale_then_rms",
    "error_norm_rms_then_scale",
    "system_matrices_1d_iwp",
    "preconditioner_taylor",
    "state_space_model_isotropic",
    "state_space_model_blockdiag",
    "state_space_model_dense",
    "strategy_filter",
    "strategy_smoother_fixedpoint",
    "strategy_smoother_fixedinterval",
    "solver",
    "solver_mle",
    "solver_dynamic",
    "error_residual_std",
    "error_state_std",
    "jacobian_materialize",
    "loss_lml_timeseries",
    "loss_lml_terminal_values",
    "ProbabilisticSolver",
    "ProbabilisticSolution",
    "StateSpaceModel",
]

_FIELD_DIMS = {"lotka_volterra": 2, "van_der_pol": 2, "fitzhugh_nagumo": 2, "burgers": None}
_FIELD_PARAMS = {"lotka_volterra": 4, "van_der_pol": 1, "fitzhugh_nagumo": 3, "burgers": 1}


@dataclasses.dataclass(frozen=True)
class Field:
    """A registered first-order autonomous vector field u' = f(u; params).

    ``params`` has shape (P,) or (B, P) for a batch of instances.
    Corresponds to ``probdiffeq.ode`` (``_probdiffeq/problems.py:283-295``):
    one Taylor coefficient in, the output is coefficient 1.
    """

    name: str
    params: Any
    jacobian: Any = None
    num_tcoeffs_in_args: int = 1
    tcoeff_indices_output: tuple = (1,)


def register_field(name, source, *, dim, num_params):
    """Register a vector field given as CUDA C++ source, compiled at run time.

    The counterpart of passing a Python callable to ``probdiffeq.ode``
    (problems.py:283-295): ``source`` defines ``struct Field`` with
    ``static constexpr int D, P`` and a generic
    ``template <typename S, typename T> PDQ_HD static void eval(const S* u, const T* p, S* out)``
    (see ``include/pdq.h``, ``pdq_register_field``).  Afterwards
    ``ode(name, params)`` describes it (isotropic and dense factorisations;
    the dense TS1 linearisation takes its Jacobian from the same definition).
    """
    if name in _FIELD_DIMS and name in _native.FIELD and _native.FIELD[name] < 1000:
        raise ValueError(f"{name!r} is a built-in field")
    _native.register_field(name, source, dim, num_params)
    _FIELD_DIMS[name] = int(dim)
    _FIELD_PARAMS[name] = int(num_params)


def ode(name, params, *, jacobian=None):
    """Describe u' = f(u) with a registered device field (problems.py:283-295)."""
    if name not in _FIELD_DIMS:
        raise ValueError(f"unknown vector field {name!r}; registered: {sorted(_FIELD_DIMS)}")
    params = torch.as_tensor(params, dtype=torch.float64)
    if params.shape[-1] != _FIELD_PARAMS[name]:
        raise ValueError(f"{name} takes {_FIELD_PARAMS[name]} parameters, got shape {tuple(params.shape)}")
    return Field(name, params, jacobian)


class jacobian_materialize:
    """Materialised Jacobians (jacobians.py:78-113); the device fields supply them exactly."""


@dataclasses.dataclass(frozen=True)
class TaylorCoefficients:
    """Taylor-mode initial derivatives u(t0), ..., u^(num)(t0), computed on the device.

    Holds the initial values and the order; the derivatives themselves are
    produced inside the solver kernels (jet recursion on the registered field).
    """

    field: Field
    y0: torch.Tensor  # (d,) or (B, d)
    num: int

    def __len__(self):
        return self.num + 1


class _JetExpand:
    def __init__(self, num):
        if num < 1:
            raise ValueError("num must be positive")
        self.num = num

    def __call__(self, vf, inits, /, *, t=0.0):
        """jetexpand_ode_*(num)(vf, (u0,), t=t0) -> (tcoeffs, info) (jet_expansion_algorithms.py:49-152)."""
        if not isinstance(vf, Field):
            raise TypeError("vf must come from probdiffeq_gb300.probdiffeq.ode(...)")
        (u0,) = inits
        return TaylorCoefficients(vf, torch.as_tensor(u0, dtype=torch.float64), self.num), {}


def jetexpand_ode_padded_scan(*, num):
    """Taylor-mode initialisation (jet_expansion_algorithms.py:49-103)."""
    return _JetExpand(num)


def jetexpand_ode_unroll(*, num):
    """Taylor-mode initialisation (jet_expansion_algorithms.py:110-152)."""
    return _JetExpand(num)


def jetexpand_ode_via_jvp(*, num):
    """Taylor coefficients by recursive forward-mode differentiation
    (jet_expansion_algorithms.py:180-225): the same exact coefficients, here
    computed by the solver kernels' jet recursion."""
    return _JetExpand(num)


def jetexpand_ode_doubling_unroll(*, num_doublings):
    """Taylor coefficients by Newton's doubling (jet_expansion_algorithms.py:228-260):
    2**num_doublings coefficients, i.e. 2**num_doublings - 1 derivatives, here
    computed by the solver kernels' jet recursion."""
    if num_doublings < 1:
        raise ValueError("num_doublings must be positive")
    return _JetExpand(2**num_doublings - 1)


class taylor_point_prior:
    """Linearise at the prior mean (taylor_points.py:150-156), the native TS1 point."""


class taylor_point_maximum_a_posteriori:
    """Linearise at the maximum-a-posteriori point (taylor_points.py:159-175);
    not native: ``constraint_ode_ts1`` raises NotImplementedError for it."""

    def __init__(self, nlstsq=None):
        self.nlstsq = nlstsq


def system_matrices_1d_iwp(num_derivatives):
    """A = flip(Pascal) and Q = the lower square root of flip(Hilbert), with a
    non-negative diagonal (utilities.py:57-71): the IWP's one-dimensional
    transition matrix and noise factor at unit step, float64 on the host.
    The kernels use the same matrices (A folded into the code as integer
    binomials, Q computed on the host in long double)."""
    import math

    import decimal

    n = num_derivatives + 1
    A = torch.tensor([[float(math.comb(n - 1 - i, j - i)) if j >= i else 0.0 for j in range(n)] for i in range(n)],
                     dtype=torch.float64)
    # Cholesky factor of flip(Hilbert) in 40-digit decimal arithmetic (the
    # matrix is ill-conditioned: a float64 factorisation loses ~4 digits)
    with decimal.localcontext(decimal.Context(prec=40)):
        one = decimal.Decimal(1)
        H = [[one / (2 * num_derivatives + 1 - i - j) for j in range(n)] for i in range(n)]
        L = [[decimal.Decimal(0)] * n for _ in range(n)]
        for j in range(n):
            L[j][j] = (H[j][j] - sum((L[j][k] * L[j][k] for k in range(j)), decimal.Decimal(0))).sqrt()
            for i in range(j + 1, n):
                L[i][j] = (H[i][j] - sum((L[i][k] * L[j][k] for k in range(j)), decimal.Decimal(0))) / L[j][j]
        Q = torch.tensor([[float(x) for x in row] for row in L], dtype=torch.float64)
    return A, Q


def preconditioner_taylor(num_derivatives):
    """The Taylor preconditioner (utilities.py:74-84): precon(dt) returns
    p_i = dt^(nu - i) / (nu - i)! and its inverse, float64 on the host."""
    import math

    powers = torch.arange(num_derivatives, -1, -1, dtype=torch.float64)
    scales = torch.tensor([float(math.factorial(int(k))) for k in powers], dtype=torch.float64)

    def precon(dt):
        dt = torch.as_tensor(dt, dtype=torch.float64)
        return torch.pow(dt, powers) / scales, torch.pow(dt, -powers) * scales

    return precon


@dataclasses.dataclass(frozen=True)
class Prior:
    """An integrated Wiener process prior (ssm_impl_*.py prior_wiener_integrated)."""

    ssm: str
    tcoeffs: TaylorCoefficients

    @property
    def num_derivatives(self):
        return self.tcoeffs.num


@dataclasses.dataclass(frozen=True)
class Constraint:
    ssm: str
    kind: str  # "ts0" | "ts1"
    field: Field
    residual_order: int = 2


class _StateSpaceModel:
    name = ""

    def prior_wiener_integrated(self, tcoeffs, /, *, is_exact=True, inexact_eps=1e-6, diffuse_derivatives=0,
                                diffuse_eps=1.0, output_scale=None):
        """IWP prior from exact Taylor coefficients (ssm_impl_isotropic.py:409-482)."""
        if not isinstance(tcoeffs, TaylorCoefficients):
            raise TypeError("tcoeffs must come from jetexpand_ode_padded_scan(...)(vf, (u0,))")
        if is_exact is not True or diffuse_derivatives or output_scale is not None:
            raise NotImplementedError("only exact initial coefficients with the default output scale are native")
        return Prior(self.name, tcoeffs)

    def constraint_ode_ts0(self, ode, /):
        if not isinstance(ode, Field):
            raise TypeError(ode)
        return Constraint(self.name, "ts0", ode)

    def constraint_ode_ts1(self, ode, /, taylor_point=None):
        """TS1 linearisation (ssm_impl_api.py:536-558): the full Jacobian (dense), its
        trace along d (isotropic, ssm_impl_isotropic.py:320-355) or its diagonal
        along d (block-diagonal, ssm_impl_blockdiag.py:147-183), at the prior mean."""
        if not isinstance(ode, Field):
            raise TypeError(ode)
        if taylor_point is not None and not isinstance(taylor_point, taylor_point_prior):
            raise NotImplementedError("only the prior-mean Taylor point (taylor_point_prior) is native")
        return Constraint(self.name, "ts1", ode)


class state_space_model_isotropic(_StateSpaceModel):
    """Isotropic factorisation (ssm_impl_isotropic.py:406-584)."""

    name = "isotropic"


class state_space_model_blockdiag(_StateSpaceModel):
    """Block-diagonal factorisation (ssm_impl_blockdiag.py:460-654)."""

    name = "blockdiag"


class state_space_model_dense(_StateSpaceModel):
    """Dense factorisation (ssm_impl_dense.py:455-732)."""

    name = "dense"


class strategy_filter:
    """estimators_and_losses.py:347-421."""

    name = "filter"
    is_suitable_for_save_at = True
    is_suitable_for_save_every_step = True
    is_suitable_for_offgrid_marginals = True


class strategy_smoother_fixedpoint:
    """estimators_and_losses.py:473-591."""

    name = "fixedpoint"
    is_suitable_for_save_at = True
    is_suitable_for_save_every_step = False
    is_suitable_for_offgrid_marginals = False


class strategy_smoother_fixedinterval:
    """estimators_and_losses.py:594-717: the smoother with a backward conditional per step.

    Native on fixed grids (``ivpsolve.solve_fixed_grid``): there every grid
    point is a checkpoint, so the fixed-point kernel's conditionals between
    checkpoints are exactly the per-step conditionals and its smoothed
    marginals are the fixed-interval smoother's (the equivalence of the
    reference's test_smoother_fixedinterval_vs_fixedpoint.py).
    """

    name = "fixedinterval"
    is_suitable_for_save_at = False
    is_suitable_for_save_every_step = True
    is_suitable_for_offgrid_marginals = True


@dataclasses.dataclass(frozen=True)
class _Solver:
    strategy: Any
    constraint: Constraint
    kind: str
    correct_asymptotic_underconfidence: bool = True

    @property
    def is_suitable_for_save_at(self):
        return self.strategy.is_suitable_for_save_at

    @property
    def is_suitable_for_save_every_step(self):
        return self.strategy.is_suitable_for_save_every_step

    @property
    def is_suitable_for_offgrid_marginals(self):
        return self.strategy.is_suitable_for_offgrid_marginals

    def offgrid_marginals(self, t, *, solution, stream=None):
        """Marginals at times off the solution's grid (solvers.py:149-203), on the GPU.

        ``solution`` is a filter or fixed-interval-smoother solution on a grid
        (``ivpsolve.solve_fixed_grid``; the smoother's solve keeps the
        filtering marginals this needs).  ``t``: a scalar, a (Q,) vector
        shared by the instances, or (B, Q).  Each query interval is
        searchsorted(grid, t) = index, with the transitions at
        output_scale[index]; t must lie strictly inside the grid's span and
        off the grid points (the reference checks neither; here a grid point
        returns its marginal and a time outside the span NaN).  Returns an
        ``ivpsolve.Normal`` with a query axis after the batch axis (none for a
        scalar ``t``).

        Block-diagonal solutions (means (B, S, d, n), factors (B, S, d, n, n),
        output scales (B, S, d)) are d independent one-dimensional isotropic
        models (ssm_impl_blockdiag.py:406-432 transitions each dimension with
        its own scale), so they run on the isotropic kernel as B * d
        instances of dimension 1.
        """
        import torch

        from . import _native
        from .ivpsolve import Normal

        if not self.is_suitable_for_offgrid_marginals:
            raise NotImplementedError
        ssm = self.constraint.ssm
        post = solution.posterior or {}
        if self.strategy.name == "fixedinterval" and "filter_mean" not in post:
            raise ValueError("off-grid marginals of a smoother need its filtering marginals: "
                             "solve with posterior=True")
        grid = solution.t if solution.t.ndim == 2 else solution.t[None]
        B = grid.shape[0]
        tq = torch.as_tensor(t, dtype=torch.float64, device=grid.device)
        scalar = tq.ndim == 0
        tq = tq.reshape(1, -1).expand(B, -1) if tq.ndim <= 1 else tq
        d = solution.ode_dim
        if ssm == "blockdiag":
            mean, chol = _blockdiag_offgrid(self.strategy.name, grid, solution, post, tq, stream)
        else:
            n = solution.u.mean_flat.shape[-2] if ssm == "isotropic" else solution.u.mean_flat.shape[-1] // d
            mean, chol = _native.offgrid_marginals(
                ssm, self.strategy.name, n - 1, d, grid, solution.u.mean_flat, solution.u.cholesky_flat,
                solution.output_scale, tq, post.get("filter_mean"), post.get("filter_chol"), stream=stream)
        if scalar:
            mean, chol = mean[:, 0], chol[:, 0]
        return Normal(mean, chol, ssm)


def _blockdiag_offgrid(strategy, grid, solution, post, tq, stream):
    """Off-grid marginals of a block-diagonal grid solution through the
    isotropic kernel: dimension j of instance b becomes instance b * d + j
    with ode_dim 1, the grid and query times repeated per dimension, the
    output scale of that dimension as its scalar scale.  Returns means
    (B, Q, d, n) and factors (B, Q, d, n, n)."""
    from . import _native

    B, S = grid.shape
    um = solution.u.mean_flat.reshape(B, S, *solution.u.mean_flat.shape[-2:])
    d, n = um.shape[-2:]
    if solution.output_scale.shape[-1] != d:
        raise ValueError("The output-scale has the wrong shape.")

    def per_dim_mean(m):  # (B, S, d, n) -> (B * d, S, n, 1)
        return m.reshape(B, S, d, n).permute(0, 2, 1, 3).reshape(B * d, S, n, 1)

    def per_dim_chol(c):  # (B, S, d, n, n) -> (B * d, S, n, n)
        return c.reshape(B, S, d, n, n).permute(0, 2, 1, 3, 4).reshape(B * d, S, n, n)

    fm, fc = post.get("filter_mean"), post.get("filter_chol")
    mean, chol = _native.offgrid_marginals(
        "isotropic", strategy, n - 1, 1, grid.repeat_interleave(d, dim=0), per_dim_mean(um),
        per_dim_chol(solution.u.cholesky_flat),
        solution.output_scale.reshape(B, S, d).permute(0, 2, 1).reshape(B * d, S),
        tq.repeat_interleave(d, dim=0), None if fm is None else per_dim_mean(fm),
        None if fc is None else per_dim_chol(fc), stream=stream)
    Q = tq.shape[1]
    mean = mean.reshape(B, d, Q, n).permute(0, 2, 1, 3).contiguous()
    chol = chol.reshape(B, d, Q, n, n).permute(0, 2, 1, 3, 4).contiguous()
    return mean, chol


ProbabilisticSolver = _Solver  # the type behind solver / solver_mle / solver_dynamic (solvers.py:72-147)
StateSpaceModel = _StateSpaceModel  # the type of the state_space_model_* factories (ssm_impl_api.py:300-587)


def __getattr__(name):
    """``ProbabilisticSolution`` (solvers.py:33-69) is ``ivpsolve.Solution``,
    imported on first use (ivpsolve imports this module)."""
    if name == "ProbabilisticSolution":
        from .ivpsolve import Solution

        return Solution
    raise AttributeError(f"module {__name__!r} has no attribute {name!r}")


def solver(*, strategy, constraint, constraint_init=None):
    """Uncalibrated solver (solvers.py:636-767)."""
    if constraint_init is not None:
        raise NotImplementedError("constraint_init is not native")
    return _Solver(strategy, constraint, "none")


def solver_mle(*, strategy, constraint, constraint_init=None, correct_asymptotic_underconfidence=True):
    """MLE calibration (solvers.py:318-480)."""
    if constraint_init is not None:
        raise NotImplementedError("constraint_init is not native")
    return _Solver(strategy, constraint, "mle", correct_asymptotic_underconfidence)


def solver_dynamic(*, strategy, constraint, constraint_init=None, re_linearize_after_calibration=False,
                   stop_gradient_through_calibration=True):
    """Dynamic calibration (solvers.py:483-633)."""
    if constraint_init is not None or re_linearize_after_calibration:
        raise NotImplementedError("constraint_init / re-linearisation are not native")
    return _Solver(strategy, constraint, "dynamic")


@dataclasses.dataclass(frozen=True)
class error_norm_scale_then_rms:
    """Error normalisation: scale by atol + rtol |reference|, then the RMS
    (solvers.py:770-791).  The native default (with the 2-norm)."""

    norm_order: Any = None


@dataclasses.dataclass(frozen=True)
class error_norm_rms_then_scale:
    """Error normalisation: the RMS, then scale by atol + rtol RMS(reference)
    (solvers.py:794-811).  Not native: the error estimators raise
    NotImplementedError for it."""

    norm_order: Any = None


def _native_error_norm(error_norm):
    """True when ``error_norm`` is the kernels' normalisation (the default)."""
    return error_norm is None or (isinstance(error_norm, error_norm_scale_then_rms) and error_norm.norm_order is None)


@dataclasses.dataclass(frozen=True)
class error_residual_std:
    """Residual-std error estimate (solvers.py:850-996), cached linearisation."""

    constraint: Constraint
    error_norm: Optional[Any] = None
    re_linearize_before_error: bool = False
    error_per_unit_step: bool = False

    def __post_init__(self):
        if not _native_error_norm(self.error_norm) or self.re_linearize_before_error or self.error_per_unit_step:
            raise NotImplementedError("only the default error_residual_std is native")


@dataclasses.dataclass(frozen=True)
class loss_lml_timeseries:
    """LML of time-series data (estimators_and_losses.py:53-105).

    Natively evaluated together with the solve by ``ivpsolve.lml_fixed_grid``.
    """

    average_pdfs: bool = True
    tcoeff_index: int = 0

    def __post_init__(self):
        if self.tcoeff_index != 0:
            raise NotImplementedError("observations of the solution (tcoeff_index=0) only")


class loss_lml_terminal_values:
    """Log-marginal likelihood of terminal-value data
    (estimators_and_losses.py:20-50): the log-pdf of ``u`` under the
    marginal's coefficient ``tcoeff_index`` observed with noise ``std``
    (``marginals.to_derivative(tcoeff_index, std).marginalise(marginals)``).

    ``loss = loss_lml_terminal_values(); loss(u, marginals=sol.u, std=std)``
    evaluates it for a batch of solutions at once (the reference's
    ``jax.vmap`` axis): ``marginals`` an ``ivpsolve.Normal`` whose leading
    axes are batch axes (e.g. ``(B, 1)`` from ``solve_adaptive_terminal_values``),
    ``u`` the data broadcastable to the observed coefficient's shape (d per
    instance), ``std`` one scalar per instance for the isotropic
    factorisation and one value per dimension for the dense and
    block-diagonal ones (or a single such container for all instances).
    Returns one log-pdf per instance.  The arithmetic is torch on the
    marginals' device, so it is differentiable through their means (the
    ``autograd.terminal_values`` sensitivities).
    """

    def __init__(self, *, tcoeff_index=0):
        self.tcoeff_index = int(tcoeff_index)

    @staticmethod
    def _raise(std, expected, u):
        msg = "The standard deviation container differs from what was expected."
        msg += f" Expected: shape={tuple(expected)}."
        msg += f" Received: shape={tuple(std.shape)}."
        msg += f" For reference: data-shape={tuple(u.shape)}."
        raise ValueError(msg)

    def __call__(self, u, /, *, marginals, std):
        import math

        k = self.tcoeff_index
        mean, chol = marginals.mean_flat, marginals.cholesky_flat
        u = torch.as_tensor(u, dtype=mean.dtype, device=mean.device)
        std = torch.as_tensor(std, dtype=mean.dtype, device=mean.device)
        log2pi = math.log(2.0 * math.pi)
        if marginals.ssm == "isotropic":
            batch = mean.shape[:-2]
            if std.shape not in ((), batch):
                self._raise(std, batch, u)
            mu = mean[..., k, :]  # (..., d)
            var = (chol[..., k, :] ** 2).sum(-1) + std**2  # one variance shared by the d dimensions
            d = mu.shape[-1]
            maha = ((u - mu) ** 2).sum(-1) / var
            return -0.5 * (maha + d * torch.log(var) + d * log2pi)
        if marginals.ssm == "blockdiag":
            batch, d = mean.shape[:-2], mean.shape[-2]
            if std.shape not in ((d,), batch + (d,)):
                self._raise(std, batch + (d,), u)
            mu = mean[..., k]  # (..., d)
            var = (chol[..., k, :] ** 2).sum(-1) + std**2  # (..., d)
            return -0.5 * (((u - mu) ** 2 / var) + torch.log(var) + log2pi).sum(-1)
        if marginals.ssm == "dense":
            d = u.shape[-1]
            batch = mean.shape[:-1]
            if std.shape not in ((d,), batch + (d,)):
                self._raise(std, batch + (d,), u)
            mu = mean[..., k * d:(k + 1) * d]
            rows = chol[..., k * d:(k + 1) * d, :]
            cov = rows @ rows.transpose(-1, -2) + torch.diag_embed(std.expand(batch + (d,)) ** 2)
            L = torch.linalg.cholesky(cov)
            w = torch.linalg.solve_triangular(L, (u - mu).unsqueeze(-1), upper=False).squeeze(-1)
            logdet = 2.0 * torch.log(torch.diagonal(L, dim1=-2, dim2=-1)).sum(-1)
            return -0.5 * ((w**2).sum(-1) + logdet + d * log2pi)
        raise ValueError(f"unknown factorisation {marginals.ssm!r}")


@dataclasses.dataclass(frozen=True)
class error_state_std:
    """State-std error estimate (solvers.py:999-1098): the posterior std of u after
    conditioning the unit-scale extrapolation on the linearised residual, times
    the local calibration; cached linearisation, derivative 0."""

    constraint: Constraint
    error_norm: Optional[Any] = None
    re_linearize_before_error: bool = False
    derivative_idx: int = 0
    error_per_unit_step: bool = False

    def __post_init__(self):
        if (not _native_error_norm(self.error_norm) or self.re_linearize_before_error or self.derivative_idx != 0
                or self.error_per_unit_step):
            raise NotImplementedError("only the default error_state_std is native")


def _native_strategy(strategy):
    if strategy.name == "fixedinterval":
        if not getattr(strategy, "_on_grid", False):
            raise NotImplementedError("strategy_smoother_fixedinterval is native with ivpsolve.solve_fixed_grid only")
        return "fixedpoint"
    return strategy.name


def _field_dim(field, y0):
    d = _FIELD_DIMS[field.name]
    return y0.shape[-1] if d is None else d


def lower(solver_obj, error, control, *, num_derivatives, y0, precision, atol, rtol, clip_dt, eps, damp):
    """Lower constructor objects to a pdq_config (include/pdq.h)."""
    from . import ensemble
    from .ivpsolve import control_integral, control_proportional_integral

    c = solver_obj.constraint
    if error is not None and error.constraint is not c:
        raise ValueError("the error estimator must use the solver's constraint")
    ctrl = control if control is not None else control_integral()
    kw = dict(safety=ctrl.safety, factor_min=ctrl.factor_min, factor_max=ctrl.factor_max)
    if isinstance(ctrl, control_proportional_integral):
        kw.update(control="proportional_integral", exponent_integral=ctrl.exponent_integral,
                  exponent_proportional=ctrl.exponent_proportional)
    else:
        kw.update(control="integral")
    kw["error"] = "state_std" if isinstance(error, error_state_std) else "residual_std"
    return ensemble.make_config(
        field=c.field.name, num_derivatives=num_derivatives, ode_dim=_field_dim(c.field, y0), ssm=c.ssm,
        constraint=c.kind, strategy=_native_strategy(solver_obj.strategy), solver=solver_obj.kind, precision=precision,
        atol=atol, rtol=rtol, clip_dt=clip_dt, eps=eps, damp=damp,
        correct_asymptotic_underconfidence=solver_obj.correct_asymptotic_underconfidence, **kw,
    )


_native_status = _native.INSTANCE_STATUS
