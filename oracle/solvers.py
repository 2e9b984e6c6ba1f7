"""Solvers, strategies, error estimators, controllers and IVP loops of the oracle.

TEST INFRASTRUCTURE ONLY.  Restates, per instance and in PyTorch:
  * ``_probdiffeq/estimators_and_losses.py`` (strategies, MarkovSequence, LML),
  * ``_probdiffeq/solvers.py`` (solver, solver_mle, solver_dynamic,
    error_residual_std, error_state_std, error norms),
  * ``_ivpsolve/controllers.py`` (I and PI control),
  * ``_ivpsolve/solvers_via_adaptive_steps.py`` (RejectionLoop, save_at,
    terminal values), ``_ivpsolve/solvers_via_fixed_steps.py``.

``jax.lax.while_loop``/``cond``/``switch`` become Python control flow with the
same branch conditions, so an instance takes exactly the reference's sequence
of attempts.  A generous ``max_attempts`` guard raises instead of looping
forever (the reference has no bound).
"""

import dataclasses
import math
from typing import Any

import torch

from . import linalg


# --------------------------------------------------------------------------
# Helpers over the three factorisations
# --------------------------------------------------------------------------


def coeff(normal, i):
    """Taylor coefficient i of a normal's mean as a (d,) vector."""
    if normal.kind == "isotropic":
        return normal.mean[i]
    if normal.kind == "blockdiag":
        return normal.mean[:, i]
    d = normal.d
    return normal.mean[i * d : (i + 1) * d]


def num_coeffs(normal):
    if normal.kind == "isotropic":
        return normal.mean.shape[0]
    if normal.kind == "blockdiag":
        return normal.mean.shape[1]
    return normal.mean.shape[0] // normal.d


@dataclasses.dataclass
class MarkovSeq:
    """MarkovSequence (estimators_and_losses.py:121-273), reverse=True."""

    marginal: Any
    conditional: Any

    def rescale_cholesky(self, factor):
        """estimators_and_losses.py:151-154."""
        return MarkovSeq(self.marginal.rescale_cholesky(factor), self.conditional.rescale_noise(factor))


@dataclasses.dataclass
class Solution:
    """ProbabilisticSolution (solvers.py:33-69)."""

    t: Any
    u: Any
    posterior: Any
    output_scale: Any
    num_steps: int
    auxiliary: Any
    fun_evals: Any
    prior: Any


# --------------------------------------------------------------------------
# Strategies (estimators_and_losses.py:347-717)
# --------------------------------------------------------------------------


class StrategyFilter:
    """strategy_filter (estimators_and_losses.py:347-421)."""

    name = "filter"
    is_smoother = False

    def init_posterior(self, u):
        return u, u

    def predict(self, posterior, transition):
        m = transition.marginalise(posterior)
        return m, m

    def apply_updates(self, prediction, updates):
        return updates, updates

    def finalize(self, posterior0, posteriors, posterior1, output_scale):
        """estimators_and_losses.py:380-391: rescale and stack."""
        marg = [posterior0.rescale_cholesky(output_scale)] + [p.rescale_cholesky(output_scale) for p in posteriors]
        return marg, marg

    def interpolate_fwd(self, posterior_t0, posterior_t1, transition_t0_t, transition_t_t1):
        """estimators_and_losses.py:393-414."""
        _, interpolated = self.predict(posterior_t0, transition_t0_t)
        return (interpolated, interpolated), (posterior_t1, interpolated)

    def interpolate_fwd_at_t1(self, posterior_t1):
        """estimators_and_losses.py:416-421."""
        return (posterior_t1, posterior_t1), (posterior_t1, posterior_t1)


class _Smoother:
    is_smoother = True

    def init_posterior(self, u):
        """estimators_and_losses.py:425-428."""
        return u, MarkovSeq(u, u.identity_conditional())

    def apply_updates(self, prediction, updates):
        """estimators_and_losses.py:430-435."""
        return updates, MarkovSeq(updates, prediction.conditional)

    def finalize(self, posterior0, posteriors, posterior1, output_scale):
        """estimators_and_losses.py:437-470."""
        posterior0 = posterior0.rescale_cholesky(output_scale)
        posteriors = [p.rescale_cholesky(output_scale) for p in posteriors]
        posterior1 = posterior1.rescale_cholesky(output_scale)
        rv_at_t1 = posterior1.conditional.marginalise(posterior1.marginal)
        conds = [p.conditional for p in posteriors]
        marginals = evaluate_marginals(rv_at_t1, conds)
        filtering = [posterior0.marginal] + [p.marginal for p in posteriors]
        return marginals, {"rv_at_t1": rv_at_t1, "conditionals": conds, "filtering": filtering}


def evaluate_marginals(terminal, conditionals):
    """Reverse scan of marginalise (estimators_and_losses.py:156-178)."""
    out = [None] * len(conditionals)
    x = terminal
    for k in range(len(conditionals) - 1, -1, -1):
        x = conditionals[k].marginalise(x)
        out[k] = x
    return out + [terminal]


class StrategyFixedPoint(_Smoother):
    """strategy_smoother_fixedpoint (estimators_and_losses.py:473-591)."""

    name = "fixedpoint"

    def predict(self, posterior, transition):
        """estimators_and_losses.py:526-532."""
        marginals, cond = transition.revert(posterior.marginal, solve_triu=linalg.solve_triu)
        cond = posterior.conditional.merge(cond)
        return marginals, MarkovSeq(marginals, cond)

    def interpolate_fwd_at_t1(self, posterior_t1):
        """estimators_and_losses.py:534-547."""
        resume = MarkovSeq(posterior_t1.marginal, posterior_t1.marginal.identity_conditional())
        return (posterior_t1.marginal, posterior_t1), (resume, resume)

    def interpolate_fwd(self, posterior_t0, posterior_t1, transition_t0_t, transition_t_t1):
        """estimators_and_losses.py:549-591."""
        _, extrapolated_t = self.predict(posterior_t0, transition_t0_t)
        previous_new = MarkovSeq(extrapolated_t.marginal, posterior_t0.marginal.identity_conditional())
        _, extrapolated_t1 = self.predict(previous_new, transition_t_t1)
        interpolated = MarkovSeq(extrapolated_t.marginal, extrapolated_t.conditional)
        step_from = MarkovSeq(posterior_t1.marginal, extrapolated_t1.conditional)
        return (interpolated.marginal, interpolated), (step_from, previous_new)


class StrategyFixedInterval(_Smoother):
    """strategy_smoother_fixedinterval (estimators_and_losses.py:594-717)."""

    name = "fixedinterval"

    def predict(self, posterior, transition):
        """estimators_and_losses.py:612-620."""
        marginals, cond = transition.revert(posterior.marginal, solve_triu=linalg.solve_triu)
        return marginals, MarkovSeq(marginals, cond)

    def interpolate_fwd(self, posterior_t0, posterior_t1, transition_t0_t, transition_t_t1):
        """estimators_and_losses.py:622-672."""
        _, solution_at_t = self.predict(posterior_t0, transition_t0_t)
        _, extrapolated_t1 = self.predict(solution_at_t, transition_t_t1)
        solution_at_t1 = MarkovSeq(posterior_t1.marginal, extrapolated_t1.conditional)
        return (solution_at_t.marginal, solution_at_t), (solution_at_t1, solution_at_t)

    def interpolate_fwd_at_t1(self, posterior_t1):
        """estimators_and_losses.py:711-717."""
        return (posterior_t1.marginal, posterior_t1), (posterior_t1, posterior_t1)


# --------------------------------------------------------------------------
# Solvers (solvers.py:72-767)
# --------------------------------------------------------------------------


class _SolverBase:
    def __init__(self, strategy, constraint):
        self.strategy, self.constraint = strategy, constraint

    def interpolate_fwd(self, t, interp_from, interp_to):
        """solvers.py:205-269."""
        output_scale = interp_to.output_scale
        tr0 = interp_from.prior.transition(t - interp_from.t, output_scale)
        tr1 = interp_from.prior.transition(interp_to.t - t, output_scale)
        (estimate, interpolated), (step_from_post, interp_from_post) = self.strategy.interpolate_fwd(
            interp_from.posterior, interp_to.posterior, tr0, tr1
        )
        step_from = dataclasses.replace(interp_to, posterior=step_from_post)
        interpolated_sol = dataclasses.replace(interp_to, t=t, posterior=interpolated, u=estimate)
        interp_from_new = dataclasses.replace(interp_from, t=t, posterior=interp_from_post)
        return interpolated_sol, (step_from, interp_from_new)

    def interpolate_fwd_at_t1(self, t, interp_from, interp_to):
        """solvers.py:271-315."""
        (estimate, interpolated), (step_from_post, interp_from_post) = self.strategy.interpolate_fwd_at_t1(
            interp_to.posterior
        )
        prev = dataclasses.replace(interp_from, t=interp_to.t, posterior=interp_from_post)
        sol = dataclasses.replace(interp_to, posterior=interpolated, u=estimate)
        acc = dataclasses.replace(interp_to, posterior=step_from_post)
        return sol, (acc, prev)

    def _init_common(self, t, prior):
        u, posterior = self.strategy.init_posterior(prior.init)
        return u, posterior


class SolverPlain(_SolverBase):
    """solver (solvers.py:636-767): no calibration."""

    name = "none"

    def init(self, t, prior, damp):
        u, posterior = self._init_common(t, prior)
        proto = u.prototype_output_scale()
        return Solution(t, u, posterior, torch.ones_like(proto), 0, None, None, prior)

    def step(self, state, dt, damp):
        """solvers.py:702-733."""
        output_scale = torch.ones_like(torch.as_tensor(state.output_scale))
        transition = state.prior.transition(dt, output_scale)
        u_pred, prediction = self.strategy.predict(state.posterior, transition)
        fx = self.constraint.linearize(u_pred, damp=damp, t=state.t + dt)
        _, reverted = fx.revert(u_pred, solve_triu=linalg.solve_triu)
        updates = reverted.apply_flat(torch.zeros_like(fx.noise.mean))
        u, posterior = self.strategy.apply_updates(prediction, updates)
        return Solution(state.t + dt, u, posterior, output_scale, state.num_steps + 1, None, fx, state.prior)

    def userfriendly_output(self, solution0, solutions, solution1):
        """solvers.py:735-767."""
        output_scale = torch.ones_like(torch.as_tensor(solutions[-1].output_scale))
        u, posterior = self.strategy.finalize(
            solution0.posterior, [s.posterior for s in solutions], solution1.posterior, output_scale
        )
        scales = [output_scale for _ in solutions]
        return u, posterior, scales


class SolverMLE(_SolverBase):
    """solver_mle (solvers.py:318-480)."""

    name = "mle"

    def __init__(self, strategy, constraint, correct_asymptotic_underconfidence=True):
        super().__init__(strategy, constraint)
        self.correct = correct_asymptotic_underconfidence

    def init(self, t, prior, damp):
        """solvers.py:348-393 (no constraint_init)."""
        u, posterior = self._init_common(t, prior)
        proto = u.prototype_output_scale()
        aux = (torch.zeros_like(proto, dtype=torch.float64), 0.0)
        return Solution(t, u, posterior, torch.ones_like(proto), 0, aux, None, prior)

    def step(self, state, dt, damp):
        """solvers.py:395-437."""
        proto = state.u.prototype_output_scale()
        transition = state.prior.transition(dt, torch.ones_like(proto))
        u, prediction = self.strategy.predict(state.posterior, transition)
        running, num_data = state.auxiliary
        fx = self.constraint.linearize(u, damp=damp, t=state.t + dt)
        observed, reverted = fx.revert(u, solve_triu=linalg.solve_triu)
        new_term = observed.residual_whitened_rms(None)
        updates = reverted.apply_flat(torch.zeros_like(fx.noise.mean))
        u, posterior = self.strategy.apply_updates(prediction, updates)
        x1 = math.sqrt(num_data / (num_data + 1)) * running
        x2 = math.sqrt(1.0 / (num_data + 1)) * new_term.to(torch.float64)
        running = torch.hypot(torch.as_tensor(x1, dtype=torch.float64), x2)
        return Solution(state.t + dt, u, posterior, state.output_scale, state.num_steps + 1, (running, num_data + 1), fx, state.prior)

    def userfriendly_output(self, solution0, solutions, solution1):
        """solvers.py:439-480."""
        running, _ = solution1.auxiliary
        output_scale = running.to(solution0.u.mean.dtype)
        if self.correct:
            output_scale = output_scale / math.sqrt(solutions[-1].num_steps)
        u, posterior = self.strategy.finalize(
            solution0.posterior, [s.posterior for s in solutions], solution1.posterior, output_scale
        )
        return u, posterior, [output_scale for _ in solutions]


class SolverDynamic(_SolverBase):
    """solver_dynamic (solvers.py:483-633), re_linearize_after_calibration=False."""

    name = "dynamic"

    def init(self, t, prior, damp):
        u, posterior = self._init_common(t, prior)
        proto = u.prototype_output_scale()
        return Solution(t, u, posterior, torch.ones_like(proto), 0, None, None, prior)

    def step(self, state, dt, damp):
        """solvers.py:549-599."""
        proto = state.u.prototype_output_scale()
        transition = state.prior.transition(dt, torch.ones_like(proto))
        u = transition.apply_flat(state.u.mean)
        fx = self.constraint.linearize(u, damp=damp, t=state.t + dt)
        observed = fx.marginalise(u)
        output_scale = observed.residual_whitened_rms(None).detach()
        transition = state.prior.transition(dt, output_scale)
        u, prediction = self.strategy.predict(state.posterior, transition)
        _, reverted = fx.revert(u, solve_triu=linalg.solve_triu)
        updates = reverted.apply_flat(torch.zeros_like(fx.noise.mean))
        u, posterior = self.strategy.apply_updates(prediction, updates)
        return Solution(state.t + dt, u, posterior, output_scale, state.num_steps + 1, None, fx, state.prior)

    def userfriendly_output(self, solution0, solutions, solution1):
        """solvers.py:601-633."""
        ones = torch.ones_like(torch.as_tensor(solutions[-1].output_scale))
        u, posterior = self.strategy.finalize(
            solution0.posterior, [s.posterior for s in solutions], solution1.posterior, ones
        )
        return u, posterior, [solution0.output_scale] + [s.output_scale for s in solutions]


# --------------------------------------------------------------------------
# Error estimators (solvers.py:770-1098)
# --------------------------------------------------------------------------


def error_norm_scale_then_rms(error_abs, reference, atol, rtol):
    """solvers.py:770-791."""
    scale = atol + rtol * torch.abs(reference)
    rel = error_abs / scale
    return linalg.vector_norm(rel) / math.sqrt(rel.numel())


class ErrorResidualStd:
    """error_residual_std (solvers.py:850-996), cached linearisation."""

    def __init__(self, constraint, error_per_unit_step=False):
        self.constraint, self.error_per_unit_step = constraint, error_per_unit_step

    def estimate_error_norm(self, previous, proposed, dt, atol, rtol, damp):
        proto = proposed.u.prototype_output_scale()
        transition = previous.prior.transition(dt, torch.ones_like(proto))
        rv = transition.apply_flat(previous.u.mean)
        linearized = proposed.fun_evals
        observed = linearized.marginalise(rv)
        scale = observed.residual_whitened_rms(None)
        observed = observed.rescale_cholesky(scale)
        error = observed.std().reshape(-1)
        rate = num_coeffs(previous.u)
        u0, u1 = coeff(previous.u, 0), coeff(proposed.u, 0)
        reference = torch.maximum(torch.abs(u0), torch.abs(u1))
        n = self.constraint.residual_order - 1
        if self.error_per_unit_step:
            n += 1
        if tuple(error.shape) not in [(1,), tuple(reference.shape)]:
            raise ValueError("The error-estimate and reference have different shapes.")
        error_abs = error * dt**n / math.factorial(n)
        error_abs = error_abs * torch.ones_like(reference)
        norm = error_norm_scale_then_rms(error_abs, reference, atol, rtol)
        return norm ** (-1.0 / rate)


class ErrorStateStd:
    """error_state_std (solvers.py:999-1098), cached linearisation."""

    def __init__(self, constraint, derivative_idx=0, error_per_unit_step=False):
        self.constraint, self.derivative_idx, self.error_per_unit_step = constraint, derivative_idx, error_per_unit_step

    def estimate_error_norm(self, previous, proposed, dt, atol, rtol, damp):
        proto = proposed.u.prototype_output_scale()
        transition = previous.prior.transition(dt, torch.ones_like(proto))
        rv = transition.apply_flat(previous.u.mean)
        rate = num_coeffs(previous.u)
        linearized = proposed.fun_evals
        observed, reverted = linearized.revert(rv, solve_triu=linalg.solve_triu)
        scale = observed.residual_whitened_rms(None)
        conditional = reverted.apply_flat(torch.zeros_like(linearized.noise.mean))
        n = self.derivative_idx
        std = conditional.std()
        if conditional.kind == "isotropic":
            err = std[n] * torch.ones_like(coeff(previous.u, n))
        elif conditional.kind == "blockdiag":
            err = std[:, n]
        else:
            d = conditional.d
            err = std[n * d : (n + 1) * d]
        err = scale * err
        reference = torch.maximum(torch.abs(coeff(previous.u, n)), torch.abs(coeff(proposed.u, n)))
        if self.error_per_unit_step:
            n += 1
        error_abs = err * dt**n / math.factorial(n)
        norm = error_norm_scale_then_rms(error_abs, reference, atol, rtol)
        return norm ** (-1.0 / rate)


# --------------------------------------------------------------------------
# Controllers (_ivpsolve/controllers.py)
# --------------------------------------------------------------------------


class ControlIntegral:
    """control_integral (controllers.py:66-84)."""

    def __init__(self, safety=0.95, factor_min=0.2, factor_max=10.0):
        self.safety, self.factor_min, self.factor_max = safety, factor_min, factor_max

    def init(self, dt):
        return ()

    def apply(self, dt, state, error_power):
        ratio = self.safety * error_power
        factor = max(self.factor_min, min(ratio, self.factor_max))
        return factor * dt, ()


class ControlPI:
    """control_proportional_integral (controllers.py:24-63)."""

    def __init__(self, safety=0.95, factor_min=0.2, factor_max=10.0, exponent_integral=0.3, exponent_proportional=0.4):
        self.safety, self.factor_min, self.factor_max = safety, factor_min, factor_max
        self.ei, self.ep = exponent_integral, exponent_proportional

    def init(self, dt):
        return 1.0

    def apply(self, dt, prev, error_power):
        gi = error_power**self.ei
        gp = (error_power / prev) ** self.ep
        ratio = self.safety * gi * gp
        factor = max(self.factor_min, min(ratio, self.factor_max))
        prev = error_power if error_power >= 1.0 else prev
        return factor * dt, prev


# --------------------------------------------------------------------------
# IVP loops (_ivpsolve/solvers_via_adaptive_steps.py, solvers_via_fixed_steps.py)
# --------------------------------------------------------------------------


@dataclasses.dataclass
class AdaptiveResult:
    t: list
    u: list  # marginals at the save points (incl. t0)
    posterior: Any
    output_scale: list
    num_steps: list
    num_attempts: int
    num_accepted: int


def solve_adaptive_save_at(
    solver,
    error,
    prior,
    save_at,
    atol,
    rtol,
    control=None,
    clip_dt=False,
    dt0=0.1,
    eps=1e-8,
    damp=0.0,
    max_attempts=10**6,
):
    """solve_adaptive_save_at (solvers_via_adaptive_steps.py:46-148) for one instance."""
    control = ControlIntegral() if control is None else control
    save_at = [float(s) for s in save_at]
    solution0 = solver.init(save_at[0], prior, damp)
    dt = float(dt0)
    step_from, interp_from, cstate = solution0, solution0, control.init(dt)
    stats = {"attempts": 0, "accepted": 0}
    solutions = []

    def step(step_from, dt, cstate, t1):
        """RejectionLoop.step / step_attempt (:249-328)."""
        acceptance = 0.9
        proposed = None
        while acceptance < 1.0:
            dt_use = min(dt, t1 - float(step_from.t)) if clip_dt else dt
            proposed = solver.step(step_from, dt_use, damp)
            ep = float(error.estimate_error_norm(step_from, proposed, dt_use, atol, rtol, damp))
            dt, cstate = control.apply(dt_use, cstate, ep)
            acceptance = ep
            stats["attempts"] += 1
            if stats["attempts"] > max_attempts:
                raise RuntimeError("oracle: attempt bound exceeded")
        stats["accepted"] += 1
        return proposed, dt, cstate

    for t_next in save_at[1:]:
        do_continue = True
        while do_continue:
            # RejectionLoop.loop (:227-247)
            if float(step_from.t) + eps < t_next:
                new_step_from, dt, cstate = step(step_from, dt, cstate, t_next)
                interp_from, step_from = step_from, new_step_from
            t = float(step_from.t)
            if t + eps < t_next:
                solution = step_from
            elif t > t_next + eps:
                solution, (step_from, interp_from) = solver.interpolate_fwd(t_next, interp_from, step_from)
            else:
                solution, (step_from, interp_from) = solver.interpolate_fwd_at_t1(t_next, interp_from, step_from)
            do_continue = float(step_from.t) + eps < t_next
        solutions.append(solution)

    u, posterior, scales = solver.userfriendly_output(solution0, solutions, step_from)
    ts = [save_at[0]] + [float(s.t) for s in solutions]
    steps = [s.num_steps for s in solutions]
    return AdaptiveResult(ts, u, posterior, scales, steps, stats["attempts"], stats["accepted"])


def solve_adaptive_terminal_values(solver, error, prior, t0, t1, atol, rtol, control=None, clip_dt=True, dt0=0.1, eps=1e-8, damp=0.0):
    """solve_adaptive_terminal_values (solvers_via_adaptive_steps.py:16-43)."""
    res = solve_adaptive_save_at(solver, error, prior, [t0, t1], atol, rtol, control, clip_dt, dt0, eps, damp)
    return res


def solve_fixed_grid(solver, prior, grid, damp=0.0):
    """solve_fixed_grid (solvers_via_fixed_steps.py:11-34)."""
    grid = [float(g) for g in grid]
    state0 = solver.init(grid[0], prior, damp)
    s = state0
    sols = []
    for a, b in zip(grid[:-1], grid[1:]):
        s = solver.step(s, b - a, damp)
        sols.append(s)
    u, posterior, scales = solver.userfriendly_output(state0, sols, s)
    return grid, u, posterior, scales, [x.num_steps for x in sols]


def solve_fixed_steps_save_at(solver, prior, t0, dt, num_steps, save_every, damp=0.0):
    """Fixed-point smoother on a uniform grid with checkpoints every ``save_every`` steps.

    This is ``solve_adaptive_save_at`` (solvers_via_adaptive_steps.py:46-148)
    when every attempt is accepted and the steps land exactly on the save
    points: each checkpoint takes the ``interp_at_t1`` branch (:362-375),
    which resets the backward conditional to the identity
    (estimators_and_losses.py:534-547).  Time follows t_k = t0 + k dt.
    """
    state0 = solver.init(t0, prior, damp)
    s = state0
    saved = []
    for k in range(1, num_steps + 1):
        s = solver.step(s, dt, damp)
        s = dataclasses.replace(s, t=t0 + k * dt)
        if k % save_every == 0:
            sol, (acc, _prev) = solver.interpolate_fwd_at_t1(s.t, s, s)
            saved.append(sol)
            s = acc
    u, posterior, scales = solver.userfriendly_output(state0, saved, s)
    return u, posterior


def solve_grid_save_every_point(solver, prior, grid, damp=0.0):
    """``solve_adaptive_save_at`` with the grid as checkpoints when every step is
    accepted and lands exactly on the next grid point (the ``interp_at_t1``
    branch at each point, solvers_via_adaptive_steps.py:362-375): the filter's
    and the fixed-point smoother's solution at every grid point.  With the
    fixed-point smoother this is the fixed-interval smoother's posterior on
    the grid (test_smoother_fixedinterval_vs_fixedpoint.py:50-86)."""
    grid = [float(g) for g in grid]
    state0 = solver.init(grid[0], prior, damp)
    s, prev = state0, state0
    saved = []
    for a, b in zip(grid[:-1], grid[1:]):
        s = solver.step(s, b - a, damp)
        s = dataclasses.replace(s, t=b)
        sol, (s, prev) = solver.interpolate_fwd_at_t1(b, prev, s)
        saved.append(sol)
    u, posterior, scales = solver.userfriendly_output(state0, saved, s)
    return AdaptiveResult(grid, u, posterior, scales, [x.num_steps for x in saved], len(saved), len(saved))


# --------------------------------------------------------------------------
# Log-marginal likelihood (estimators_and_losses.py:20-105, 180-218)
# --------------------------------------------------------------------------


def evaluate_lml(u, terminal, conditionals, models, average_pdfs=True, solve_triu=linalg.lstsq_svd):
    """MarkovSequence.evaluate_lml (estimators_and_losses.py:180-218)."""
    observed, reverted = models[-1].revert(terminal, solve_triu=solve_triu)
    pdf = observed.logpdf(u[-1])
    rv = reverted.apply_flat(u[-1])
    num = 1
    for k in range(len(conditionals) - 1, -1, -1):
        predicted = conditionals[k].marginalise(rv)
        observed, reverted = models[k].revert(predicted, solve_triu=solve_triu)
        pdf_n = observed.logpdf(u[k])
        rv = reverted.apply_flat(u[k])
        if average_pdfs:
            pdf = (pdf * num + pdf_n) / (num + 1)
        else:
            pdf = pdf + pdf_n
        num += 1
    return pdf


def loss_lml_timeseries(u, posterior, std, average_pdfs=True, tcoeff_index=0):
    """loss_lml_timeseries (estimators_and_losses.py:53-105), isotropic/dense posteriors.

    ``u`` holds one observation per marginal (len(conditionals) + 1 of them),
    each shaped like the ODE state; ``std`` one noise value per observation.
    """
    terminal = posterior["rv_at_t1"]
    conds = posterior["conditionals"]
    if len(u) != len(conds) + 1:
        raise ValueError("The standard deviation container differs from what was expected.")
    models = [terminal.to_derivative(tcoeff_index, std[k]) for k in range(len(u))]
    if terminal.kind == "isotropic":
        data = [x.reshape(1, -1) for x in u]
    else:
        data = list(u)
    return evaluate_lml(data, terminal, conds, models, average_pdfs=average_pdfs)


def loss_lml_terminal_values(u, marginal, std, tcoeff_index=0):
    """loss_lml_terminal_values (estimators_and_losses.py:20-50)."""
    model = marginal.to_derivative(tcoeff_index, std)
    marg = model.marginalise(marginal)
    if marginal.kind == "isotropic":
        data = u.reshape(1, -1)
    elif marginal.kind == "blockdiag":
        data = u.reshape(-1, 1)
    else:
        data = u
    return marg.logpdf(data)


def offgrid_marginals(solver, t, result, prior):
    """solver.offgrid_marginals(t, solution=...) (solvers.py:149-203).

    ``result`` is a save-every-step or fixed-grid solution.  The query t must
    lie strictly inside (t0, t1) and off the grid (the reference does not
    check either).  index = searchsorted(ts, t); the strategies'
    interpolate_offgrid_marginals: the filter predicts from the marginal at
    ts[index-1] (estimators_and_losses.py:403-414); the fixed-interval smoother
    reverts the filtering marginal at ts[index-1] to t and t to ts[index], and
    marginalises the smoothed marginal at ts[index] through the second
    backward conditional (:674-709).  The transitions use
    output_scale[index] (JAX clamps the index for the MLE solver's shorter
    scale array; its entries are all equal).
    """
    if solver.strategy.name == "fixedpoint":
        raise NotImplementedError
    ts = torch.tensor([float(s) for s in result.t], dtype=torch.float64)
    index = int(torch.searchsorted(ts, torch.tensor(float(t), dtype=torch.float64)))
    t0, t1 = float(ts[index - 1]), float(ts[index])
    scale = result.output_scale[min(index, len(result.output_scale) - 1)]
    transition_t0_t = prior.transition(t - t0, scale)
    transition_t_t1 = prior.transition(t1 - t, scale)
    if solver.strategy.name == "filter":
        return transition_t0_t.marginalise(result.posterior[index - 1])
    filtering = result.posterior["filtering"][index - 1]
    extrapolated_t, _ = transition_t0_t.revert(filtering, solve_triu=linalg.solve_triu)
    _, conditional_t1_to_t = transition_t_t1.revert(extrapolated_t, solve_triu=linalg.solve_triu)
    return conditional_t1_to_t.marginalise(result.u[index])


def solve_adaptive_save_every_step(solver, error, prior, t0, t1, atol, rtol, control=None, clip_dt=False, dt0=0.1, eps=1e-8, damp=0.0):
    """Python-loop save-every-step solver (util/test_util.py:10-66)."""
    control = ControlIntegral() if control is None else control
    solution0 = solver.init(t0, prior, damp)
    dt, step_from, interp_from, cstate = float(dt0), solution0, solution0, control.init(dt0)
    solutions = []
    attempts = [0]

    def step(step_from, dt, cstate):
        acceptance = 0.9
        while acceptance < 1.0:
            dt_use = min(dt, t1 - float(step_from.t)) if clip_dt else dt
            proposed = solver.step(step_from, dt_use, damp)
            ep = float(error.estimate_error_norm(step_from, proposed, dt_use, atol, rtol, damp))
            dt, cstate = control.apply(dt_use, cstate, ep)
            acceptance = ep
            attempts[0] += 1
        return proposed, dt, cstate

    while float(step_from.t) < t1:
        if float(step_from.t) + eps < t1:
            new, dt, cstate = step(step_from, dt, cstate)
            interp_from, step_from = step_from, new
        t = float(step_from.t)
        if t + eps < t1:
            solution = step_from
        elif t > t1 + eps:
            solution, (step_from, interp_from) = solver.interpolate_fwd(t1, interp_from, step_from)
        else:
            solution, (step_from, interp_from) = solver.interpolate_fwd_at_t1(t1, interp_from, step_from)
        solutions.append(solution)
    u, posterior, scales = solver.userfriendly_output(solution0, solutions, step_from)
    ts = [t0] + [float(s.t) for s in solutions]
    return AdaptiveResult(ts, u, posterior, scales, [s.num_steps for s in solutions], attempts[0], len(solutions))
