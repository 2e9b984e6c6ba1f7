"""The LML-gradient configuration shared by tests and the benchmark.

FitzHugh--Nagumo (benchmarks/C0_taylor-init-fitzhughnagumo.py:119-131) with
parameters theta = (a, b, c), u0 = (-1, 1).  Observations at t_k = k * dt *
save_every, k = 0..num_obs-1 (the grid's every save_every-th point, t0
included so the 200 backward conditionals of the smoother line up with the
data, len(data) = len(conditionals) + 1 as evaluate_lml requires), generated
from a DOP853 (rtol = atol = 1e-12) solution at theta* = (0.2, 0.2, 3.0) plus
N(0, 0.01^2) noise, numpy seed 0.
"""

import numpy as np
import scipy.integrate

THETA_STAR = np.array([0.2, 0.2, 3.0])
U0 = np.array([-1.0, 1.0])
STD = 0.01


def fhn(t, u, a, b, c):
    return [c * (u[0] - u[0] ** 3 / 3 + u[1]), -(u[0] - a - b * u[1]) / c]


def observations(t1=20.0, dt=0.01, save_every=10, seed=0):
    num_steps = int(round(t1 / dt))
    num_obs = num_steps // save_every + 1
    t_obs = np.arange(num_obs) * dt * save_every
    sol = scipy.integrate.solve_ivp(fhn, (0.0, t1), U0, t_eval=t_obs, args=tuple(THETA_STAR), method="DOP853",
                                    rtol=1e-12, atol=1e-12)
    rng = np.random.default_rng(seed)
    data = sol.y.T + STD * rng.standard_normal(sol.y.T.shape)
    return num_steps, data


def theta_samples(B, seed=0):
    rng = np.random.default_rng(seed)
    return THETA_STAR[None, :] + 0.05 * rng.standard_normal((B, 3))
