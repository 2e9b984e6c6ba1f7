"""The five benchmark workloads: seeded synthetic inputs with the shapes,
sizes and distributions of the configurations they stand for.

The reference publishes no dataset or benchmark inputs (its benchmarks draw
work-precision plots from problems built in the scripts themselves), so every
input here is generated from a seed:

* ``lv_ensemble``: Lotka--Volterra, (a, b, c, d) = (0.5, 0.05, 0.5, 0.05)
  * exp(0.2 z), z ~ N(0, 1), y0 ~ U[10, 30]^2, t in [0, 50]
  (benchmarks/A0_work-precision-lotka-volterra.py:99-110 for the field and
  the nominal parameters).  ``lv_ensemble(1)`` with nominal parameters and
  y0 = (20, 20) is the single-instance configuration.
* ``vdp_dense``: van der Pol, mu = exp(U[0, ln mu_max]), y0 = (2, 0),
  t in [0, 2 mu], 100 uniform save points.
* ``burgers_blockdiag``: periodic viscous Burgers (nu = 0.01) on d points,
  u0 = sum_{k=1..8} a_k sin(2 pi k x + phi_k), a_k ~ N(0, 1/k^2),
  phi_k ~ U[0, 2 pi) (benchmarks/A5_work-precision-burgers-pde.py:32-78
  builds its problem the same way from random Fourier modes).
* ``fhn_lml``: FitzHugh--Nagumo (benchmarks/C0_taylor-init-fitzhughnagumo.py:119-131),
  theta = (a, b, c), u0 = (-1, 1); observations at t_k = k dt save_every from
  a DOP853 (rtol = atol = 1e-12) solution at theta* = (0.2, 0.2, 3.0) plus
  N(0, 0.01^2) noise; theta samples ~ N(theta*, 0.05^2 I).

The generators return CPU tensors (float64) or numpy arrays; callers move
them to the device.
"""

import math

import numpy as np

LV_NOMINAL = (0.5, 0.05, 0.5, 0.05)
LV_T_SPAN = (0.0, 50.0)


def lv_ensemble(B, seed=0):
    """(params (B, 4), y0 (B, 2)) of the Lotka--Volterra ensemble, float64 CPU tensors."""
    import torch

    g = torch.Generator().manual_seed(seed)
    nominal = torch.tensor(LV_NOMINAL, dtype=torch.float64)
    params = nominal * torch.exp(0.2 * torch.randn((B, 4), generator=g, dtype=torch.float64))
    y0 = 10.0 + 20.0 * torch.rand((B, 2), generator=g, dtype=torch.float64)
    return params, y0


def lv_truth(params, y0, t1=LV_T_SPAN[1], h=1e-3):
    """Terminal values of the Lotka--Volterra instances by the classical
    fourth-order Runge--Kutta method on a fixed grid of step h, vectorised
    over the instances (numpy float64; error ~1e-12 relative at h = 1e-3 on
    this distribution).  The accuracy yardstick for the solver's terminal
    values, not a solver under test."""
    p = np.asarray(params, dtype=np.float64)
    u = np.array(y0, dtype=np.float64)
    a, b, c, d = p[:, 0], p[:, 1], p[:, 2], p[:, 3]

    def f(x):
        y01 = x[:, 0] * x[:, 1]
        return np.stack([a * x[:, 0] - b * y01, d * y01 - c * x[:, 1]], axis=1)

    steps = int(round(t1 / h))
    for _ in range(steps):
        k1 = f(u)
        k2 = f(u + 0.5 * h * k1)
        k3 = f(u + 0.5 * h * k2)
        k4 = f(u + h * k3)
        u = u + (h / 6.0) * (k1 + 2.0 * k2 + 2.0 * k3 + k4)
    return u


def vdp_dense(B=4096, mu_max=1000.0, num_save=100, seed=0):
    """(mu (B,), save_at (B, num_save), y0 (B, 2)) of the stiff van der Pol batch."""
    import torch

    g = torch.Generator().manual_seed(seed)
    mu = torch.exp(torch.rand(B, generator=g, dtype=torch.float64) * math.log(mu_max))
    save_at = (torch.linspace(0.0, 1.0, num_save, dtype=torch.float64)[None, :] * 2.0 * mu[:, None]).contiguous()
    y0 = torch.tensor([[2.0, 0.0]], dtype=torch.float64).expand(B, 2).contiguous()
    return mu, save_at, y0


def burgers_u0(B=64, d=4096):
    """(B, d) initial conditions of the Burgers batch (instance s from seed s), numpy float64."""
    rows = []
    x = np.arange(d) / d
    k = np.arange(1, 9)
    for s in range(B):
        g = np.random.default_rng(s)
        amp = g.normal(0.0, 1.0 / k)
        phase = g.uniform(0.0, 2 * np.pi, size=8)
        rows.append((amp[:, None] * np.sin(2 * np.pi * k[:, None] * x[None, :] + phase[:, None])).sum(axis=0))
    return np.stack(rows)


# FitzHugh--Nagumo LML problem
FHN_THETA_STAR = np.array([0.2, 0.2, 3.0])
FHN_U0 = np.array([-1.0, 1.0])
FHN_STD = 0.01


def _fhn(t, u, a, b, c):
    return [c * (u[0] - u[0] ** 3 / 3 + u[1]), -(u[0] - a - b * u[1]) / c]


def fhn_observations(t1=20.0, dt=0.01, save_every=10, seed=0):
    """(num_steps, data (num_obs, 2)): observations at t_k = k dt save_every,
    k = 0..num_obs-1 (t0 included, so len(data) = number of backward
    conditionals + 1 as evaluate_lml requires)."""
    import scipy.integrate

    num_steps = int(round(t1 / dt))
    num_obs = num_steps // save_every + 1
    t_obs = np.arange(num_obs) * dt * save_every
    sol = scipy.integrate.solve_ivp(_fhn, (0.0, t1), FHN_U0, t_eval=t_obs, args=tuple(FHN_THETA_STAR),
                                    method="DOP853", rtol=1e-12, atol=1e-12)
    rng = np.random.default_rng(seed)
    data = sol.y.T + FHN_STD * rng.standard_normal(sol.y.T.shape)
    return num_steps, data


def fhn_theta_samples(B, seed=0):
    rng = np.random.default_rng(seed)
    return FHN_THETA_STAR[None, :] + 0.05 * rng.standard_normal((B, 3))
