"""Vector fields and Taylor-mode initialisation of the oracle (test infrastructure only).

Vector fields (each written once, generic over plain tensors and truncated
Taylor series so the same code yields f, its Jacobian and the Taylor-mode
initial derivatives):

  * Lotka--Volterra, as ``probdiffeq/backend/ode.py:45-49`` with the four
    parameters made explicit,
  * first-order van der Pol u' = (u1, mu((1 - u0^2) u1 - u0)),
  * FitzHugh--Nagumo, as ``benchmarks/C0_taylor-init-fitzhughnagumo.py:122-129``
    with (a, b, c) made explicit,
  * viscous Burgers with the central-difference flux stencil of
    ``benchmarks/A5_work-precision-burgers-pde.py:124-134`` on a periodic grid.

Taylor-mode initialisation restates ``jetexpand_ode_padded_scan``
(``_probdiffeq/jet_expansion_algorithms.py:49-103``): the derivatives
u(t0), u'(t0), ..., u^(num)(t0) of the ODE solution, computed here by
truncated power-series arithmetic (the published Taylor-mode recurrence:
with u(t) = sum_k a_k (t - t0)^k, (k + 1) a_{k+1} = [f(u)]_k), and returned as
derivatives u^(k) = k! a_k, like the reference (jet with factorial scaling,
``backend/func.py:21-25``).
"""

import math

import torch


class Series:
    """Truncated Taylor series with normalised coefficients, shape (K+1, *state)."""

    def __init__(self, c):
        self.c = c

    @staticmethod
    def _lift(x, like):
        if isinstance(x, Series):
            return x.c
        z = torch.zeros_like(like.c)
        z[0] = x
        return z

    def __add__(self, o):
        return Series(self.c + Series._lift(o, self))

    __radd__ = __add__

    def __sub__(self, o):
        return Series(self.c - Series._lift(o, self))

    def __rsub__(self, o):
        return Series(Series._lift(o, self) - self.c)

    def __neg__(self):
        return Series(-self.c)

    def __mul__(self, o):
        if not isinstance(o, Series):
            return Series(self.c * o)
        a, b = self.c, o.c
        K = a.shape[0]
        out = torch.zeros(torch.broadcast_shapes(a.shape, b.shape), dtype=a.dtype)
        for k in range(K):
            acc = 0.0
            for j in range(k + 1):
                acc = acc + a[j] * b[k - j]
            out[k] = acc
        return Series(out)

    __rmul__ = __mul__

    def __truediv__(self, o):
        if isinstance(o, Series):
            raise NotImplementedError("series division is not needed by the registered fields")
        return Series(self.c / o)

    def __pow__(self, k: int):
        out = self
        for _ in range(k - 1):
            out = out * self
        return out

    def __getitem__(self, idx):
        return Series(self.c[(slice(None), idx)])

    def roll(self, shift):
        return Series(torch.roll(self.c, shifts=shift, dims=-1))


def stack(xs):
    if isinstance(xs[0], Series) or any(isinstance(x, Series) for x in xs):
        like = next(x for x in xs if isinstance(x, Series))
        return Series(torch.stack([Series._lift(x, like) if not isinstance(x, Series) else x.c for x in xs], dim=-1))
    return torch.stack(list(xs), dim=-1)


def roll(x, shift):
    if isinstance(x, Series):
        return x.roll(shift)
    return torch.roll(x, shifts=shift, dims=-1)


# --------------------------------------------------------------------------
# Vector fields f(u, params) (autonomous)
# --------------------------------------------------------------------------


def lotka_volterra(u, p):
    """backend/ode.py:45-49 with params p = (a, b, c, d)."""
    a, b, c, d = p[0], p[1], p[2], p[3]
    y01 = u[0] * u[1]
    return stack([a * u[0] - b * y01, -c * u[1] + d * y01])


def van_der_pol(u, p):
    """First-order van der Pol, p = (mu,)."""
    mu = p[0]
    return stack([u[1] + 0.0 * u[0], mu * ((1.0 - u[0] * u[0]) * u[1] - u[0])])


def fitzhugh_nagumo(u, p):
    """benchmarks/C0_taylor-init-fitzhughnagumo.py:122-129, p = (a, b, c)."""
    a, b, c = p[0], p[1], p[2]
    du1 = c * (u[0] - u[0] * u[0] * u[0] / 3.0 + u[1])
    du2 = -(1.0 / c) * (u[0] - a - b * u[1])
    return stack([du1, du2])


def burgers(u, p):
    """Viscous Burgers, periodic central differences, p = (nu,); d = len(u).

    Flux-form stencil of benchmarks/A5_work-precision-burgers-pde.py:124-134
    with dx = 1/d and periodic neighbours (roll) instead of zero ghosts.
    """
    nu = p[0]
    d = u.c.shape[-1] if isinstance(u, Series) else u.shape[-1]
    dx = 1.0 / d
    left, right = roll(u, 1), roll(u, -1)
    flux_term = (right * right - left * left) / (4.0 * dx)
    lap = (right - 2.0 * u + left) / (dx * dx)
    return -flux_term + nu * lap


FIELDS = {
    "lotka_volterra": lotka_volterra,
    "van_der_pol": van_der_pol,
    "fitzhugh_nagumo": fitzhugh_nagumo,
    "burgers": burgers,
}


def jacobian(field, u, p):
    """Materialised df/du via forward-mode autodiff (jacobians.py:93-98)."""
    return torch.func.jacfwd(lambda x: field(x, p))(u)


def taylor_derivatives(field, u0, p, num):
    """Derivatives u, u', ..., u^(num) at t0 (jet_expansion_algorithms.py:49-103).

    Returns a tensor (num + 1, d).
    """
    u0 = torch.as_tensor(u0, dtype=torch.float64)
    K = num + 1
    a = torch.zeros((K,) + tuple(u0.shape), dtype=u0.dtype)
    a[0] = u0
    for k in range(num):
        s = Series(a.clone())
        fs = field(s, p)
        a[k + 1] = fs.c[k] / (k + 1)
    fact = torch.tensor([math.factorial(k) for k in range(K)], dtype=u0.dtype)
    return a * fact.reshape((K,) + (1,) * u0.ndim)
