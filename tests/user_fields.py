"""CUDA C++ sources of vector fields registered at run time in the tests."""

LOTKA_VOLTERRA = """
struct Field {
  static constexpr int D = 2;
  static constexpr int P = 4;
  template <typename S, typename T>
  PDQ_HD static void eval(const S* u, const T* p, S* out) {
    S y01 = u[0] * u[1];
    out[0] = p[0] * u[0] - p[1] * y01;
    out[1] = p[3] * y01 - p[2] * u[1];
  }
};
"""

# Brusselator: u0' = a + u0^2 u1 - (b + 1) u0,  u1' = b u0 - u0^2 u1
BRUSSELATOR = """
struct Field {
  static constexpr int D = 2;
  static constexpr int P = 2;
  template <typename S, typename T>
  PDQ_HD static void eval(const S* u, const T* p, S* out) {
    const S u0sq_u1 = u[0] * u[0] * u[1];
    out[0] = u0sq_u1 - (p[1] + T(1)) * u[0] + p[0];
    out[1] = p[1] * u[0] - u0sq_u1;
  }
};
"""

# Lorenz-63 (three dimensions): sigma, rho, beta
LORENZ = """
struct Field {
  static constexpr int D = 3;
  static constexpr int P = 3;
  template <typename S, typename T>
  PDQ_HD static void eval(const S* u, const T* p, S* out) {
    out[0] = p[0] * (u[1] - u[0]);
    out[1] = u[0] * (p[1] - u[2]) - u[1];
    out[2] = u[0] * u[1] - p[2] * u[2];
  }
};
"""

BROKEN = """
struct Field {
  static constexpr int D = 2;
  static constexpr int P = 1;
  template <typename S, typename T>
  PDQ_HD static void eval(const S* u, const T* p, S* out) { out[0] = no_such_symbol; out[1] = u[0]; }
};
"""


def brusselator(u, p):
    """The same fields for the oracle (``oracle.problems.stack`` handles Taylor series too)."""
    from oracle.problems import stack

    a, b = p[0], p[1]
    u0sq_u1 = u[0] * u[0] * u[1]
    return stack([u0sq_u1 - (b + 1.0) * u[0] + a, b * u[0] - u0sq_u1])


def lorenz(u, p):
    from oracle.problems import stack

    s, r, b = p[0], p[1], p[2]
    return stack([s * (u[1] - u[0]), u[0] * (r - u[2]) - u[1], u[0] * u[1] - b * u[2]])


# FitzHugh--Nagumo, as the built-in field (the LML configuration's problem)
FITZHUGH_NAGUMO = """
struct Field {
  static constexpr int D = 2;
  static constexpr int P = 3;
  template <typename S, typename T>
  PDQ_HD static void eval(const S* u, const T* p, S* out) {
    const T a = p[0], b = p[1], c = p[2];
    out[0] = c * (u[0] - u[0] * u[0] * u[0] * (T(1) / T(3)) + u[1]);
    out[1] = -(T(1) / c) * (u[0] - a - b * u[1]);
  }
};
"""


# Block-diagonal stencils (struct Stencil): the viscous Burgers stencil of the
# built-in field, and Allen--Cahn, u_t = eps^2 u_xx + u - u^3 (periodic
# central differences), with the oracle's definition below
BURGERS_STENCIL = """
struct Stencil {
  static constexpr int P = 1;
  template <typename S, typename T>
  PDQ_HD static S eval(const S& left, const S& mid, const S& right, const T* p, T inv_dx) {
    const S flux = (right * right - left * left) * (T(0.25) * inv_dx);
    const S lap = (right - T(2) * mid + left) * (inv_dx * inv_dx);
    return -flux + p[0] * lap;
  }
};
"""

ALLEN_CAHN_STENCIL = """
struct Stencil {
  static constexpr int P = 1;
  template <typename S, typename T>
  PDQ_HD static S eval(const S& left, const S& mid, const S& right, const T* p, T inv_dx) {
    const S lap = (right - T(2) * mid + left) * (inv_dx * inv_dx);
    return p[0] * lap + mid - mid * mid * mid;
  }
};
"""


def allen_cahn(u, p):
    from oracle.problems import Series, roll

    d = u.c.shape[-1] if isinstance(u, Series) else u.shape[-1]
    inv_dx = float(d)
    left, right = roll(u, 1), roll(u, -1)
    lap = (right - 2.0 * u + left) * (inv_dx * inv_dx)
    return lap * p[0] + u - u * u * u
