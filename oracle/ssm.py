"""State-space-model factorisations of the oracle (test infrastructure only).

Restates ``probdiffeq/_probdiffeq/ssm_impl_isotropic.py``,
``ssm_impl_blockdiag.py``, ``ssm_impl_dense.py`` and
``probdiffeq/util/cholesky_util.py``, ``_probdiffeq/utilities.py``.

Conventions of the reference are kept:
  * isotropic: mean (n, d), one Cholesky factor (n, n);
  * blockdiag: mean (d, n), Cholesky factors (d, n, n), output scale (d,);
  * dense: mean (n*d,) coefficient-major [u, u', ...], Cholesky (n*d, n*d).
Taylor "coefficients" are derivatives (u, u', u'', ...).
"""

import math

import torch

from . import linalg

# --------------------------------------------------------------------------
# Square-root utilities (util/cholesky_util.py, _probdiffeq/utilities.py)
# --------------------------------------------------------------------------


def revert_conditional(R_X_F, R_X, R_YX, solve_triu):
    """QR-based revert of a Gaussian conditional (util/cholesky_util.py:27-82)."""
    k = R_YX.shape[0]
    top = torch.cat([R_YX, torch.zeros((k, R_X.shape[1]), dtype=R_X.dtype)], dim=1)
    bottom = torch.cat([R_X_F, R_X], dim=1)
    R = linalg.qr_r(torch.cat([top, bottom], dim=0))
    d_out = R_YX.shape[1]
    R_Y = R[:d_out, :d_out]
    R12 = R[:d_out, d_out:]
    G = solve_triu(R_Y, R12).T
    R_XY = R[d_out:, d_out:]
    return R_Y, (R_XY, G)


def sum_of_sqrtm_factors(R_stack):
    """R with R^T R = sum R_i^T R_i (util/cholesky_util.py:89-95)."""
    return linalg.qr_r(torch.cat(R_stack, dim=0))


def cholesky_hilbert(n: int):
    """Cholesky factor of the n x n Hilbert matrix (util/cholesky_util.py:106-176).

    Kahan's recurrence for K = 0: column j of U from the downward recurrence,
    then column scaling by sqrt(2i+1) and the f-vector.
    """
    K = 0.0
    dr = torch.sqrt(torch.arange(K + 1, K + 2 * n, 2, dtype=torch.float64))
    f = torch.ones(n, dtype=torch.float64) * (1.0 + K)
    for idx in range(1, n):
        prev = f[idx - 1].item()
        f[idx] = (((prev / idx) * (K + 2.0 * idx)) / (K + idx)) * (K + 2.0 * idx + 1.0)
    f = 1.0 / f
    U = torch.eye(n, dtype=torch.float64)
    for j in range(1, n):
        g = U[:, j].clone()
        for kk in range(j):
            i = j - 1 - kk
            g[i] = (g[i + 1] / (j - i)) * (K + (i + 1) + (j + 1))
        U[:, j] = g
    U = U * (dr[:, None] * f[None, :])
    return torch.tril(U.T)


def system_matrices_1d_iwp(num_derivatives: int):
    """A = flip(Pascal), Q = lower sqrt of flip(Hilbert) (_probdiffeq/utilities.py:57-71)."""
    n = num_derivatives + 1
    # _pascal(x)[0][i, j] = binom(i, j); the reference's factorial is
    # exp(lgamma(n + 1)), which makes binom(i, j > i) = 0 (backend/np.py:8-9).
    pascal = torch.tensor(
        [[float(math.comb(i, j)) if j <= i else 0.0 for j in range(n)] for i in range(n)],
        dtype=torch.float64,
    )
    A = torch.flip(pascal, dims=(0, 1))
    Q = cholesky_hilbert(n)
    Q_flipped = torch.flip(Q, dims=(0,))
    Q = linalg.qr_r(Q_flipped.T).T
    scale = torch.sign(torch.diagonal(Q))
    scale = torch.where(scale == 0.0, torch.ones_like(scale), scale)
    Q = Q * scale[None, :]
    return A, Q


def preconditioner_taylor(num_derivatives: int):
    """p_i = dt^(nu-i)/(nu-i)!, p_inv_i = dt^-(nu-i) (nu-i)! (_probdiffeq/utilities.py:74-84)."""
    powers = torch.arange(num_derivatives, -1, -1, dtype=torch.float64)
    scales = torch.tensor([math.factorial(int(k)) for k in powers], dtype=torch.float64)

    def precon(dt):
        dt = torch.as_tensor(dt, dtype=torch.float64)
        p = torch.pow(dt, powers) / scales
        p_inv = torch.pow(dt, -powers) * scales
        return p, p_inv

    return precon


# --------------------------------------------------------------------------
# Isotropic factorisation (ssm_impl_isotropic.py)
# --------------------------------------------------------------------------


class IsoNormal:
    """IsotropicNormal (ssm_impl_isotropic.py:146-292)."""

    kind = "isotropic"

    def __init__(self, mean, cholesky):
        self.mean = mean  # (n, d)
        self.cholesky = cholesky  # (n, n)

    @staticmethod
    def from_mean_and_std(mean, std):
        """ssm_impl_isotropic.py:161-178; std is one scalar per coefficient."""
        return IsoNormal(mean, torch.diag(std))

    def residual_whitened_rms(self, u=None):
        """ssm_impl_isotropic.py:203-207."""
        res = self.mean if u is None else self.mean - u
        res = linalg.solve_tril(self.cholesky, res)
        return linalg.vector_norm(res.reshape(-1)) / math.sqrt(self.mean.numel())

    def rescale_cholesky(self, factor):
        """ssm_impl_isotropic.py:209-211."""
        return IsoNormal(self.mean, factor * self.cholesky)

    def std(self):
        """Row norms of the Cholesky factor (ssm_impl_isotropic.py:193-197)."""
        return torch.sqrt(torch.sum(self.cholesky**2, dim=1))

    def logpdf(self, u):
        """ssm_impl_isotropic.py:217-236: sum over the d columns."""
        total = 0.0
        chol = linalg.qr_r(self.cholesky.T).T
        diag = torch.diagonal(chol)
        slogdet = torch.sum(torch.log(torch.abs(diag)))
        for j in range(self.mean.shape[1]):
            dx = u[:, j] - self.mean[:, j]
            w = linalg.solve_triu(chol.T, dx, trans="T")
            maha = torch.dot(w, w)
            total = total - 0.5 * (2.0 * slogdet + maha + dx.numel() * math.log(2 * math.pi))
        return total

    def to_multivariate_normal(self):
        """ssm_impl_isotropic.py:238-249."""
        n, d = self.mean.shape
        cov = self.cholesky @ self.cholesky.T
        full = torch.einsum("nm,dt->ndmt", cov, torch.eye(d, dtype=cov.dtype)).reshape(n * d, n * d)
        return self.mean.reshape(-1), full

    def identity_conditional(self):
        """ssm_impl_isotropic.py:260-266."""
        n, d = self.mean.shape
        noise = IsoNormal(torch.zeros((n, d), dtype=self.mean.dtype), torch.zeros((n, n), dtype=self.mean.dtype))
        return IsoCond.from_linop_and_noise(torch.eye(n, dtype=self.mean.dtype), noise)

    def prototype_output_scale(self):
        return torch.ones((), dtype=self.mean.dtype)

    def to_derivative(self, i, std):
        """ssm_impl_isotropic.py:271-278: observe coefficient i with noise std."""
        n, d = self.mean.shape
        linop = torch.zeros((1, n), dtype=self.mean.dtype)
        linop[0, i] = 1.0
        noise = IsoNormal(torch.zeros((1, d), dtype=self.mean.dtype), torch.reshape(std, (1, 1)))
        return IsoCond.from_linop_and_noise(linop, noise)

    def select(self, i):
        return IsoNormal(self.mean[i], self.cholesky[i])


class IsoCond:
    """IsotropicLatentCond (ssm_impl_isotropic.py:72-140)."""

    def __init__(self, A, noise, to_latent, to_observed):
        self.A, self.noise, self.to_latent, self.to_observed = A, noise, to_latent, to_observed

    @staticmethod
    def from_linop_and_noise(A, noise):
        """ssm_impl_api.py:66-76."""
        d_out, d_in = A.shape
        return IsoCond(A, noise, torch.ones(d_in, dtype=A.dtype), torch.ones(d_out, dtype=A.dtype))

    def apply_flat(self, x):
        """ssm_impl_isotropic.py:75-79."""
        x = self.to_latent[:, None] * x
        mean = (self.to_observed[:, None] * self.A) @ x + self.noise.mean
        chol = torch.abs(self.to_observed[:, None]) * self.noise.cholesky
        return IsoNormal(mean, chol)

    def marginalise(self, rv):
        """ssm_impl_isotropic.py:81-89."""
        mean = self.to_latent[:, None] * rv.mean
        chol = self.to_latent[:, None] * rv.cholesky
        R = sum_of_sqrtm_factors(((self.A @ chol).T, self.noise.cholesky.T))
        chol_new = R.T
        mean_new = self.to_observed[:, None] * (self.A @ mean + self.noise.mean)
        chol_new = torch.abs(self.to_observed[:, None]) * chol_new
        return IsoNormal(mean_new, chol_new)

    def merge(self, other):
        """ssm_impl_isotropic.py:91-105 (self outer, other inner)."""
        T = self.to_latent * other.to_observed
        g = self.A @ (T[:, None] * other.A)
        xi = self.A @ (T[:, None] * other.noise.mean) + self.noise.mean
        R1 = (self.A @ (torch.abs(T[:, None]) * other.noise.cholesky)).T
        R2 = self.noise.cholesky.T
        Xi = sum_of_sqrtm_factors((R1, R2))
        return IsoCond(g, IsoNormal(xi, Xi.T), other.to_latent, self.to_observed)

    def revert(self, rv, solve_triu=linalg.solve_triu):
        """ssm_impl_isotropic.py:107-133."""
        mean = self.to_latent[:, None] * rv.mean
        chol = torch.abs(self.to_latent[:, None]) * rv.cholesky
        r_obs, (r_cor, gain) = revert_conditional(
            (self.A @ chol).T, chol.T, self.noise.cholesky.T, solve_triu
        )
        mean_observed = self.A @ mean + self.noise.mean
        mean_corrected = mean - gain @ mean_observed
        corrected = IsoNormal(mean_corrected, r_cor.T)
        cond_new = IsoCond(gain, corrected, 1.0 / self.to_observed, 1.0 / self.to_latent)
        observed = IsoNormal(
            self.to_observed[:, None] * mean_observed,
            torch.abs(self.to_observed[:, None]) * r_obs.T,
        )
        return observed, cond_new

    def preconditioner_apply(self):
        """ssm_impl_isotropic.py:135-140."""
        A = self.to_observed[:, None] * self.A * self.to_latent[None, :]
        mean = self.to_observed[:, None] * self.noise.mean
        chol = torch.abs(self.to_observed[:, None]) * self.noise.cholesky
        return IsoCond.from_linop_and_noise(A, IsoNormal(mean, chol))

    def rescale_noise(self, factor):
        return IsoCond(self.A, self.noise.rescale_cholesky(factor), self.to_latent, self.to_observed)


class IsoPrior:
    """IsotropicWienerIntegrated (ssm_impl_isotropic.py:358-378)."""

    def __init__(self, init, output_scale, A, q_sqrtm, precon):
        self.init, self.output_scale = init, output_scale
        self.A, self.q_sqrtm, self.precon = A, q_sqrtm, precon

    def transition(self, dt, output_scale=1.0):
        output_scale = torch.as_tensor(output_scale, dtype=self.A.dtype)
        if output_scale.shape != ():
            raise ValueError(f"The base-scale has the wrong shape. Expected: (). Received: {tuple(output_scale.shape)}.")
        dt = torch.as_tensor(dt, dtype=self.A.dtype)
        scale = torch.sqrt(torch.abs(dt)) * self.output_scale * output_scale
        n, d = self.init.mean.shape
        noise = IsoNormal(torch.zeros((n, d), dtype=self.A.dtype), scale * self.q_sqrtm)
        p, p_inv = self.precon(dt)
        return IsoCond(self.A, noise, p_inv.to(self.A.dtype), p.to(self.A.dtype))


class IsoTs0:
    """IsotropicOdeTs0 (ssm_impl_isotropic.py:298-317), first-order ODE."""

    residual_order = 2  # ssm_impl_api.py:176: num_tcoeffs_in_args + 1

    def __init__(self, vf, output_index=1, num_in=1):
        self.vf, self.output_index, self.num_in = vf, output_index, num_in

    def linearize(self, rv, damp, t):
        fx = -self.vf(rv.mean[: self.num_in], t)  # (d,)
        n = rv.mean.shape[0]
        bias = IsoNormal(fx[None, :], torch.full((1, 1), float(damp), dtype=rv.mean.dtype))
        linop = torch.zeros((1, n), dtype=rv.mean.dtype)
        linop[0, self.output_index] = 1.0
        return IsoCond.from_linop_and_noise(linop, bias)


class IsoTs1:
    """IsotropicResidual (ssm_impl_isotropic.py:320-355) for the ODE residual u' - f(u).

    The residual comes from ``problems.residual_from_ode`` (problems.py:518-532);
    the Jacobian of the flat residual (1, d) w.r.t. the mean (n, d) is
    materialised and traced along d (jacobians.py:100-106), then divided by d,
    so every dimension shares the (1, n) linear operator; the bias is
    r(m) - J m.
    """

    residual_order = 2  # num_tcoeffs_in_args of the residual = 1 + 1 (ssm_impl_api.py:163-165)

    def __init__(self, vf, output_index=1, num_in=1):
        self.vf, self.output_index, self.num_in = vf, output_index, num_in

    def residual(self, x, t):
        return (x[self.output_index] - self.vf(x[: self.num_in], t))[None, :]  # (1, d)

    def linearize(self, rv, damp, t):
        mean = rv.mean
        n, d = mean.shape
        fx = self.residual(mean, t)
        jac = torch.func.jacfwd(lambda x: self.residual(x, t))(mean)  # (1, d, n, d)
        trace = torch.diagonal(jac, dim1=1, dim2=3).sum(-1) / d       # (1, n)
        bias = IsoNormal(fx - trace @ mean, torch.full((1, 1), float(damp), dtype=mean.dtype))
        return IsoCond.from_linop_and_noise(trace, bias)


class IsoSSM:
    """state_space_model_isotropic (ssm_impl_isotropic.py:406-482)."""

    def prior_wiener_integrated(self, tcoeffs, std=None, output_scale=None):
        """tcoeffs: (n, d) derivatives; exact coefficients have std 0 (:519-554)."""
        n = tcoeffs.shape[0]
        if std is None:
            std = torch.zeros(n, dtype=tcoeffs.dtype)
        init = IsoNormal.from_mean_and_std(tcoeffs, std)
        if output_scale is None:
            output_scale = torch.ones((), dtype=tcoeffs.dtype)
        A, Q = system_matrices_1d_iwp(n - 1)
        return IsoPrior(init, torch.as_tensor(output_scale, dtype=tcoeffs.dtype), A.to(tcoeffs.dtype), Q.to(tcoeffs.dtype), preconditioner_taylor(n - 1))

    def constraint_ode_ts0(self, vf):
        return IsoTs0(vf)

    def constraint_ode_ts1(self, vf):
        return IsoTs1(vf)


# --------------------------------------------------------------------------
# Block-diagonal factorisation (ssm_impl_blockdiag.py)
# --------------------------------------------------------------------------


class BdNormal:
    """BlockDiagNormal (ssm_impl_blockdiag.py:215-391); mean (d, n), chol (d, n, n)."""

    kind = "blockdiag"

    def __init__(self, mean, cholesky):
        self.mean, self.cholesky = mean, cholesky

    def residual_whitened_rms(self, u=None):
        """ssm_impl_blockdiag.py:285-292: one value per dimension."""
        res = self.mean if u is None else self.mean - u
        w = linalg.solve_tril(self.cholesky, res)  # (d, k)
        return torch.sqrt(torch.sum(w * w, dim=-1)) / math.sqrt(self.mean.shape[-1])

    def rescale_cholesky(self, factor):
        return BdNormal(self.mean, factor[..., None, None] * self.cholesky)

    def std(self):
        """(d, n) row norms (ssm_impl_blockdiag.py:269-274)."""
        return torch.sqrt(torch.sum(self.cholesky**2, dim=-1))

    def logpdf(self, u):
        """ssm_impl_blockdiag.py:302-316: sum over dimensions."""
        total = 0.0
        for j in range(self.mean.shape[0]):
            chol = linalg.qr_r(self.cholesky[j].T).T
            dx = u[j] - self.mean[j]
            w = linalg.solve_triu(chol.T, dx, trans="T")
            slogdet = torch.sum(torch.log(torch.abs(torch.diagonal(chol))))
            total = total - 0.5 * (2.0 * slogdet + torch.dot(w, w) + dx.numel() * math.log(2 * math.pi))
        return total

    def to_multivariate_normal(self):
        d, n = self.mean.shape
        cov = self.cholesky @ self.cholesky.transpose(-1, -2)
        full = torch.einsum("dnm,dt->ndmt", cov, torch.eye(d, dtype=cov.dtype)).reshape(n * d, n * d)
        return self.mean.T.reshape(-1), full

    def identity_conditional(self):
        d, n = self.mean.shape
        z = torch.zeros
        noise = BdNormal(z((d, n), dtype=self.mean.dtype), z((d, n, n), dtype=self.mean.dtype))
        A = torch.eye(n, dtype=self.mean.dtype).expand(d, n, n).clone()
        return BdCond.from_linop_and_noise(A, noise)

    def prototype_output_scale(self):
        return torch.ones(self.mean.shape[0], dtype=self.mean.dtype)

    def to_derivative(self, i, std):
        """ssm_impl_blockdiag.py:367-377: observe coefficient i of every
        dimension with noise std (d,); linop (d, 1, n) selects it."""
        d, n = self.mean.shape
        linop = torch.zeros((d, 1, n), dtype=self.mean.dtype)
        linop[:, 0, i] = 1.0
        std = torch.as_tensor(std, dtype=self.mean.dtype).reshape(d)
        noise = BdNormal(torch.zeros((d, 1), dtype=self.mean.dtype), std.reshape(d, 1, 1).clone())
        return BdCond.from_linop_and_noise(linop, noise)

    def select(self, i):
        return BdNormal(self.mean[i], self.cholesky[i])


class BdCond:
    """BlockDiagLatentCond (ssm_impl_blockdiag.py:16-113)."""

    def __init__(self, A, noise, to_latent, to_observed):
        self.A, self.noise, self.to_latent, self.to_observed = A, noise, to_latent, to_observed

    @staticmethod
    def from_linop_and_noise(A, noise):
        d, d_out, d_in = A.shape
        return BdCond(A, noise, torch.ones((d, d_in), dtype=A.dtype), torch.ones((d, d_out), dtype=A.dtype))

    def apply_flat(self, x):
        """ssm_impl_blockdiag.py:19-26."""
        s = self.to_latent * x
        m_new = self.to_observed * (torch.einsum("dij,dj->di", self.A, s) + self.noise.mean)
        c_new = torch.abs(self.to_observed[:, :, None]) * self.noise.cholesky
        return BdNormal(m_new, c_new)

    def marginalise(self, rv):
        """ssm_impl_blockdiag.py:28-43."""
        mean = self.to_latent * rv.mean
        chol = torch.abs(self.to_latent[:, :, None]) * rv.cholesky
        mean_marg = torch.einsum("ijk,ik->ij", self.A, mean) + self.noise.mean
        chol1 = (self.A @ chol).transpose(-1, -2)
        chol2 = self.noise.cholesky.transpose(-1, -2)
        R = torch.stack([sum_of_sqrtm_factors((chol1[j], chol2[j])) for j in range(chol1.shape[0])])
        mean_new = self.to_observed * mean_marg
        chol_new = torch.abs(self.to_observed[:, :, None]) * R.transpose(-1, -2)
        return BdNormal(mean_new, chol_new)

    def merge(self, other):
        """ssm_impl_blockdiag.py:45-67."""
        T = self.to_latent * other.to_observed
        A1, A2 = self.A, T[:, :, None] * other.A
        g = A1 @ A2
        xi = torch.einsum("dij,dj->di", A1, T * other.noise.mean) + self.noise.mean
        C1, C2 = self.noise.cholesky, torch.abs(T[:, :, None]) * other.noise.cholesky
        R1 = (A1 @ C2).transpose(-1, -2)
        R2 = C1.transpose(-1, -2)
        Xi = torch.stack([sum_of_sqrtm_factors((R1[j], R2[j])) for j in range(R1.shape[0])])
        return BdCond(g, BdNormal(xi, Xi.transpose(-1, -2)), other.to_latent, self.to_observed)

    def revert(self, rv, solve_triu=linalg.solve_triu):
        """ssm_impl_blockdiag.py:69-102."""
        mean = self.to_latent * rv.mean
        chol = torch.abs(self.to_latent[:, :, None]) * rv.cholesky
        outs = [
            revert_conditional(
                (self.A[j] @ chol[j]).T, chol[j].T, self.noise.cholesky[j].T, solve_triu
            )
            for j in range(chol.shape[0])
        ]
        r_obs = torch.stack([o[0] for o in outs])
        r_cor = torch.stack([o[1][0] for o in outs])
        gain = torch.stack([o[1][1] for o in outs])
        mean_observed = torch.einsum("dij,dj->di", self.A, mean) + self.noise.mean
        mean_corrected = mean - torch.einsum("dij,dj->di", gain, mean_observed)
        corrected = BdNormal(mean_corrected, r_cor.transpose(-1, -2))
        bwd = BdCond(gain, corrected, 1.0 / self.to_observed, 1.0 / self.to_latent)
        observed = BdNormal(
            self.to_observed * mean_observed,
            torch.abs(self.to_observed[:, :, None]) * r_obs.transpose(-1, -2),
        )
        return observed, bwd

    def preconditioner_apply(self):
        """ssm_impl_blockdiag.py:104-113."""
        A = self.to_observed[:, :, None] * self.A * self.to_latent[:, None, :]
        mean = self.to_observed * self.noise.mean
        chol = torch.abs(self.to_observed[:, :, None]) * self.noise.cholesky
        return BdCond(A, BdNormal(mean, chol), torch.ones_like(self.to_latent), torch.ones_like(self.to_observed))

    def rescale_noise(self, factor):
        return BdCond(self.A, self.noise.rescale_cholesky(factor), self.to_latent, self.to_observed)


class BdPrior:
    """BlockDiagWienerIntegrated (ssm_impl_blockdiag.py:397-432)."""

    def __init__(self, init, output_scale, a, q_sqrtm, precon):
        self.init, self.output_scale = init, output_scale
        self.a, self.q_sqrtm, self.precon = a, q_sqrtm, precon

    def transition(self, dt, output_scale):
        dt = torch.as_tensor(dt, dtype=self.a.dtype)
        p, p_inv = self.precon(dt)
        output_scale = torch.as_tensor(output_scale, dtype=self.a.dtype)
        if output_scale.shape != self.output_scale.shape:
            raise ValueError("The output-scale has the wrong shape.")
        s = self.output_scale * output_scale
        d = s.shape[0]
        n = self.a.shape[0]
        mean = torch.zeros((d, n), dtype=self.a.dtype)
        chol = torch.sqrt(torch.abs(dt)) * s[:, None, None] * self.q_sqrtm[None]
        A = self.a.expand(d, n, n).clone()
        return BdCond(A, BdNormal(mean, chol), p_inv.to(self.a.dtype).expand(d, n).clone(), p.to(self.a.dtype).expand(d, n).clone())


class BdTs0:
    """BlockDiagOdeTs0 (ssm_impl_blockdiag.py:123-144)."""

    residual_order = 2

    def __init__(self, vf, output_index=1, num_in=1):
        self.vf, self.output_index, self.num_in = vf, output_index, num_in

    def linearize(self, rv, damp, t):
        u = rv.mean[:, : self.num_in].T  # (num_in, d)
        fx = -self.vf(u, t)  # (d,)
        d, n = rv.mean.shape
        bias = BdNormal(fx[:, None], float(damp) * torch.ones((d, 1, 1), dtype=rv.mean.dtype))
        linop = torch.zeros((d, 1, n), dtype=rv.mean.dtype)
        linop[:, 0, self.output_index] = 1.0
        return BdCond.from_linop_and_noise(linop, bias)


class BdTs1:
    """BlockDiagResidual (ssm_impl_blockdiag.py:147-183) for the ODE residual u' - f(u).

    The Jacobian of the residual (1, d) w.r.t. the coefficients (n, d) is
    materialised and its diagonal along d taken (jacobians.py:108-113): the
    (d, 1, n) per-dimension operators J_j = d r_j / d x[:, j]; the bias is
    r(m) - J m per dimension.
    """

    residual_order = 2

    def __init__(self, vf, output_index=1, num_in=1):
        self.vf, self.output_index, self.num_in = vf, output_index, num_in

    def residual(self, x, t):  # x (n, d) -> (1, d)
        return (x[self.output_index] - self.vf(x[: self.num_in], t))[None, :]

    def linearize(self, rv, damp, t):
        x = rv.mean.T  # (n, d)
        d, n = rv.mean.shape
        fx = self.residual(x, t).T  # (d, 1)
        jac = torch.func.jacfwd(lambda z: self.residual(z, t))(x)  # (1, d, n, d)
        diag = torch.diagonal(jac, dim1=1, dim2=3).permute(2, 0, 1)  # (d, 1, n)
        fx = fx - torch.einsum("din,dn->di", diag, rv.mean)
        bias = BdNormal(fx, float(damp) * torch.ones((d, 1, 1), dtype=rv.mean.dtype))
        return BdCond.from_linop_and_noise(diag, bias)


class BdSSM:
    """state_space_model_blockdiag (ssm_impl_blockdiag.py:460-547)."""

    def prior_wiener_integrated(self, tcoeffs, std=None, output_scale=None):
        """tcoeffs (n, d) derivatives; stored as mean (d, n)."""
        n, d = tcoeffs.shape
        if std is None:
            std = torch.zeros((n, d), dtype=tcoeffs.dtype)
        chol = std.T[:, :, None] * torch.eye(n, dtype=tcoeffs.dtype)[None]
        init = BdNormal(tcoeffs.T.clone(), chol)
        if output_scale is None:
            output_scale = torch.ones(d, dtype=tcoeffs.dtype)
        a, q = system_matrices_1d_iwp(n - 1)
        return BdPrior(init, output_scale, a.to(tcoeffs.dtype), q.to(tcoeffs.dtype), preconditioner_taylor(n - 1))

    def constraint_ode_ts0(self, vf):
        return BdTs0(vf)

    def constraint_ode_ts1(self, vf):
        return BdTs1(vf)


# --------------------------------------------------------------------------
# Dense factorisation (ssm_impl_dense.py)
# --------------------------------------------------------------------------


class DenseNormal:
    """DenseNormal (ssm_impl_dense.py:108-231); mean (N,), chol (N, N)."""

    kind = "dense"

    def __init__(self, mean, cholesky, d):
        self.mean, self.cholesky, self.d = mean, cholesky, d

    def residual_whitened_rms(self, u=None):
        """ssm_impl_dense.py:156-160."""
        dx = -self.mean if u is None else u - self.mean
        w = linalg.solve_tril(self.cholesky, dx)
        return linalg.vector_norm(w) / math.sqrt(self.mean.numel())

    def rescale_cholesky(self, factor):
        return DenseNormal(self.mean, factor * self.cholesky, self.d)

    def std(self):
        """|qr_r(row)| = row norms (ssm_impl_dense.py:144-150), shape (N,)."""
        return torch.sqrt(torch.sum(self.cholesky**2, dim=1))

    def logpdf(self, u):
        """ssm_impl_dense.py:170-180."""
        chol = linalg.qr_r(self.cholesky.T).T
        slogdet = torch.sum(torch.log(torch.abs(torch.diagonal(chol))))
        dx = u - self.mean
        w = linalg.solve_tril(chol, dx)
        return -0.5 * torch.dot(w, w) - dx.numel() / 2 * math.log(2 * math.pi) - slogdet

    def to_multivariate_normal(self):
        return self.mean, self.cholesky @ self.cholesky.T

    def identity_conditional(self):
        N = self.mean.shape[0]
        noise = DenseNormal(torch.zeros(N, dtype=self.mean.dtype), torch.zeros((N, N), dtype=self.mean.dtype), self.d)
        return DenseCond.from_linop_and_noise(torch.eye(N, dtype=self.mean.dtype), noise)

    def prototype_output_scale(self):
        return torch.ones((), dtype=self.mean.dtype)

    def to_derivative(self, i, std):
        """ssm_impl_dense.py:206-217; std (d,)."""
        N, d = self.mean.shape[0], self.d
        linop = torch.zeros((d, N), dtype=self.mean.dtype)
        linop[:, i * d : (i + 1) * d] = torch.eye(d, dtype=self.mean.dtype)
        noise = DenseNormal(torch.zeros(d, dtype=self.mean.dtype), torch.diag(std), d)
        return DenseCond.from_linop_and_noise(linop, noise)

    def select(self, i):
        return DenseNormal(self.mean[i], self.cholesky[i], self.d)

    def coefficients(self):
        """Mean as (n, d) derivatives."""
        return self.mean.reshape(-1, self.d)


class DenseCond:
    """DenseLatentCond (ssm_impl_dense.py:15-84)."""

    def __init__(self, A, noise, to_latent, to_observed):
        self.A, self.noise, self.to_latent, self.to_observed = A, noise, to_latent, to_observed

    @staticmethod
    def from_linop_and_noise(A, noise):
        d_out, d_in = A.shape
        return DenseCond(A, noise, torch.ones(d_in, dtype=A.dtype), torch.ones(d_out, dtype=A.dtype))

    def apply_flat(self, x):
        """ssm_impl_dense.py:18-22."""
        x = self.to_latent * x
        mean = self.to_observed * (self.A @ x + self.noise.mean)
        chol = torch.abs(self.to_observed[:, None]) * self.noise.cholesky
        return DenseNormal(mean, chol, self.noise.d)

    def marginalise(self, rv):
        """ssm_impl_dense.py:24-33."""
        mean = self.to_latent * rv.mean
        chol = self.to_latent[:, None] * rv.cholesky
        R = sum_of_sqrtm_factors(((self.A @ chol).T, self.noise.cholesky.T))
        mean_new = self.to_observed * (self.A @ mean + self.noise.mean)
        chol_new = torch.abs(self.to_observed[:, None]) * R.T
        return DenseNormal(mean_new, chol_new, self.noise.d)

    def merge(self, other):
        """ssm_impl_dense.py:35-49."""
        T = self.to_latent * other.to_observed
        g = self.A @ (T[:, None] * other.A)
        xi = self.A @ (T * other.noise.mean) + self.noise.mean
        R1 = (self.A @ (torch.abs(T[:, None]) * other.noise.cholesky)).T
        R2 = self.noise.cholesky.T
        Xi = sum_of_sqrtm_factors((R1, R2))
        return DenseCond(g, DenseNormal(xi, Xi.T, self.noise.d), other.to_latent, self.to_observed)

    def revert(self, rv, solve_triu=linalg.solve_triu):
        """ssm_impl_dense.py:51-77."""
        mean = self.to_latent * rv.mean
        chol = torch.abs(self.to_latent[:, None]) * rv.cholesky
        r_obs, (r_cor, gain) = revert_conditional((self.A @ chol).T, chol.T, self.noise.cholesky.T, solve_triu)
        mean_observed = self.A @ mean + self.noise.mean
        mean_corrected = mean - gain @ mean_observed
        corrected = DenseNormal(mean_corrected, r_cor.T, rv.d)
        cond_new = DenseCond(gain, corrected, 1.0 / self.to_observed, 1.0 / self.to_latent)
        observed = DenseNormal(self.to_observed * mean_observed, torch.abs(self.to_observed[:, None]) * r_obs.T, self.noise.d)
        return observed, cond_new

    def preconditioner_apply(self):
        """ssm_impl_dense.py:79-84."""
        A = self.to_observed[:, None] * self.A * self.to_latent[None, :]
        mean = self.to_observed * self.noise.mean
        chol = torch.abs(self.to_observed[:, None]) * self.noise.cholesky
        return DenseCond.from_linop_and_noise(A, DenseNormal(mean, chol, self.noise.d))

    def rescale_noise(self, factor):
        return DenseCond(self.A, self.noise.rescale_cholesky(factor), self.to_latent, self.to_observed)


class DensePrior:
    """DenseWienerIntegrated (ssm_impl_dense.py:337-363)."""

    def __init__(self, init, d, A, Q, precon):
        self.init, self.d, self.A, self.Q, self.precon = init, d, A, Q, precon
        self.output_scale = torch.ones((), dtype=A.dtype)

    def transition(self, dt, output_scale=1.0):
        output_scale = torch.as_tensor(output_scale, dtype=self.A.dtype)
        if output_scale.shape != ():
            raise ValueError("The output-scale has the wrong shape.")
        dt = torch.as_tensor(dt, dtype=self.A.dtype)
        p, p_inv = self.precon(dt)
        p = torch.repeat_interleave(p.to(self.A.dtype), self.d)
        p_inv = torch.repeat_interleave(p_inv.to(self.A.dtype), self.d)
        N = self.A.shape[0]
        noise = DenseNormal(torch.zeros(N, dtype=self.A.dtype), torch.sqrt(torch.abs(dt)) * output_scale * self.Q, self.d)
        return DenseCond(self.A, noise, p_inv, p)


class DenseTs0:
    """DenseOdeTs0 (ssm_impl_dense.py:237-259)."""

    residual_order = 2

    def __init__(self, vf, d, output_index=1, num_in=1):
        self.vf, self.d, self.output_index, self.num_in = vf, d, output_index, num_in

    def linearize(self, rv, damp, t):
        coeffs = rv.mean.reshape(-1, self.d)
        fx = -self.vf(coeffs[: self.num_in], t)
        N = rv.mean.shape[0]
        linop = torch.zeros((self.d, N), dtype=rv.mean.dtype)
        k = self.output_index
        linop[:, k * self.d : (k + 1) * self.d] = torch.eye(self.d, dtype=rv.mean.dtype)
        noise = DenseNormal(fx, float(damp) * torch.eye(self.d, dtype=rv.mean.dtype), self.d)
        return DenseCond.from_linop_and_noise(linop, noise)


class DenseTs1:
    """DenseResidual (ssm_impl_dense.py:262-334) for the ODE residual u' - f(u).

    Residual from ``problems.residual_from_ode`` (problems.py:518-532), the
    linearisation point from ``taylor_point_prior`` (taylor_points.py:150-156),
    the Jacobian materialised (jacobians.py:93-98); ``jac`` returns df/du.
    """

    residual_order = 2  # num_tcoeffs_in_args of the residual = 1 + 1

    def __init__(self, vf, jac, d):
        self.vf, self.jac, self.d = vf, jac, d

    def linearize(self, rv, damp, t):
        d = self.d
        xi = rv.mean
        coeffs = xi.reshape(-1, d)
        N = xi.shape[0]
        r = coeffs[1] - self.vf(coeffs[:1], t)
        J = torch.zeros((d, N), dtype=xi.dtype)
        J[:, :d] = -self.jac(coeffs[0], t)
        J[:, d : 2 * d] = torch.eye(d, dtype=xi.dtype)
        fx = r - J @ xi
        noise = DenseNormal(fx, float(damp) * torch.eye(d, dtype=xi.dtype), d)
        return DenseCond.from_linop_and_noise(J, noise)


class DenseSSM:
    """state_space_model_dense (ssm_impl_dense.py:455-514)."""

    def prior_wiener_integrated(self, tcoeffs, std=None):
        n, d = tcoeffs.shape
        if std is None:
            std = torch.zeros((n, d), dtype=tcoeffs.dtype)
        init = DenseNormal(tcoeffs.reshape(-1).clone(), torch.diag(std.reshape(-1)), d)
        a, q = system_matrices_1d_iwp(n - 1)
        eye = torch.eye(d, dtype=torch.float64)
        A = torch.kron(a, eye).to(tcoeffs.dtype)
        Q = torch.kron(q, eye).to(tcoeffs.dtype)
        return DensePrior(init, d, A, Q, preconditioner_taylor(n - 1))

    def constraint_ode_ts0(self, vf, d):
        return DenseTs0(vf, d)

    def constraint_ode_ts1(self, vf, jac, d):
        return DenseTs1(vf, jac, d)
