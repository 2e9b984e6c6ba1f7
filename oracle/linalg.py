"""Linear algebra shim of the oracle (test infrastructure only).

Restates ``probdiffeq/backend/linalg.py``.

``qr_r`` follows ``backend/linalg.py:8-37``: the R factor of a reduced QR
decomposition, differentiated with the reference's custom rule
``R_dot = Q^T M_dot`` (Q treated as a constant).  ``qr_r_exact`` uses
PyTorch's own QR derivative (the true derivative of the triangular factor)
so that the two differentiation conventions can be compared.
"""

import torch

_MODE = {"qr": "reference"}


def set_qr_derivative(mode: str) -> None:
    """Select 'reference' (Q constant, backend/linalg.py:13-37) or 'exact'."""
    if mode not in ("reference", "exact"):
        raise ValueError(mode)
    _MODE["qr"] = mode


class _QrR(torch.autograd.Function):
    """R of a reduced QR with the reference's custom JVP (backend/linalg.py:13-37).

    Forward: R = qr(M, mode='reduced').R.  The JVP is R_dot = Q^T M_dot, so
    the VJP (its transpose) is M_bar = Q R_bar.
    """

    @staticmethod
    def forward(ctx, m):
        q, r = torch.linalg.qr(m, mode="reduced")
        ctx.save_for_backward(q)
        return r

    @staticmethod
    def backward(ctx, r_bar):
        (q,) = ctx.saved_tensors
        return q @ r_bar


def qr_r(m):
    """R factor of reduced QR (backend/linalg.py:8-10)."""
    if _MODE["qr"] == "reference" and m.requires_grad:
        return _QrR.apply(m)
    return torch.linalg.qr(m, mode="reduced").R


def solve_triu(matrix, rhs, trans=0):
    """solve_triangular(lower=False) (backend/linalg.py:48-49)."""
    b = rhs if rhs.ndim == matrix.ndim else rhs.unsqueeze(-1)
    if trans in (1, "T"):
        x = torch.linalg.solve_triangular(matrix.transpose(-1, -2), b, upper=False)
    else:
        x = torch.linalg.solve_triangular(matrix, b, upper=True)
    return x if rhs.ndim == matrix.ndim else x.squeeze(-1)


def solve_tril(matrix, rhs, trans=0):
    """solve_triangular(lower=True) (backend/linalg.py:52-53)."""
    b = rhs if rhs.ndim == matrix.ndim else rhs.unsqueeze(-1)
    if trans in (1, "T"):
        x = torch.linalg.solve_triangular(matrix.transpose(-1, -2), b, upper=True)
    else:
        x = torch.linalg.solve_triangular(matrix, b, upper=False)
    return x if rhs.ndim == matrix.ndim else x.squeeze(-1)


def lstsq_svd(matrix, rhs):
    """Minimum-norm least squares via SVD (backend/linalg.py:60-61).

    ``jnp.linalg.lstsq`` uses an SVD with rcond = eps * max(shape); the
    pseudo-inverse below uses the same cut-off.
    """
    m, n = matrix.shape[-2], matrix.shape[-1]
    u, s, vh = torch.linalg.svd(matrix, full_matrices=False)
    eps = torch.finfo(matrix.dtype).eps
    cutoff = eps * max(m, n) * s.max()
    s_inv = torch.where(s > cutoff, 1.0 / torch.where(s > cutoff, s, torch.ones_like(s)), torch.zeros_like(s))
    b = rhs if rhs.ndim == matrix.ndim else rhs.unsqueeze(-1)
    x = vh.transpose(-1, -2) @ (s_inv.unsqueeze(-1) * (u.transpose(-1, -2) @ b))
    return x if rhs.ndim == matrix.ndim else x.squeeze(-1)


def vector_norm(x):
    """2-norm over all entries (backend/linalg.py:40-41 with ord=None on vectors)."""
    return torch.sqrt(torch.sum(x * x))
