"""Batched FP64 numerical primitives of the oracle (TEST INFRASTRUCTURE ONLY).

All functions accept arrays with arbitrary leading batch dimensions and act on
the trailing one or two axes.
"""
import numpy as np

LOG_2PI = float(np.log(2.0 * np.pi))


def canon(L):
    """Flip column signs of a lower-triangular factor so its diagonal is >= 0.

    ``tria`` is only defined up to the signs of the columns of its result
    (parsmooth/_utils.py:22-24 leaves them to LAPACK).  Every quantity the
    smoother produces is invariant under those flips, so the oracle and the
    CUDA kernels both return this canonical representative.
    """
    L = np.asarray(L, dtype=float)
    k = min(L.shape[-1], L.shape[-2])
    d = np.diagonal(L[..., :k, :k], axis1=-2, axis2=-1)
    s = np.where(d < 0, -1.0, 1.0)
    out = L.copy()
    out[..., :, :k] *= s[..., None, :]
    return out


def tria(A):
    """Lower-triangular ``L`` with ``L @ L.T == A @ A.T`` via QR of ``A.T``.

    Follows parsmooth/_utils.py:22-24 (``qr(A.T, mode='economic').R.T``),
    batched over leading axes, canonicalised with :func:`canon`.
    """
    A = np.asarray(A, dtype=float)
    R = np.linalg.qr(np.swapaxes(A, -1, -2), mode="r")
    return canon(np.swapaxes(R, -1, -2))


def solve_lower(L, B):
    """Solve ``L X = B`` for lower-triangular ``L`` (batched)."""
    return np.linalg.solve(L, B)


def solve_upper(U, B):
    """Solve ``U X = B`` for upper-triangular ``U`` (batched)."""
    return np.linalg.solve(U, B)


def mT(A):
    return np.swapaxes(A, -1, -2)


def mv(A, x):
    """Batched matrix-vector product."""
    return np.einsum("...ij,...j->...i", A, x)


def cholesky_update(chol, v, multiplier):
    """Rank-1 update/downdate of a lower Cholesky factor.

    Restates parsmooth/_utils.py:39-81 (the column sweep of Algorithm 3.1 of
    Krause & Igel, written as a scan over columns): for each column ``j`` the
    diagonal ``d``, the running vector ``omega`` and the scalar ``b`` are
    updated; the strictly upper part is zeroed and every non-finite entry of the
    result is replaced by zero (parsmooth/_utils.py:80).
    """
    chol = np.asarray(chol, dtype=float)
    n = chol.shape[-1]
    diag = np.diagonal(chol, axis1=-2, axis2=-1).copy()
    omega = np.array(v, dtype=float, copy=True) * np.ones(chol.shape[:-1])
    b = np.ones(chol.shape[:-2])
    out = np.zeros(np.broadcast_shapes(chol.shape, omega.shape[:-1] + (n, n)))
    new_diag = np.zeros(out.shape[:-1])
    with np.errstate(all="ignore"):
        for j in range(n):
            d = diag[..., j]
            w = omega[..., j]
            nd = np.sqrt(d * d + multiplier / b * w * w)
            gamma = d * d * b + multiplier * w * w
            col = chol[..., :, j]
            omega = omega - (w / d)[..., None] * col
            out[..., :, j] = nd[..., None] * (col / d[..., None] + (multiplier * w / gamma)[..., None] * omega)
            b = b + multiplier * (w / d) ** 2
            new_diag[..., j] = nd
    idx = np.arange(n)
    out[..., idx, idx] = new_diag
    out = np.tril(out)
    return np.where(np.isfinite(out), out, 0.0)


def cholesky_update_many(chol, vs, multiplier):
    """Apply :func:`cholesky_update` for each row of ``vs`` in turn (parsmooth/_utils.py:13-19)."""
    vs = np.asarray(vs, dtype=float)
    for k in range(vs.shape[-2]):
        chol = cholesky_update(chol, vs[..., k, :], multiplier)
    return chol


def mvn_loglikelihood(x, chol):
    """Log-density of ``N(0, chol chol^T)`` at ``x`` (parsmooth/_utils.py:152-160)."""
    x = np.asarray(x, dtype=float)
    dim = chol.shape[-1]
    y = np.linalg.solve(chol, x[..., None])[..., 0]
    diag = np.diagonal(chol, axis1=-2, axis2=-1)
    const = np.sum(np.log(np.abs(diag)), axis=-1) + dim * LOG_2PI / 2.0
    return -0.5 * np.sum(y * y, axis=-1) - const
