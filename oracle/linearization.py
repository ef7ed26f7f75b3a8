"""Oracle linearisations (TEST INFRASTRUCTURE ONLY).

Each method maps ``(model, x)`` with ``model = FunctionalModel(f, q)`` and
``x`` an ``MVNSqrt`` (or ``MVNStandard``) to ``(F, chol_or_cov, b)`` such that
``f(x') + q ~= F x' + b + N(0, chol chol^T)``.  Inputs may carry leading batch
axes (one linearisation point per time step).
"""
import math

import numpy as np

from .core import tria, cholesky_update_many, mT, mv
from .types import MVNSqrt, MVNStandard, ConditionalMomentsModel, are_inputs_compatible


# ----------------------------------------------------------------------------- sigma points

def cubature_weights(n):
    """Spherical cubature: ``2n`` points ``+-sqrt(n) e_i``, equal weights.

    parsmooth/linearization/_cubature.py:63-85.  Returns ``(wm, wc, xi)`` with
    ``xi`` of shape ``(n_points, n)`` (unit sigma points as rows).
    """
    wm = np.full(2 * n, 1.0 / (2 * n))
    xi = np.concatenate([np.eye(n), -np.eye(n)], axis=0) * np.sqrt(n)
    return wm, wm.copy(), xi


def unscented_weights(n, alpha=1.0, beta=0.0, kappa=None):
    """Unscented transform with ``lambda = alpha^2 (n + kappa) - n``.

    parsmooth/linearization/_unscented.py:42-101; the code's default is
    ``kappa = 3 + n`` (:64-65).  Returns ``(wm, wc, xi)`` where ``xi`` rows are
    ``0, +sqrt(n+lambda) e_i, -sqrt(n+lambda) e_i`` in the chol's column basis.
    """
    if kappa is None:
        kappa = 3.0 + n
    lam = alpha ** 2 * (n + kappa) - n
    wm = np.full(2 * n + 1, 1.0 / (2 * (n + lam)))
    wm[0] = lam / (n + lam)
    wc = wm.copy()
    wc[0] = lam / (n + lam) + (1 - alpha ** 2 + beta)
    scale = np.sqrt(n + lam)
    xi = np.concatenate([np.zeros((1, n)), scale * np.eye(n), -scale * np.eye(n)], axis=0)
    return wm, wc, xi


def hermite_coefficients(order):
    """Physicists' Hermite polynomials ``H_0..H_order``, highest power first.

    Recurrence ``H_k = 2x H_{k-1} - 2(k-1) H_{k-2}`` as in
    parsmooth/linearization/_gh.py:129-151.
    """
    H = [np.array([1.0]), np.array([2.0, 0.0])]
    for k in range(2, order + 1):
        H.append(2 * np.append(H[k - 1], 0.0) - 2 * (k - 1) * np.pad(H[k - 2], (2, 0)))
    return H


def gauss_hermite_weights(n, order=3):
    """Tensor-product Gauss-Hermite rule with ``order**n`` points.

    parsmooth/linearization/_gh.py:73-126: 1-D roots of ``H_p`` (via
    ``np.roots``), 1-D weights ``2^(p-1) p! sqrt(pi) / (p^2 H_{p-1}(x_i)^2)``,
    products over dimensions scaled by ``pi^(-n/2)``, points ``sqrt(2) x``.
    Point ``k`` takes, in dimension ``r``, root number ``(k // p^r) % p``.
    Returns ``(wm, wc, xi)`` with ``xi`` rows the unit points.
    """
    p = order
    H = hermite_coefficients(p)
    roots = np.flip(np.roots(H[-1]))
    w1 = np.array([2 ** (p - 1) * math.factorial(p) * np.sqrt(np.pi) /
                   (p ** 2 * np.polyval(H[p - 1], roots[i]) ** 2) for i in range(p)])
    k = np.arange(p ** n)
    table = np.stack([(k // p ** r) % p for r in range(n)], axis=0)  # (n, p^n)
    wm = np.prod(w1[table], axis=0) / np.sqrt(np.pi) ** n
    xi = (np.sqrt(2.0) * roots[table]).T
    return wm, wm.copy(), np.real(xi)


def sigma_points(rule, m, chol):
    """Points ``m + chol @ xi_k`` for each unit point ``xi_k`` (rows of ``rule[2]``)."""
    wm, wc, xi = rule
    pts = m[..., None, :] + np.einsum("...ij,kj->...ki", chol, xi)
    return pts, wm, wc


# ----------------------------------------------------------------------------- methods

class _Method:
    """Base of the four linearisation methods; instances are callables ``(model, x)``."""
    name = ""

    def __call__(self, model, x):
        if isinstance(model, ConditionalMomentsModel):
            c_m, c_cov_or_chol = model
            if isinstance(x, MVNSqrt):
                return self.sqrt_conditional(c_m, c_cov_or_chol, x)
            return self.standard_conditional(c_m, c_cov_or_chol, x)
        f, q = model
        are_inputs_compatible(x, q)
        if isinstance(x, MVNSqrt):
            return self.sqrt(f, x, q)
        return self.standard(f, x, q)


class Extended(_Method):
    """First-order Taylor linearisation (parsmooth/linearization/_extended.py:9-70)."""
    name = "extended"

    def sqrt(self, f, x, q):
        m = np.asarray(x.mean, dtype=float)
        F = f.jacobian(m)
        b = f(m) - mv(F, m) + q.mean
        chol = np.broadcast_to(q.chol, F.shape[:-2] + np.shape(q.chol)).copy()
        return F, chol, b

    def standard(self, f, x, q):
        m = np.asarray(x.mean, dtype=float)
        F = f.jacobian(m)
        b = f(m) - mv(F, m) + q.mean
        cov = np.broadcast_to(q.cov, F.shape[:-2] + np.shape(q.cov)).copy()
        return F, cov, b

    # parsmooth/linearization/_extended.py:43-56
    def sqrt_conditional(self, c_m, c_chol, x):
        m = np.asarray(x.mean, dtype=float)
        F = c_m.jacobian(m)
        return F, c_chol(m), c_m(m) - mv(F, m)

    def standard_conditional(self, c_m, c_cov, x):
        m = np.asarray(x.mean, dtype=float)
        F = c_m.jacobian(m)
        return F, c_cov(m), c_m(m) - mv(F, m)


class _SigmaPointMethod(_Method):
    """Statistical linear regression on sigma points.

    parsmooth/linearization/_sigma_points.py:63-100 (``linearize_functional``
    and ``_linearize_functional_common``).
    """

    def rule(self, n):
        raise NotImplementedError

    def _common(self, f, m, chol):
        pts, wm, wc = sigma_points(self.rule(m.shape[-1]), m, chol)
        f_pts = f(pts)
        m_f = np.einsum("k,...kd->...d", wm, f_pts)
        psi = np.einsum("k,...kn,...kd->...nd", wc, pts - m[..., None, :], f_pts - m_f[..., None, :])
        # F_x = cho_solve((chol, lower), Psi_x).T  (_sigma_points.py:98)
        tmp = np.linalg.solve(chol, psi)
        F = mT(np.linalg.solve(mT(chol), tmp))
        return F, pts, wc, f_pts, m_f

    def sqrt(self, f, x, q):
        m = np.asarray(x.mean, dtype=float)
        chol = np.asarray(x.chol, dtype=float)
        F, pts, wc, f_pts, m_f = self._common(f, m, chol)
        sqrt_phi = np.sqrt(wc)[:, None] * (f_pts - m_f[..., None, :])  # (..., N, d)
        n_sigma, d_out = sqrt_phi.shape[-2:]
        if n_sigma >= d_out:
            sqrt_phi = tria(mT(sqrt_phi))
        else:
            pad = np.zeros(sqrt_phi.shape[:-2] + (d_out, d_out - n_sigma))
            sqrt_phi = np.concatenate([mT(sqrt_phi), pad], axis=-1)
        chol_q = np.broadcast_to(q.chol, sqrt_phi.shape[:-2] + np.shape(q.chol))
        chol_L = tria(np.concatenate([sqrt_phi, chol_q], axis=-1))
        chol_L = cholesky_update_many(chol_L, mT(F @ chol), -1.0)
        return F, chol_L, m_f - mv(F, m) + q.mean

    # parsmooth/linearization/_sigma_points.py:25-60
    def sqrt_conditional(self, c_m, c_chol, x):
        m = np.asarray(x.mean, dtype=float)
        chol = np.asarray(x.chol, dtype=float)
        F, pts, wc, f_pts, m_f = self._common(c_m, m, chol)
        sqrt_phi = tria(mT(np.sqrt(wc)[:, None] * (f_pts - m_f[..., None, :])))
        chol_pts = c_chol(pts)                                     # (..., N, d, d)
        temp = np.sqrt(wc)[:, None, None] * chol_pts
        temp = np.swapaxes(temp, -3, -2)                           # (..., d, N, d)
        temp = temp.reshape(temp.shape[:-2] + (-1,))               # (..., d, N d)
        chol_L = tria(np.concatenate([sqrt_phi, temp], axis=-1))
        chol_L = cholesky_update_many(chol_L, mT(F @ chol), -1.0)
        return F, chol_L, m_f - mv(F, m)

    def standard_conditional(self, c_m, c_cov, x):
        m = np.asarray(x.mean, dtype=float)
        cov = np.asarray(x.cov, dtype=float)
        chol = np.linalg.cholesky(cov)
        F, pts, wc, f_pts, m_f = self._common(c_m, m, chol)
        v_f = np.einsum("k,...kij->...ij", wc, c_cov(pts))
        d = f_pts - m_f[..., None, :]
        phi = np.einsum("k,...ki,...kj->...ij", wc, d, d)
        temp = F @ chol
        return F, phi - temp @ mT(temp) + v_f, m_f - mv(F, m)

    def standard(self, f, x, q):
        m = np.asarray(x.mean, dtype=float)
        cov = np.asarray(x.cov, dtype=float)
        chol = np.linalg.cholesky(cov)
        F, pts, wc, f_pts, m_f = self._common(f, m, chol)
        d = f_pts - m_f[..., None, :]
        phi = np.einsum("k,...ki,...kj->...ij", wc, d, d)
        L = phi - F @ cov @ mT(F) + q.cov
        return F, 0.5 * (L + mT(L)), m_f - mv(F, m) + q.mean


class Cubature(_SigmaPointMethod):
    name = "cubature"

    def rule(self, n):
        return cubature_weights(n)


class Unscented(_SigmaPointMethod):
    name = "unscented"

    def __init__(self, alpha=1.0, beta=0.0, kappa=None):
        self.alpha, self.beta, self.kappa = alpha, beta, kappa

    def rule(self, n):
        return unscented_weights(n, self.alpha, self.beta, self.kappa)


class GaussHermite(_SigmaPointMethod):
    name = "gauss_hermite"

    def __init__(self, order=3):
        self.order = order

    def rule(self, n):
        return gauss_hermite_weights(n, self.order)


extended = Extended()
cubature = Cubature()
unscented = Unscented()
gauss_hermite = GaussHermite()
