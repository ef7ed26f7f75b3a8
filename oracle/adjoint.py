"""Reverse-mode gradient of the filter log-likelihood (TEST INFRASTRUCTURE ONLY).

The reference obtains ``d ell / d theta`` by ``jax.grad`` through its parallel filter
(parsmooth/parallel/_filtering.py:13-61 with ``return_loglikelihood``, the sum of
:149-154).  At a fixed nominal trajectory that log-likelihood is the exact marginal
log-likelihood of the linearised Gaussian model

    x_0 ~ N(m0, L0 L0^T),  x_t = F_t x_{t-1} + b_t + q_t,  q_t ~ N(0, cQ_t cQ_t^T),
    y_t = H_t x_t + c_t + r_t,  r_t ~ N(0, cR_t cR_t^T),

whose per-step parameters are what the linearisation (parsmooth/linearization/*.py)
returns.  Its gradient with respect to every per-step parameter follows from the
posterior moments of the same model (Fisher's identity,
``grad ell = E[grad log p(x, y) | y]``), which the RTS smoother supplies: with the
smoothing element ``x_{t-1} = E_{t-1} x_t + g_{t-1} + D_{t-1} w`` (_smoothing.py:72-85)
and the smoothed ``x_t ~ N(ms_t, Ls_t Ls_t^T)``, the transition residual
``e_t = x_t - F_t x_{t-1} - b_t`` has mean ``ms_t - F_t ms_{t-1} - b_t`` and a square
root of its covariance ``[(I - F_t E_{t-1}) Ls_t, F_t D_{t-1}]``, and

    d ell / d F_t = Q_t^-1 E[e_t x_{t-1}^T],   d ell / d b_t = Q_t^-1 E[e_t],
    d ell / d Q_t = (Q_t^-1 E[e_t e_t^T] Q_t^-1 - Q_t^-1) / 2,

with the same forms for the observation residual ``y_t - H_t x_t - c_t`` and for the
prior.  Everything is written in the whitened form ``Z = cQ^-1 [sqrt(Cov e), E e]``,
``A = Z Z^T - I``, so ``d ell / d cQ_any = cQ^-T A cQ^-1 L`` for any factor ``L`` of the
same covariance.  This module computes those quantities with the FP64 oracle (its
filter, smoother and elements), and the chain to model parameters; the tests check it
against central differences of the oracle's log-likelihood.
"""
import numpy as np

from . import parallel as par
from .core import mT, mv, solve_lower, solve_upper, tria
from .types import MVNSqrt


def _whiten(c, W):
    """``c^-1 W`` for lower-triangular ``c`` (batched)."""
    return solve_lower(c, W)


def _unwhiten_T(c, X):
    """``c^-T X`` for lower-triangular ``c`` (batched)."""
    return solve_upper(mT(c), X)


def linearised_model(observations, x0, transition_model, observation_model, linearization_method,
                     nominal_trajectory=None):
    """The per-step parameters the parallel filter runs on (parsmooth/parallel/_filtering.py:29-33)."""
    T = np.asarray(observations).shape[0]
    nx = np.asarray(x0.mean).shape[-1]
    if nominal_trajectory is None:
        nominal_trajectory = par._default_nominal(type(x0), T + 1, nx)
    n_prev = MVNSqrt(*(np.asarray(v, dtype=float)[:-1] for v in nominal_trajectory))
    n_next = MVNSqrt(*(np.asarray(v, dtype=float)[1:] for v in nominal_trajectory))
    F, cQ, b = linearization_method(transition_model, n_prev)
    H, cR, c = linearization_method(observation_model, n_next)
    return F, cQ, b, H, cR, c


def filter_adjoint(observations, x0, transition_model, observation_model, linearization_method,
                   nominal_trajectory=None):
    """Gradient of the filter's summed log-likelihood with respect to the linearised model.

    Returns ``(ell, adj)`` with ``adj`` a dict of per-step arrays ``F`` (T, nx, nx), ``b``
    (T, nx), ``A_q`` (T, nx, nx) (the whitened ``Z Z^T - I`` of the transition residual),
    ``H`` (T, ny, nx), ``c`` (T, ny), ``A_r`` (T, ny, ny), the per-step linearisation
    (``lin``: F, cQ, b, H, cR, c), and the prior's ``m0`` (nx,) and ``L0`` (nx, nx) (lower
    triangle: the filter reads only that part of the prior factor).
    """
    ys = np.asarray(observations, dtype=float)
    T = ys.shape[0]
    m0, L0 = (np.asarray(v, dtype=float) for v in x0)
    nx = m0.shape[-1]
    if nominal_trajectory is None:
        nominal_trajectory = par._default_nominal(type(x0), T + 1, nx)
    F, cQ, b, H, cR, c = linearised_model(ys, x0, transition_model, observation_model, linearization_method,
                                          nominal_trajectory)
    filt, ell = par.filtering(ys, x0, transition_model, observation_model, linearization_method,
                              nominal_trajectory, return_loglikelihood=True)
    fm, fL = (np.asarray(v) for v in filt)
    sm_traj = par.smoothing(transition_model, filt, linearization_method, nominal_trajectory)
    sm, sL = (np.asarray(v) for v in sm_traj)
    _, E, D = par.sqrt_smoother_elements(F, cQ, b, fm[:-1], fL[:-1])
    I = np.eye(nx)
    # transition residual e_t = x_t - F x_{t-1} - b, t = 1..T (arrays indexed t-1)
    m_prev, m_next, L_next = sm[:-1], sm[1:], sL[1:]
    e_mean = m_next - mv(F, m_prev) - b
    M = I - F @ E
    W = np.concatenate([M @ L_next, F @ D, e_mean[..., None]], axis=-1)
    Z = _whiten(cQ, W)
    A_q = Z @ mT(Z) - I
    # Q^-1 E[e x_{t-1}^T] = cQ^-T (Z1 (E L)^T - Z2 D^T + z_e m_{t-1}^T)
    Z1, Z2, ze = Z[..., :nx], Z[..., nx:2 * nx], Z[..., 2 * nx]
    Fbar = _unwhiten_T(cQ, Z1 @ mT(E @ L_next) - Z2 @ mT(D) + ze[..., None] * m_prev[..., None, :])
    bbar = _unwhiten_T(cQ, ze[..., None])[..., 0]
    # observation residual r_t = y_t - H x_t - c
    ny = ys.shape[-1]
    r_mean = ys - mv(H, m_next) - c
    Wy = np.concatenate([H @ L_next, r_mean[..., None]], axis=-1)
    Zy = _whiten(cR, Wy)
    A_r = Zy @ mT(Zy) - np.eye(ny)
    Zy1, zr = Zy[..., :nx], Zy[..., nx]
    Hbar = _unwhiten_T(cR, zr[..., None] * m_next[..., None, :] - Zy1 @ mT(L_next))
    cbar = _unwhiten_T(cR, zr[..., None])[..., 0]
    # prior
    d0 = sm[0] - m0
    Z0 = _whiten(L0, np.concatenate([sL[0], d0[:, None]], axis=-1))
    m0bar = _unwhiten_T(L0, Z0[:, nx:])[:, 0]
    L0bar = np.tril(_unwhiten_T(L0, Z0 @ Z0.T - I))
    adj = {"F": Fbar, "b": bbar, "A_q": A_q, "H": Hbar, "c": cbar, "A_r": A_r, "m0": m0bar, "L0": L0bar,
           "lin": (F, cQ, b, H, cR, c)}
    return ell, adj


def noise_chol_adjoint(A, c, L):
    """``sum_t d ell / d L`` for a noise factor ``L`` whose covariance enters every step's
    ``c_t c_t^T`` additively (``c_t c_t^T = Omega_t + L L^T``): ``cQ^-T A cQ^-1 L``, summed,
    lower triangle (the kernels read only that part)."""
    Y = _whiten(c, np.broadcast_to(L, c.shape[:-2] + L.shape).copy())
    return np.tril(np.sum(_unwhiten_T(c, A @ Y), axis=0))


def linear_model_adjoints(adj, Lq, Lr):
    """Adjoints of a linear model pair's own arrays: transition matrix, noise mean and
    factor, observation matrix, noise mean and factor, summed over the steps."""
    return {"trans_matrix": adj["F"].sum(0), "trans_noise_mean": adj["b"].sum(0),
            "trans_noise_chol": noise_chol_adjoint(adj["A_q"], adj["lin"][1], Lq),
            "obs_matrix": adj["H"].sum(0), "obs_noise_mean": adj["c"].sum(0),
            "obs_noise_chol": noise_chol_adjoint(adj["A_r"], adj["lin"][4], Lr),
            "m0": adj["m0"], "L0": adj["L0"]}


def param_adjoint(adj, which, lin_plus, lin_minus, h):
    """``d ell / d p`` for one scalar model parameter ``p`` that enters the step-wise
    linearisation of one model (``which`` 0 transition, 1 observation), from that
    linearisation evaluated at ``p + h`` and ``p - h`` (central differences of the local,
    per-step map; the filter and smoother are not differentiated numerically):
    ``sum_t tr(Fbar^T dF) + bbar . db + tr(Qbar d(cQ cQ^T))`` with
    ``tr(Qbar d(c c^T)) = tr(A c^-1 dc)`` in the whitened form."""
    Fp, cp, bp = lin_plus
    Fm, cm, bm = lin_minus
    dF, dc, db = (Fp - Fm) / (2 * h), (cp - cm) / (2 * h), (bp - bm) / (2 * h)
    if which == 0:
        Fbar, bbar, A, c = adj["F"], adj["b"], adj["A_q"], adj["lin"][1]
    else:
        Fbar, bbar, A, c = adj["H"], adj["c"], adj["A_r"], adj["lin"][4]
    # d(c c^T) = dc c^T + c dc^T, and the derivative of a factor of a fixed covariance is
    # not unique; contracting with Qbar = c^-T A c^-1 / 2 makes it so:
    # tr(Qbar (dc c^T + c dc^T)) = tr(c^-T A c^-1 dc c^T) = tr(A c^-1 dc)
    X = _whiten(c, dc)
    return float(np.sum(Fbar * dF) + np.sum(bbar * db) + np.einsum("tij,tji->", A, X))


def transition_adjoint_predicted_form(F, cQ, b, fm, fL, sm, sL):
    """The transition part of :func:`filter_adjoint` written with the filter's predicted moments
    instead of the residual ``e_t`` (the form the GPU kernel computes): with ``Lp`` the predicted
    factor from ``tria([[F Lf, cQ], [Lf, 0]])`` (whose lower-left block is ``Phi21 = E Lp``),
    ``d = ms_t - mp_t`` and ``[Y, y] = Lp^-1 [Ls_t, d]``,
    ``dl/dQ = Lp^-T (Y Y^T - I + y y^T) Lp^-1 / 2``, ``dl/db = Lp^-T y`` and
    ``dl/dF = Lp^-T ((Y Y^T - I) Phi21^T + y ms_{t-1}^T)``.  ``fm, fL`` / ``sm, sL``: filtered
    and smoothed trajectories (T + 1 states).  Returns ``(Fbar, bbar, Qbar)`` per step."""
    nx = cQ.shape[-1]
    Phi = tria(np.concatenate([np.concatenate([F @ fL[:-1], cQ], -1),
                               np.concatenate([fL[:-1], np.zeros_like(cQ)], -1)], -2))
    Lp, P21 = Phi[..., :nx, :nx], Phi[..., nx:, :nx]
    d = sm[1:] - (mv(F, fm[:-1]) + b)
    Y = solve_lower(Lp, np.concatenate([sL[1:], d[..., None]], -1))
    Y1, y = Y[..., :nx], Y[..., nx]
    Ap = Y1 @ mT(Y1) - np.eye(nx)
    N = Ap + y[..., None] * y[..., None, :]
    Fbar = _unwhiten_T(Lp, Ap @ mT(P21) + y[..., None] * sm[:-1][..., None, :])
    bbar = _unwhiten_T(Lp, y[..., None])[..., 0]
    Qbar = 0.5 * _unwhiten_T(Lp, mT(_unwhiten_T(Lp, N)))
    return Fbar, bbar, Qbar
