"""Oracle sequential square-root filter and RTS smoother (TEST INFRASTRUCTURE ONLY).

Restates parsmooth/sequential/_filtering.py:11-108 and
parsmooth/sequential/_smoothing.py:12-77: one step at a time, the parallel
path's association-independent counterpart.
"""
import numpy as np

from .core import tria, mv, mvn_loglikelihood
from .types import MVNSqrt, are_inputs_compatible


def _lin_one(method, model, x):
    return method(model, type(x)(*(np.asarray(v, dtype=float) for v in x)))


def sqrt_predict(F, cholQ, b, m, L):
    """parsmooth/sequential/_filtering.py:80-86."""
    return mv(F, m) + b, tria(np.concatenate([F @ L, cholQ], axis=-1))


def sqrt_update(H, cholR, c, m, L, y):
    """parsmooth/sequential/_filtering.py:89-108; returns ``(m, L, ell)``."""
    nx = m.shape[-1]
    ny = y.shape[-1]
    y_diff = y - (mv(H, m) + c)
    M = np.block([[H @ L, cholR], [L, np.zeros((nx, ny))]])
    S = tria(M)
    L_new = S[ny:, ny:]
    G = S[ny:, :ny]
    Iy = S[:ny, :ny]
    m_new = m + G @ np.linalg.solve(Iy, y_diff)
    return m_new, L_new, float(mvn_loglikelihood(y_diff, Iy))


def standard_predict(F, Q, b, m, P):
    """parsmooth/sequential/_filtering.py:56-62."""
    return mv(F, m) + b, Q + F @ P @ F.T


def standard_update(H, R, c, m, P, y):
    """parsmooth/sequential/_filtering.py:65-77."""
    y_diff = y - (H @ m + c)
    S = R + H @ P @ H.T
    chol_S = np.linalg.cholesky(S)
    G = P @ np.linalg.solve(S, H).T
    return m + G @ y_diff, P - G @ S @ G.T, float(mvn_loglikelihood(y_diff, chol_S))


def filtering(observations, x0, transition_model, observation_model, linearization_method,
              nominal_trajectory=None, return_loglikelihood=False):
    """Sequential filter (parsmooth/sequential/_filtering.py:11-53).

    Without a nominal trajectory each step linearises at the running state.
    """
    ys = np.asarray(observations, dtype=float)
    if nominal_trajectory is not None:
        are_inputs_compatible(x0, nominal_trajectory)
    sqrt = isinstance(x0, MVNSqrt)
    kind = type(x0)
    m, C = (np.asarray(v, dtype=float) for v in x0)
    ms, Cs = [m], [C]
    ell = 0.0
    for t, y in enumerate(ys):
        ref = kind(m, C) if nominal_trajectory is None else kind(*(np.asarray(v)[t] for v in nominal_trajectory))
        F, Qc, b = _lin_one(linearization_method, transition_model, ref)
        m, C = (sqrt_predict if sqrt else standard_predict)(F, Qc, b, m, C)
        ref = kind(m, C) if nominal_trajectory is None else kind(*(np.asarray(v)[t + 1] for v in nominal_trajectory))
        H, Rc, c = _lin_one(linearization_method, observation_model, ref)
        m, C, inc = (sqrt_update if sqrt else standard_update)(H, Rc, c, m, C, y)
        ell += inc
        ms.append(m)
        Cs.append(C)
    res = kind(np.stack(ms), np.stack(Cs))
    return (res, ell) if return_loglikelihood else res


def sqrt_smooth(F, cholQ, b, mf, Lf, ms, Ls):
    """parsmooth/sequential/_smoothing.py:60-77."""
    nx = F.shape[0]
    Phi = np.block([[F @ Lf, cholQ], [Lf, np.zeros_like(F)]])
    TP = tria(Phi)
    Phi11 = TP[:nx, :nx]
    Phi21 = TP[nx:, :nx]
    Phi22 = TP[nx:, nx:]
    gain = np.linalg.solve(Phi11.T, Phi21.T).T
    mean = mf + gain @ (ms - (b + F @ mf))
    chol = tria(np.concatenate([Phi22, gain @ Ls], axis=1))
    return mean, chol


def standard_smooth(F, Q, b, mf, Pf, ms, Ps):
    """parsmooth/sequential/_smoothing.py:46-57."""
    S = F @ Pf @ F.T + Q
    gain = Pf @ np.linalg.solve(S, F).T
    return mf + gain @ (ms - (b + F @ mf)), Pf + gain @ (Ps - S) @ gain.T


def smoothing(transition_model, filter_trajectory, linearization_method, nominal_trajectory=None):
    """Sequential RTS smoother (parsmooth/sequential/_smoothing.py:12-42)."""
    if nominal_trajectory is not None:
        are_inputs_compatible(filter_trajectory, nominal_trajectory)
    sqrt = isinstance(filter_trajectory, MVNSqrt)
    kind = type(filter_trajectory)
    fm, fc = (np.asarray(v, dtype=float) for v in filter_trajectory)
    T = fm.shape[0] - 1
    sm, sc = fm[-1], fc[-1]
    out_m, out_c = [sm], [sc]
    for t in range(T - 1, -1, -1):
        ref = kind(sm, sc) if nominal_trajectory is None else kind(*(np.asarray(v)[t] for v in nominal_trajectory))
        F, Qc, b = _lin_one(linearization_method, transition_model, ref)
        sm, sc = (sqrt_smooth if sqrt else standard_smooth)(F, Qc, b, fm[t], fc[t], sm, sc)
        out_m.append(sm)
        out_c.append(sc)
    return kind(np.stack(out_m[::-1]), np.stack(out_c[::-1]))
