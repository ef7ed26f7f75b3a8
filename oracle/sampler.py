"""Pathwise posterior sampler (TEST INFRASTRUCTURE ONLY).

Restates parsmooth/_pathwise_sampler.py:13-127 with the standard-normal draws
passed in explicitly (``eps`` of shape (T + 1, n_samples, nx), the array the
reference draws from its key at :74), so that a device implementation can be
compared sample by sample.
"""
import numpy as np

from .core import tria, mT, mv
from . import methods
from .parallel import associative_scan
from .types import MVNSqrt


def _make_mvn(m, cov_or_chol, eps, sqrt):
    """parsmooth/_pathwise_sampler.py:81-90: m + L eps, L the (Cholesky) factor."""
    L = cov_or_chol if sqrt else np.linalg.cholesky(cov_or_chol)
    return m[..., None, :] + np.einsum("...ij,...sj->...si", L, eps)


def _gain_and_inc(F, cov_or_chol, b, mf, cf, eps, sqrt):
    """parsmooth/_pathwise_sampler.py:93-127, batched over the steps."""
    nx = F.shape[-1]
    if sqrt:
        Phi = np.block([[F @ cf, cov_or_chol], [cf, np.zeros_like(F)]])
        TP = tria(Phi)
        Phi11, Phi21, inc_L = TP[..., :nx, :nx], TP[..., nx:, :nx], TP[..., nx:, nx:]
        gain = mT(np.linalg.solve(mT(Phi11), mT(Phi21)))
        inc_m = mf - mv(gain, mv(F, mf) + b)
        return gain, _make_mvn(inc_m, inc_L, eps, True)
    S = F @ cf @ mT(F) + cov_or_chol
    gain = cf @ mT(np.linalg.solve(S, F))
    inc_Sig = cf - gain @ S @ mT(gain)
    inc_m = mf - mv(gain, mv(F, mf) + b)
    return gain, _make_mvn(inc_m, inc_Sig, eps, False)


def sampling(eps, transition_model, filter_trajectory, linearization_method, nominal_trajectory=None,
             parallel=True):
    """parsmooth/methods.py:79-91 -> _par_sampling / _seq_sampling with explicit ``eps``.

    Returns (T + 1, n_samples, nx) sampled trajectories."""
    sqrt = isinstance(filter_trajectory, MVNSqrt)
    fm, fc = (np.asarray(v, dtype=float) for v in filter_trajectory)
    Tp1, nx = fm.shape
    eps = np.asarray(eps, dtype=float)
    if nominal_trajectory is None:   # parsmooth/methods.py:86-87: the smoothed trajectory
        nominal_trajectory = methods.smoothing(transition_model, filter_trajectory, linearization_method, None,
                                               parallel)
    nm, nc = (np.asarray(v, dtype=float)[:-1] for v in nominal_trajectory)
    F, cq, b = linearization_method(transition_model, type(filter_trajectory)(nm, nc))
    gains, incs = _gain_and_inc(F, cq, b, fm[:-1], fc[:-1], eps[1:], sqrt)
    last = _make_mvn(fm[-1], fc[-1], eps[0], sqrt)
    if not parallel:
        xs = np.empty((Tp1, eps.shape[1], nx))
        xs[-1] = last
        for t in range(Tp1 - 2, -1, -1):
            xs[t] = np.einsum("ij,sj->si", gains[t], xs[t + 1]) + incs[t]
        return xs
    Gs = np.concatenate([gains, np.zeros((1, nx, nx))])
    es = np.concatenate([incs, last[None]])

    def op(e1, e2):
        G1, x1 = e1
        G2, x2 = e2
        return G2 @ G1, np.einsum("...ij,...sj->...si", G2, x1) + x2

    _, xs = associative_scan(op, (Gs, es), reverse=True)
    return xs
