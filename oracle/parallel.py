"""Oracle parallel-in-time filter and smoother (TEST INFRASTRUCTURE ONLY).

Restates parsmooth/parallel/{_operators,_filtering,_smoothing}.py in batched
NumPy.  ``associative_scan`` restates the odd/even recursion of
``jax.lax.associative_scan`` so the oracle combines elements in the same
order as the reference; ``sequential_scan`` is a plain left fold used as a
second, association-independent truth.
"""
import numpy as np

from .core import tria, mT, mv, mvn_loglikelihood
from .types import MVNSqrt, are_inputs_compatible


# ----------------------------------------------------------------------------- scans

def _interleave(a, b):
    n = a.shape[0] + b.shape[0]
    out = np.empty((n,) + a.shape[1:], dtype=np.result_type(a, b))
    out[0::2] = a
    out[1::2] = b
    return out


def _odd_even_scan(fn, elems):
    n = elems[0].shape[0]
    if n < 2:
        return elems
    reduced = fn(tuple(e[0:-1:2] for e in elems), tuple(e[1::2] for e in elems))
    odd = _odd_even_scan(fn, reduced)
    if n % 2 == 0:
        even = fn(tuple(o[:-1] for o in odd), tuple(e[2::2] for e in elems))
    else:
        even = fn(odd, tuple(e[2::2] for e in elems))
    even = tuple(np.concatenate([e[:1], r], axis=0) for e, r in zip(elems, even))
    return tuple(_interleave(e, o) for e, o in zip(even, odd))


def associative_scan(fn, elems, reverse=False):
    """Inclusive scan with the association order of ``jax.lax.associative_scan``.

    ``fn(a, b)`` receives batched tuples, ``a`` the earlier partial results.
    With ``reverse=True`` the sequence is flipped first, so ``a`` is then the
    partial result over *later* indices (parsmooth/parallel/_smoothing.py:33-34).
    """
    elems = tuple(np.asarray(e, dtype=float) for e in elems)
    if reverse:
        elems = tuple(e[::-1] for e in elems)
    out = _odd_even_scan(fn, elems)
    if reverse:
        out = tuple(o[::-1] for o in out)
    return out


def sequential_scan(fn, elems, reverse=False):
    """Inclusive left fold, element by element (independent association order)."""
    elems = tuple(np.asarray(e, dtype=float) for e in elems)
    n = elems[0].shape[0]
    order = range(n - 1, -1, -1) if reverse else range(n)
    outs = [np.empty_like(e) for e in elems]
    acc = None
    for k in order:
        cur = tuple(e[k:k + 1] for e in elems)
        acc = cur if acc is None else fn(acc, cur)
        for o, a in zip(outs, acc):
            o[k] = a[0]
    return tuple(outs)


# ----------------------------------------------------------------------------- operators

def sqrt_filtering_operator(elem1, elem2):
    """Square-root filtering combine (parsmooth/parallel/_operators.py:43-77), batched."""
    A1, b1, U1, eta1, Z1 = elem1
    A2, b2, U2, eta2, Z2 = elem2
    nx = Z2.shape[-2]
    I = np.broadcast_to(np.eye(nx), A1.shape)
    Xi = np.block([[mT(U1) @ Z2, I], [Z2, np.zeros_like(A1)]])
    T = tria(Xi)
    Xi11 = T[..., :nx, :nx]
    Xi21 = T[..., nx:, :nx]
    Xi22 = T[..., nx:, nx:]
    W = mT(np.linalg.solve(Xi11, mT(U1) @ mT(A2)))           # A2 U1 Xi11^-T
    A = A2 @ A1 - W @ mT(Xi21) @ A1
    V = np.linalg.solve(Xi11, mT(U1))                          # Xi11^-1 U1^T
    M = I - mT(V) @ mT(Xi21)
    b = mv(A2 @ M, b1 + mv(U1 @ mT(U1), eta2)) + b2
    U = tria(np.concatenate([W, U2], axis=-1))
    G = mT(np.linalg.solve(mT(Xi11), mT(Xi21)))               # Xi21 Xi11^-1
    eta = mv(mT(A1) @ (I - G @ mT(U1)), eta2 - mv(Z2 @ mT(Z2), b1)) + eta1
    Z = tria(np.concatenate([mT(A1) @ Xi22, Z1], axis=-1))
    return A, b, U, eta, Z


def sqrt_smoothing_operator(elem1, elem2):
    """Square-root smoothing combine (parsmooth/parallel/_operators.py:104-125), batched."""
    g1, E1, D1 = elem1
    g2, E2, D2 = elem2
    g = mv(E2, g1) + g2
    E = E2 @ E1
    D = tria(np.concatenate([E2 @ D1, D2], axis=-1))
    return g, E, D


def standard_filtering_operator(elem1, elem2):
    """Covariance-form filtering combine (parsmooth/parallel/_operators.py:7-40), batched."""
    A1, b1, C1, eta1, J1 = elem1
    A2, b2, C2, eta2, J2 = elem2
    I = np.broadcast_to(np.eye(b1.shape[-1]), A1.shape)
    IpCJ = I + C1 @ J2
    IpJC = I + J2 @ C1
    AIpCJ_inv = mT(np.linalg.solve(mT(IpCJ), mT(A2)))
    AIpJC_inv = mT(np.linalg.solve(mT(IpJC), A1))
    A = AIpCJ_inv @ A1
    b = mv(AIpCJ_inv, b1 + mv(C1, eta2)) + b2
    C = AIpCJ_inv @ C1 @ mT(A2) + C2
    eta = mv(AIpJC_inv, eta2 - mv(J2, b1)) + eta1
    J = AIpJC_inv @ J2 @ A1 + J1
    return A, b, C, eta, J


def standard_smoothing_operator(elem1, elem2):
    """Covariance-form smoothing combine (parsmooth/parallel/_operators.py:80-101)."""
    g1, E1, L1 = elem1
    g2, E2, L2 = elem2
    return mv(E2, g1) + g2, E2 @ E1, E2 @ L1 @ mT(E2) + L2


# ----------------------------------------------------------------------------- elements

def sqrt_filter_elements(F, cholQ, b, H, cholR, c, y, m0, L0):
    """Per-step square-root filtering elements, batched over the leading axis.

    parsmooth/parallel/_filtering.py:115-146.  ``m0, L0`` are the per-step
    priors (the true prior at step 0 and zeros elsewhere, :106-108).
    """
    nx = cholQ.shape[-1]
    ny = cholR.shape[-1]
    m1 = mv(F, m0) + b
    N1 = tria(np.concatenate([F @ L0, cholQ], axis=-1))
    zeros = np.zeros(N1.shape[:-2] + (nx, ny))
    Psi = np.block([[H @ N1, cholR], [N1, zeros]])
    TP = tria(Psi)
    Psi11 = TP[..., :ny, :ny]
    Psi21 = TP[..., ny:ny + nx, :ny]
    U = TP[..., ny:ny + nx, ny:]
    K = mT(np.linalg.solve(mT(Psi11), mT(Psi21)))            # Psi21 Psi11^-1
    HF = H @ F
    A = F - K @ HF
    b_sqr = m1 + mv(K, y - mv(H, m1) - c)
    Z = mT(np.linalg.solve(Psi11, HF))                         # (Psi11^-1 H F)^T
    eta = mv(mT(np.linalg.solve(mT(Psi11), mT(Z))), y - mv(H, b) - c)
    if nx > ny:
        Z = np.concatenate([Z, np.zeros(Z.shape[:-2] + (nx, nx - ny))], axis=-1)
    else:
        Z = tria(Z)
    return A, b_sqr, U, eta, Z


def standard_filter_elements(F, Q, b, H, R, c, y, m0, P0):
    """Covariance-form filtering elements (parsmooth/parallel/_filtering.py:78-97)."""
    m = mv(F, m0) + b
    P = F @ P0 @ mT(F) + Q
    S = H @ P @ mT(H) + R
    S_invH = np.linalg.solve(S, H)
    K = mT(S_invH @ P)
    A = F - K @ H @ F
    b_std = m + mv(K, y - mv(H, m) - c)
    C = P - K @ S @ mT(K)
    temp = mT(S_invH @ F)
    eta = mv(temp, y - mv(H, b) - c)
    J = temp @ H @ F
    return A, b_std, C, eta, J


def sqrt_smoother_elements(F, cholQ, b, m, L):
    """Per-step square-root smoothing elements (parsmooth/parallel/_smoothing.py:72-85)."""
    nx = cholQ.shape[-1]
    Phi = np.block([[F @ L, cholQ], [L, np.zeros_like(cholQ)]])
    TP = tria(Phi)
    Phi11 = TP[..., :nx, :nx]
    Phi21 = TP[..., nx:, :nx]
    D = TP[..., nx:, nx:]
    E = mT(np.linalg.solve(mT(Phi11), mT(Phi21)))
    g = m - mv(E, mv(F, m) + b)
    return g, E, D


def standard_smoother_elements(F, Q, b, m, P):
    """Covariance-form smoothing elements (parsmooth/parallel/_smoothing.py:60-69)."""
    Pp = F @ P @ mT(F) + Q
    E = mT(np.linalg.solve(Pp, F @ P))
    g = m - mv(E, mv(F, m) + b)
    L = P - E @ Pp @ mT(E)
    return g, E, L


# ----------------------------------------------------------------------------- drivers

def _default_nominal(kind, T, nx):
    mean = np.zeros((T, nx))
    chol = np.repeat(np.eye(nx)[None], T, axis=0)
    return kind(mean, chol)


def filtering(observations, x0, transition_model, observation_model, linearization_method,
              nominal_trajectory=None, return_loglikelihood=False, scan=associative_scan):
    """Parallel filter (parsmooth/parallel/_filtering.py:13-61).

    Default nominal is zero means with identity square roots (:25-28).
    Returns ``T+1`` states (the prior prepended, :45-46) and optionally the
    summed log-likelihood (:53-60).
    """
    ys = np.asarray(observations, dtype=float)
    T = ys.shape[0]
    m0, c0 = (np.asarray(v, dtype=float) for v in x0)
    nx = m0.shape[-1]
    if nominal_trajectory is not None:
        are_inputs_compatible(x0, nominal_trajectory)
    else:
        nominal_trajectory = _default_nominal(type(x0), T + 1, nx)
    sqrt = isinstance(x0, MVNSqrt)
    if T == 0:  # an empty sequence: the trajectory is the prior alone
        res = type(x0)(m0[None], c0[None])
        return (res, 0.0) if return_loglikelihood else res
    n_prev = type(x0)(*(np.asarray(v, dtype=float)[:-1] for v in nominal_trajectory))
    n_next = type(x0)(*(np.asarray(v, dtype=float)[1:] for v in nominal_trajectory))
    F, Q_, b = linearization_method(transition_model, n_prev)
    H, R_, c = linearization_method(observation_model, n_next)
    ms = np.concatenate([m0[None], np.zeros((T - 1, nx))])
    Cs = np.concatenate([c0[None], np.zeros((T - 1, nx, nx))])
    if sqrt:
        elems = sqrt_filter_elements(F, Q_, b, H, R_, c, ys, ms, Cs)
        op = sqrt_filtering_operator
    else:
        elems = standard_filter_elements(F, Q_, b, H, R_, c, ys, ms, Cs)
        op = standard_filtering_operator
    _, fm, fc, _, _ = scan(op, elems)
    fm = np.concatenate([m0[None], fm])
    fc = np.concatenate([c0[None], fc])
    res = type(x0)(fm, fc)
    if return_loglikelihood:
        if sqrt:
            ells = sqrt_loglikelihood(F, Q_, b, H, R_, c, fm[:-1], fc[:-1], ys)
        else:
            ells = standard_loglikelihood(F, Q_, b, H, R_, c, fm[:-1], fc[:-1], ys)
        return res, float(np.sum(ells))
    return res


def sqrt_loglikelihood(F, cholQ, b, H, cholR, c, m, L, y):
    """Per-step predictive log-likelihood (parsmooth/parallel/_filtering.py:149-154)."""
    pm = mv(F, m) + b
    pc = tria(np.concatenate([F @ L, cholQ], axis=-1))
    om = mv(H, pm) + c
    oc = tria(np.concatenate([H @ pc, cholR], axis=-1))
    return mvn_loglikelihood(y - om, oc)


def standard_loglikelihood(F, Q, b, H, R, c, m, P, y):
    """Covariance-form per-step log-likelihood (parsmooth/parallel/_filtering.py:157-163)."""
    pm = mv(F, m) + b
    pP = F @ P @ mT(F) + Q
    om = mv(H, pm) + c
    oP = H @ pP @ mT(H) + R
    return mvn_loglikelihood(y - om, np.linalg.cholesky(oP))


def smoothing(transition_model, filter_trajectory, linearization_method, nominal_trajectory=None,
              scan=associative_scan):
    """Parallel smoother (parsmooth/parallel/_smoothing.py:14-57)."""
    fm, fc = (np.asarray(v, dtype=float) for v in filter_trajectory)
    Tp1, nx = fm.shape
    if nominal_trajectory is not None:
        are_inputs_compatible(filter_trajectory, nominal_trajectory)
    else:
        nominal_trajectory = _default_nominal(type(filter_trajectory), Tp1, nx)
    sqrt = isinstance(filter_trajectory, MVNSqrt)
    if Tp1 == 1:
        return type(filter_trajectory)(fm, fc)
    nom = type(filter_trajectory)(*(np.asarray(v, dtype=float)[:-1] for v in nominal_trajectory))
    F, Q_, b = linearization_method(transition_model, nom)
    if sqrt:
        g, E, D = sqrt_smoother_elements(F, Q_, b, fm[:-1], fc[:-1])
        op = sqrt_smoothing_operator
    else:
        g, E, D = standard_smoother_elements(F, Q_, b, fm[:-1], fc[:-1])
        op = standard_smoothing_operator
    g = np.concatenate([g, fm[-1:]])
    E = np.concatenate([E, np.zeros((1, nx, nx))])
    D = np.concatenate([D, fc[-1:]])
    sm, _, sc = scan(op, (g, E, D), reverse=True)
    return type(filter_trajectory)(sm, sc)
