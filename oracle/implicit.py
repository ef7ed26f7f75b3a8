"""Implicit-function derivative of the iterated smoother (TEST INFRASTRUCTURE ONLY).

Restates the custom VJP of the reference's fixed point (parsmooth/_utils.py:108-133).  At the
fixed point ``x* = f(x*, theta)`` reached after ``n_iter`` counted calls, a cotangent ``x_bar``
of ``x*`` maps to ``theta_bar = (df/dtheta)^T u`` where ``u`` comes from the fixed-point
iteration ``u <- x_bar + (df/dx)^T u`` started at ``u = x_bar`` and run for ``n_iter + 1``
calls (criterion ``i < n_iter + 1``, :118-122), i.e. the truncated Neumann series
``u = sum_{k=0}^{n_iter+1} ((df/dx)^T)^k x_bar`` with every Jacobian evaluated at ``x*``.

The oracle has no automatic differentiation, so it forms the same number in forward form: for
a parameter direction ``e_j``, ``x_bar^T sum_k (df/dx)^k (df/dtheta) e_j``, which equals
``u^T (df/dtheta) e_j``.  Every Jacobian-vector product is a central difference of the FP64
oracle's filter-smoother map.  For the log-likelihood of ``iterated_smoothing(...,
return_loglikelihood=True)`` (parsmooth/methods.py:72-75) the cotangent is ``x_bar =
d ell / d x*`` of the final filtering pass, and the total derivative is
``d ell / d theta = (d ell / d theta)|_{x*} + x_bar^T dx*/dtheta``.
"""
import numpy as np

from . import methods as M
from .types import MVNSqrt


def _pack(x):
    """Trajectory -> flat vector of its means and the lower triangles of its factors."""
    m, L = np.asarray(x.mean, float), np.asarray(x.chol, float)
    il = np.tril_indices(L.shape[-1])
    return np.concatenate([m.ravel(), L[:, il[0], il[1]].ravel()])


def _unpack(v, T1, nx):
    il = np.tril_indices(nx)
    m = v[:T1 * nx].reshape(T1, nx)
    L = np.zeros((T1, nx, nx))
    L[:, il[0], il[1]] = v[T1 * nx:].reshape(T1, -1)
    return MVNSqrt(m, L)


def iterated_loglikelihood_grad(make_models, theta, ys, x0, method, x_star, n_iter, h_x=1e-6, h_theta=1e-6):
    """``d ell / d theta`` of the reference's iterated smoother with ``return_loglikelihood`` at
    the fixed point ``x_star`` (an ``MVNSqrt`` trajectory) after ``n_iter`` calls.

    ``make_models(theta) -> (transition_model, observation_model)``.  Returns
    ``(grad, parts)`` with ``parts`` holding the direct term and the fixed-point term."""
    theta = np.asarray(theta, float)
    T1, nx = np.shape(x_star.mean)
    xs = _pack(x_star)

    def f(v, th):
        tm, om = make_models(th)
        return _pack(M.filter_smoother(ys, x0, tm, om, method, _unpack(v, T1, nx), True))

    def ell(v, th):
        tm, om = make_models(th)
        _, e = M.filtering(ys, x0, tm, om, method, _unpack(v, T1, nx), True, return_loglikelihood=True)
        return e

    def jvp(fun, v, d, h):
        s = np.max(np.abs(d))
        if s == 0:
            return 0.0 * fun(v, theta)
        dn = d / s
        return s * (fun(v + h * dn, theta) - fun(v - h * dn, theta)) / (2 * h)

    direct, through = np.zeros(len(theta)), np.zeros(len(theta))
    for j in range(len(theta)):
        e = np.zeros(len(theta))
        e[j] = h_theta
        direct[j] = (ell(xs, theta + e) - ell(xs, theta - e)) / (2 * h_theta)
        w = (f(xs, theta + e) - f(xs, theta - e)) / (2 * h_theta)   # (df/dtheta) e_j
        acc = w.copy()
        for _ in range(n_iter + 1):                                  # terms k = 1 .. n_iter + 1
            w = jvp(f, xs, w, h_x)
            acc = acc + w
        through[j] = jvp(ell, xs, acc, h_x)
    return direct + through, {"direct": direct, "fixed_point": through}
