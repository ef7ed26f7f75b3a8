"""The oracle's restatement of the reference's fixed-point derivative (parsmooth/_utils.py:108-133)
on the bearings iterated smoother, checked against central differences of the converged
iterated log-likelihood (CPU)."""
import numpy as np

import oracle as O
from oracle import implicit
from oracle import models as OM


def bearings_theta_models(theta, Q1, dt=0.01, s2=(1.0, 1.0)):
    """theta = (s1x, s1y, log q, log sigma): Q = q Q1, R = sigma^2 I."""
    q, sigma = np.exp(theta[2]), np.exp(theta[3])
    tm = O.FunctionalModel(OM.CoordinatedTurn(dt), O.MVNSqrt(np.zeros(5), np.linalg.cholesky(q * Q1)))
    om = O.FunctionalModel(OM.Bearings((theta[0], theta[1]), s2), O.MVNSqrt(np.zeros(2), sigma * np.eye(2)))
    return tm, om


def converged_problem(T=60, seed=3, n_iter=20):
    from sqrt_parallel_smoothers_gb300 import data
    w = data.bearings_workload(T, seed=seed)
    Q1, _ = OM.bearings_noise(1.0, 5.0, 0.05, 0.01)
    ys = w["ys"].astype(float)
    m0 = np.array([0.1, 0.2, 1.0, 0.0, 1.0])
    nom = O.MVNSqrt(np.repeat(m0[None], T + 1, 0), np.repeat(np.eye(5)[None], T + 1, 0))
    theta = np.array([-1.5, 0.5, np.log(0.1), np.log(0.05)])
    return ys, m0, nom, Q1, theta, n_iter


def iterated_ell(theta, ys, m0, nom, Q1, n_iter, with_traj=False, history=None):
    tm, om = bearings_theta_models(theta, Q1)

    def crit(i, prev, cur):
        if history is not None:
            history.append(float(np.mean((prev.mean - cur.mean) ** 2)))
        return i < n_iter

    traj, ell = O.methods.iterated_smoothing(ys, O.MVNSqrt(m0, np.eye(5)), tm, om, O.linearization.cubature, nom,
                                             True, criterion=crit, return_loglikelihood=True)
    return (traj, ell) if with_traj else ell


def test_implicit_derivative_matches_converged_finite_differences():
    ys, m0, nom, Q1, theta, n_iter = converged_problem()
    hist = []
    x_star, _ = iterated_ell(theta, ys, m0, nom, Q1, n_iter, with_traj=True, history=hist)
    assert hist[-1] < 1e-20                        # converged to rounding: the last calls do not move
    grad, parts = implicit.iterated_loglikelihood_grad(lambda th: bearings_theta_models(th, Q1), theta, ys,
                                                      O.MVNSqrt(m0, np.eye(5)), O.linearization.cubature, x_star,
                                                      n_iter)
    h = 1e-5
    fd = []
    for j in range(4):
        e = np.zeros(4)
        e[j] = h
        fd.append((iterated_ell(theta + e, ys, m0, nom, Q1, n_iter) -
                   iterated_ell(theta - e, ys, m0, nom, Q1, n_iter)) / (2 * h))
    fd = np.array(fd)
    rel = np.abs(grad - fd) / np.maximum(np.abs(fd), 1.0)
    assert np.all(rel < 1e-5), (grad, fd, rel)
    # the nominal's dependence on theta contributes
    assert np.max(np.abs(parts["fixed_point"]) / np.maximum(np.abs(fd), 1.0)) > 1e-4
