"""The oracle's reverse-mode gradient of the filter log-likelihood (smoothed moments, Fisher's
identity) against central differences of the oracle's parallel filter log-likelihood
(parsmooth/parallel/_filtering.py:13-61 with return_loglikelihood), FP64, CPU."""
import numpy as np
import pytest

import oracle as O
from oracle import adjoint
from oracle import models as OM

from _systems import lgssm


def _ell(ys, m0, L0, F, Lq, bq, H, Lr, cr, nominal=None):
    tm = O.FunctionalModel(OM.LinearFunction(F), O.MVNSqrt(bq, Lq))
    om = O.FunctionalModel(OM.LinearFunction(H), O.MVNSqrt(cr, Lr))
    _, ell = O.parallel.filtering(ys, O.MVNSqrt(m0, L0), tm, om, O.linearization.extended, nominal,
                                  return_loglikelihood=True)
    return ell


def _fd(f, x, h=1e-6, mask=None):
    g = np.zeros_like(x)
    for idx in np.ndindex(x.shape):
        if mask is not None and not mask[idx]:
            continue
        e = np.zeros_like(x)
        e[idx] = h
        g[idx] = (f(x + e) - f(x - e)) / (2 * h)
    return g


@pytest.mark.parametrize("nx,ny", [(4, 2), (3, 3), (2, 1)])
def test_linear_model_adjoints_match_finite_differences(nx, ny):
    s = lgssm(nx, ny, 25, seed=nx * 10 + ny)
    ys = s["ys"].astype(float)
    m0, L0 = s["chol_x0"].mean, s["chol_x0"].chol
    args = dict(F=s["F"], Lq=s["cholQ"], bq=s["b"], H=s["H"], Lr=s["cholR"], cr=s["c"])
    tm = O.FunctionalModel(OM.LinearFunction(s["F"]), O.MVNSqrt(s["b"], s["cholQ"]))
    om = O.FunctionalModel(OM.LinearFunction(s["H"]), O.MVNSqrt(s["c"], s["cholR"]))
    ell, adj = adjoint.filter_adjoint(ys, O.MVNSqrt(m0, L0), tm, om, O.linearization.extended)
    got = adjoint.linear_model_adjoints(adj, s["cholQ"], s["cholR"])
    assert np.isclose(ell, _ell(ys, m0, L0, **args))
    low_x, low_y = np.tril(np.ones((nx, nx), bool)), np.tril(np.ones((ny, ny), bool))
    checks = {
        "trans_matrix": ("F", None), "trans_noise_mean": ("bq", None), "trans_noise_chol": ("Lq", low_x),
        "obs_matrix": ("H", None), "obs_noise_mean": ("cr", None), "obs_noise_chol": ("Lr", low_y),
    }
    for key, (arg, mask) in checks.items():
        def f(v, arg=arg):
            a = dict(args)
            a[arg] = v
            return _ell(ys, m0, L0, **a)
        fd = _fd(f, np.array(args[arg], float), mask=mask)
        np.testing.assert_allclose(got[key], fd, rtol=1e-5, atol=1e-6 * max(1.0, np.abs(fd).max()), err_msg=key)
    fd_m0 = _fd(lambda v: _ell(ys, v, L0, **args), np.array(m0, float))
    np.testing.assert_allclose(got["m0"], fd_m0, rtol=1e-5, atol=1e-7)
    fd_L0 = _fd(lambda v: _ell(ys, m0, v, **args), np.array(L0, float), mask=low_x)
    np.testing.assert_allclose(got["L0"], fd_L0, rtol=1e-5, atol=1e-7)


def test_linear_model_adjoint_at_a_nominal_is_independent_of_it():
    """For a linear model the linearisation does not depend on the nominal, nor does the gradient."""
    s = lgssm(3, 2, 20, seed=5)
    ys = s["ys"].astype(float)
    x0 = O.MVNSqrt(s["chol_x0"].mean, s["chol_x0"].chol)
    tm = O.FunctionalModel(OM.LinearFunction(s["F"]), O.MVNSqrt(s["b"], s["cholQ"]))
    om = O.FunctionalModel(OM.LinearFunction(s["H"]), O.MVNSqrt(s["c"], s["cholR"]))
    nom = O.MVNSqrt(s["m_nominal"], np.repeat(np.eye(3)[None], 21, 0))
    _, a1 = adjoint.filter_adjoint(ys, x0, tm, om, O.linearization.cubature, nom)
    _, a2 = adjoint.filter_adjoint(ys, x0, tm, om, O.linearization.extended)
    for k in ("F", "b", "H", "c", "A_q", "A_r"):
        np.testing.assert_allclose(a1[k], a2[k], atol=1e-9)


def _bearings_models(theta, Q1, dt=0.01, s2=(1.0, 1.0)):
    q, sigma = np.exp(theta[2]), np.exp(theta[3])
    tm = O.FunctionalModel(OM.CoordinatedTurn(dt), O.MVNSqrt(np.zeros(5), np.linalg.cholesky(q * Q1)))
    om = O.FunctionalModel(OM.Bearings((theta[0], theta[1]), s2), O.MVNSqrt(np.zeros(2), sigma * np.eye(2)))
    return tm, om


def bearings_theta_gradient(method, theta, ys, x0, nom, Q1, h=1e-6):
    """d ell / d (s1x, s1y, log q, log sigma) at a fixed nominal from the oracle adjoint: the sensor
    coordinates through the per-step observation linearisation, the noise scales through the
    noise factors (L_Q = sqrt(q) chol(Q1): d L_Q / d log q = L_Q / 2; d L_R / d log sigma = L_R)."""
    tm, om = _bearings_models(theta, Q1)
    ell, adj = adjoint.filter_adjoint(ys, x0, tm, om, method, nom)
    T = ys.shape[0]
    n_next = O.MVNSqrt(nom.mean[1:], nom.chol[1:])
    g = np.zeros(4)
    for j in range(2):
        e = np.zeros(4)
        e[j] = h
        lp = method(_bearings_models(theta + e, Q1)[1], n_next)
        lm = method(_bearings_models(theta - e, Q1)[1], n_next)
        g[j] = adjoint.param_adjoint(adj, 1, lp, lm, h)
    Lq, Lr = tm.mvn.chol, om.mvn.chol
    g[2] = np.sum(adjoint.noise_chol_adjoint(adj["A_q"], adj["lin"][1], Lq) * (0.5 * Lq))
    g[3] = np.sum(adjoint.noise_chol_adjoint(adj["A_r"], adj["lin"][4], Lr) * Lr)
    assert adj["F"].shape[0] == T
    return ell, g


@pytest.mark.parametrize("method", ["cubature", "extended", "unscented"])
def test_bearings_parameter_gradient_matches_finite_differences(method):
    from sqrt_parallel_smoothers_gb300 import data
    T = 40
    w = data.bearings_workload(T, seed=7)
    ys = w["ys"].astype(float)
    Q1, _ = OM.bearings_noise(1.0, 5.0, 0.05, 0.01)
    m0 = np.array([0.1, 0.2, 1.0, 0.0, 1.0])
    x0 = O.MVNSqrt(m0, np.eye(5))
    rng = np.random.RandomState(1)
    nom = O.MVNSqrt(np.repeat(m0[None], T + 1, 0) + 0.05 * rng.randn(T + 1, 5),
                    np.repeat(0.3 * np.eye(5)[None], T + 1, 0))
    theta = np.array([-1.5, 0.5, np.log(0.1), np.log(0.05)])
    lin = getattr(O.linearization, method)
    ell, g = bearings_theta_gradient(lin, theta, ys, x0, nom, Q1)

    def ell_of(th):
        tm, om = _bearings_models(th, Q1)
        return O.parallel.filtering(ys, x0, tm, om, lin, nom, return_loglikelihood=True)[1]

    h = 1e-6
    fd = np.array([(ell_of(theta + h * e) - ell_of(theta - h * e)) / (2 * h) for e in np.eye(4)])
    assert np.isclose(ell, ell_of(theta))
    np.testing.assert_allclose(g, fd, rtol=2e-6, atol=1e-6 * np.abs(fd).max())


@pytest.mark.parametrize("method", ["extended", "cubature"])
def test_predicted_moment_form_equals_residual_form(method):
    """The GPU kernel's transition contraction (predicted moments, no state differences) equals
    the residual form of filter_adjoint: dl/dF, dl/db and dl/dQ = cQ^-T A_q cQ^-1 / 2."""
    from sqrt_parallel_smoothers_gb300 import data
    T = 30
    w = data.bearings_workload(T, seed=4)
    ys = w["ys"].astype(float)
    Q1, _ = OM.bearings_noise(1.0, 5.0, 0.05, 0.01)
    m0 = np.array([0.1, 0.2, 1.0, 0.0, 1.0])
    x0 = O.MVNSqrt(m0, np.eye(5))
    tm, om = _bearings_models(np.array([-1.5, 0.5, np.log(0.1), np.log(0.05)]), Q1)
    lin = getattr(O.linearization, method)
    nom = O.MVNSqrt(np.repeat(m0[None], T + 1, 0), np.repeat(0.3 * np.eye(5)[None], T + 1, 0))
    _, adj = adjoint.filter_adjoint(ys, x0, tm, om, lin, nom)
    F, cQ, b = adj["lin"][:3]
    filt = O.parallel.filtering(ys, x0, tm, om, lin, nom)
    sm = O.parallel.smoothing(tm, filt, lin, nom)
    Fbar, bbar, Qbar = adjoint.transition_adjoint_predicted_form(F, cQ, b, np.asarray(filt[0]), np.asarray(filt[1]),
                                                                 np.asarray(sm[0]), np.asarray(sm[1]))
    Qbar_res = 0.5 * adjoint._unwhiten_T(cQ, np.swapaxes(adjoint._unwhiten_T(cQ, adj["A_q"]), -1, -2))
    for got, ref in ((Fbar, adj["F"]), (bbar, adj["b"]), (Qbar, Qbar_res)):
        np.testing.assert_allclose(got, ref, rtol=1e-7, atol=1e-9 * np.abs(ref).max())
