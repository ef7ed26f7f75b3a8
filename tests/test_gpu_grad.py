"""Forward-mode (tangent-linear) gradients of the filter log-likelihood, checked
against central finite differences of the FP64 oracle (h = 1e-3 for the
bearings parameters, as the reference's parameter-estimation study uses them;
h = 1e-5 for the linear-model entries).

Tolerances: FP64 runs 1e-6 relative (finite-difference truncation dominates),
FP32 runs 1e-3 relative on these short sequences."""
import numpy as np
import pytest
import torch

import oracle as O
import sqrt_parallel_smoothers_gb300 as S
from tests._parity import linear_pair, np_

pytestmark = pytest.mark.gpu


def _oracle_ell(ys, m0, L0, A, b, cQ, H, c, cR, method, nom=None):
    tm = O.FunctionalModel(O.models.LinearFunction(A), O.MVNSqrt(b, cQ))
    om = O.FunctionalModel(O.models.LinearFunction(H), O.MVNSqrt(c, cR))
    _, ell = O.methods.filtering(ys, O.MVNSqrt(m0, L0), tm, om, method, nom, True, return_loglikelihood=True)
    return ell


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-6), (torch.float32, 1e-3)])
@pytest.mark.parametrize("method", ["extended", "cubature"])
def test_linear_directions_vs_fd(dtype, tol, method):
    rng = np.random.RandomState(0)
    T = 40
    A = np.array([[0.9, 0.1], [-0.2, 0.95]])
    H = np.array([[1.0, 0.0], [0.3, 1.0]])
    b, c = rng.randn(2) * 0.1, rng.randn(2) * 0.1
    cQ = np.array([[0.3, 0.0], [0.1, 0.2]])
    cR = np.array([[0.5, 0.0], [0.2, 0.4]])
    m0, L0 = np.zeros(2), np.eye(2)
    from sqrt_parallel_smoothers_gb300.data import lgssm_data
    _, ys = lgssm_data(m0, A, H, cR @ cR.T, cQ @ cQ.T, b, c, T, random_state=1)
    ys = ys.astype(np.float64)
    dA = np.array([[1.0, 0.0], [0.0, 0.0]])
    dH = np.array([[0.0, 0.0], [1.0, 0.0]])
    dcQ = np.array([[1.0, 0.0], [0.0, 0.0]])
    dcR = np.array([[0.0, 0.0], [0.0, 1.0]])
    db = np.array([0.0, 1.0])
    dirs_np = [dict(A=dA), dict(H=dH), dict(cQ=dcQ), dict(cR=dcR, b=db)]
    meth = {"extended": O.linearization.extended, "cubature": O.linearization.cubature}[method]
    h = 1e-5
    fd = []
    for d in dirs_np:
        def at(e):
            return _oracle_ell(ys, m0, L0, A + e * d.get("A", 0), b + e * d.get("b", 0), cQ + e * d.get("cQ", 0),
                               H + e * d.get("H", 0), c, cR + e * d.get("cR", 0), meth)
        fd.append((at(h) - at(-h)) / (2 * h))
    _, gt = linear_pair(A, b, cQ)
    _, go = linear_pair(H, c, cR)
    dirs = [(S.ModelTangent(matrix=torch.as_tensor(dA)), S.ModelTangent()),
            (S.ModelTangent(), S.ModelTangent(matrix=torch.as_tensor(dH))),
            (S.ModelTangent(noise_chol=torch.as_tensor(dcQ)), S.ModelTangent()),
            (S.ModelTangent(noise_mean=torch.as_tensor(db)), S.ModelTangent(noise_chol=torch.as_tensor(dcR)))]
    ell, grad = S.filter_loglikelihood_grad(torch.as_tensor(ys, dtype=dtype),
                                            S.MVNSqrt(torch.as_tensor(m0), torch.as_tensor(L0)), gt, go,
                                            getattr(S.linearization, method), None, dirs)
    ref_ell = _oracle_ell(ys, m0, L0, A, b, cQ, H, c, cR, meth)
    assert abs(float(ell) - ref_ell) <= tol * abs(ref_ell)
    g = np_(grad)
    for k in range(4):
        assert abs(g[k] - fd[k]) <= tol * max(1.0, abs(fd[k])), (k, g[k], fd[k])


def _bearings_ell_oracle(theta, ys, m0, nom, Q1, dt=0.01, s2=(1.0, 1.0)):
    s1 = (theta[0], theta[1])
    q, sigma = np.exp(theta[2]), np.exp(theta[3])
    tm = O.FunctionalModel(O.models.CoordinatedTurn(dt), O.MVNSqrt(np.zeros(5), np.linalg.cholesky(q * Q1)))
    om = O.FunctionalModel(O.models.Bearings(s1, s2), O.MVNSqrt(np.zeros(2), sigma * np.eye(2)))
    _, ell = O.methods.filtering(ys, O.MVNSqrt(m0, np.eye(5)), tm, om, O.linearization.cubature, nom, True,
                                 return_loglikelihood=True)
    return ell


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-5), (torch.float32, 2e-3)])
def test_bearings_theta_gradient_autograd(dtype, tol):
    T = 300
    w = S.data.bearings_workload(T, seed=4)
    Q1, _ = S.data.bearings_noise(1.0, 5.0, 0.05, 0.01)
    ys = w["ys"].astype(np.float64)
    m0 = np.array([0.1, 0.2, 1.0, 0.0, 1.0])
    nom_m = np.repeat(m0[None], T + 1, 0)
    nom_L = np.repeat(np.eye(5)[None], T + 1, 0)
    theta0 = np.array([-1.5, 0.5, np.log(0.1), np.log(0.05)])
    h = 1e-3
    fd = []
    for k in range(4):
        e = np.zeros(4)
        e[k] = h
        fd.append((_bearings_ell_oracle(theta0 + e, ys, m0, O.MVNSqrt(nom_m, nom_L), Q1) -
                   _bearings_ell_oracle(theta0 - e, ys, m0, O.MVNSqrt(nom_m, nom_L), Q1)) / (2 * h))
    fd = np.array(fd)
    theta = torch.tensor(theta0, dtype=torch.float64, requires_grad=True)
    ell = S.BearingsLogLikelihood.apply(theta, torch.as_tensor(ys, dtype=dtype),
                                        S.MVNSqrt(torch.as_tensor(m0), torch.eye(5, dtype=torch.float64)),
                                        S.MVNSqrt(torch.as_tensor(nom_m), torch.as_tensor(nom_L)), Q1, 0.01,
                                        (1.0, 1.0), S.linearization.cubature, None, None)
    ell.backward()
    g = theta.grad.numpy()
    rel = np.abs(g - fd) / np.maximum(np.abs(fd), 1.0)
    assert np.all(rel <= tol), (g, fd, rel)


def _bearings_iterated_ell_oracle(theta, ys, m0, nom, Q1, n_iter, dt=0.01, s2=(1.0, 1.0)):
    s1 = (theta[0], theta[1])
    q, sigma = np.exp(theta[2]), np.exp(theta[3])
    tm = O.FunctionalModel(O.models.CoordinatedTurn(dt), O.MVNSqrt(np.zeros(5), np.linalg.cholesky(q * Q1)))
    om = O.FunctionalModel(O.models.Bearings(s1, s2), O.MVNSqrt(np.zeros(2), sigma * np.eye(2)))
    _, ell = O.methods.iterated_smoothing(ys, O.MVNSqrt(m0, np.eye(5)), tm, om, O.linearization.cubature, nom,
                                          True, criterion=lambda i, *_: i < n_iter, return_loglikelihood=True)
    return ell


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-5), (torch.float32, 2e-3)])
def test_bearings_theta_gradient_through_iterations(dtype, tol):
    """d/dtheta of the iterated smoother's log-likelihood (5 Gauss-Newton calls, the nominal's
    dependence on theta included) against central differences of the oracle's iterated
    log-likelihood."""
    T, n_iter = 150, 5
    w = S.data.bearings_workload(T, seed=3)
    Q1, _ = S.data.bearings_noise(1.0, 5.0, 0.05, 0.01)
    ys = w["ys"].astype(np.float64)
    m0 = np.array([0.1, 0.2, 1.0, 0.0, 1.0])
    nom_m = np.repeat(m0[None], T + 1, 0)
    nom_L = np.repeat(np.eye(5)[None], T + 1, 0)
    theta0 = np.array([-1.5, 0.5, np.log(0.1), np.log(0.05)])
    h = 1e-4
    fd = []
    for k in range(4):
        e = np.zeros(4)
        e[k] = h
        fd.append((_bearings_iterated_ell_oracle(theta0 + e, ys, m0, O.MVNSqrt(nom_m, nom_L), Q1, n_iter) -
                   _bearings_iterated_ell_oracle(theta0 - e, ys, m0, O.MVNSqrt(nom_m, nom_L), Q1, n_iter)) / (2 * h))
    fd = np.array(fd)
    theta = torch.tensor(theta0, dtype=torch.float64, requires_grad=True)
    ell = S.BearingsLogLikelihood.apply(theta, torch.as_tensor(ys, dtype=dtype),
                                        S.MVNSqrt(torch.as_tensor(m0), torch.eye(5, dtype=torch.float64)),
                                        S.MVNSqrt(torch.as_tensor(nom_m), torch.as_tensor(nom_L)), Q1, 0.01,
                                        (1.0, 1.0), S.linearization.cubature, None, None, n_iter)
    ell_ref = _bearings_iterated_ell_oracle(theta0, ys, m0, O.MVNSqrt(nom_m, nom_L), Q1, n_iter)
    assert abs(float(ell.detach()) - ell_ref) <= tol * abs(ell_ref)
    ell.backward()
    g = theta.grad.numpy()
    rel = np.abs(g - fd) / np.maximum(np.abs(fd), 1.0)
    assert np.all(rel <= tol), (g, fd, rel)
    # the nominal's dependence matters: the fixed-nominal filter gradient differs
    dirs_only = S.BearingsLogLikelihood.apply(theta.detach().clone().requires_grad_(True),
                                              torch.as_tensor(ys, dtype=dtype),
                                              S.MVNSqrt(torch.as_tensor(m0), torch.eye(5, dtype=torch.float64)),
                                              S.MVNSqrt(torch.as_tensor(nom_m), torch.as_tensor(nom_L)), Q1, 0.01,
                                              (1.0, 1.0), S.linearization.cubature, None, None)
    assert abs(float(dirs_only.detach()) - float(ell.detach())) > 1e-6 * abs(float(ell.detach()))


def test_iterated_gradient_equals_implicit_derivative_at_fixed_point():
    """At a converged bearings fixed point (20 calls, FP64) the derivative of the unrolled
    iteration (ss_iterated_grad) equals the reference's implicit-function derivative
    (parsmooth/_utils.py:108-133: the truncated Neumann series of n_iter + 1 adjoint sweeps),
    restated in oracle/implicit.py."""
    from oracle import implicit
    from tests.test_oracle_implicit import bearings_theta_models, converged_problem, iterated_ell
    ys, m0, nom, Q1, theta0, n_iter = converged_problem()
    x_star, _ = iterated_ell(theta0, ys, m0, nom, Q1, n_iter, with_traj=True)
    ref, _ = implicit.iterated_loglikelihood_grad(lambda th: bearings_theta_models(th, Q1), theta0, ys,
                                                 O.MVNSqrt(m0, np.eye(5)), O.linearization.cubature, x_star, n_iter)
    theta = torch.tensor(theta0, dtype=torch.float64, requires_grad=True)
    ell = S.BearingsLogLikelihood.apply(theta, torch.as_tensor(ys),
                                        S.MVNSqrt(torch.as_tensor(m0), torch.eye(5, dtype=torch.float64)),
                                        S.MVNSqrt(torch.as_tensor(nom.mean), torch.as_tensor(nom.chol)), Q1, 0.01,
                                        (1.0, 1.0), S.linearization.cubature, None, None, n_iter)
    ell.backward()
    g = theta.grad.numpy()
    rel = np.abs(g - ref) / np.maximum(np.abs(ref), 1.0)
    assert np.all(rel <= 1e-6), (g, ref, rel)
