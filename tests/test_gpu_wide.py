"""Six- to eight-state models on the thread-per-chunk kernels, against the FP64 oracle.

A 2-D constant-acceleration target (nx = 6: position, velocity, acceleration; linear
transition) seen through two bearings (ny = 2) with the iterated sigma-point smoother; a
six- to eight-state Ricker population (nonlinear transition, linear counts); random
linear systems at (8, 1).  FP64 within 1e-9 of the oracle (1e-8 where the sigma-point
regression of a nonlinear model enters), FP32 within a position RMSE of 1 % of FP64's."""
import numpy as np
import pytest
import torch

import oracle as O
from oracle import models as OM
import sqrt_parallel_smoothers_gb300 as S
from sqrt_parallel_smoothers_gb300 import models as GM
from tests._parity import assert_rel, np_
from tests._systems import lgssm

pytestmark = pytest.mark.gpu


def constant_acceleration(dt=0.05, q=1e-5):
    """x = (px, py, vx, vy, ax, ay), white-noise jerk of intensity q."""
    I2, Z2 = np.eye(2), np.zeros((2, 2))
    F = np.block([[I2, dt * I2, dt ** 2 / 2 * I2], [Z2, I2, dt * I2], [Z2, Z2, I2]])
    Q = q * np.block([[dt ** 5 / 20 * I2, dt ** 4 / 8 * I2, dt ** 3 / 6 * I2],
                      [dt ** 4 / 8 * I2, dt ** 3 / 3 * I2, dt ** 2 / 2 * I2],
                      [dt ** 3 / 6 * I2, dt ** 2 / 2 * I2, dt * I2]])
    return F, Q


def ca_bearings_problem(T, seed=0, sigma=0.02):
    F, Q = constant_acceleration()
    rng = np.random.RandomState(seed)
    cQ = np.linalg.cholesky(Q)
    s1, s2 = (-1.5, 0.5), (1.0, 1.0)
    x = np.array([0.1, 0.2, 0.1, 0.05, 0.0, 0.0])
    xs, ys = [x], []
    h = OM.Bearings(s1, s2, d_in=6)
    for _ in range(T):
        x = F @ x + cQ @ rng.randn(6)
        xs.append(x)
        ys.append(h(x) + sigma * rng.randn(2))
    m0 = np.array([0.1, 0.2, 0.1, 0.05, 0.0, 0.0])
    L0 = np.diag([0.1, 0.1, 0.1, 0.1, 0.05, 0.05])
    return dict(F=F, cQ=cQ, s1=s1, s2=s2, sigma=sigma, m0=m0, L0=L0, ys=np.array(ys), xs=np.array(xs))


@pytest.mark.parametrize("method,tol", [("cubature", 1e-8), ("unscented", 1e-8), ("extended", 1e-9)])
def test_constant_acceleration_bearings_iterated_fp64(method, tol):
    p = ca_bearings_problem(60, seed=1)
    cR = p["sigma"] * np.eye(2)
    ot = O.FunctionalModel(OM.LinearFunction(p["F"]), O.MVNSqrt(np.zeros(6), p["cQ"]))
    oo = O.FunctionalModel(OM.Bearings(p["s1"], p["s2"], d_in=6), O.MVNSqrt(np.zeros(2), cR))
    gt = S.FunctionalModel(GM.LinearModel(p["F"]), S.MVNSqrt(torch.zeros(6, dtype=torch.float64),
                                                              torch.as_tensor(p["cQ"])))
    go = S.FunctionalModel(GM.Bearings(p["s1"], p["s2"], d_in=6), S.MVNSqrt(torch.zeros(2, dtype=torch.float64),
                                                                            torch.as_tensor(cR)))
    T = p["ys"].shape[0]
    nom_o = O.MVNSqrt(np.repeat(p["m0"][None], T + 1, 0), np.repeat(p["L0"][None], T + 1, 0))
    ref, ell_ref = O.methods.iterated_smoothing(p["ys"], O.MVNSqrt(p["m0"], p["L0"]), ot, oo,
                                                getattr(O.linearization, method), nom_o, True,
                                                criterion=lambda i, *_: i < 5, return_loglikelihood=True)
    nom = S.MVNSqrt(torch.as_tensor(nom_o.mean), torch.as_tensor(nom_o.chol))
    res, ell = S.iterated_smoothing(torch.as_tensor(p["ys"]), S.MVNSqrt(torch.as_tensor(p["m0"]),
                                                                         torch.as_tensor(p["L0"])),
                                    gt, go, getattr(S.linearization, method), nom,
                                    criterion=S.FixedIterations(5), return_loglikelihood=True)
    assert_rel(res.mean, ref.mean, tol, "means")
    L = np_(res.chol)
    assert_rel(L @ np.swapaxes(L, -1, -2), ref.chol @ np.swapaxes(ref.chol, -1, -2), tol, "covariances")
    assert abs(float(ell) - ell_ref) <= tol * max(1.0, abs(ell_ref))


def test_constant_acceleration_bearings_fp32_rmse():
    """FP32 (staged kernels at nx = 6) against FP64 on a longer track (the FP64 oracle's 10 calls
    converge on it, position RMSE 0.006): position RMSE within 1 %."""
    p = ca_bearings_problem(400, seed=2)
    cR = p["sigma"] * np.eye(2)
    gt = S.FunctionalModel(GM.LinearModel(p["F"]), S.MVNSqrt(torch.zeros(6, dtype=torch.float64),
                                                              torch.as_tensor(p["cQ"])))
    go = S.FunctionalModel(GM.Bearings(p["s1"], p["s2"], d_in=6), S.MVNSqrt(torch.zeros(2, dtype=torch.float64),
                                                                            torch.as_tensor(cR)))
    x0 = S.MVNSqrt(torch.as_tensor(p["m0"]), torch.as_tensor(p["L0"]))
    T = p["ys"].shape[0]
    rmse = {}
    for dtype in (torch.float64, torch.float32):
        nom = S.MVNSqrt(torch.as_tensor(np.repeat(p["m0"][None], T + 1, 0)),
                        torch.as_tensor(np.repeat(p["L0"][None], T + 1, 0)))
        res = S.iterated_smoothing(torch.as_tensor(p["ys"], dtype=dtype), x0, gt, go, S.linearization.cubature,
                                   nom, criterion=S.FixedIterations(10))
        m = np_(res.mean)
        assert np.all(np.isfinite(m))
        rmse[dtype] = float(np.sqrt(np.mean(np.sum((m[:, :2] - p["xs"][:, :2]) ** 2, -1))))
    assert abs(rmse[torch.float32] - rmse[torch.float64]) <= 0.01 * rmse[torch.float64], rmse


@pytest.mark.parametrize("nx,ny,method", [(7, 2, "cubature"), (8, 2, "unscented"), (7, 1, "extended"),
                                           (6, 3, "gauss_hermite")])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_ricker_population_filter_smoother(nx, ny, method, dtype):
    """Ricker transition (nonlinear, elementwise; growth a = 0.5, stable about its fixed point
    log a) with linear counts of the first ny species."""
    rng = np.random.RandomState(nx * 10 + ny)
    T = 40 if method == "gauss_hermite" else 80
    a = 0.5
    cQ = np.tril(0.05 * rng.rand(nx, nx)) + 0.2 * np.eye(nx)
    H = np.eye(ny, nx) + 0.1 * rng.rand(ny, nx)
    cR = 0.3 * np.eye(ny)
    x = np.full(nx, np.log(a))
    ys = []
    for _ in range(T):
        x = OM.Ricker(a)(x) + cQ @ rng.randn(nx)
        ys.append(H @ x + cR @ rng.randn(ny))
    ys = np.array(ys)
    m0, L0 = np.full(nx, np.log(a)), 0.5 * np.eye(nx)
    ot = O.FunctionalModel(OM.Ricker(a), O.MVNSqrt(np.zeros(nx), cQ))
    oo = O.FunctionalModel(OM.LinearFunction(H), O.MVNSqrt(np.zeros(ny), cR))
    lin_o = getattr(O.linearization, method)
    nom_o = O.MVNSqrt(np.repeat(m0[None], T + 1, 0), np.repeat(L0[None], T + 1, 0))
    ref = O.methods.filter_smoother(ys, O.MVNSqrt(m0, L0), ot, oo, lin_o, nom_o)
    gt = S.FunctionalModel(GM.Ricker(a, d=nx), S.MVNSqrt(torch.zeros(nx, dtype=torch.float64), torch.as_tensor(cQ)))
    go = S.FunctionalModel(GM.LinearModel(H), S.MVNSqrt(torch.zeros(ny, dtype=torch.float64), torch.as_tensor(cR)))
    nom = S.MVNSqrt(torch.as_tensor(nom_o.mean), torch.as_tensor(nom_o.chol))
    res = S.filter_smoother(torch.as_tensor(ys, dtype=dtype), S.MVNSqrt(torch.as_tensor(m0), torch.as_tensor(L0)),
                            gt, go, getattr(S.linearization, method), nom)
    tol = 1e-8 if dtype == torch.float64 else 2e-3
    assert_rel(res.mean, ref.mean, tol, "means")
    L = np_(res.chol)
    assert_rel(L @ np.swapaxes(L, -1, -2), ref.chol @ np.swapaxes(ref.chol, -1, -2), tol, "covariances")


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-9), (torch.float32, 5e-3)])
def test_linear_8_1_ragged_batch(dtype, tol):
    s = lgssm(8, 1, 5, seed=8)
    from sqrt_parallel_smoothers_gb300.data import lgssm_data
    lengths = [35, 0, 70, 12]
    ys = [lgssm_data(s["x0"].mean, s["F"], s["H"], s["R"], s["Q"], s["b"], s["c"], max(T, 1),
                     random_state=i)[1][:T] for i, T in enumerate(lengths)]
    ot = O.FunctionalModel(OM.LinearFunction(s["F"]), O.MVNSqrt(s["b"], s["cholQ"]))
    oo = O.FunctionalModel(OM.LinearFunction(s["H"]), O.MVNSqrt(s["c"], s["cholR"]))
    gt = S.FunctionalModel(GM.LinearModel(s["F"]), S.MVNSqrt(torch.as_tensor(s["b"]), torch.as_tensor(s["cholQ"])))
    go = S.FunctionalModel(GM.LinearModel(s["H"]), S.MVNSqrt(torch.as_tensor(s["c"]), torch.as_tensor(s["cholR"])))
    x0o = O.MVNSqrt(s["chol_x0"].mean, s["chol_x0"].chol)
    x0 = S.MVNSqrt(torch.as_tensor(x0o.mean), torch.as_tensor(x0o.chol))
    packed = torch.as_tensor(np.concatenate([y.reshape(-1, 1) for y in ys]).astype(np.float64), dtype=dtype)
    offsets = np.concatenate([[0], np.cumsum(lengths)])
    res = S.filter_smoother(packed, x0, gt, go, S.linearization.extended, None, offsets=offsets)
    m, L = np_(res.mean), np_(res.chol)
    start = 0
    for y, T in zip(ys, lengths):
        ref = O.methods.filter_smoother(y.astype(float).reshape(T, 1), x0o, ot, oo, O.linearization.extended)
        sl = slice(start, start + T + 1)
        assert_rel(m[sl], ref.mean, tol, f"means T={T}")
        P = L[sl] @ np.swapaxes(L[sl], -1, -2)
        assert_rel(P, ref.chol @ np.swapaxes(ref.chol, -1, -2), tol, f"covariances T={T}")
        start += T + 1
