"""Pin the oracle to the reference's own saved outputs (CPU).

* ``ieks.npz``: 100-iteration extended smoother on the bearings fixture,
  compared to 3 decimals as in the reference's tests/test_bearings_only.py:67-72.
* ``robustness_small.npz``: FP32 GPU log-likelihoods of the reference's
  20-iteration extended/cubature smoothers (notebooks/robustness_100runs.py).
  The reference's values are FP32, so a run may settle on another fixed point
  in FP32 than in FP64; the test requires most runs to agree to 1e-5 (extended).
  The covariance-form values of the same study pin the oracle's covariance form,
  and record the study's finding: FP32 covariance-form cubature fails (NaN)
  where the square-root form does not.
"""
import os

import numpy as np
import pytest

from oracle import linearization as LZ
from oracle import methods as M
from oracle import models as OM
from oracle.types import MVNSqrt, FunctionalModel

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def bearings_models(qc, qw, r, dt=0.01):
    Q, R = OM.bearings_noise(qc, qw, r, dt)
    tm = FunctionalModel(OM.CoordinatedTurn(dt), MVNSqrt(np.zeros(5), np.linalg.cholesky(Q)))
    om = FunctionalModel(OM.Bearings([-1.5, 0.5], [1.0, 1.0]), MVNSqrt(np.zeros(2), np.linalg.cholesky(R)))
    return tm, om


def test_ieks_golden():
    ys = np.load(os.path.join(GOLD, "bearings_ys.npy")).astype(float)
    gold = np.load(os.path.join(GOLD, "ieks.npz"))
    tm, om = bearings_models(0.01, 0.1, 0.5)
    x0 = MVNSqrt(np.array([-1.0, -1.0, 0.0, 0.0, 0.0]), np.eye(5))
    res = M.iterated_smoothing(ys, x0, tm, om, LZ.extended, None, True, criterion=lambda i, *_: i < 100)
    cov = res.chol[1:] @ np.swapaxes(res.chol[1:], -1, -2)
    np.testing.assert_array_almost_equal(res.mean[1:], gold["mean"], decimal=3)
    np.testing.assert_array_almost_equal(cov, gold["cov"], decimal=3)


def _robustness_ell(lin, T, run, ys):
    tm, om = bearings_models(0.01, 0.1, 0.5)
    x0 = MVNSqrt(np.array([-4.0, -1.0, 2.0, 7.0, 3.0]), np.eye(5))
    nom = MVNSqrt(np.repeat(np.array([[-1.0, -1.0, 6.0, 4.0, 2.0]]), T + 1, 0), np.repeat(np.eye(5)[None], T + 1, 0))
    _, ell = M.iterated_smoothing(ys[run, :T].astype(float), x0, tm, om, lin, nom, True,
                                  criterion=lambda i, *_: i < 20, return_loglikelihood=True)
    return ell


@pytest.mark.parametrize("T", [20, 30, 40, 50, 80, 100])
def test_robustness_loglikelihood_extended(T):
    d = np.load(os.path.join(GOLD, "robustness_small.npz"))
    ti = list(d["Ts"]).index(T)
    rel = []
    for run in range(d["ys"].shape[0]):
        ell = _robustness_ell(LZ.extended, T, run, d["ys"])
        g = float(d["ell_extended"][ti, run])
        rel.append(abs(ell - g) / abs(g))
    rel = np.array(rel)
    assert np.mean(rel < 1e-5) >= 0.8, rel


def test_robustness_loglikelihood_cubature_t50():
    # FP32 cancellation in the reference's SLR downdate makes its FP32 cubature
    # values noisy; an FP64 restatement agrees to 1e-2 on most runs.
    d = np.load(os.path.join(GOLD, "robustness_small.npz"))
    ti = list(d["Ts"]).index(50)
    rel = []
    for run in range(d["ys"].shape[0]):
        ell = _robustness_ell(LZ.cubature, 50, run, d["ys"])
        g = float(d["ell_cubature"][ti, run])
        rel.append(abs(ell - g) / abs(g))
    assert np.mean(np.array(rel) < 1e-2) >= 0.8, rel


def _robustness_ell_standard(lin, T, run, ys):
    """The covariance-form run of the same study (notebooks/robustness_100runs.py, std models)."""
    from oracle.types import MVNStandard
    Q, R = OM.bearings_noise(0.01, 0.1, 0.5, 0.01)
    tm = FunctionalModel(OM.CoordinatedTurn(0.01), MVNStandard(np.zeros(5), Q))
    om = FunctionalModel(OM.Bearings([-1.5, 0.5], [1.0, 1.0]), MVNStandard(np.zeros(2), R))
    x0 = MVNStandard(np.array([-4.0, -1.0, 2.0, 7.0, 3.0]), np.eye(5))
    nom = MVNStandard(np.repeat(np.array([[-1.0, -1.0, 6.0, 4.0, 2.0]]), T + 1, 0),
                      np.repeat(np.eye(5)[None], T + 1, 0))
    _, ell = M.iterated_smoothing(ys[run, :T].astype(float), x0, tm, om, lin, nom, True,
                                  criterion=lambda i, *_: i < 20, return_loglikelihood=True)
    return ell


@pytest.mark.parametrize("T", [20, 50, 100])
def test_robustness_loglikelihood_extended_standard(T):
    # the reference's FP32 covariance-form extended smoother: the oracle's covariance form
    # (FP64) agrees to 1e-5 on most runs, as the square-root form does
    d = np.load(os.path.join(GOLD, "robustness_small.npz"))
    ti = list(d["Ts"]).index(T)
    rel = []
    for run in range(d["ys"].shape[0]):
        g = float(d["ell_extended_std"][ti, run])
        rel.append(abs(_robustness_ell_standard(LZ.extended, T, run, d["ys"]) - g) / abs(g))
    assert np.mean(np.array(rel) < 1e-5) >= 0.8, rel


def test_robustness_covariance_form_cubature_fails_in_fp32_only():
    # the reference's robustness finding at T = 100: its FP32 covariance-form cubature smoother
    # returns NaN on every run while its FP32 square-root form is finite; in FP64 the
    # covariance form is finite too, so the failure is the FP32 arithmetic of that form
    d = np.load(os.path.join(GOLD, "robustness_small.npz"))
    ti = list(d["Ts"]).index(100)
    assert np.isnan(d["ell_cubature_std"][ti]).all()
    assert np.isfinite(d["ell_cubature"][ti]).all()
    for run in range(0, d["ys"].shape[0], 4):
        assert np.isfinite(_robustness_ell_standard(LZ.cubature, 100, run, d["ys"]))


def _icks_one_call(form):
    """One filter-smoother call of the bearings cubature smoother with the reference's
    ``icks.npz`` trajectory (prior prepended) as the nominal: a fixed point of the map
    stays where it is (tests/test_bearings_only.py:25-65 of the reference)."""
    from oracle.types import MVNStandard
    ys = np.load(os.path.join(GOLD, "bearings_ys.npy")).astype(float)
    gold = np.load(os.path.join(GOLD, "icks.npz"))
    m0 = np.array([-1.0, -1.0, 0.0, 0.0, 0.0])
    mean = np.concatenate([m0[None], gold["mean"]])
    cov = np.concatenate([np.eye(5)[None], gold["cov"]])
    if form == "sqrt":
        tm, om = bearings_models(0.01, 0.1, 0.5)
        x0, nom = MVNSqrt(m0, np.eye(5)), MVNSqrt(mean, np.linalg.cholesky(cov))
    else:
        Q, R = OM.bearings_noise(0.01, 0.1, 0.5, 0.01)
        tm = FunctionalModel(OM.CoordinatedTurn(0.01), MVNStandard(np.zeros(5), Q))
        om = FunctionalModel(OM.Bearings([-1.5, 0.5], [1.0, 1.0]), MVNStandard(np.zeros(2), R))
        x0, nom = MVNStandard(m0, np.eye(5)), MVNStandard(mean, cov)
    res = M.filter_smoother(ys, x0, tm, om, LZ.cubature, nom, True)
    return np.abs(res.mean[1:] - gold["mean"]), res.mean


@pytest.mark.parametrize("form", ["sqrt", "std"])
def test_icks_fixed_point(form):
    # icks.npz is NOT a fixed point of the reference's cubature map as the code stands:
    # one FP64 call from it moves the means by 0.18 (max) / 0.026 (mean) in both forms,
    # while the same check on ieks.npz with the extended map moves them by < 1e-13
    # (test_ieks_fixed_point).  The call lands on the oracle's own converged cubature
    # trajectory, so the gap is in the fixture, not in which fixed point is reached.
    move, mean = _icks_one_call(form)
    assert 0.15 < move.max() < 0.22 and 0.02 < move.mean() < 0.035, (move.max(), move.mean())
    tm, om = bearings_models(0.01, 0.1, 0.5)
    ys = np.load(os.path.join(GOLD, "bearings_ys.npy")).astype(float)
    conv = M.iterated_smoothing(ys, MVNSqrt(np.array([-1.0, -1.0, 0.0, 0.0, 0.0]), np.eye(5)), tm, om,
                                LZ.cubature, None, True, criterion=lambda i, *_: i < 100)
    assert np.abs(mean - conv.mean).max() < 1e-3


def test_ieks_fixed_point():
    ys = np.load(os.path.join(GOLD, "bearings_ys.npy")).astype(float)
    gold = np.load(os.path.join(GOLD, "ieks.npz"))
    m0 = np.array([-1.0, -1.0, 0.0, 0.0, 0.0])
    tm, om = bearings_models(0.01, 0.1, 0.5)
    nom = MVNSqrt(np.concatenate([m0[None], gold["mean"]]),
                  np.linalg.cholesky(np.concatenate([np.eye(5)[None], gold["cov"]])))
    res = M.filter_smoother(ys, MVNSqrt(m0, np.eye(5)), tm, om, LZ.extended, nom, True)
    assert np.abs(res.mean[1:] - gold["mean"]).max() < 1e-10
