"""Covariance-form (MVNStandard) inputs, the reference's standard filter and smoother: the
GPU factors them, computes in square-root form and returns covariances; results match the
oracle's covariance-form path (parsmooth/parallel/_operators.py:7-40, 80-101)."""
import numpy as np
import pytest
import torch

import oracle as O
import sqrt_parallel_smoothers_gb300 as S
from oracle import models as OM
from sqrt_parallel_smoothers_gb300 import models as GM
from tests._parity import assert_rel
from tests._systems import lgssm

pytestmark = pytest.mark.gpu


def _linear_std_pair(A, b, Q):
    o = O.FunctionalModel(OM.LinearFunction(A), O.MVNStandard(np.asarray(b, float), np.asarray(Q, float)))
    g = S.FunctionalModel(GM.LinearModel(A), S.MVNStandard(torch.as_tensor(b), torch.as_tensor(Q)))
    return o, g


@pytest.mark.parametrize("method", ["extended", "cubature"])
def test_standard_filter_smoother_linear(method):
    s = lgssm(4, 2, 60, seed=13)
    ot, gt = _linear_std_pair(s["F"], s["b"], s["Q"])
    oo, go = _linear_std_pair(s["H"], s["c"], s["R"])
    x0 = s["x0"]
    ys = s["ys"].astype(np.float64)
    ref_f, ref_ell = O.methods.filtering(ys, O.MVNStandard(x0.mean, x0.cov), ot, oo,
                                         getattr(O.linearization, method), None, True, return_loglikelihood=True)
    ref_s = O.methods.smoothing(ot, ref_f, getattr(O.linearization, method), None, True)
    gx0 = S.MVNStandard(torch.as_tensor(x0.mean), torch.as_tensor(x0.cov))
    filt, ell = S.filtering(torch.as_tensor(ys), gx0, gt, go, getattr(S.linearization, method), None,
                            return_loglikelihood=True)
    assert isinstance(filt, S.MVNStandard)
    sm = S.smoothing(gt, filt, getattr(S.linearization, method))
    assert isinstance(sm, S.MVNStandard)
    assert_rel(filt.mean, ref_f.mean, 1e-9, "filtered mean")
    assert_rel(filt.cov, ref_f.cov, 1e-9, "filtered cov")
    assert abs(float(ell) - ref_ell) <= 1e-9 * abs(ref_ell)
    assert_rel(sm.mean, ref_s.mean, 1e-9, "smoothed mean")
    assert_rel(sm.cov, ref_s.cov, 1e-9, "smoothed cov")


def test_standard_iterated_bearings():
    """Covariance-form iterated cubature smoother on the bearings model (3 calls from the
    prior mean broadcast) against the oracle's covariance-form operators."""
    T = 80
    w = S.data.bearings_workload(T, seed=2)
    Q, R = w["Q"], w["R"]
    ot = O.FunctionalModel(O.models.CoordinatedTurn(0.01), O.MVNStandard(np.zeros(5), Q))
    oo = O.FunctionalModel(O.models.Bearings((-1.5, 0.5), (1.0, 1.0)), O.MVNStandard(np.zeros(2), R))
    gt = S.FunctionalModel(GM.CoordinatedTurn(0.01), S.MVNStandard(torch.zeros(5, dtype=torch.float64),
                                                                    torch.as_tensor(Q)))
    go = S.FunctionalModel(GM.Bearings((-1.5, 0.5), (1.0, 1.0)), S.MVNStandard(torch.zeros(2, dtype=torch.float64),
                                                                               torch.as_tensor(R)))
    m0 = np.array([0.1, 0.2, 1.0, 0.0, 1.0])
    ys = w["ys"].astype(np.float64)
    nom = (np.repeat(m0[None], T + 1, 0), np.repeat(np.eye(5)[None], T + 1, 0))
    ref, ref_ell = O.methods.iterated_smoothing(ys, O.MVNStandard(m0, np.eye(5)), ot, oo, O.linearization.cubature,
                                                O.MVNStandard(*nom), True, criterion=lambda i, *_: i < 3,
                                                return_loglikelihood=True)
    res, ell = S.iterated_smoothing(torch.as_tensor(ys), S.MVNStandard(torch.as_tensor(m0),
                                                                       torch.eye(5, dtype=torch.float64)),
                                    gt, go, S.linearization.cubature,
                                    S.MVNStandard(torch.as_tensor(nom[0]), torch.as_tensor(nom[1])),
                                    criterion=lambda i, *_: i < 3, return_loglikelihood=True)
    assert isinstance(res, S.MVNStandard)
    assert_rel(res.mean, ref.mean, 1e-8, "mean")
    assert_rel(res.cov, ref.cov, 1e-8, "cov")
    assert abs(float(ell) - ref_ell) <= 1e-8 * abs(ref_ell)


def test_standard_linearize():
    rng = np.random.RandomState(0)
    Q, R = S.data.bearings_noise(0.1, 0.5, 0.05, 0.01)
    om = O.FunctionalModel(O.models.Bearings((-1.5, 0.5), (1.0, 1.0)), O.MVNStandard(np.zeros(2), R))
    gm = S.FunctionalModel(GM.Bearings((-1.5, 0.5), (1.0, 1.0)), S.MVNStandard(torch.zeros(2, dtype=torch.float64),
                                                                               torch.as_tensor(R)))
    m = rng.randn(5)
    A = rng.randn(5, 5) * 0.3
    P = A @ A.T + 0.1 * np.eye(5)
    for name in ("extended", "cubature"):
        Fo, Qo, bo = getattr(O.linearization, name)(om, O.MVNStandard(m, P))
        Fg, Qg, bg = S.linearize(gm, S.MVNStandard(torch.as_tensor(m), torch.as_tensor(P)),
                                 getattr(S.linearization, name))
        assert_rel(Fg, Fo, 1e-9, name + " F")
        assert_rel(Qg, Qo, 1e-9, name + " Q")
        assert_rel(bg, bo, 1e-9, name + " b")
