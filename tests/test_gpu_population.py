"""Conditional-moments models (parsmooth ConditionalMomentsModel) on the reference's population
workload: a Ricker-map transition with constant conditional covariance and Poisson counts
(notebooks/population_model.py), iterated smoothers in square-root and covariance form
against the oracle."""
import numpy as np
import pytest
import torch

import oracle as O
import sqrt_parallel_smoothers_gb300 as S
from oracle import models as OM
from tests._parity import assert_rel, cov

pytestmark = pytest.mark.gpu

LAM, Q = 10.0, np.array([[0.3 ** 2]])


def _oracle_models(sqrt):
    f = O.ConditionalMomentsModel(OM.Ricker(), OM.ConstantCovariance(Q, chol=sqrt))
    h = O.ConditionalMomentsModel(OM.PoissonExpMean(LAM), OM.PoissonExpCovariance(LAM, chol=sqrt))
    return f, h


def _gpu_models(sqrt):
    mean_f, cov_f, mean_h, cov_h, chol_f, chol_h = S.models.population_parameters(LAM, Q)
    return (S.ConditionalMomentsModel(mean_f, chol_f if sqrt else cov_f),
            S.ConditionalMomentsModel(mean_h, chol_h if sqrt else cov_h))


@pytest.mark.parametrize("method", ["extended", "cubature", "gauss_hermite"])
def test_population_linearize(method):
    _, h = _oracle_models(True)
    _, gh = _gpu_models(True)
    rng = np.random.RandomState(2)
    m = rng.randn(6, 1) * 0.5
    L = np.abs(rng.randn(6, 1, 1)) * 0.4 + 0.1
    Fo, Lo, bo = getattr(O.linearization, method)(h, O.MVNSqrt(m, L))
    Fg, Lg, bg = S.linearize(gh, S.MVNSqrt(torch.as_tensor(m), torch.as_tensor(L)), getattr(S.linearization, method))
    assert_rel(Fg, Fo, 1e-10, "F")
    assert_rel(cov(Lg), cov(Lo), 1e-10, "chol")
    assert_rel(bg, bo, 1e-10, "b")


@pytest.mark.parametrize("method", ["extended", "cubature"])
@pytest.mark.parametrize("sqrt", [True, False])
def test_population_iterated_vs_oracle(method, sqrt):
    """The reference's population workload (T = 128, 10 iterations, FP64) from a
    well-conditioned start: the nominal means log((y + 1) / lam) read off the counts.  From a
    random nominal, undamped Gauss-Newton on this chaotic map leaves the data's basin (the
    oracle itself overflows within three iterations), and rounding differences then grow
    without bound, so such a start says nothing about parity."""
    T = 128
    _, ys = S.data.population_data(T)
    m0 = np.array([np.log(7.0)])
    P0 = np.array([[0.25]])
    m_nom = np.concatenate([m0[None], np.log((ys + 1.0) / LAM)], 0)
    P_nom = np.repeat(0.5 * np.eye(1)[None], T + 1, 0)
    of, oh = _oracle_models(sqrt)
    gf, gh = _gpu_models(sqrt)
    if sqrt:
        ox0, onom = O.MVNSqrt(m0, np.linalg.cholesky(P0)), O.MVNSqrt(m_nom, P_nom)
        gx0 = S.MVNSqrt(torch.as_tensor(m0), torch.as_tensor(np.linalg.cholesky(P0)))
        gnom = S.MVNSqrt(torch.as_tensor(m_nom), torch.as_tensor(P_nom))
    else:
        ox0, onom = O.MVNStandard(m0, P0), O.MVNStandard(m_nom, P_nom)
        gx0 = S.MVNStandard(torch.as_tensor(m0), torch.as_tensor(P0))
        gnom = S.MVNStandard(torch.as_tensor(m_nom), torch.as_tensor(P_nom))
    ref = O.methods.iterated_smoothing(ys, ox0, of, oh, getattr(O.linearization, method), onom, True,
                                       criterion=lambda i, *_: i < 10)
    res = S.iterated_smoothing(torch.as_tensor(ys), gx0, gf, gh, getattr(S.linearization, method), gnom,
                               criterion=lambda i, *_: i < 10)
    assert_rel(res.mean, ref.mean, 1e-8, "mean")
    if sqrt:
        assert_rel(cov(res.chol), cov(ref.chol), 1e-8, "cov")
    else:
        assert_rel(res.cov, ref.cov, 1e-8, "cov")
