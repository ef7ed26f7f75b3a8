"""Oracle sequential steps (CPU): the square-root and covariance-form predict, update and RTS
smoothing steps against their closed forms and against each other, porting the relations of
the reference's tests/test_sequential_filter.py:24-250 and
tests/test_sequential_smoother.py:24-200 (these steps are the sequential oracle the parallel
path is checked against)."""
import numpy as np
import pytest

from oracle import sequential as S
from oracle.core import mvn_loglikelihood
from tests._systems import get_system


def _cov(L):
    return L @ L.T


@pytest.mark.parametrize("dim_x", [1, 2, 3])
@pytest.mark.parametrize("seed", [0, 42])
def test_predict_values_and_forms(dim_x, seed):
    np.random.seed(seed)
    x, chol_x, F, Q, cholQ, b, _ = get_system(dim_x, dim_x)
    ms, Ls = S.sqrt_predict(F, cholQ, b, chol_x.mean, chol_x.chol)
    m, P = S.standard_predict(F, Q, b, x.mean, x.cov)
    for mean, cov in ((ms, _cov(Ls)), (m, P)):
        np.testing.assert_allclose(mean, F @ x.mean + b, atol=1e-10)
        np.testing.assert_allclose(cov, Q + F @ x.cov @ F.T, atol=1e-10)


@pytest.mark.parametrize("dim_x", [1, 2, 3])
@pytest.mark.parametrize("dim_y", [1, 2, 3])
@pytest.mark.parametrize("seed", [0, 42])
def test_update_values_and_forms(dim_x, dim_y, seed):
    np.random.seed(seed)
    x, chol_x, H, R, cholR, c, y = get_system(dim_x, dim_y)
    ms, Ls, ell_s = S.sqrt_update(H, cholR, c, chol_x.mean, chol_x.chol, y)
    m, P, ell = S.standard_update(H, R, c, x.mean, x.cov, y)
    res = y - H @ x.mean - c
    Sy = H @ x.cov @ H.T + R
    K = x.cov @ np.linalg.solve(Sy, H).T
    expected_ell = mvn_loglikelihood(res, np.linalg.cholesky(Sy))
    for mean, cov, e in ((ms, _cov(Ls), ell_s), (m, P, ell)):
        np.testing.assert_allclose(mean, x.mean + K @ res, atol=1e-9)
        np.testing.assert_allclose(cov, x.cov - K @ H @ x.cov, atol=1e-9)
        np.testing.assert_allclose(e, expected_ell, atol=1e-9)


@pytest.mark.parametrize("dim_x", [1, 3])
@pytest.mark.parametrize("dim_y", [1, 2, 3])
@pytest.mark.parametrize("seed", [0, 42])
def test_update_without_information(dim_x, dim_y, seed):
    np.random.seed(seed)
    x, chol_x, H, R, cholR, c, y = get_system(dim_x, dim_y)
    ms, Ls, ell_s = S.sqrt_update(H, 1e4 * cholR, c, chol_x.mean, chol_x.chol, y)
    m, P, ell = S.standard_update(H, 1e8 * R, c, x.mean, x.cov, y)
    np.testing.assert_allclose(ell, ell_s, atol=1e-3)
    for mean, cov in ((ms, _cov(Ls)), (m, P)):
        np.testing.assert_allclose(mean, x.mean, atol=1e-3)
        np.testing.assert_allclose(cov, x.cov, atol=1e-3)


def _smooth_pair(dim_x):
    xf, chol_xf, F, Q, cholQ, b, _ = get_system(dim_x, dim_x)
    xs, chol_xs, *_ = get_system(dim_x, dim_x)
    return xf, chol_xf, F, Q, cholQ, b, xs, chol_xs


@pytest.mark.parametrize("dim_x", [1, 2, 3])
@pytest.mark.parametrize("seed", [0, 42])
def test_smooth_one_values_and_forms(dim_x, seed):
    np.random.seed(seed)
    xf, chol_xf, F, Q, cholQ, b, xs, chol_xs = _smooth_pair(dim_x)
    m_s, L_s = S.sqrt_smooth(F, cholQ, b, chol_xf.mean, chol_xf.chol, chol_xs.mean, chol_xs.chol)
    m, P = S.standard_smooth(F, Q, b, xf.mean, xf.cov, xs.mean, xs.cov)
    m_ = F @ xf.mean + b
    P_ = F @ xf.cov @ F.T + Q
    G = xf.cov @ np.linalg.solve(P_.T, F).T
    for mean, cov in ((m_s, _cov(L_s)), (m, P)):
        np.testing.assert_allclose(mean, xf.mean + G @ (xs.mean - m_), atol=1e-9)
        np.testing.assert_allclose(cov, xf.cov + G @ (xs.cov - P_) @ G.T, atol=1e-9)


@pytest.mark.parametrize("dim_x", [1, 3])
@pytest.mark.parametrize("seed", [0, 42])
def test_smooth_one_without_process_noise(dim_x, seed):
    np.random.seed(seed)
    xf, chol_xf, F, Q, cholQ, b, xs, chol_xs = _smooth_pair(dim_x)
    m_s, L_s = S.sqrt_smooth(F, 0 * cholQ, b, chol_xf.mean, chol_xf.chol, chol_xs.mean, chol_xs.chol)
    m, P = S.standard_smooth(F, 0 * Q, b, xf.mean, xf.cov, xs.mean, xs.cov)
    G = np.linalg.pinv(F)
    m_ = F @ xf.mean + b
    P_ = F @ xf.cov @ F.T
    for mean, cov in ((m_s, _cov(L_s)), (m, P)):
        np.testing.assert_allclose(mean, xf.mean + G @ (xs.mean - m_), atol=1e-5)
        np.testing.assert_allclose(cov, xf.cov + G @ (xs.cov - P_) @ G.T, atol=1e-5)


@pytest.mark.parametrize("dim_x", [1, 3])
@pytest.mark.parametrize("seed", [0, 42])
def test_smooth_one_with_infinite_process_noise(dim_x, seed):
    np.random.seed(seed)
    xf, chol_xf, F, Q, cholQ, b, xs, chol_xs = _smooth_pair(dim_x)
    m_s, L_s = S.sqrt_smooth(F, 1e6 * cholQ, b, chol_xf.mean, chol_xf.chol, chol_xs.mean, chol_xs.chol)
    m, P = S.standard_smooth(F, 1e12 * Q, b, xf.mean, xf.cov, xs.mean, xs.cov)
    for mean, cov in ((m_s, _cov(L_s)), (m, P)):
        np.testing.assert_allclose(mean, xf.mean, atol=1e-5)
        np.testing.assert_allclose(cov, xf.cov, atol=1e-5)


@pytest.mark.parametrize("dim_x", [1, 3])
@pytest.mark.parametrize("dim_y", [2, 3])
@pytest.mark.parametrize("seed", [0, 42])
@pytest.mark.parametrize("with_nominal", [False, True])
def test_all_filters_and_smoothers_agree(dim_x, dim_y, seed, with_nominal):
    # tests/test_sequential_filter.py:186-250 and tests/test_sequential_smoother.py:123-200 of
    # the reference: on a linear system the four linearisations, in square-root and covariance
    # form, with or without a nominal trajectory, give one filter and one smoother
    from oracle import linearization as LZ
    from oracle.types import MVNSqrt, MVNStandard
    from tests._systems import lgssm
    from tests.test_oracle_filter_smoother import _models
    T = 5
    s = lgssm(dim_x, dim_y, T, seed)
    means_f, means_s = [], []
    for lin in (LZ.extended, LZ.cubature, LZ.gauss_hermite, LZ.unscented):
        for sqrt in (True, False):
            tm, om = _models(s, sqrt)
            x0 = s["chol_x0"] if sqrt else s["x0"]
            nom = None
            if with_nominal:
                eye = np.repeat(np.eye(dim_x)[None], T + 1, 0)
                nom = (MVNSqrt if sqrt else MVNStandard)(s["m_nominal"], eye)
            filt = S.filtering(s["ys"], x0, tm, om, lin, nom)
            means_f.append(filt.mean)
            means_s.append(S.smoothing(tm, filt, lin, nom).mean)
    for got in means_f[1:]:
        np.testing.assert_allclose(got, means_f[0], atol=1e-8)
    for got in means_s[1:]:
        np.testing.assert_allclose(got, means_s[0], atol=1e-8)
