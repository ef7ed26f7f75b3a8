"""Oracle filter/smoother relations (CPU), porting the reference's
tests/test_parallel_operators.py:17-89, test_parallel_filter.py:26-122,
test_parallel_smoother.py:26-99, test_iterated_smoother.py:26-69 and
test_sequential_filter.py:120-184."""
import numpy as np
import pytest

from oracle import linearization as LZ
from oracle import methods as M
from oracle import models as OM
from oracle import parallel as P
from oracle import sequential as S
from oracle.types import MVNSqrt, MVNStandard, FunctionalModel
from tests._systems import get_system, lgssm

LINS = [LZ.cubature, LZ.extended]


def _tril_rand(n):
    a = np.random.rand(n, n)
    a[np.triu_indices(n, 1)] = 0.0
    return a


@pytest.mark.parametrize("dim_x", [1, 2, 3])
@pytest.mark.parametrize("seed", [0, 42])
def test_filtering_operator_sqrt_vs_standard(dim_x, seed):
    np.random.seed(seed)
    A1, A2 = np.random.randn(dim_x, dim_x), np.random.randn(dim_x, dim_x)
    b1, b2 = np.random.randn(dim_x), np.random.randn(dim_x)
    U1, U2 = _tril_rand(dim_x), _tril_rand(dim_x)
    eta1, eta2 = np.random.randn(dim_x), np.random.randn(dim_x)
    Z1, Z2 = _tril_rand(dim_x), _tril_rand(dim_x)
    std = P.standard_filtering_operator(
        (A1[None], b1[None], (U1 @ U1.T)[None], eta1[None], (Z1 @ Z1.T)[None]),
        (A2[None], b2[None], (U2 @ U2.T)[None], eta2[None], (Z2 @ Z2.T)[None]))
    sq = P.sqrt_filtering_operator((A1[None], b1[None], U1[None], eta1[None], Z1[None]),
                                   (A2[None], b2[None], U2[None], eta2[None], Z2[None]))
    np.testing.assert_allclose(std[0], sq[0], atol=1e-6, rtol=1e-6)
    np.testing.assert_allclose(std[1], sq[1], atol=1e-6, rtol=1e-6)
    np.testing.assert_allclose(std[3], sq[3], atol=1e-6, rtol=1e-6)
    np.testing.assert_allclose(std[2], sq[2] @ np.swapaxes(sq[2], -1, -2), atol=1e-6, rtol=1e-6)
    np.testing.assert_allclose(std[4], sq[4] @ np.swapaxes(sq[4], -1, -2), atol=1e-6, rtol=1e-6)


@pytest.mark.parametrize("dim_x", [1, 2, 3])
@pytest.mark.parametrize("seed", [0, 42])
def test_smoothing_operator_sqrt_vs_standard(dim_x, seed):
    np.random.seed(seed)
    g1, g2 = np.random.randn(dim_x), np.random.randn(dim_x)
    E1, E2 = np.random.randn(dim_x, dim_x), np.random.randn(dim_x, dim_x)
    D1, D2 = _tril_rand(dim_x), _tril_rand(dim_x)
    std = P.standard_smoothing_operator((g1[None], E1[None], (D1 @ D1.T)[None]),
                                        (g2[None], E2[None], (D2 @ D2.T)[None]))
    sq = P.sqrt_smoothing_operator((g1[None], E1[None], D1[None]), (g2[None], E2[None], D2[None]))
    np.testing.assert_allclose(std[0], sq[0], atol=1e-10)
    np.testing.assert_allclose(std[1], sq[1], atol=1e-10)
    np.testing.assert_allclose(std[2], sq[2] @ np.swapaxes(sq[2], -1, -2), atol=1e-10)


def _models(sys_, sqrt=True):
    F, H = sys_["F"], sys_["H"]
    if sqrt:
        return (FunctionalModel(OM.LinearFunction(F), MVNSqrt(sys_["b"], sys_["cholQ"])),
                FunctionalModel(OM.LinearFunction(H), MVNSqrt(sys_["c"], sys_["cholR"])))
    return (FunctionalModel(OM.LinearFunction(F), MVNStandard(sys_["b"], sys_["Q"])),
            FunctionalModel(OM.LinearFunction(H), MVNStandard(sys_["c"], sys_["R"])))


@pytest.mark.parametrize("dim_x", [1, 2, 3])
@pytest.mark.parametrize("dim_y", [1, 2, 3])
@pytest.mark.parametrize("seed", [0, 42])
@pytest.mark.parametrize("lin", LINS, ids=lambda m: m.name)
def test_parallel_vs_sequential_filter(dim_x, dim_y, seed, lin):
    s = lgssm(dim_x, dim_y, 10, seed)
    tm, om = _models(s, True)
    tms, oms = _models(s, False)
    nom = MVNSqrt(s["m_nominal"], np.repeat(np.eye(dim_x)[None], 11, 0))
    noms = MVNStandard(s["m_nominal"], np.repeat(np.eye(dim_x)[None], 11, 0))
    seq, seq_ell = S.filtering(s["ys"], s["x0"], tms, oms, lin, noms, return_loglikelihood=True)
    par, par_ell = P.filtering(s["ys"], s["chol_x0"], tm, om, lin, nom, return_loglikelihood=True)
    sqs, sqs_ell = S.filtering(s["ys"], s["chol_x0"], tm, om, lin, nom, return_loglikelihood=True)
    np.testing.assert_allclose(par.mean, seq.mean, atol=1e-9)
    np.testing.assert_allclose(par.chol @ np.swapaxes(par.chol, -1, -2), seq.cov, atol=1e-9)
    np.testing.assert_allclose(sqs.mean, seq.mean, atol=1e-9)
    assert par_ell == pytest.approx(seq_ell, rel=1e-9)
    assert sqs_ell == pytest.approx(seq_ell, rel=1e-9)


@pytest.mark.parametrize("dim_x", [1, 2, 3])
@pytest.mark.parametrize("dim_y", [1, 2, 3])
@pytest.mark.parametrize("seed", [0, 42])
@pytest.mark.parametrize("lin", LINS, ids=lambda m: m.name)
def test_parallel_vs_sequential_smoother(dim_x, dim_y, seed, lin):
    s = lgssm(dim_x, dim_y, 10, seed)
    tm, om = _models(s, True)
    nom = MVNSqrt(s["m_nominal"], np.repeat(np.eye(dim_x)[None], 11, 0))
    filt = S.filtering(s["ys"], s["chol_x0"], tm, om, lin, nom)
    seq = S.smoothing(tm, filt, lin)
    par = P.smoothing(tm, filt, lin)
    np.testing.assert_allclose(par.mean, seq.mean, atol=1e-9)
    np.testing.assert_allclose(par.chol @ np.swapaxes(par.chol, -1, -2),
                               seq.chol @ np.swapaxes(seq.chol, -1, -2), atol=1e-9)


@pytest.mark.parametrize("dim_x", [1, 2])
@pytest.mark.parametrize("dim_y", [1, 2])
@pytest.mark.parametrize("lin", LINS, ids=lambda m: m.name)
def test_iterated_linear_equals_rts(dim_x, dim_y, lin):
    s = lgssm(dim_x, dim_y, 5, 0)
    tm, om = _models(s, True)
    nom = MVNSqrt(s["m_nominal"], np.repeat(np.eye(dim_x)[None], 6, 0))
    filt = S.filtering(s["ys"], s["chol_x0"], tm, om, lin, nom)
    rts = S.smoothing(tm, filt, lin)
    it = M.iterated_smoothing(s["ys"], s["chol_x0"], tm, om, lin, nom, True, criterion=lambda i, *_: i < 5)
    np.testing.assert_allclose(it.mean, rts.mean, atol=1e-9)


@pytest.mark.parametrize("dim_x", [1, 3])
@pytest.mark.parametrize("dim_y", [2, 3])
@pytest.mark.parametrize("seed", [0, 42])
@pytest.mark.parametrize("lin", LINS, ids=lambda m: m.name)
def test_filter_no_info(dim_x, dim_y, seed, lin):
    np.random.seed(seed)
    x0, chol_x0, F, Q, cholQ, b, _ = get_system(dim_x, dim_x)
    _, _, H, R, cholR, c, _ = get_system(dim_x, dim_y)
    cholR = 1e6 * cholR
    ys = np.random.randn(3, dim_y)
    tm = FunctionalModel(OM.LinearFunction(F), MVNSqrt(b, cholQ))
    om = FunctionalModel(OM.LinearFunction(H), MVNSqrt(c, cholR))
    expected = [x0.mean]
    for _ in range(3):
        expected.append(F @ expected[-1] + b)
    res = P.filtering(ys, chol_x0, tm, om, lin, None)
    np.testing.assert_allclose(res.mean, expected, atol=1e-3, rtol=1e-3)


@pytest.mark.parametrize("dim", [1, 3])
@pytest.mark.parametrize("seed", [0, 42])
@pytest.mark.parametrize("lin", LINS, ids=lambda m: m.name)
def test_filter_infinite_info(dim, seed, lin):
    np.random.seed(seed)
    x0, chol_x0, _, Q, cholQ, b, _ = get_system(dim, dim)
    _, _, _, R, cholR, c, _ = get_system(dim, dim)
    cholR = 1e-3 * cholR
    ys = np.random.randn(3, dim)
    tm = FunctionalModel(OM.LinearFunction(np.eye(dim)), MVNSqrt(b, cholQ))
    om = FunctionalModel(OM.LinearFunction(np.eye(dim)), MVNSqrt(c, cholR))
    res = P.filtering(ys, chol_x0, tm, om, lin, None)
    np.testing.assert_allclose(res.mean[1:], ys - c, atol=1e-3, rtol=1e-3)


@pytest.mark.parametrize("dim_x", [1, 2, 3])
@pytest.mark.parametrize("dim_y", [1, 2, 3])
@pytest.mark.parametrize("seed", [0, 42])
@pytest.mark.parametrize("lin", LINS, ids=lambda m: m.name)
def test_elements_sqrt_vs_standard(dim_x, dim_y, seed, lin):
    # tests/test_parallel_filter.py:26-75 and tests/test_parallel_smoother.py:26-55 of the
    # reference: one step's filtering and smoothing elements at a nominal N(m, I) of a linear
    # system, square-root against covariance form, and the linearised model is the system itself
    np.random.seed(seed)
    x0, chol_x0, F, Q, cholQ, b, _ = get_system(dim_x, dim_x)
    _, _, H, R, cholR, c, _ = get_system(dim_x, dim_y)
    m_nom = np.random.randn(dim_x)
    y = np.random.randn(dim_y)
    s = dict(F=F, H=H, Q=Q, R=R, cholQ=cholQ, cholR=cholR, b=b, c=c)
    (tm_s, om_s), (tm, om) = _models(s, True), _models(s, False)
    Fs, cQs, bs = lin(tm_s, MVNSqrt(m_nom, np.eye(dim_x)))
    Hs, cRs, cs = lin(om_s, MVNSqrt(m_nom, np.eye(dim_x)))
    Fc, Qc, bc = lin(tm, MVNStandard(m_nom, np.eye(dim_x)))
    Hc, Rc, cc = lin(om, MVNStandard(m_nom, np.eye(dim_x)))
    for got, want in ((Fs, F), (bs, b), (Hs, H), (cs, c), (cQs @ cQs.T, Q), (cRs @ cRs.T, R),
                      (Fc, F), (bc, b), (Hc, H), (cc, c), (Qc, Q), (Rc, R)):
        np.testing.assert_allclose(got, want, atol=1e-9)

    A1, b1, U, eta1, Z = P.sqrt_filter_elements(Fs, cQs, bs, Hs, cRs, cs, y, chol_x0.mean, chol_x0.chol)
    A2, b2, C, eta2, J = P.standard_filter_elements(Fc, Qc, bc, Hc, Rc, cc, y, x0.mean, x0.cov)
    np.testing.assert_allclose(A1, A2, atol=1e-9)
    np.testing.assert_allclose(b1, b2, atol=1e-9)
    np.testing.assert_allclose(eta1, eta2, atol=1e-9)
    np.testing.assert_allclose(U @ U.T, C, atol=1e-9)
    np.testing.assert_allclose(Z @ Z.T, J, atol=1e-9)

    g1, E1, D = P.sqrt_smoother_elements(Fs, cQs, bs, chol_x0.mean, chol_x0.chol)
    g2, E2, L = P.standard_smoother_elements(Fc, Qc, bc, x0.mean, x0.cov)
    np.testing.assert_allclose(g1, g2, atol=1e-9)
    np.testing.assert_allclose(E1, E2, atol=1e-9)
    np.testing.assert_allclose(D @ D.T, L, atol=1e-9)
