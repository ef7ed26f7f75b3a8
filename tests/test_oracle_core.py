"""Oracle primitives (CPU): tria, rank-1 updates, log-likelihood, scans, quadrature rules.

Ports the relations of the reference's tests/test_math_utils.py:16-54 (the
tfp comparison is replaced by the defining identity L L^T = C C^T +- v v^T).
"""
import numpy as np
import pytest

import oracle as O
from oracle import parallel as P
from oracle import linearization as LZ


@pytest.mark.parametrize("shape", [(3, 5), (4, 4), (2, 7), (6, 9)])
def test_tria_factor(shape):
    rng = np.random.RandomState(0)
    A = rng.randn(8, *shape)
    L = O.tria(A)
    np.testing.assert_allclose(L @ np.swapaxes(L, -1, -2), A @ np.swapaxes(A, -1, -2), atol=1e-12)
    assert np.all(np.triu(L, 1) == 0)
    assert np.all(np.diagonal(L, axis1=-2, axis2=-1) >= 0)


@pytest.mark.parametrize("multiplier", [1.0, -0.1])
@pytest.mark.parametrize("seed", [0, 42, 666])
@pytest.mark.parametrize("dim_x", [2, 3, 10, 11])
def test_cholesky_update(multiplier, seed, dim_x):
    np.random.seed(seed)
    cholQ = np.random.rand(dim_x, dim_x)
    cholQ[np.triu_indices(dim_x, 1)] = 0.0
    v = np.random.randn(dim_x)
    expected = cholQ @ cholQ.T + multiplier * np.outer(v, v)
    if min(np.linalg.eigvals(expected).real) <= 1e-6:
        pytest.skip("not positive definite")
    res = O.cholesky_update(cholQ, v, multiplier)
    np.testing.assert_allclose(res @ res.T, expected, rtol=1e-4)


@pytest.mark.parametrize("multiplier", [1.0, -0.1])
@pytest.mark.parametrize("seed", [0, 1, 2, 42, 666])
@pytest.mark.parametrize("dim_x", [2, 3, 10, 11])
def test_cholesky_update_many(multiplier, seed, dim_x):
    np.random.seed(seed)
    cholQ = np.random.rand(dim_x, dim_x)
    cholQ[np.triu_indices(dim_x, 1)] = 0.0
    v = np.random.rand(3, dim_x)
    expected = cholQ @ cholQ.T + multiplier * sum(np.outer(v[k], v[k]) for k in range(3))
    if min(np.linalg.eigvals(expected).real) <= 1e-6:
        pytest.skip("not positive definite")
    res = O.cholesky_update_many(cholQ, v, multiplier)
    np.testing.assert_allclose(res @ res.T, expected, rtol=1e-4)


def test_cholesky_downdate_failure_is_zeroed():
    # a downdate that leaves the cone: the reference maps non-finite entries to 0 (parsmooth/_utils.py:80)
    res = O.cholesky_update(np.eye(2), np.array([2.0, 0.0]), -1.0)
    assert np.all(np.isfinite(res))
    assert res[0, 0] == 0.0


def test_mvn_loglikelihood():
    from scipy.stats import multivariate_normal
    rng = np.random.RandomState(3)
    L = np.tril(rng.rand(3, 3)) + np.eye(3)
    x = rng.randn(3)
    ref = multivariate_normal(np.zeros(3), L @ L.T).logpdf(x)
    assert O.mvn_loglikelihood(x, L) == pytest.approx(ref, rel=1e-12)


def test_associative_scan_matches_fold():
    rng = np.random.RandomState(1)
    for n in [1, 2, 3, 7, 16, 33]:
        A = rng.randn(n, 3, 3) * 0.5
        b = rng.randn(n, 3)

        def op(e1, e2):
            return e2[0] @ e1[0], np.einsum("...ij,...j->...i", e2[0], e1[1]) + e2[1]

        a1, b1 = P.associative_scan(op, (A, b))
        a2, b2 = P.sequential_scan(op, (A, b))
        np.testing.assert_allclose(a1, a2, atol=1e-12)
        np.testing.assert_allclose(b1, b2, atol=1e-12)
        r1 = P.associative_scan(op, (A, b), reverse=True)
        r2 = P.sequential_scan(op, (A, b), reverse=True)
        np.testing.assert_allclose(r1[1], r2[1], atol=1e-12)


@pytest.mark.parametrize("n", [1, 2, 3])
@pytest.mark.parametrize("order", [2, 3, 4, 5])
def test_gauss_hermite_moments(n, order):
    wm, wc, xi = LZ.gauss_hermite_weights(n, order)
    assert wm.sum() == pytest.approx(1.0, abs=1e-12)
    np.testing.assert_allclose(xi.T @ (wm[:, None] * xi), np.eye(n), atol=1e-12)
    np.testing.assert_allclose(wm @ xi, np.zeros(n), atol=1e-12)


def test_unscented_default_kappa():
    # the code's default is kappa = 3 + n (parsmooth/linearization/_unscented.py:64-65)
    wm, wc, xi = LZ.unscented_weights(2)
    lam = 1.0 * (2 + 5) - 2
    assert wm[0] == pytest.approx(lam / (2 + lam))
    assert wm.sum() == pytest.approx(1.0)
    np.testing.assert_allclose(xi.T @ (wc[:, None] * xi), np.eye(2), atol=1e-12)


def test_fixed_point_known_answer():
    # tests/test_math_utils.py:57-67 of the reference: x <- 0.7 x + 0.5 from 1 converges to 0.5 / 0.3
    from oracle.methods import fixed_point
    x, calls = fixed_point(lambda x: 0.7 * x + 0.5, 1.0, lambda i, *_: i < 500)
    assert x == pytest.approx(0.5 / 0.3, rel=1e-7, abs=1e-7)
    assert calls == 500


@pytest.mark.parametrize("n", [1, 2, 10])
def test_fixed_point_calls_f_n_times(n):
    # parsmooth/_utils.py:136-146: the loop starts at (1, x0, f(x0)), so `i < n` makes n calls of f
    from oracle.methods import fixed_point
    seen = []

    def f(x):
        seen.append(x)
        return x + 1

    x, calls = fixed_point(f, 0, lambda i, *_: i < n)
    assert len(seen) == n and calls == n and x == n
