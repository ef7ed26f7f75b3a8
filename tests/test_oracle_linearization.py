"""Oracle linearisations (CPU), porting the reference's tests/test_linearization.py:67-239."""
import numpy as np
import pytest

from oracle import linearization as LZ
from oracle import models as OM
from oracle.types import MVNSqrt, MVNStandard, FunctionalModel

METHODS = [LZ.extended, LZ.cubature, LZ.gauss_hermite, LZ.unscented]


class Elementwise:
    """Elementwise f with derivative df (for the sqrt-vs-standard checks)."""

    def __init__(self, f, df):
        self.f, self.df = f, df

    def __call__(self, x):
        return self.f(x)

    def jacobian(self, x):
        x = np.asarray(x)
        return np.einsum("...i,ij->...ij", self.df(x), np.eye(x.shape[-1]))


FUNCS = {"sin": Elementwise(np.sin, np.cos), "cos": Elementwise(np.cos, lambda x: -np.sin(x)),
         "exp": Elementwise(np.exp, np.exp), "arctan": Elementwise(np.arctan, lambda x: 1 / (1 + x * x))}


def _rand_chol(n):
    c = np.random.rand(n, n)
    c[np.triu_indices(n, 1)] = 0
    return c


@pytest.mark.parametrize("dim_x", [1, 3])
@pytest.mark.parametrize("seed", [0, 42])
@pytest.mark.parametrize("method", METHODS, ids=lambda m: m.name)
@pytest.mark.parametrize("sqrt", [True, False])
def test_linear_functional(dim_x, seed, method, sqrt):
    np.random.seed(seed)
    a = np.random.randn(dim_x, dim_x)
    c = np.random.randn(dim_x)
    m_x = np.random.randn(dim_x)
    m_q = np.random.randn(dim_x)
    chol_x = _rand_chol(dim_x)
    chol_q = _rand_chol(dim_x)
    if sqrt:
        x, q = MVNSqrt(m_x, chol_x), MVNSqrt(m_q, chol_q)
    else:
        x, q = MVNStandard(m_x, chol_x @ chol_x.T), MVNStandard(m_q, chol_q @ chol_q.T)

    class Affine(OM.LinearFunction):
        def __call__(self, x):
            return super().__call__(x) + c

    fun = Affine(a)
    F, Q, rem = method(FunctionalModel(fun, q), x)
    if sqrt:
        Q = Q @ Q.T
    xp = np.random.randn(dim_x)
    np.testing.assert_allclose(a, F, atol=1e-7)
    np.testing.assert_allclose(fun(xp) + m_q, F @ xp + rem, atol=1e-7)
    np.testing.assert_allclose(chol_q @ chol_q.T, Q, atol=1e-7)


@pytest.mark.parametrize("dim_x", [1, 3])
@pytest.mark.parametrize("seed", [0, 42])
@pytest.mark.parametrize("method", METHODS, ids=lambda m: m.name)
@pytest.mark.parametrize("name", list(FUNCS))
def test_sqrt_vs_std(dim_x, seed, method, name):
    np.random.seed(seed)
    m_x = np.random.randn(dim_x)
    m_q = np.random.randn(dim_x)
    chol_x = _rand_chol(dim_x)
    chol_q = _rand_chol(dim_x)
    f = FUNCS[name]
    sF, sL, sb = method(FunctionalModel(f, MVNSqrt(m_x, chol_x)), MVNSqrt(m_q, chol_q))
    F, Q, b = method(FunctionalModel(f, MVNStandard(m_x, chol_x @ chol_x.T)),
                     MVNStandard(m_q, chol_q @ chol_q.T))
    np.testing.assert_allclose(sF, F, atol=1e-10)
    np.testing.assert_allclose(sb, b, atol=1e-10)
    np.testing.assert_allclose(Q, sL @ sL.T, atol=1e-10)


@pytest.mark.parametrize("model", ["ct", "bearings"])
def test_model_jacobians_complex_step(model):
    rng = np.random.RandomState(0)
    f = OM.CoordinatedTurn(0.01) if model == "ct" else OM.Bearings([-1.5, 0.5], [1.0, 1.0])
    for x in [rng.randn(5), np.array([0.3, -0.2, 1.0, 0.5, 1e-8])]:
        J = f.jacobian(x)
        h = 1e-7
        num = np.stack([(f(x + h * e) - f(x - h * e)) / (2 * h) for e in np.eye(5)], axis=-1)
        np.testing.assert_allclose(J, num, atol=1e-6)


def test_batched_equals_single():
    rng = np.random.RandomState(5)
    f = OM.CoordinatedTurn(0.01)
    Q, _ = OM.bearings_noise(0.1, 0.5, 0.05, 0.01)
    q = MVNSqrt(np.zeros(5), np.linalg.cholesky(Q))
    m = rng.randn(4, 5)
    L = np.tril(rng.rand(4, 5, 5)) + np.eye(5)
    for method in METHODS:
        Fb, Lb, bb = method(FunctionalModel(f, q), MVNSqrt(m, L))
        for k in range(4):
            F1, L1, b1 = method(FunctionalModel(f, q), MVNSqrt(m[k], L[k]))
            np.testing.assert_allclose(Fb[k], F1, atol=1e-13)
            np.testing.assert_allclose(bb[k], b1, atol=1e-13)
            np.testing.assert_allclose(Lb[k] @ Lb[k].T, L1 @ L1.T, atol=1e-13)


# ----------------------------------------------------------------------------- conditional models
# The reference's tests/test_linearization.py:108-239 relations for ConditionalMomentsModel:
# exactness on a linear-Gaussian conditional model, and square-root vs covariance form on the
# population model's moments (Ricker transition, Poisson observation).

class _AffineMean:
    """E[y | x] = a x + b m_q + c (with a Jacobian for the extended method)."""

    def __init__(self, a, b, m_q, c):
        self.a, self.off = a, b @ m_q + c

    def __call__(self, x):
        return np.einsum("ij,...j->...i", self.a, np.asarray(x, dtype=float)) + self.off

    def jacobian(self, x):
        x = np.asarray(x, dtype=float)
        return np.broadcast_to(self.a, x.shape[:-1] + self.a.shape).copy()


def _conditional_chol(b, chol_q):
    """A square factor of b Q b^T: [b L_q, 0] when b has more rows than columns, else tria(b L_q)."""
    ny, nq = b.shape
    bl = b @ chol_q
    if ny > nq:
        return np.concatenate([bl, np.zeros((ny, ny - nq))], axis=1)
    from oracle.core import tria
    return tria(bl)


@pytest.mark.parametrize("dim_x", [1, 3])
@pytest.mark.parametrize("dim_q", [1, 2, 3])
@pytest.mark.parametrize("seed", [0, 42])
@pytest.mark.parametrize("method", METHODS, ids=lambda m: m.name)
@pytest.mark.parametrize("sqrt", [True, False])
def test_linear_conditional(dim_x, dim_q, seed, method, sqrt):
    from oracle.types import ConditionalMomentsModel
    np.random.seed(seed)
    a = np.random.randn(dim_x, dim_x)
    b = np.random.randn(dim_x, dim_q)
    c = np.random.randn(dim_x)
    m_x = np.random.randn(dim_x)
    m_q = np.random.randn(dim_q)
    chol_x = _rand_chol(dim_x)
    chol_q = _rand_chol(dim_q)
    mean = _AffineMean(a, b, m_q, c)
    if sqrt:
        # the factor itself (b L_q padded or triangularised), as the reference's test passes it
        fac = _conditional_chol(b, chol_q)
        model = ConditionalMomentsModel(mean, lambda x, fac=fac: np.broadcast_to(
            fac, np.shape(x)[:-1] + fac.shape).copy())
        x = MVNSqrt(m_x, chol_x)
    else:
        model = ConditionalMomentsModel(mean, OM.ConstantCovariance(b @ chol_q @ chol_q.T @ b.T))
        x = MVNStandard(m_x, chol_x @ chol_x.T)
    F, Q, rem = method(model, x)
    if sqrt:
        Q = Q @ Q.T
    xp = np.random.randn(dim_x)
    np.testing.assert_allclose(a, F, atol=1e-7)
    np.testing.assert_allclose(mean(xp), F @ xp + rem, atol=1e-7)
    np.testing.assert_allclose((b @ chol_q) @ (b @ chol_q).T, Q, atol=1e-7)


@pytest.mark.parametrize("seed", [0, 42])
@pytest.mark.parametrize("method", METHODS, ids=lambda m: m.name)
@pytest.mark.parametrize("which", ["ricker_transition", "poisson_observation"])
def test_sqrt_vs_std_conditional(seed, method, which):
    from oracle.types import ConditionalMomentsModel
    np.random.seed(seed)
    m_x = np.random.randn(1)
    chol_x = np.random.rand(1, 1)
    if which == "ricker_transition":
        mean = OM.Ricker()
        cov, chol = OM.ConstantCovariance(0.3 ** 2), OM.ConstantCovariance(0.3 ** 2, chol=True)
    else:
        mean = OM.PoissonExpMean(10.0)
        cov, chol = OM.PoissonExpCovariance(10.0), OM.PoissonExpCovariance(10.0, chol=True)
    sF, sL, sb = method(ConditionalMomentsModel(mean, chol), MVNSqrt(m_x, chol_x))
    F, Q, b = method(ConditionalMomentsModel(mean, cov), MVNStandard(m_x, chol_x @ chol_x.T))
    np.testing.assert_allclose(sF, F, atol=1e-10)
    np.testing.assert_allclose(sb, b, atol=1e-10)
    np.testing.assert_allclose(Q, sL @ sL.T, atol=1e-10)
