"""Oracle model functions with analytic Jacobians (TEST INFRASTRUCTURE ONLY).

Each model is a callable ``f(x)`` vectorised over leading axes, with
``jacobian(x)`` returning ``df/dx`` of shape ``(..., d_out, d_in)``.  The
extended linearisation of the reference takes ``jax.jacfwd`` of the user
function (parsmooth/linearization/_extended.py:48-49); the oracle uses these
hand-derived Jacobians instead, cross-checked against complex-step
derivatives in ``tests/test_oracle_models.py``.
"""
import numpy as np


class LinearFunction:
    """``f(x) = A x`` (tests/_lgssm.py:5-18 and 21-35)."""

    def __init__(self, A):
        self.A = np.asarray(A, dtype=float)
        self.d_out, self.d_in = self.A.shape

    def __call__(self, x):
        return np.einsum("ij,...j->...i", self.A, x)

    def jacobian(self, x):
        x = np.asarray(x)
        return np.broadcast_to(self.A, x.shape[:-1] + self.A.shape).copy()


class CoordinatedTurn:
    """Coordinated-turn transition, state ``(x, y, vx, vy, w)``.

    Follows tests/bearings/bearings_utils.py:7-44 (same as
    notebooks/bearing_data.py:11-44), including the small-turn-rate branch
    ``|w| < 1e-6`` that replaces ``sin(w dt)/w`` by ``dt`` and
    ``(cos(w dt) - 1)/w`` by ``0``.
    """

    d_in = d_out = 5

    def __init__(self, dt):
        self.dt = float(dt)

    def _coeffs(self, w):
        dt = self.dt
        small = np.abs(w) < 1e-6
        c = np.cos(w * dt)
        s = np.sin(w * dt)
        wsafe = np.where(small, 1.0, w)
        sw = np.where(small, dt, s / wsafe)           # sin(w dt) / w
        cw = np.where(small, 0.0, (c - 1.0) / wsafe)  # (cos(w dt) - 1) / w
        # derivatives with respect to w (zero in the small branch, as jacfwd of lax.cond gives)
        dsw = np.where(small, 0.0, dt * c / wsafe - s / wsafe ** 2)
        dcw = np.where(small, 0.0, -dt * s / wsafe - (c - 1.0) / wsafe ** 2)
        return c, s, sw, cw, dsw, dcw, small

    def __call__(self, x):
        x = np.asarray(x, dtype=float)
        c, s, sw, cw, *_ = self._coeffs(x[..., 4])
        x0, x1, x2, x3, w = (x[..., i] for i in range(5))
        return np.stack([x0 + sw * x2 - cw * x3,
                         x1 + cw * x2 + sw * x3,
                         c * x2 + s * x3,
                         -s * x2 + c * x3,
                         w], axis=-1)

    def jacobian(self, x):
        x = np.asarray(x, dtype=float)
        c, s, sw, cw, dsw, dcw, _ = self._coeffs(x[..., 4])
        dt = self.dt
        x2, x3 = x[..., 2], x[..., 3]
        J = np.zeros(x.shape[:-1] + (5, 5))
        J[..., 0, 0] = 1.0
        J[..., 0, 2] = sw
        J[..., 0, 3] = -cw
        J[..., 0, 4] = dsw * x2 - dcw * x3
        J[..., 1, 1] = 1.0
        J[..., 1, 2] = cw
        J[..., 1, 3] = sw
        J[..., 1, 4] = dcw * x2 + dsw * x3
        J[..., 2, 2] = c
        J[..., 2, 3] = s
        J[..., 2, 4] = -dt * s * x2 + dt * c * x3
        J[..., 3, 2] = -s
        J[..., 3, 3] = c
        J[..., 3, 4] = -dt * c * x2 - dt * s * x3
        J[..., 4, 4] = 1.0
        return J


class Bearings:
    """Two bearings ``atan2(y - s_y, x - s_x)`` (tests/bearings/bearings_utils.py:47-69)."""

    d_out = 2

    def __init__(self, s1, s2, d_in=5):
        self.s1 = np.asarray(s1, dtype=float)
        self.s2 = np.asarray(s2, dtype=float)
        self.d_in = d_in

    def __call__(self, x):
        x = np.asarray(x)
        return np.stack([np.arctan2(x[..., 1] - self.s1[1], x[..., 0] - self.s1[0]),
                         np.arctan2(x[..., 1] - self.s2[1], x[..., 0] - self.s2[0])], axis=-1)

    def jacobian(self, x):
        x = np.asarray(x, dtype=float)
        J = np.zeros(x.shape[:-1] + (2, self.d_in))
        for k, s in enumerate((self.s1, self.s2)):
            dx = x[..., 0] - s[0]
            dy = x[..., 1] - s[1]
            r2 = dx * dx + dy * dy
            J[..., k, 0] = -dy / r2
            J[..., k, 1] = dx / r2
        return J


def bearings_noise(qc, qw, r, dt):
    """Process and observation covariances of the bearings model.

    Follows tests/bearings/bearings_utils.py:72-115 (``make_parameters``).
    """
    Q = np.array([[qc * dt ** 3 / 3, 0, qc * dt ** 2 / 2, 0, 0],
                  [0, qc * dt ** 3 / 3, 0, qc * dt ** 2 / 2, 0],
                  [qc * dt ** 2 / 2, 0, qc * dt, 0, 0],
                  [0, qc * dt ** 2 / 2, 0, qc * dt, 0],
                  [0, 0, 0, 0, dt * qw]])
    R = r ** 2 * np.eye(2)
    return Q, R


class Ricker:
    """``a + x - exp(x)`` elementwise (notebooks/population_model.py:9-35, a = log 44.7)."""

    def __init__(self, a=np.log(44.7)):
        self.a = float(a)

    def __call__(self, x):
        x = np.asarray(x, dtype=float)
        return self.a + x - np.exp(x)

    def jacobian(self, x):
        x = np.asarray(x, dtype=float)
        return np.eye(x.shape[-1]) * (1.0 - np.exp(x))[..., None, :]


class ConstantCovariance:
    """``x -> Q`` (and its Cholesky factor with ``chol=True``), batched
    (notebooks/population_model.py:38-65)."""

    def __init__(self, Q, chol=False):
        Q = np.atleast_2d(np.asarray(Q, dtype=float))
        self.M = np.linalg.cholesky(Q) if chol else Q

    def __call__(self, x):
        x = np.asarray(x, dtype=float)
        return np.broadcast_to(self.M, x.shape[:-1] + self.M.shape).copy()


class PoissonExpMean:
    """``E[y | x] = lam exp(x)`` (notebooks/population_model.py:83-98)."""

    def __init__(self, lam, d_out=1):
        self.lam, self.d_out = float(lam), int(d_out)

    def __call__(self, x):
        x = np.asarray(x, dtype=float)
        return self.lam * np.exp(x[..., :self.d_out])

    def jacobian(self, x):
        x = np.asarray(x, dtype=float)
        J = np.zeros(x.shape[:-1] + (self.d_out, x.shape[-1]))
        for k in range(self.d_out):
            J[..., k, k] = self.lam * np.exp(x[..., k])
        return J


class PoissonExpCovariance:
    """``Cov[y | x] = diag(lam exp(x))`` or its square root with ``chol=True``
    (notebooks/population_model.py:101-118)."""

    def __init__(self, lam, d_out=1, chol=False):
        self.lam, self.d_out, self.chol = float(lam), int(d_out), chol

    def __call__(self, x):
        x = np.asarray(x, dtype=float)
        v = self.lam * np.exp(x[..., :self.d_out])
        if self.chol:
            v = np.sqrt(v)
        out = np.zeros(x.shape[:-1] + (self.d_out, self.d_out))
        for k in range(self.d_out):
            out[..., k, k] = v[..., k]
        return out
