"""Device model registry.

``parsmooth`` linearises arbitrary JAX callables.  CUDA kernels cannot call
Python, so a ``FunctionalModel`` here must wrap one of these models; each
selects a C++ functor compiled into the library (``csrc/ss_models.cuh``).
Calling a model evaluates it with torch for convenience (host or device);
the smoother itself never does.
"""
import math

import torch

from . import _lib


class DeviceModel:
    """Base class: ``kind`` (C enum), dimensions and scalar parameters."""
    kind = -1
    d_in = d_out = 0

    def params(self):
        return [0.0, 0.0, 0.0, 0.0]

    def matrix(self):
        return None


class LinearModel(DeviceModel):
    """``f(x) = A x`` (the reference tests' ``transition_function``/``observation_function``,
    tests/_lgssm.py:5-35)."""
    kind = _lib.SS_MODEL_LINEAR

    def __init__(self, A):
        self.A = torch.as_tensor(A, dtype=torch.float64).detach().cpu()
        if self.A.ndim != 2:
            raise ValueError("LinearModel expects a matrix")
        self.d_out, self.d_in = self.A.shape

    def matrix(self):
        return self.A

    def __call__(self, x):
        x = torch.as_tensor(x)
        return x @ self.A.to(x.dtype).to(x.device).T

    def __repr__(self):
        return f"LinearModel({self.d_out}x{self.d_in})"


class CoordinatedTurn(DeviceModel):
    """Coordinated-turn transition of state ``(x, y, vx, vy, w)`` with step ``dt``
    (tests/bearings/bearings_utils.py:7-44)."""
    kind = _lib.SS_MODEL_COORDINATED_TURN
    d_in = d_out = 5

    def __init__(self, dt):
        self.dt = float(dt)

    def params(self):
        return [self.dt, 0.0, 0.0, 0.0]

    def __call__(self, x):
        x = torch.as_tensor(x)
        w = x[..., 4]
        c, s = torch.cos(w * self.dt), torch.sin(w * self.dt)
        small = w.abs() < 1e-6
        wsafe = torch.where(small, torch.ones_like(w), w)
        sw = torch.where(small, torch.full_like(w, self.dt), s / wsafe)
        cw = torch.where(small, torch.zeros_like(w), (c - 1) / wsafe)
        x0, x1, x2, x3 = x[..., 0], x[..., 1], x[..., 2], x[..., 3]
        return torch.stack([x0 + sw * x2 - cw * x3, x1 + cw * x2 + sw * x3, c * x2 + s * x3,
                            -s * x2 + c * x3, w], dim=-1)

    def __repr__(self):
        return f"CoordinatedTurn(dt={self.dt})"


class Bearings(DeviceModel):
    """Bearings ``atan2(y - s_y, x - s_x)`` from two sensors ``s1``, ``s2``
    (tests/bearings/bearings_utils.py:47-69).  ``d_in`` is the state dimension."""
    kind = _lib.SS_MODEL_BEARINGS
    d_out = 2

    def __init__(self, s1, s2, d_in=5):
        self.s1 = [float(v) for v in s1]
        self.s2 = [float(v) for v in s2]
        self.d_in = int(d_in)

    def params(self):
        return self.s1 + self.s2

    def __call__(self, x):
        x = torch.as_tensor(x)
        return torch.stack([torch.atan2(x[..., 1] - self.s1[1], x[..., 0] - self.s1[0]),
                            torch.atan2(x[..., 1] - self.s2[1], x[..., 0] - self.s2[0])], dim=-1)

    def __repr__(self):
        return f"Bearings(s1={self.s1}, s2={self.s2})"


class Ricker(DeviceModel):
    """Ricker map on the log scale, elementwise ``f(x) = a + x - exp(x)`` with ``a = log 44.7``
    by default (notebooks/population_model.py:9-21).  Use it in a ``FunctionalModel`` with
    additive Gaussian noise, or through :func:`population_parameters` as the reference's
    conditional-moments transition (constant conditional covariance ``Q``)."""
    kind = _lib.SS_MODEL_RICKER

    def __init__(self, a=math.log(44.7), d=1, Q=None):
        self.a = float(a)
        self.d_in = self.d_out = int(d)
        self.Q = None if Q is None else torch.as_tensor(Q, dtype=torch.float64).reshape(self.d_in, self.d_in)

    def params(self):
        return [self.a, 0.0, 0.0, 0.0]

    def __call__(self, x):
        x = torch.as_tensor(x)
        return self.a + x - torch.exp(x)

    # conditional moments (the reference's _mean/_cov/_chol_transition_function)
    def conditional_mean(self, x):
        return self(x)

    def conditional_cov(self, x):
        return self.Q

    def conditional_chol(self, x):
        return torch.linalg.cholesky(self.Q)

    def noise_chol(self):
        return torch.linalg.cholesky(self.Q)

    def __repr__(self):
        return f"Ricker(a={self.a}, d={self.d_in})"


class PoissonExp(DeviceModel):
    """Poisson counts with log-intensity x: ``E[y_k | x] = Var[y_k | x] = lam exp(x_k)`` for the
    first ``d_out`` state components (notebooks/population_model.py:83-118).  A
    conditional-moments model: ``ConditionalMomentsModel(m.conditional_mean,
    m.conditional_cov)`` (or ``m.conditional_chol``)."""
    kind = _lib.SS_MODEL_POISSON_EXP
    conditional = True

    def __init__(self, lam, d_in=1, d_out=1):
        self.lam = float(lam)
        self.d_in, self.d_out = int(d_in), int(d_out)
        if self.d_out > self.d_in:
            raise ValueError("PoissonExp observes at most d_in components")

    def params(self):
        return [self.lam, 0.0, 0.0, 0.0]

    def __call__(self, x):
        x = torch.as_tensor(x)
        return self.lam * torch.exp(x[..., :self.d_out])

    def conditional_mean(self, x):
        return self(x)

    def conditional_cov(self, x):
        return torch.diag_embed(self(x))

    def conditional_chol(self, x):
        return torch.diag_embed(torch.sqrt(self(x)))

    def noise_chol(self):
        return torch.zeros(self.d_out, self.d_out, dtype=torch.float64)

    def __repr__(self):
        return f"PoissonExp(lam={self.lam})"


def population_parameters(lam, Q):
    """The reference's population model ``make_parameters(lam, Q)``
    (notebooks/population_model.py:121-169) with device models: the conditional mean,
    covariance and square-root functions of the Ricker transition and the Poisson
    observation, ``(mean_f, cov_f, mean_h, cov_h, chol_f, chol_h)``."""
    f = Ricker(Q=Q)
    h = PoissonExp(lam)
    return (f.conditional_mean, f.conditional_cov, h.conditional_mean, h.conditional_cov, f.conditional_chol,
            h.conditional_chol)


def bearings_parameters(qc, qw, r, dt, s1, s2):
    """``(Q, R, observation_function, transition_function)`` as the reference's
    ``make_parameters`` (tests/bearings/bearings_utils.py:72-115), with device models."""
    Q = torch.tensor([[qc * dt ** 3 / 3, 0, qc * dt ** 2 / 2, 0, 0],
                      [0, qc * dt ** 3 / 3, 0, qc * dt ** 2 / 2, 0],
                      [qc * dt ** 2 / 2, 0, qc * dt, 0, 0],
                      [0, qc * dt ** 2 / 2, 0, qc * dt, 0],
                      [0, 0, 0, 0, dt * qw]], dtype=torch.float64)
    R = r ** 2 * torch.eye(2, dtype=torch.float64)
    return Q, R, Bearings(s1, s2), CoordinatedTurn(dt)


def conditional_owner(model):
    """The device model behind a ``ConditionalMomentsModel`` built from its bound methods."""
    owner = getattr(model.conditional_mean, "__self__", None)
    if isinstance(owner, DeviceModel) and getattr(model.conditional_covariance_or_cholesky, "__self__", None) is owner:
        return owner
    raise NotImplementedError(
        "a ConditionalMomentsModel on the GPU must use the conditional moments of one device model "
        "(e.g. ConditionalMomentsModel(PoissonExp(lam).conditional_mean, PoissonExp(lam).conditional_cov) "
        "built from the same object, or population_parameters)")


def as_device_model(function):
    """Return ``function`` if it is a registry model, else raise ``NotImplementedError``."""
    if isinstance(function, DeviceModel):
        return function
    raise NotImplementedError(
        "the GPU smoother needs a device model (LinearModel, CoordinatedTurn, Bearings, Ricker, PoissonExp); "
        f"got {function!r}. Arbitrary Python callables cannot run inside CUDA kernels.")
