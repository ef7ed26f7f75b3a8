"""Seeded synthetic workloads for the smoother (host side, NumPy).

The reference ships no dataset for this path; its experiments simulate data.
These generators restate the reference's simulators so that benchmarks and
tests run on inputs with the same shapes and distributions:

* :func:`lgssm_data` - linear Gaussian SSM, tests/_lgssm.py:42-95 (FP32 draws).
* :func:`bearings_data` - coordinated-turn target seen by two bearings
  sensors, notebooks/bearing_data.py:137-198.  The reference propagates the
  state with ``scipy.linalg.expm`` of the 4x4 turn generator; here the same
  matrix exponential is evaluated in closed form (it is the coordinated-turn
  matrix), vectorised over a batch of sequences.
* workload builders for the five benchmark configurations (constant-velocity
  linear model, bearings model, ragged batch, adjoint batch, large random
  stable linear model).
"""
import numpy as np

BEARINGS_S1 = (-1.5, 0.5)
BEARINGS_S2 = (1.0, 1.0)


def lgssm_data(x0, A, H, R, Q, b, c, T, random_state=None, chol_R=None):
    """Simulate ``x_{t+1} = A x_t + b + q``, ``y = H x + c + r`` in FP32 (tests/_lgssm.py:42-95)."""
    if random_state is None or isinstance(random_state, (int, np.integer)):
        random_state = np.random.RandomState(random_state)
    ny, nx = R.shape[0], Q.shape[0]
    normals = random_state.randn(T, nx + ny).astype(np.float32)
    chol_R = np.linalg.cholesky(R) if chol_R is None else chol_R
    chol_Q = np.linalg.cholesky(Q)
    x = np.array(x0, dtype=np.float32)
    ys = np.empty((T, ny), dtype=np.float32)
    xs = np.empty((T + 1, nx), dtype=np.float32)
    xs[0] = x
    for i in range(T):
        x = A @ x + chol_Q @ normals[i, :nx] + b
        xs[i + 1] = x
        ys[i] = H @ x + chol_R @ normals[i, nx:] + c
    return xs, ys


def bearings_noise(qc, qw, r, dt):
    """Process/observation covariances of the bearings model (tests/bearings/bearings_utils.py:72-115)."""
    Q = np.array([[qc * dt ** 3 / 3, 0, qc * dt ** 2 / 2, 0, 0],
                  [0, qc * dt ** 3 / 3, 0, qc * dt ** 2 / 2, 0],
                  [qc * dt ** 2 / 2, 0, qc * dt, 0, 0],
                  [0, qc * dt ** 2 / 2, 0, qc * dt, 0],
                  [0, 0, 0, 0, dt * qw]])
    return Q, r ** 2 * np.eye(2)


def bearings_data(x0, dt, r, T, s1=BEARINGS_S1, s2=BEARINGS_S2, q=10.0, random_state=None):
    """Simulate one bearings-only sequence (notebooks/bearing_data.py:154-198).

    Turn rates ``a_t = 1 + q dt cumsum(N(0,1))``, state propagated by the
    exact exponential of the turn generator, bearings noise ``r * N(0,1)``.
    Returns ``(true_states (T+1, 5), observations (T, 2))`` in FP32.
    """
    if random_state is None or isinstance(random_state, (int, np.integer)):
        random_state = np.random.RandomState(random_state)
    a_s = (1 + q * dt * np.cumsum(random_state.randn(T))).astype(np.float32)
    normals = random_state.randn(T, 2).astype(np.float32)
    return _bearings_propagate(np.asarray(x0, np.float32)[None], dt, r, a_s[None], normals[None],
                               s1, s2)


def _bearings_propagate(x0, dt, r, a_s, normals, s1, s2):
    B, T = a_s.shape
    x = np.array(x0, dtype=np.float64)
    states = np.zeros((B, T + 1, 5), dtype=np.float32)
    ys = np.empty((B, T, 2), dtype=np.float32)
    states[:, 0, :4] = x
    s1 = np.asarray(s1, np.float32)
    s2 = np.asarray(s2, np.float32)
    for i in range(T):
        a = a_s[:, i].astype(np.float64)
        c, s = np.cos(a * dt), np.sin(a * dt)
        sa = np.where(a == 0, dt, s / np.where(a == 0, 1, a))
        ca = np.where(a == 0, 0.0, (1 - c) / np.where(a == 0, 1, a))
        px, py, vx, vy = x.T
        x = np.stack([px + sa * vx + ca * vy, py - ca * vx + sa * vy, c * vx + s * vy, -s * vx + c * vy], 1)
        x = x.astype(np.float32).astype(np.float64)
        ys[:, i, 0] = np.arctan2(x[:, 1] - s1[1], x[:, 0] - s1[0]) + r * normals[:, i, 0]
        ys[:, i, 1] = np.arctan2(x[:, 1] - s2[1], x[:, 0] - s2[0]) + r * normals[:, i, 1]
        states[:, i + 1, :4] = x
        states[:, i + 1, 4] = a_s[:, i]
    return states[0] if B == 1 else states, ys[0] if B == 1 else ys


# ----------------------------------------------------------------------------- workloads

def cv_model(dt=0.1, q=0.1, r=0.5):
    """2-D constant-velocity model, nx=4, ny=2: ``(F, Q, H, R)``."""
    I2 = np.eye(2)
    F = np.block([[I2, dt * I2], [np.zeros((2, 2)), I2]])
    Q = q * np.block([[dt ** 3 / 3 * I2, dt ** 2 / 2 * I2], [dt ** 2 / 2 * I2, dt * I2]])
    H = np.block([I2, np.zeros((2, 2))])
    return F, Q, H, r * I2


def cv_workload(T=1000, seed=0):
    """Constant-velocity workload (dt=0.1, q=0.1, R=0.5 I, m0=0, P0=I), simulated from ``seed``."""
    F, Q, H, R = cv_model()
    xs, ys = lgssm_data(np.zeros(4), F, H, R, Q, np.zeros(4), np.zeros(2), T, seed)
    return dict(F=F, Q=Q, H=H, R=R, m0=np.zeros(4), P0=np.eye(4), ys=ys, xs=xs)


BEARINGS_M0 = np.array([-4.0, -1.0, 2.0, 7.0, 3.0])


def bearings_workload(T, seed=0, qc=0.1, qw=0.5, sigma=0.05, dt=0.01):
    """Bearings-only coordinated-turn workload for one sequence of length ``T``.

    Data from :func:`bearings_data` with ``x0=(0.1, 0.2, 1, 0)``, ``q=10`` and
    bearing noise ``sigma``; model noise from :func:`bearings_noise` with
    ``qc``/``qw``; prior ``m0=(-4,-1,2,7,3)``, ``P0=I``.
    """
    xs, ys = bearings_data([0.1, 0.2, 1.0, 0.0], dt, sigma, T, q=10.0, random_state=seed)
    Q, R = bearings_noise(qc, qw, sigma, dt)
    return dict(Q=Q, R=R, dt=dt, m0=BEARINGS_M0.copy(), P0=np.eye(5), ys=ys, xs=xs)


def ragged_lengths(B, lo=50, hi=5000, seed=0):
    """Lengths drawn log-uniform in ``[lo, hi]`` and rounded, from ``seed``."""
    rng = np.random.RandomState(seed)
    return np.round(np.exp(rng.uniform(np.log(lo), np.log(hi), size=B))).astype(np.int64)


def bearings_batch(lengths, qc=0.1, qw=0.5, sigma=0.05, dt=0.01, seed0=0):
    """Ragged batch of bearings sequences; sequence ``i`` is simulated from seed ``seed0 + i``.

    Returns packed observations ``(sum T_i, 2)``, ``offsets (B+1,)`` and packed
    true states ``(sum (T_i + 1), 5)``.
    """
    lengths = np.asarray(lengths, dtype=np.int64)
    B = len(lengths)
    Tmax = int(lengths.max()) if B else 0
    a_s = np.empty((B, Tmax), np.float32)
    normals = np.empty((B, Tmax, 2), np.float32)
    for i, T in enumerate(lengths):
        rs = np.random.RandomState(seed0 + i)
        a_s[i, :T] = (1 + 10.0 * dt * np.cumsum(rs.randn(T))).astype(np.float32)
        normals[i, :T] = rs.randn(T, 2).astype(np.float32)
        a_s[i, T:] = a_s[i, T - 1] if T else 1.0
        normals[i, T:] = 0
    x0 = np.tile(np.array([0.1, 0.2, 1.0, 0.0], np.float32), (B, 1))
    states, ys = _bearings_propagate(x0, dt, sigma, a_s, normals, BEARINGS_S1, BEARINGS_S2)
    if B == 1:
        states, ys = states[None], ys[None]
    offsets = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64)
    ys_p = np.concatenate([ys[i, :T] for i, T in enumerate(lengths)]) if B else np.zeros((0, 2), np.float32)
    xs_p = np.concatenate([states[i, :T + 1] for i, T in enumerate(lengths)])
    Q, R = bearings_noise(qc, qw, sigma, dt)
    return dict(Q=Q, R=R, dt=dt, m0=BEARINGS_M0.copy(), P0=np.eye(5), ys=ys_p, offsets=offsets,
                xs=xs_p, lengths=lengths)


def large_state_model(nx=32, ny=16, seed=0):
    """Random stable linear SSM: ``F = 0.98 * Haar orthogonal``, ``Q = L L^T / nx``, ``H ~ N(0, 1/nx)``, ``R = 0.1 I``."""
    rng = np.random.RandomState(seed)
    G = rng.randn(nx, nx)
    Qm, Rm = np.linalg.qr(G)
    Qm = Qm * np.sign(np.diag(Rm))[None, :]
    F = 0.98 * Qm
    L = rng.randn(nx, nx)
    Q = L @ L.T / nx
    H = rng.randn(ny, nx) / np.sqrt(nx)
    R = 0.1 * np.eye(ny)
    return F, Q, H, R


def population_data(T, Q=0.3 ** 2, lam=10.0, x0=np.log(7.0), seed=40):
    """Stochastic Ricker map with Poisson counts (notebooks/population_model.py:172-208):
    x_{t+1} = log 44.7 + x_t - exp(x_t) + N(0, Q), y_t ~ Poisson(lam exp(x_t)) for t = 1..T,
    seeded with NumPy.  Returns ``(xs (T+1, 1), ys (T, 1))``."""
    rng = np.random.RandomState(seed)
    xs = np.empty((T + 1, 1))
    ys = np.empty((T, 1))
    xs[0] = x0
    for t in range(T):
        xs[t + 1] = np.log(44.7) + xs[t] - np.exp(xs[t]) + np.sqrt(Q) * rng.randn(1)
        ys[t] = rng.poisson(lam * np.exp(xs[t + 1]))
    return xs, ys
