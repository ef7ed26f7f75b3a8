"""Random test systems, restating the reference's test helpers.

``get_system`` follows tests/_test_utils.py:6-22 of the reference (random mean,
random lower-triangular factors from ``np.random.rand``, ``H = eye(ny, nx)``),
seeded through the legacy global ``np.random`` state as the reference does.
"""
import numpy as np

from oracle.types import MVNSqrt, MVNStandard


def get_system(dim_x, dim_y):
    m = np.random.randn(dim_x)
    cholP = np.random.rand(dim_x, dim_x)
    cholP[np.triu_indices(dim_x, 1)] = 0.0
    P = cholP @ cholP.T
    cholR = np.random.rand(dim_y, dim_y)
    cholR[np.triu_indices(dim_y, 1)] = 0.0
    R = cholR @ cholR.T
    H = np.eye(dim_y, dim_x)
    c = np.random.randn(dim_y)
    y = np.random.randn(dim_y)
    return MVNStandard(m, P), MVNSqrt(m, cholP), H, R, cholR, c, y


def lgssm(dim_x, dim_y, T, seed):
    """A random linear system and FP32 data (tests/test_parallel_filter.py:165-183 setup)."""
    from sqrt_parallel_smoothers_gb300.data import lgssm_data
    np.random.seed(seed)
    x0, chol_x0, F, Q, cholQ, b, _ = get_system(dim_x, dim_x)
    _, _, H, R, cholR, c, _ = get_system(dim_x, dim_y)
    m_nominal = np.random.randn(T + 1, dim_x)
    _, ys = lgssm_data(x0.mean, F, H, R, Q, b, c, T, random_state=np.random.RandomState(seed + 1000))
    return dict(x0=x0, chol_x0=chol_x0, F=F, Q=Q, cholQ=cholQ, b=b, H=H, R=R, cholR=cholR, c=c, ys=ys,
                m_nominal=m_nominal)


def canon_np(L):
    """Flip columns of lower-triangular factors so the diagonal is >= 0."""
    L = np.array(L, dtype=float)
    d = np.diagonal(L, axis1=-2, axis2=-1)
    s = np.where(d < 0, -1.0, 1.0)
    return L * s[..., None, :]
