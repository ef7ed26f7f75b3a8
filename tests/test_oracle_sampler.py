"""Oracle pathwise sampler (CPU), porting the relation of the reference's
tests/test_sampler.py:27-72: on a linear system the sample means and variances of the drawn
trajectories match the smoothed marginals (rtol = atol = 1e-2 with 100 000 draws), in the
square-root and the covariance form; and with the same standard normals the parallel
(associative-scan) and the sequential sampler draw the same trajectories."""
import numpy as np
import pytest

from oracle import linearization as LZ
from oracle import methods as M
from oracle import sampler as OS
from tests._systems import lgssm
from tests.test_oracle_filter_smoother import _models

T = 10
N_SAMPLES = 100_000


def _filtered_and_smoothed(s, sqrt, lin):
    tm, om = _models(s, sqrt)
    x0 = s["chol_x0"] if sqrt else s["x0"]
    filt = M.filtering(s["ys"], x0, tm, om, lin, None, True)
    smooth = M.smoothing(tm, filt, lin, None, True)
    return tm, filt, smooth


@pytest.mark.parametrize("dim_x", [1, 3])
@pytest.mark.parametrize("dim_y", [2, 3])
@pytest.mark.parametrize("lin", [LZ.cubature, LZ.extended], ids=lambda m: m.name)
@pytest.mark.parametrize("sqrt", [True, False])
def test_sample_marginals_match_the_smoother(dim_x, dim_y, lin, sqrt):
    s = lgssm(dim_x, dim_y, T, 0)
    tm, filt, smooth = _filtered_and_smoothed(s, sqrt, lin)
    eps = np.random.RandomState(123).randn(T + 1, N_SAMPLES, dim_x)
    xs = OS.sampling(eps, tm, filt, lin, smooth, parallel=True)
    cov = smooth.chol @ np.swapaxes(smooth.chol, -1, -2) if sqrt else smooth.cov
    np.testing.assert_allclose(xs.mean(1), smooth.mean, rtol=1e-2, atol=1e-2)
    np.testing.assert_allclose(xs.var(1), np.diagonal(cov, axis1=1, axis2=2), rtol=1e-2, atol=1e-2)


@pytest.mark.parametrize("dim_x", [1, 3])
@pytest.mark.parametrize("sqrt", [True, False])
def test_parallel_equals_sequential_sampler(dim_x, sqrt):
    s = lgssm(dim_x, 2, T, 1)
    tm, filt, smooth = _filtered_and_smoothed(s, sqrt, LZ.extended)
    eps = np.random.RandomState(7).randn(T + 1, 64, dim_x)
    par = OS.sampling(eps, tm, filt, LZ.extended, smooth, parallel=True)
    seq = OS.sampling(eps, tm, filt, LZ.extended, smooth, parallel=False)
    np.testing.assert_allclose(par, seq, atol=1e-10)


def test_default_nominal_is_the_smoothed_trajectory():
    # parsmooth/methods.py:86-87
    s = lgssm(3, 2, T, 2)
    tm, filt, smooth = _filtered_and_smoothed(s, True, LZ.cubature)
    eps = np.random.RandomState(9).randn(T + 1, 16, 3)
    np.testing.assert_allclose(OS.sampling(eps, tm, filt, LZ.cubature),
                               OS.sampling(eps, tm, filt, LZ.cubature, smooth), atol=1e-12)
