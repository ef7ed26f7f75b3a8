"""Pathwise posterior sampler (parsmooth.sampling): the GPU draws match the oracle's
restatement sample by sample for the same standard normals, and the draws' moments match
the smoother's."""
import numpy as np
import pytest
import torch

import oracle as O
import sqrt_parallel_smoothers_gb300 as S
from oracle import sampler as OS
from tests._parity import assert_rel, bearings_pair, linear_pair

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("method", ["extended", "cubature"])
def test_sampler_matches_oracle_bearings(method):
    (ot, oo), (gt, go) = bearings_pair(0.1, 0.5, 0.05)
    T, n = 60, 17
    w = S.data.bearings_workload(T, seed=6)
    ys = w["ys"].astype(np.float64)
    m0 = np.array([0.1, 0.2, 1.0, 0.0, 1.0])
    filt = O.methods.filtering(ys, O.MVNSqrt(m0, np.eye(5)), ot, oo, getattr(O.linearization, method), None, True)
    eps = np.random.RandomState(1).randn(T + 1, n, 5)
    ref = OS.sampling(eps, ot, filt, getattr(O.linearization, method))
    got = S.sampling(None, n, gt, S.MVNSqrt(torch.as_tensor(filt.mean), torch.as_tensor(filt.chol)),
                     getattr(S.linearization, method), eps=eps)
    assert got.shape == (T + 1, n, 5)
    # each side linearises at its own smoothed trajectory (the default nominal), which agree
    # to ~1e-10; the recursion over 60 steps carries that to a few 1e-9
    assert_rel(got, ref, 1e-8, "samples")


def test_sampler_ragged_batch_and_explicit_nominal():
    rng = np.random.RandomState(3)
    F = np.array([[1.0, 0.1], [0.0, 1.0]])
    ot, gt = linear_pair(F, np.zeros(2), np.linalg.cholesky(0.1 * np.eye(2)))
    oo, go = linear_pair(np.eye(1, 2), np.zeros(1), np.linalg.cholesky(0.5 * np.eye(1)))
    lengths = np.array([20, 0, 7])
    Tm, n = int(lengths.max()), 5
    ys = rng.randn(3, Tm, 1)
    eps = rng.randn(3, Tm + 1, n, 2)
    fm = np.zeros((3, Tm + 1, 2))
    fL = np.zeros((3, Tm + 1, 2, 2))
    refs = []
    for i, T in enumerate(lengths):
        f = O.methods.filtering(ys[i, :T], O.MVNSqrt(np.zeros(2), np.eye(2)), ot, oo, O.linearization.extended,
                                None, True)
        fm[i, :T + 1], fL[i, :T + 1] = f.mean, f.chol
        nom = O.MVNSqrt(np.zeros((T + 1, 2)), np.repeat(np.eye(2)[None], T + 1, 0))
        refs.append(OS.sampling(eps[i, :T + 1], ot, f, O.linearization.extended, nom))
    nom_g = S.MVNSqrt(torch.zeros(3, Tm + 1, 2, dtype=torch.float64),
                      torch.eye(2, dtype=torch.float64).expand(3, Tm + 1, 2, 2).contiguous())
    got = S.sampling(None, n, gt, S.MVNSqrt(torch.as_tensor(fm), torch.as_tensor(fL)), S.linearization.extended,
                     nom_g, lengths=lengths, eps=eps)
    for i, T in enumerate(lengths):
        assert_rel(got[i, :T + 1], refs[i], 1e-10, f"seq {i}")


def test_sampler_moments_match_the_smoother():
    """With a seed: the mean and covariance of 20 000 draws match the smoothed mean and
    covariance to Monte-Carlo accuracy (5 standard errors)."""
    rng = np.random.RandomState(7)
    F = np.array([[1.0, 0.1], [0.0, 1.0]])
    ot, gt = linear_pair(F, np.zeros(2), np.linalg.cholesky(0.1 * np.eye(2)))
    oo, go = linear_pair(np.eye(1, 2), np.zeros(1), np.linalg.cholesky(0.5 * np.eye(1)))
    ys = torch.as_tensor(rng.randn(40, 1))
    x0 = S.MVNSqrt(torch.zeros(2, dtype=torch.float64), torch.eye(2, dtype=torch.float64))
    filt = S.filtering(ys, x0, gt, go, S.linearization.extended)
    sm = S.smoothing(gt, filt, S.linearization.extended)
    n = 20_000
    xs = S.sampling(123, n, gt, filt, S.linearization.extended)
    mean = xs.mean(1)
    cov_s = sm.chol @ sm.chol.transpose(-1, -2)
    se = torch.sqrt(torch.diagonal(cov_s, dim1=-2, dim2=-1) / n)
    assert bool(((mean - sm.mean).abs() <= 5 * se + 1e-12).all())
    d = xs - mean[:, None]
    emp = torch.einsum("tsi,tsj->tij", d, d) / (n - 1)
    assert float((emp - cov_s).abs().max()) <= 0.05 * float(cov_s.abs().max())


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-9), (torch.float32, 2e-3)])
def test_sampler_parallel_in_time_long_sequence(dtype, tol):
    """Few draws of a long sequence take the parallel-in-time sampler (chunk maps composed,
    scanned and replayed, as the reference's _par_sampling composes its affine maps); the
    draws equal the oracle's for the same normals and the same nominal."""
    (ot, oo), (gt, go) = bearings_pair(0.1, 0.5, 0.05)
    T, n = 3000, 2
    w = S.data.bearings_batch(np.array([T]), seed0=4)
    ys = w["ys"].astype(np.float64)
    m0 = np.array([0.1, 0.2, 1.0, 0.0, 1.0])
    filt = O.methods.filtering(ys, O.MVNSqrt(m0, np.eye(5)), ot, oo, O.linearization.extended, None, True)
    nom = O.methods.smoothing(ot, filt, O.linearization.extended, None, True)
    eps = np.random.RandomState(2).randn(T + 1, n, 5)
    ref = OS.sampling(eps, ot, filt, O.linearization.extended, nom)
    got = S.sampling(None, n, gt, S.MVNSqrt(torch.as_tensor(np.ascontiguousarray(filt.mean), dtype=dtype),
                                            torch.as_tensor(np.ascontiguousarray(filt.chol), dtype=dtype)),
                     S.linearization.extended, S.MVNSqrt(torch.as_tensor(np.ascontiguousarray(nom.mean), dtype=dtype),
                                                         torch.as_tensor(np.ascontiguousarray(nom.chol), dtype=dtype)),
                     eps=torch.as_tensor(eps, dtype=dtype))
    assert got.shape == (T + 1, n, 5)
    assert_rel(got, ref, tol, "samples")


def test_sampler_parallel_in_time_ragged_batch():
    rng = np.random.RandomState(5)
    F = np.array([[1.0, 0.1], [0.0, 1.0]])
    ot, gt = linear_pair(F, np.zeros(2), np.linalg.cholesky(0.1 * np.eye(2)))
    oo, go = linear_pair(np.eye(1, 2), np.zeros(1), np.linalg.cholesky(0.5 * np.eye(1)))
    lengths = np.array([500, 0, 130, 64, 1])
    Tm, n = int(lengths.max()), 3
    ys = rng.randn(len(lengths), Tm, 1)
    eps = rng.randn(len(lengths), Tm + 1, n, 2)
    fm = np.zeros((len(lengths), Tm + 1, 2))
    fL = np.zeros((len(lengths), Tm + 1, 2, 2))
    refs = []
    for i, T in enumerate(lengths):
        f = O.methods.filtering(ys[i, :T], O.MVNSqrt(np.zeros(2), np.eye(2)), ot, oo, O.linearization.extended,
                                None, True)
        fm[i, :T + 1], fL[i, :T + 1] = f.mean, f.chol
        nom = O.MVNSqrt(np.zeros((T + 1, 2)), np.repeat(np.eye(2)[None], T + 1, 0))
        refs.append(OS.sampling(eps[i, :T + 1], ot, f, O.linearization.extended, nom))
    nom_g = S.MVNSqrt(torch.zeros(len(lengths), Tm + 1, 2, dtype=torch.float64),
                      torch.eye(2, dtype=torch.float64).expand(len(lengths), Tm + 1, 2, 2).contiguous())
    got = S.sampling(None, n, gt, S.MVNSqrt(torch.as_tensor(fm), torch.as_tensor(fL)), S.linearization.extended,
                     nom_g, lengths=lengths, eps=eps)
    for i, T in enumerate(lengths):
        assert_rel(got[i, :T + 1], refs[i], 1e-10, f"seq {i}")
