"""Large-state (dense, warp-per-item) path: linear models with nx = 8 and 32 against the
oracle, on ragged batches whose scans have several levels (chunk 8, group 2)."""
import numpy as np
import pytest
import torch

import oracle as O
import sqrt_parallel_smoothers_gb300 as S
from tests._parity import assert_rel, cov, linear_pair

pytestmark = pytest.mark.gpu

DIMS = [(8, 4), (32, 16)]
LENGTHS = np.array([37, 1, 0, 70])


def _system(nx, ny, seed=0):
    F, Q, H, R = S.data.large_state_model(nx, ny, seed)
    rng = np.random.RandomState(seed + 1)
    qm, rm = 0.05 * rng.randn(nx), 0.05 * rng.randn(ny)
    ot, gt = linear_pair(F, qm, np.linalg.cholesky(Q))
    oo, go = linear_pair(H, rm, np.linalg.cholesky(R))
    return (F, Q, H, R, qm, rm), (ot, oo), (gt, go)


def _observations(sysm, lengths, seed=0):
    F, Q, H, R, qm, rm = sysm
    nx, ny = F.shape[0], H.shape[0]
    rng = np.random.RandomState(seed + 7)
    cQ, cR = np.linalg.cholesky(Q), np.linalg.cholesky(R)
    ys = np.zeros((len(lengths), int(lengths.max()), ny))
    for i, T in enumerate(lengths):
        x = rng.randn(nx)
        for t in range(T):
            x = F @ x + qm + cQ @ rng.randn(nx)
            ys[i, t] = H @ x + rm + cR @ rng.randn(ny)
    return ys


def _prior(nx, seed=3):
    rng = np.random.RandomState(seed)
    m0 = 0.3 * rng.randn(nx)
    L0 = np.linalg.cholesky(np.eye(nx) + 0.1 * np.ones((nx, nx)))
    return m0, L0


@pytest.mark.parametrize("nx,ny", DIMS)
@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-9), (torch.float32, 2e-3)])
def test_dense_filter_and_smoother_vs_oracle(nx, ny, dtype, tol):
    sysm, (ot, oo), (gt, go) = _system(nx, ny)
    ys = _observations(sysm, LENGTHS)
    m0, L0 = _prior(nx)
    x0 = S.MVNSqrt(torch.as_tensor(m0), torch.as_tensor(L0))
    filt, ell = S.filtering(torch.as_tensor(ys, dtype=dtype), x0, gt, go, S.linearization.extended, None,
                            return_loglikelihood=True, lengths=LENGTHS, chunk=8, group=2)
    smooth = S.smoothing(gt, filt, S.linearization.extended, None, lengths=LENGTHS, chunk=8, group=2)
    for i, T in enumerate(LENGTHS):
        ref_f, ref_ell = O.methods.filtering(ys[i, :T], O.MVNSqrt(m0, L0), ot, oo, O.linearization.extended,
                                             None, True, return_loglikelihood=True)
        assert_rel(filt.mean[i, :T + 1], ref_f.mean, tol, f"seq {i} filtered mean")
        assert_rel(cov(filt.chol[i, :T + 1]), cov(ref_f.chol), tol, f"seq {i} filtered cov")
        if T > 0:
            assert abs(float(ell[i]) - ref_ell) <= tol * max(1.0, abs(ref_ell)), (i, float(ell[i]), ref_ell)
        ref_s = O.methods.smoothing(ot, ref_f, O.linearization.extended, None, True)
        assert_rel(smooth.mean[i, :T + 1], ref_s.mean, tol, f"seq {i} smoothed mean")
        assert_rel(cov(smooth.chol[i, :T + 1]), cov(ref_s.chol), tol, f"seq {i} smoothed cov")


@pytest.mark.parametrize("nx,ny", DIMS)
@pytest.mark.parametrize("method", ["extended", "cubature"])
def test_dense_iterated_vs_oracle(nx, ny, method):
    """Two filter-smoother calls from the default nominal (the reference's extra first pass
    included); a linear model makes every rule exact, so both rules give the oracle's result."""
    sysm, (ot, oo), (gt, go) = _system(nx, ny, seed=5)
    lengths = np.array([50, 19])
    ys = _observations(sysm, lengths, seed=5)
    m0, L0 = _prior(nx)
    x0 = S.MVNSqrt(torch.as_tensor(m0), torch.as_tensor(L0))
    res, ell, info = S.iterated_smoothing(torch.as_tensor(ys), x0, gt, go, getattr(S.linearization, method),
                                          None, criterion=lambda i, *_: i < 2, return_loglikelihood=True,
                                          lengths=lengths, return_info=True, chunk=8, group=2)
    for i, T in enumerate(lengths):
        ref, ref_ell = O.methods.iterated_smoothing(ys[i, :T], O.MVNSqrt(m0, L0), ot, oo,
                                                    O.linearization.extended, None, True,
                                                    criterion=lambda k, *_: k < 2, return_loglikelihood=True)
        assert_rel(res.mean[i, :T + 1], ref.mean, 1e-9, f"seq {i} mean")
        assert_rel(cov(res.chol[i, :T + 1]), cov(ref.chol), 1e-9, f"seq {i} cov")
        assert abs(float(ell[i]) - ref_ell) <= 1e-9 * abs(ref_ell)
    assert int(info["iterations"][0]) == 2
    assert int(info["flags"].abs().sum()) == 0


def test_dense_default_criterion_stops_after_one_call():
    """Linear model: the first counted call reproduces the initial pass, so the default test
    (mean squared change > 1e-6) stops after exactly one call, as in the reference."""
    sysm, _, (gt, go) = _system(32, 16, seed=2)
    lengths = np.array([120])
    ys = _observations(sysm, lengths, seed=2)
    m0, L0 = _prior(32)
    res, info = S.iterated_smoothing(torch.as_tensor(ys[0]), S.MVNSqrt(torch.as_tensor(m0), torch.as_tensor(L0)),
                                     gt, go, S.linearization.extended, None, return_info=True, chunk=16)
    assert int(info["iterations"]) == 1
    assert torch.isfinite(res.mean).all()


@pytest.mark.parametrize("nx,ny", DIMS)
def test_dense_linearize_is_exact(nx, ny):
    sysm, _, (gt, go) = _system(nx, ny)
    F, Q, H, R, qm, rm = sysm
    rng = np.random.RandomState(0)
    pts = S.MVNSqrt(torch.as_tensor(rng.randn(5, nx)), torch.as_tensor(np.repeat(np.eye(nx)[None], 5, 0)))
    for method in (S.linearization.extended, S.linearization.cubature):
        Fg, cg, bg = S.linearize(go, pts, method)
        assert_rel(Fg, np.repeat(H[None], 5, 0), 1e-12, "F")
        assert_rel(cov(cg), np.repeat(R[None], 5, 0), 1e-12, "chol")
        assert_rel(bg, np.repeat(rm[None], 5, 0), 1e-12, "b")


def test_dense_large_workload_fp32_tracks_fp64():
    """A slice of the large-state workload (nx = 32, ny = 16, B = 4, T = 4096, ten calls):
    the FP32 smoothed means stay within 1e-3 (relative to their scale) of the FP64 ones and
    the factors are finite and lower triangular."""
    sysm, _, (gt, go) = _system(32, 16, seed=11)
    lengths = np.full(4, 4096)
    ys = _observations(sysm, lengths, seed=11)
    m0, L0 = _prior(32)
    out = {}
    for dt in (torch.float32, torch.float64):
        x0 = S.MVNSqrt(torch.as_tensor(m0), torch.as_tensor(L0))
        res = S.iterated_smoothing(torch.as_tensor(ys, dtype=dt), x0, gt, go, S.linearization.cubature, None,
                                   criterion=lambda i, *_: i < 10, lengths=lengths)
        out[dt] = res
    a, b = out[torch.float32], out[torch.float64]
    assert torch.isfinite(a.chol).all() and torch.isfinite(a.mean).all()
    assert float(torch.triu(a.chol, 1).abs().max()) == 0.0
    assert_rel(a.mean, b.mean, 1e-3, "fp32 vs fp64 means")
    assert_rel(cov(a.chol), cov(b.chol), 1e-3, "fp32 vs fp64 covariances")


@pytest.fixture
def per_sequence_covariance():
    S.set_large_state_options(per_sequence_covariance=True)
    yield
    S.set_large_state_options(per_sequence_covariance=False)


def _equal_batch(nx, ny, B=3, T=45, seed=9):
    sysm, (ot, oo), (gt, go) = _system(nx, ny, seed=seed)
    lengths = np.full(B, T)
    ys = _observations(sysm, lengths, seed=seed)
    m0, L0 = _prior(nx)
    return lengths, ys, m0, L0, (ot, oo), (gt, go)


@pytest.mark.parametrize("nx,ny", DIMS)
@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-9), (torch.float32, 2e-3)])
def test_dense_shared_covariance_vs_oracle(nx, ny, dtype, tol):
    """Equally long sequences with one prior: the factor recursion is computed once for the
    batch (shared-covariance mode); every sequence still matches the oracle."""
    lengths, ys, m0, L0, (ot, oo), (gt, go) = _equal_batch(nx, ny)
    x0 = S.MVNSqrt(torch.as_tensor(m0), torch.as_tensor(L0))
    filt, ell = S.filtering(torch.as_tensor(ys, dtype=dtype), x0, gt, go, S.linearization.extended, None,
                            return_loglikelihood=True, lengths=lengths, chunk=8, group=2)
    res, ell2, info = S.iterated_smoothing(torch.as_tensor(ys, dtype=dtype), x0, gt, go, S.linearization.cubature,
                                           None, criterion=lambda i, *_: i < 2, return_loglikelihood=True,
                                           lengths=lengths, return_info=True, chunk=8, group=2)
    for i, T in enumerate(lengths):
        ref_f, ref_ell = O.methods.filtering(ys[i], O.MVNSqrt(m0, L0), ot, oo, O.linearization.extended, None, True,
                                             return_loglikelihood=True)
        assert_rel(filt.mean[i], ref_f.mean, tol, f"seq {i} filtered mean")
        assert_rel(cov(filt.chol[i]), cov(ref_f.chol), tol, f"seq {i} filtered cov")
        assert abs(float(ell[i]) - ref_ell) <= tol * abs(ref_ell)
        ref_s = O.methods.smoothing(ot, ref_f, O.linearization.extended, None, True)
        assert_rel(res.mean[i], ref_s.mean, tol, f"seq {i} smoothed mean")
        assert_rel(cov(res.chol[i]), cov(ref_s.chol), tol, f"seq {i} smoothed cov")
        assert abs(float(ell2[i]) - ref_ell) <= tol * abs(ref_ell)
    assert int(info["flags"].abs().sum()) == 0


@pytest.mark.parametrize("nx,ny", DIMS)
def test_dense_shared_equals_per_sequence(nx, ny, per_sequence_covariance):
    """Shared-covariance and per-sequence computation agree to rounding (FP64), including the
    tolerance criterion that stops sequences on their own."""
    lengths, ys, m0, L0, _, (gt, go) = _equal_batch(nx, ny, B=5, T=64, seed=4)
    x0 = S.MVNSqrt(torch.as_tensor(m0), torch.as_tensor(L0))
    out = {}
    for per_seq in (True, False):
        S.set_large_state_options(per_sequence_covariance=per_seq)
        res, info = S.iterated_smoothing(torch.as_tensor(ys), x0, gt, go, S.linearization.extended, None,
                                         lengths=lengths, return_info=True, chunk=8, group=2)
        out[per_seq] = (res, info)
    a, b = out[True][0], out[False][0]
    assert_rel(a.mean, b.mean, 1e-11, "means")
    assert_rel(cov(a.chol), cov(b.chol), 1e-11, "covariances")
    assert torch.equal(out[True][1]["iterations"], out[False][1]["iterations"])


def test_dense_filter_prefix_at_full_size():
    """The large-state workload's size (B = 16, T = 131 072, nx = 32, ny = 16, one prior), FP64:
    filtering is causal, so each sequence's first 300 filtered states equal the oracle's
    filter of its first 300 observations."""
    sysm, (ot, oo), (gt, go) = _system(32, 16, seed=21)
    F, Q, H, R, qm, rm = sysm
    B, T, P = 16, 131_072, 300
    rng = np.random.RandomState(5)
    ys = rng.randn(B, T, 16)
    ys[:, :P] = _observations(sysm, np.full(B, P), seed=5)
    m0, L0 = _prior(32)
    filt = S.filtering(torch.as_tensor(ys), S.MVNSqrt(torch.as_tensor(m0), torch.as_tensor(L0)), gt, go,
                       S.linearization.extended, None, lengths=np.full(B, T), chunk=32)
    for i in (0, B - 1):
        ref = O.methods.filtering(ys[i, :P], O.MVNSqrt(m0, L0), ot, oo, O.linearization.extended, None, True)
        assert_rel(filt.mean[i, :P + 1], ref.mean, 1e-9, f"seq {i} prefix mean")
        assert_rel(cov(filt.chol[i, :P + 1]), cov(ref.chol), 1e-9, f"seq {i} prefix cov")
    assert torch.isfinite(filt.mean).all()
