"""Iterated smoother through the CUDA path for every sigma-point rule, and long
bearings sequences in FP64 (parsmooth/methods.py:54-76 with the linearisations
of parsmooth/linearization/{_unscented,_gh,_cubature}.py).

The unscented and Gauss-Hermite rules run through the staged linearisation
kernel of the iterated loop here (FP64 with the reference's Cholesky-downdate
regression, FP32 with the residual form), on a ragged batch against the FP64
oracle."""
import numpy as np
import pytest
import torch

import oracle as O
import sqrt_parallel_smoothers_gb300 as S
from tests._parity import GPU_LIN, ORACLE_LIN, assert_rel, bearings_pair, cov

pytestmark = pytest.mark.gpu

PRIOR = np.array([0.1, 0.2, 1.0, 0.0, 1.0])


@pytest.mark.parametrize("method", ["unscented", "gauss_hermite", "cubature", "extended"])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_ragged_iterated_all_rules_vs_oracle(method, dtype):
    # FP64 starts from the reference's default nominal (one extra pass at zero means, identity
    # factors); FP32 from the prior mean broadcast, where Gauss-Newton does not wander (from the
    # default nominal some of these tracks reach means of a few hundred by the fourth call, and
    # FP32 and FP64 iterates drift apart there by more than FP32 rounding).
    lengths = np.array([3, 40, 1, 120, 17, 0, 64])
    (ot, oo), (gt, go) = bearings_pair(0.1, 0.5, 0.05)
    batch = S.data.bearings_batch(lengths, seed0=11)
    x0 = S.MVNSqrt(torch.as_tensor(PRIOR), torch.eye(5, dtype=torch.float64))
    n_states = int(lengths.sum()) + len(lengths)
    nom = None if dtype == torch.float64 else \
        S.MVNSqrt(torch.as_tensor(PRIOR, dtype=dtype).expand(n_states, 5).contiguous(),
                  torch.eye(5, dtype=dtype).expand(n_states, 5, 5).contiguous())
    res, ell = S.iterated_smoothing(torch.as_tensor(batch["ys"], dtype=dtype), x0, gt, go, GPU_LIN[method], nom,
                                    criterion=lambda i, *_: i < 4, return_loglikelihood=True,
                                    offsets=batch["offsets"], chunk=4, group=2)
    tol = 1e-9 if dtype == torch.float64 else 5e-3
    off = batch["offsets"]
    for i, T in enumerate(lengths):
        ys = batch["ys"][off[i]:off[i + 1]].astype(float)
        onom = None if nom is None else O.MVNSqrt(np.repeat(PRIOR[None], T + 1, 0), np.repeat(np.eye(5)[None], T + 1, 0))
        ref, ref_ell = O.methods.iterated_smoothing(ys, O.MVNSqrt(PRIOR, np.eye(5)), ot, oo, ORACLE_LIN[method],
                                                    onom, True, criterion=lambda k, *_: k < 4,
                                                    return_loglikelihood=True)
        a, b = off[i] + i, off[i + 1] + i + 1
        assert_rel(res.mean[a:b], ref.mean, tol, f"{method} seq {i} mean")
        assert_rel(cov(res.chol[a:b]), cov(ref.chol), tol, f"{method} seq {i} cov")
        if T > 0:
            assert abs(float(ell[i]) - ref_ell) <= tol * max(1.0, abs(ref_ell)), (i, float(ell[i]), ref_ell)


@pytest.mark.parametrize("seed", [1, 4])
@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-9), (torch.float32, 5e-3)])
def test_long_bearings_iterated_vs_oracle(seed, dtype, tol):
    """One 2000-step bearings sequence (the headline model: qc = 0.1, qw = 0.5, sigma = 0.05),
    10 cubature calls from the prior mean broadcast.  Seeds whose Gauss-Newton iteration
    converges (oracle mean-squared change 1e-11 and 1e-14 by the tenth call), so the
    comparison is not between wandering iterates."""
    T = 2000
    (ot, oo), (gt, go) = bearings_pair(0.1, 0.5, 0.05)
    w = S.data.bearings_batch(np.array([T]), seed0=seed)
    ys = w["ys"].astype(float)
    nom = (np.repeat(PRIOR[None], T + 1, 0), np.repeat(np.eye(5)[None], T + 1, 0))
    ref = O.methods.iterated_smoothing(ys, O.MVNSqrt(PRIOR, np.eye(5)), ot, oo, O.linearization.cubature,
                                       O.MVNSqrt(*nom), True, criterion=lambda i, *_: i < 10)
    x0 = S.MVNSqrt(torch.as_tensor(PRIOR, dtype=dtype), torch.eye(5, dtype=dtype))
    res = S.iterated_smoothing(torch.as_tensor(ys, dtype=dtype), x0, gt, go, S.linearization.cubature,
                               S.MVNSqrt(torch.as_tensor(nom[0], dtype=dtype), torch.as_tensor(nom[1], dtype=dtype)),
                               criterion=lambda i, *_: i < 10)
    assert_rel(res.mean, ref.mean, tol, "mean")
    assert_rel(cov(res.chol), cov(ref.chol), tol, "cov")


def test_fp32_long_divergent_sequence_stays_finite():
    """The single-sequence sweep's longest case (T = 1e5, headline model, 10 cubature calls from
    the prior mean broadcast, simulator seed 30003) diverges as a Gauss-Newton iteration (FP64
    means reach 2e7).  Its FP32 run once turned non-finite on the ninth call, when row sums of
    squares in the combine's reflectors overflowed; with the FP32 range guard of the reflectors
    every call stays finite, and no status bit is raised."""
    T = 100_000
    (_, _), (gt, go) = bearings_pair(0.1, 0.5, 0.05)
    w = S.data.bearings_batch(np.array([T]), qc=0.1, qw=0.5, sigma=0.05, dt=0.01, seed0=30_003)
    dt = torch.float32
    m0 = torch.as_tensor(PRIOR, dtype=dt)
    nom = S.MVNSqrt(m0.expand(T + 1, 5).contiguous(), torch.eye(5, dtype=dt).expand(T + 1, 5, 5).contiguous())
    for n in (9, 10):
        res, info = S.iterated_smoothing(torch.as_tensor(w["ys"], dtype=dt), S.MVNSqrt(m0, torch.eye(5, dtype=dt)),
                                         gt, go, S.linearization.cubature, nom, criterion=S.FixedIterations(n),
                                         return_info=True)
        assert torch.isfinite(res.mean).all() and torch.isfinite(res.chol).all(), n
        assert int(info["flags"].reshape(-1)[0]) == 0
