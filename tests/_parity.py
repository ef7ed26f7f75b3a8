"""Helpers for GPU-vs-oracle parity tests: matching model pairs and tolerances."""
import numpy as np
import torch

import oracle as O
import sqrt_parallel_smoothers_gb300 as S
from oracle import models as OM
from sqrt_parallel_smoothers_gb300 import models as GM

ORACLE_LIN = {"extended": O.linearization.extended, "cubature": O.linearization.cubature,
              "unscented": O.linearization.unscented, "gauss_hermite": O.linearization.gauss_hermite}
GPU_LIN = {"extended": S.linearization.extended, "cubature": S.linearization.cubature,
           "unscented": S.linearization.unscented, "gauss_hermite": S.linearization.gauss_hermite}


def linear_pair(A, b, cholQ):
    """The same linear model with Gaussian noise for the oracle and the GPU."""
    o = O.FunctionalModel(OM.LinearFunction(A), O.MVNSqrt(np.asarray(b, float), np.asarray(cholQ, float)))
    g = S.FunctionalModel(GM.LinearModel(A), S.MVNSqrt(torch.as_tensor(b), torch.as_tensor(cholQ)))
    return o, g


def bearings_pair(qc, qw, r, dt=0.01, s1=(-1.5, 0.5), s2=(1.0, 1.0)):
    Q, R = OM.bearings_noise(qc, qw, r, dt)
    cQ, cR = np.linalg.cholesky(Q), np.linalg.cholesky(R)
    ot = O.FunctionalModel(OM.CoordinatedTurn(dt), O.MVNSqrt(np.zeros(5), cQ))
    oo = O.FunctionalModel(OM.Bearings(s1, s2), O.MVNSqrt(np.zeros(2), cR))
    gt = S.FunctionalModel(GM.CoordinatedTurn(dt), S.MVNSqrt(torch.zeros(5), torch.as_tensor(cQ)))
    go = S.FunctionalModel(GM.Bearings(s1, s2), S.MVNSqrt(torch.zeros(2), torch.as_tensor(cR)))
    return (ot, oo), (gt, go)


def np_(t):
    return t.detach().cpu().double().numpy() if isinstance(t, torch.Tensor) else np.asarray(t, float)


def assert_rel(actual, expected, rtol, what=""):
    """max |a - e| <= rtol * max(1, max |e|): a norm-wise relative bound."""
    a, e = np_(actual), np_(expected)
    assert a.shape == e.shape, (what, a.shape, e.shape)
    scale = max(1.0, float(np.max(np.abs(e))) if e.size else 1.0)
    err = float(np.max(np.abs(a - e))) if e.size else 0.0
    assert err <= rtol * scale, f"{what}: max abs err {err:.3e} > {rtol:.1e} * {scale:.3e}"


def cov(L):
    L = np_(L)
    return L @ np.swapaxes(L, -1, -2)
