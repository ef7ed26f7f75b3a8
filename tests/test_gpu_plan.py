"""IteratedSmootherPlan: the graph-replayed iterated smoother equals the direct call
(iterated_smoothing, parsmooth/methods.py:54-76), with its batch cut into concurrent
sequence groups (streams > 1) as well, and through the host-buffer path."""
import numpy as np
import pytest
import torch

import sqrt_parallel_smoothers_gb300 as S
from sqrt_parallel_smoothers_gb300 import models as GM
from tests._parity import assert_rel

pytestmark = pytest.mark.gpu

LENGTHS = np.array([60, 3, 0, 140, 97, 1, 33, 250])
M0 = np.array([0.1, 0.2, 1.0, 0.0, 1.0])


def _setup(dtype):
    w = S.data.bearings_batch(LENGTHS, seed0=5)
    Q, R = S.data.bearings_noise(0.1, 0.5, 0.05, 0.01)
    tm = S.FunctionalModel(GM.CoordinatedTurn(0.01), S.MVNSqrt(torch.zeros(5, dtype=dtype),
                                                               torch.as_tensor(np.linalg.cholesky(Q), dtype=dtype)))
    om = S.FunctionalModel(GM.Bearings((-1.5, 0.5), (1.0, 1.0)),
                           S.MVNSqrt(torch.zeros(2, dtype=dtype), torch.as_tensor(np.linalg.cholesky(R), dtype=dtype)))
    n_states = int(LENGTHS.sum()) + len(LENGTHS)
    m0 = torch.as_tensor(M0, dtype=dtype)
    x0 = S.MVNSqrt(m0, torch.eye(5, dtype=dtype))
    nom = S.MVNSqrt(m0.expand(n_states, 5).contiguous(), torch.eye(5, dtype=dtype).expand(n_states, 5, 5).contiguous())
    ys = torch.as_tensor(w["ys"], dtype=dtype)
    return ys, w["offsets"], x0, tm, om, nom


@pytest.mark.parametrize("streams", [1, 2, 3])
def test_plan_matches_direct_call(streams):
    ys, offsets, x0, tm, om, nom = _setup(torch.float64)
    crit = S.FixedIterations(4)
    ref, ref_ell = S.iterated_smoothing(ys, x0, tm, om, S.linearization.cubature, nom, criterion=crit,
                                        return_loglikelihood=True, offsets=offsets, chunk=8, group=2)
    plan = S.IteratedSmootherPlan(ys, x0, tm, om, S.linearization.cubature, nom, criterion=crit,
                                  return_loglikelihood=True, offsets=offsets, chunk=8, group=2, streams=streams)
    plan.run()
    torch.cuda.synchronize()
    got = plan.result()
    # the sequence groups may have fewer scan levels than the whole batch (their longest
    # sequence is shorter), which changes only the association of the combines
    assert_rel(got.mean, ref.mean, 1e-10, "mean")
    assert_rel(got.chol, ref.chol, 1e-10, "chol")
    assert_rel(plan.ell, ref_ell, 1e-10, "ell")
    if streams > 1:
        assert len(plan._groups) == streams


def test_plan_replay_and_host_path():
    ys, offsets, x0, tm, om, nom = _setup(torch.float32)
    plan = S.IteratedSmootherPlan(ys, x0, tm, om, S.linearization.cubature, nom, criterion=S.FixedIterations(3),
                                  offsets=offsets, streams=2)
    plan.run()
    torch.cuda.synchronize()
    first = plan.mean.clone()
    ys_host = ys.clone().pin_memory()
    m_host = torch.empty(plan.mean.shape, dtype=torch.float32).pin_memory()
    L_host = torch.empty(plan.chol.shape, dtype=torch.float32).pin_memory()
    plan.run_host(ys_host, m_host, L_host)
    torch.cuda.synchronize()
    assert torch.equal(m_host, first.cpu())                      # replays are deterministic
    assert torch.equal(L_host, plan.chol.cpu())
    # new observations in place: the replay follows them
    ys2 = ys.clone()
    ys2[:, 0] += 0.01
    plan.set_observations(ys2.cuda())
    plan.run()
    torch.cuda.synchronize()
    assert not torch.equal(plan.mean, first)
    assert torch.isfinite(plan.mean).all()


def test_pipelined_host_path_matches():
    """run_host(pipelined=True) alternates the plan with a twin and copies out on a second
    stream; every call still returns that call's smoothed trajectory."""
    ys, offsets, x0, tm, om, nom = _setup(torch.float32)
    plan = S.IteratedSmootherPlan(ys, x0, tm, om, S.linearization.cubature, nom, criterion=S.FixedIterations(3),
                                  offsets=offsets, streams=2)
    ys_host = ys.clone().pin_memory()
    m_ref = torch.empty(plan.mean.shape, dtype=torch.float32).pin_memory()
    L_ref = torch.empty(plan.chol.shape, dtype=torch.float32).pin_memory()
    plan.run_host(ys_host, m_ref, L_ref)
    torch.cuda.synchronize()
    outs = []
    for k in range(4):
        yk = ys_host.clone()
        yk[:, 0] += 0.001 * k
        yk = yk.pin_memory()
        m_host = torch.empty_like(m_ref).pin_memory()
        L_host = torch.empty_like(L_ref).pin_memory()
        plan.run_host(yk, m_host, L_host, pipelined=True)
        outs.append((m_host, L_host))
    plan.sync_host()
    torch.cuda.synchronize()
    assert torch.equal(outs[0][0], m_ref) and torch.equal(outs[0][1], L_ref)
    for k in range(1, 4):
        assert not torch.equal(outs[k][0], outs[k - 1][0])       # each call saw its own observations
    # the twin plan (odd calls) computes what the plan itself computes
    plan.run_host(ys_host, m_ref, L_ref)
    torch.cuda.synchronize()
    m_twin = torch.empty_like(m_ref).pin_memory()
    L_twin = torch.empty_like(L_ref).pin_memory()
    if plan._flip == 0:
        plan.run_host(ys_host, torch.empty_like(m_ref).pin_memory(), None, pipelined=True)
    plan.run_host(ys_host, m_twin, L_twin, pipelined=True)
    plan.sync_host()
    torch.cuda.synchronize()
    assert torch.equal(m_twin, m_ref) and torch.equal(L_twin, L_ref)
