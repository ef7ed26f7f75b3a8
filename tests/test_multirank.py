"""The multi-GPU form of the benchmark is weak scaling over independent batches: each rank
smooths its own sequences with no data-path collective, and the job's step time is the
slowest rank's.  Exercised here with two gloo ranks on the CPU (the per-rank work is the
oracle's filter on the rank's first sequences)."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        import oracle as O
        import sqrt_parallel_smoothers_gb300 as S
        lengths, batch = bench.rank_batch(S, 6, rank)
        # per-rank work: the oracle filter on this rank's first two (short) sequences
        Q, R = S.data.bearings_noise(bench.QC, bench.QW, bench.SIGMA, bench.DT)
        tm = O.FunctionalModel(O.models.CoordinatedTurn(bench.DT), O.MVNSqrt(np.zeros(5), np.linalg.cholesky(Q)))
        om = O.FunctionalModel(O.models.Bearings(bench.S1, bench.S2), O.MVNSqrt(np.zeros(2), np.linalg.cholesky(R)))
        ells = []
        for i in range(2):
            ys = batch["ys"][batch["offsets"][i]:batch["offsets"][i] + 40].astype(float)
            _, ell = O.methods.filtering(ys, O.MVNSqrt(bench.PRIOR_M0, np.eye(5)), tm, om, O.linearization.extended,
                                         None, True, return_loglikelihood=True)
            ells.append(float(ell))
        ms = 10.0 + rank            # rank 1 is the slow one
        job_ms = bench.max_over_ranks(torch, dist, ms, "cpu")
        gathered = [None] * world
        dist.all_gather_object(gathered, {"lengths": lengths.tolist(), "first_ys": batch["ys"][:3].tolist(),
                                          "ells": ells, "job_ms": job_ms,
                                          "value": bench.job_value(world, int(lengths.sum()), job_ms)})
        if rank == 0:
            out.put(gathered)
    finally:
        dist.destroy_process_group()


def test_two_rank_weak_scaling_bookkeeping():
    world = 2
    ctx = mp.get_context("spawn")
    out = ctx.SimpleQueue()
    mp.start_processes(_rank_main, args=(world, _free_port(), out), nprocs=world, join=True, start_method="spawn")
    g = out.get()
    assert g[0]["lengths"] == g[1]["lengths"]                    # same length draw on every rank
    assert not np.allclose(g[0]["first_ys"], g[1]["first_ys"])  # but each rank's own sequences
    assert g[0]["ells"] != g[1]["ells"]
    assert g[0]["job_ms"] == g[1]["job_ms"] == pytest.approx(11.0)   # the slowest rank's time
    sum_T = int(np.sum(g[0]["lengths"]))
    assert g[0]["value"] == pytest.approx(world * sum_T / 11e-3)
