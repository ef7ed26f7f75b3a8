"""Benchmark: smoother timesteps/s on one GB300, FP32 batched vs FP64 plain.

Workload (the batched configuration): B = 1024 independent bearings-only
sequences (coordinated-turn state, two bearings sensors, dt = 0.01), lengths
drawn log-uniform in [50, 5000] (seed 0), sequence i simulated from seed i
(+ 1024 * rank), iterated square-root cubature smoother: 10 filter-smoother
calls from the prior mean broadcast, FP32.  One step = the whole 10-call
smoother over the batch, replayed from one CUDA graph at the scan geometry
and number of concurrent sequence groups the autotuner picks.  ``value`` =
sum_i T_i / device time of a step (inputs resident, L2 flushed between
steps); ``e2e`` = the same through ``IteratedSmootherPlan.run_host`` with
pinned host observations in and the smoothed trajectory out every step
(copy-out overlapped with the next step).  The FP64 plain path (B = 1,
T = 5000, FP64, same method) is timed beside it, and the per-kernel times
for the roofline come from a single-stream replay of the same geometry.

``--impl reference`` times the reference algorithm on the host CPU (the
FP64 NumPy port in ``oracle/``: the reference's JAX code cannot be
installed here) on a bounded sample of the same workload, with one process
per host core.
"""
import argparse
import datetime
import json
import os
import subprocess
import sys
import threading
import time

for _v in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
    os.environ.setdefault(_v, "1")

import numpy as np  # noqa: E402

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "smoother timesteps/s on 1 GB300: FP32 batched vs FP64 plain at fixed RMSE"
UNIT = "timesteps/s"
B_DEFAULT = 1024
N_ITER = 10
S1, S2 = (-1.5, 0.5), (1.0, 1.0)
DT, QC, QW, SIGMA = 0.01, 0.1, 0.5, 0.05
FP64_PLAIN_T = 5000
# prior centred on the simulator's initial state (x, y, vx, vy) = (0.1, 0.2, 1, 0) with
# the simulator's mean turn rate 1, P0 = I; the initial trajectory is this mean broadcast
PRIOR_M0 = np.array([0.1, 0.2, 1.0, 0.0, 1.0])


def workload_config(B, lengths, C, G):
    return {"workload": f"bearings-only coordinated-turn, iterated sqrt cubature smoother, B={B} ragged "
                        f"T~logU[50,5000], {N_ITER} filter-smoother calls from the prior mean broadcast, FP32, "
                        f"one CUDA graph",
            "batch": int(B), "sum_T": int(np.sum(lengths)), "max_T": int(np.max(lengths)),
            "iterations": N_ITER, "init": "prior mean broadcast", "prior": "m0=(0.1,0.2,1,0,1), P0=I",
            "nx": 5, "ny": 2, "linearization": "cubature", "chunk": C, "group": G,
            "l2": "flushed between timed steps (256 MiB write)", "parallelism": "batch of sequences"}


# ----------------------------------------------------------------------------- reference arm

def _oracle_smooth(ys, m0):
    import oracle as O
    Q, R = O.models.bearings_noise(QC, QW, SIGMA, DT)
    tm = O.FunctionalModel(O.models.CoordinatedTurn(DT), O.MVNSqrt(np.zeros(5), np.linalg.cholesky(Q)))
    om = O.FunctionalModel(O.models.Bearings(S1, S2), O.MVNSqrt(np.zeros(2), np.linalg.cholesky(R)))
    T = ys.shape[0]
    nom = O.MVNSqrt(np.repeat(m0[None], T + 1, 0), np.repeat(np.eye(5)[None], T + 1, 0))
    return O.methods.iterated_smoothing(ys.astype(np.float64), O.MVNSqrt(m0, np.eye(5)), tm, om,
                                        O.linearization.cubature, nom, True, criterion=lambda i, *_: i < N_ITER)


def _oracle_task(args):
    ys, m0 = args
    return float(np.sum(_oracle_smooth(ys, m0).mean))


def _oracle_means_task(args):
    ys, m0 = args
    return _oracle_smooth(ys, m0).mean


def oracle_accuracy_sample(batch, lengths, mean32, mean64, conv, every=32):
    """Smoothed means of a fixed sample of the batch (every ``every``-th sequence) from the FP64
    CPU oracle (a spawn pool over the host cores), against which the FP32 and FP64 GPU results
    of the same sequences are compared: position RMSE vs the simulated truth per sequence, and
    the largest difference of the smoothed means themselves."""
    import multiprocessing as mp
    idx = list(range(0, len(lengths), every))
    off = batch["offsets"]
    tasks = [(batch["ys"][off[i]:off[i + 1]], PRIOR_M0.copy()) for i in idx]
    with mp.get_context("spawn").Pool(min(len(tasks), os.cpu_count() or 1)) as pool:
        ref = pool.map(_oracle_means_task, tasks, chunksize=1)
    xs = batch["xs"].astype(np.float64)
    r_or, r32, r64, d32, d64 = [], [], [], [], []
    for i, m in zip(idx, ref):
        a, b = off[i] + i, off[i + 1] + i + 1
        truth = xs[a + 1:b, :2]
        for out, mean in ((r_or, m), (r32, mean32[a:b]), (r64, mean64[a:b])):
            d = mean[1:, :2] - truth
            out.append(float(np.sqrt(np.mean(np.sum(d * d, axis=1)))))
        scale = max(1.0, float(np.abs(m).max()))
        d32.append(float(np.abs(mean32[a:b] - m).max()) / scale)
        d64.append(float(np.abs(mean64[a:b] - m).max()) / scale)
    r_or, r32, r64 = map(np.array, (r_or, r32, r64))
    rel32 = np.abs(r32 - r_or) / np.maximum(r_or, 1e-12)
    c = np.asarray(conv)[idx]
    out = {"sequences": len(idx), "sample": f"one sequence in every {every} of the batch (sum T = "
                                            f"{int(np.sum(lengths[idx]))})",
           "frac_fp32_rmse_within_1pct_of_oracle_all": float(np.mean(rel32 <= 0.01)),
           "frac_fp32_rmse_within_1pct_of_oracle_converged": float(np.mean(rel32[c] <= 0.01)) if c.any() else None,
           "frac_fp32_rmse_within_1pct_of_oracle_not_converged": float(np.mean(rel32[~c] <= 0.01))
           if (~c).any() else None,
           "converged": int(c.sum()),
           "fp32_rmse_rel_diff_median": float(np.median(rel32)),
           "fp64_gpu_vs_oracle_max_rel_mean_diff": float(np.max(d64)),
           "fp64_gpu_vs_oracle_max_rel_mean_diff_converged": float(np.max(np.array(d64)[c])) if c.any() else None,
           "fp32_gpu_vs_oracle_max_rel_mean_diff_converged": float(np.max(np.array(d32)[c])) if c.any() else None,
           "oracle": "FP64 NumPy restatement of the reference, 10 calls from the prior mean broadcast"}
    return out


def cpu_sample(lengths, batch, budget_steps):
    """The first sequences of the batch whose lengths sum to about ``budget_steps``."""
    idx, tot = [], 0
    for i, T in enumerate(lengths):
        if tot >= budget_steps:
            break
        idx.append(i)
        tot += int(T)
    off = batch["offsets"]
    return [batch["ys"][off[i]:off[i + 1]] for i in idx], tot


def run_cpu(seqs, processes):
    tasks = [(y, PRIOR_M0.copy()) for y in seqs]
    t0 = time.perf_counter()
    if processes <= 1:
        for t in tasks:
            _oracle_task(t)
    else:
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(processes) as pool:
            pool.map(_oracle_task, tasks, chunksize=1)
    return time.perf_counter() - t0


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from sqrt_parallel_smoothers_gb300 import data
    lengths = data.ragged_lengths(B_DEFAULT, seed=0)
    cores = os.cpu_count() or 1
    sub = lengths[:max(cores * 2, 8)]
    batch = data.bearings_batch(sub, qc=QC, qw=QW, sigma=SIGMA, dt=DT)
    seqs, tot = cpu_sample(sub, batch, budget_steps=1500 * cores)
    import multiprocessing as mp
    times = []
    with mp.get_context("spawn").Pool(cores) as pool:
        tasks = [(y, PRIOR_M0.copy()) for y in seqs]
        for k in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            pool.map(_oracle_task, tasks, chunksize=1)
            if k >= args.warmup:
                times.append(time.perf_counter() - t0)
    t = float(np.mean(times))
    value = tot / t
    sample = f"{len(seqs)} sequences (sum T = {tot}) of the B=1024 batch, {N_ITER} calls, one process per core"
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(B_DEFAULT, lengths, 0, 0),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "reference JAX 0.4.30 is not installable offline; its algorithm is timed as the FP64 "
                    "NumPy port in oracle/"}
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------------------- GPU arm

class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every ``period_ms`` from before the
    warm-up to the end of the timed region.  Each sample carries nvidia-smi's own timestamp
    (so pipe buffering does not matter); :meth:`stop` keeps the samples taken inside the timed
    window ``[t0, t1]`` (``window: "timed"``) or, when the window is shorter than the sampling
    period and holds none, the last sample before ``t1`` (``window: "nearest"``, taken under the
    warm-up's load of the same work)."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    NAMES = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")

    def __init__(self, gpu_index, period_ms=25, exe="nvidia-smi"):
        self.gpu = gpu_index
        self.period_ms = int(period_ms)
        self.exe = exe
        self.fields = self.FIELDS + ",timestamp"
        self.proc = None
        self.lines = []                  # (host arrival time, line)

    def _spawn(self):
        try:
            self.proc = subprocess.Popen([self.exe, f"--id={self.gpu}", f"--query-gpu={self.fields}",
                                          "--format=csv,noheader,nounits", "-lms", str(self.period_ms)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, args=(self.proc,), daemon=True)
        self.thread.start()

    def start(self, first_line_timeout=2.0):
        """Start sampling; return once the first sample has arrived, nvidia-smi has exited or
        the timeout has passed.  If nvidia-smi exits without a sample (an interval or a field
        it does not take), sample again every 200 ms without the timestamp field (the samples
        are then stamped with their arrival time)."""
        self._spawn()
        if self.proc is None:
            return
        t_end = time.monotonic() + first_line_timeout
        while not self.lines and self.proc.poll() is None and time.monotonic() < t_end:
            time.sleep(0.005)
        if not self.lines and self.proc.poll() is not None and self.period_ms < 200:
            self.thread.join(timeout=5)
            self.period_ms, self.fields = 200, self.FIELDS
            self._spawn()

    def _read(self, proc):
        for line in proc.stdout:
            self.lines.append((time.time(), line.strip()))

    @staticmethod
    def _stamp(text, fallback):
        try:
            return datetime.datetime.strptime(text.strip(), "%Y/%m/%d %H:%M:%S.%f").timestamp()
        except ValueError:
            return fallback

    def stop(self, t0=None, t1=None):
        """Stop sampling and summarise the samples of the timed window ``[t0, t1]`` (host
        ``time.time()`` values; every sample when they are not given)."""
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        if t1 is not None:
            # let the sample that straddles t1 be taken
            t_end = time.time() + self.period_ms / 1000.0
            while time.time() < t_end and self.proc.poll() is None:
                time.sleep(0.005)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=5)
        samples = []
        for arrived, ln in list(self.lines):
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm, smax = float(parts[1]), float(parts[2])
            except ValueError:
                continue
            t = self._stamp(parts[9], arrived) if len(parts) > 9 else arrived
            samples.append((t, sm, smax, {nm for nm, v in zip(self.NAMES, parts[5:9])
                                          if v.lower().startswith("active")}))
        window = "all"
        if t0 is not None and t1 is not None:
            inside = [s for s in samples if t0 <= s[0] <= t1]
            if inside:
                samples, window = inside, "timed"
            else:
                before = [s for s in samples if s[0] <= t1]
                samples, window = (before[-1:], "nearest") if before else (samples, "all")
        sm = [s[1] for s in samples]
        reasons = set().union(*[s[3] for s in samples]) if samples else set()
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(s[2] for s in samples) if samples else None,
                "reasons": sorted(reasons), "samples": len(sm), "period_ms": self.period_ms, "window": window}


def models(torch, S, dtype):
    Q, R = S.data.bearings_noise(QC, QW, SIGMA, DT)
    cQ = torch.as_tensor(np.linalg.cholesky(Q), dtype=dtype)
    cR = torch.as_tensor(np.linalg.cholesky(R), dtype=dtype)
    tm = S.FunctionalModel(S.models.CoordinatedTurn(DT), S.MVNSqrt(torch.zeros(5, dtype=dtype), cQ))
    om = S.FunctionalModel(S.models.Bearings(S1, S2), S.MVNSqrt(torch.zeros(2, dtype=dtype), cR))
    return tm, om


def make_plan(torch, S, ys, offsets, dtype, chunk=0, group=0, graph=True, profile=False, criterion=None,
              streams=1):
    tm, om = models(torch, S, dtype)
    m0 = torch.as_tensor(PRIOR_M0, dtype=dtype)
    x0 = S.MVNSqrt(m0, torch.eye(5, dtype=dtype))
    n_states = int(ys.shape[0]) + len(offsets) - 1
    nom = S.MVNSqrt(m0.expand(n_states, 5).contiguous(), torch.eye(5, dtype=dtype).expand(n_states, 5, 5).contiguous())
    return S.IteratedSmootherPlan(torch.as_tensor(ys, dtype=dtype), x0, tm, om, S.linearization.cubature, nom,
                                  criterion=criterion or S.FixedIterations(N_ITER), offsets=offsets, chunk=chunk,
                                  group=group, graph=graph, profile=profile, streams=streams)


def time_plan(torch, plan, steps, warmup, flush=None, sampler=None):
    if sampler is not None:
        sampler.start()
    for _ in range(warmup):
        plan.run()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    t0 = time.time()
    for k in range(steps):
        if flush is not None:
            flush.add_(1)
        ev[k][0].record()
        plan.run()
        ev[k][1].record()
    torch.cuda.synchronize()
    t1 = time.time()
    clocks = sampler.stop(t0, t1) if sampler is not None else None
    return [a.elapsed_time(b) for a, b in ev], clocks


def measure_fp32_peak(torch):
    """FP32 CUDA-core throughput of this GPU: a cuBLAS SGEMM of 8192^3 with TF32 off (best of 5,
    CUDA events), TFLOP/s."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        n = 8192
        a = torch.randn(n, n, device="cuda")
        b = torch.randn(n, n, device="cuda")
        c = a @ b
        best = float("inf")
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b, out=c)
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        del a, b, c
        torch.cuda.empty_cache()
        return 2.0 * n ** 3 / (best * 1e-3) / 1e12
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def position_rmse(mean, xs, offsets):
    """Per-sequence RMSE of smoothed (x, y) positions against the simulated truth."""
    out = []
    for i in range(len(offsets) - 1):
        a, b = offsets[i] + i, offsets[i + 1] + i + 1
        d = mean[a + 1:b, :2] - xs[a + 1:b, :2]
        out.append(float(np.sqrt(np.mean(np.sum(d * d, axis=1)))))
    return np.array(out)


# per-step algorithmic bytes (FP32, nx=5, ny=2) of each kernel: the compulsory
# reads and writes of its inputs and outputs in minimal form (lower-triangular
# factors counted by their 15 entries); see the design notes for the derivation.
ALG_BYTES_PER_STEP = {
    "lin": 4 * (20 + 60),            # nominal state in, F/cQ/bq/H/cR/c out
    "filter_leaf": 4 * (60 + 2),     # linearised model + observation in
    "filter_walk": 4 * (60 + 2 + 45),  # ... in, smoothing element out
    "smoother_walk": 4 * (45 + 20),  # smoothing element in, smoothed state out
}
# Whole filter-smoother pass, per timestep and call, at nx = 5, ny = 2 (FP32): the observation
# (2 floats), the nominal state in (5 + 15), the smoothed state out (5 + 15) and the filtered
# hand-off between the filter and the smoother written and read (2 x 20): 82 floats.
PASS_ALG_BYTES_PER_STEP = 4 * (2 + 20 + 20 + 2 * 20)
# Executed FP32 operations per timestep of each per-step kernel (flops: FFMA and FFMA2 count 2 and
# 4, FADD/FMUL 1 and FADD2/FMUL2 2), from one ncu capture of the first call of this workload's
# kernels on its first 128 sequences (sm__sass_thread_inst_executed_op_{ffma,fadd,fmul,ffma2,
# fadd2,fmul2}_pred_on.sum / 133,357 timesteps; no FFMA2/FADD2/FMUL2 were executed).
FP32_FLOPS_PER_STEP = {"lin": 1761, "filter_leaf": 1868, "filter_walk": 3103, "smoother_walk": 555}
# DRAM bytes (read + write) per timestep of each kernel, from one ncu capture of this workload
# (bytes of one launch / 1,101,870 timesteps)
TRAFFIC_BYTES_PER_STEP = {"lin": 314, "filter_leaf": 269, "filter_walk": 426, "smoother_walk": 257}


def _timed(torch, flush, fn, reps=3):
    fn()
    torch.cuda.synchronize()
    times = []
    for _ in range(reps):
        flush.add_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    return float(np.median(times)) * 1e3, out


def adjoint_section(torch, S, flush):
    """Gradient of the batch pseudo-log-likelihood w.r.t. (s1x, s1y, log q, log sigma): bearings model,
    B = 64 sequences of T = 5000, FP32, from the reverse pass (filter, smoother scan, per-step
    contraction) and from the tangent-linear filter (one pass per parameter), both checked against
    central differences (h = 1e-3) of the FP64 filter.  Then p = 32 (every entry of F and of the
    process-noise square root of the constant-velocity model, nx = 4) on the same batch shape."""
    B, T = 64, 5000
    batch = S.data.bearings_batch(np.full(B, T), qc=QC, qw=QW, sigma=SIGMA, dt=DT, seed0=20_000)
    Q1, _ = S.data.bearings_noise(1.0, QW / QC, SIGMA, DT)
    theta0 = np.array([S1[0], S1[1], np.log(QC), np.log(SIGMA)])
    m0 = torch.as_tensor(PRIOR_M0)
    x0 = S.MVNSqrt(m0, torch.eye(5, dtype=torch.float64))
    n_states = B * (T + 1)
    nom = S.MVNSqrt(m0.expand(n_states, 5).contiguous(), torch.eye(5, dtype=torch.float64).expand(n_states, 5, 5))
    ys32 = torch.as_tensor(batch["ys"], dtype=torch.float32)

    def ell_grad(theta, ys, mode):
        th = torch.tensor(theta, dtype=torch.float64, requires_grad=True)
        ell = S.BearingsLogLikelihood.apply(th, ys, x0, nom, Q1, DT, S2, S.linearization.cubature, None,
                                            batch["offsets"], 0, mode)
        ell.backward()
        return float(ell.detach()), th.grad.numpy()

    ms_rev, (ell32, g_rev) = _timed(torch, flush, lambda: ell_grad(theta0, ys32, "reverse"))
    ms_tan, (_, g_tan) = _timed(torch, flush, lambda: ell_grad(theta0, ys32, "tangent"))
    h = 1e-3
    ys64 = torch.as_tensor(batch["ys"], dtype=torch.float64)
    fd = np.array([(ell_grad(theta0 + h * e, ys64, "tangent")[0] - ell_grad(theta0 - h * e, ys64, "tangent")[0])
                   / (2 * h) for e in np.eye(4)])
    rel_rev = np.abs(g_rev - fd) / np.abs(fd)
    rel_tan = np.abs(g_tan - fd) / np.abs(fd)
    out = {"B": B, "T": T, "dtype": "f32", "ms": ms_rev, "ell": ell32, "grad": g_rev.tolist(),
           "fd_grad_fp64": fd.tolist(), "rel_err": rel_rev.tolist(), "max_rel_err": float(np.max(rel_rev)),
           "method": "reverse pass: filter + smoother scan + per-step contraction of the smoothed moments "
                     "(Fisher's identity), cost independent of the parameter count",
           "tangent": {"ms": ms_tan, "grad": g_tan.tolist(), "max_rel_err": float(np.max(rel_tan)),
                       "method": "tangent-linear filter, one pass per parameter"}}
    out["p32"] = _adjoint_p32(torch, S, flush, B, T)
    return out


def _adjoint_p32(torch, S, flush, B, T):
    """d ell / d (F, L_Q) of a random stable linear model at nx = 4, ny = 2 (the large-state
    construction: F = 0.98 Haar orthogonal, Q = L L^T / nx, H ~ N(0, 1/nx), R = 0.1 I): 16 + 16
    parameters, B sequences of T steps, from one FP32 reverse pass, checked against central
    differences of the FP64 filter log-likelihood (h = 1e-5 for F, 1e-6 for the lower-triangle
    entries of L_Q, which the library reads alone)."""
    F, Q, H, R = S.data.large_state_model(4, 2, seed=3)
    ys = np.concatenate([S.data.lgssm_data(np.zeros(4), F, H, R, Q, np.zeros(4), np.zeros(2), T, 30_000 + i)[1]
                         for i in range(B)])
    offsets = np.arange(B + 1, dtype=np.int64) * T
    Lq, Lr = np.linalg.cholesky(Q), np.linalg.cholesky(R)
    x0 = S.MVNSqrt(torch.zeros(4, dtype=torch.float64), torch.eye(4, dtype=torch.float64))

    def models(F_, Lq_):
        tm = S.FunctionalModel(S.models.LinearModel(F_), S.MVNSqrt(torch.zeros(4, dtype=torch.float64),
                                                                   torch.as_tensor(Lq_)))
        om = S.FunctionalModel(S.models.LinearModel(H), S.MVNSqrt(torch.zeros(2, dtype=torch.float64),
                                                                  torch.as_tensor(Lr)))
        return tm, om

    tm, om = models(F, Lq)
    ys32 = torch.as_tensor(ys, dtype=torch.float32)
    ys64 = torch.as_tensor(ys, dtype=torch.float64)

    def reverse():
        _, adj = S.filter_loglikelihood_adjoint(ys32, x0, tm, om, S.linearization.extended, None, offsets=offsets,
                                                model_params=False)
        return np.concatenate([adj["trans_matrix"].sum(0).cpu().numpy().ravel(),
                               adj["trans_noise_chol"].sum(0).cpu().numpy().ravel()])

    def ell64(F_, Lq_):
        t_, o_ = models(F_, Lq_)
        _, ell = S.filtering(ys64, x0, t_, o_, S.linearization.extended, None, offsets=offsets,
                             return_loglikelihood=True)
        return float(ell.sum())

    ms_rev, g_rev = _timed(torch, flush, reverse)
    fd = np.zeros(32)
    for k in range(16):
        for off, h in ((0, 1e-5), (16, 1e-6)):
            if off and k // 4 < k % 4:
                continue
            E = np.zeros(16)
            E[k] = h
            E = E.reshape(4, 4)
            fd[off + k] = ((ell64(F + E, Lq) - ell64(F - E, Lq)) if off == 0 else
                           (ell64(F, Lq + E) - ell64(F, Lq - E))) / (2 * h)
    rel = np.abs(g_rev - fd) / np.maximum(np.abs(fd), 1e-3 * np.abs(fd).max())
    return {"workload": f"random stable linear model nx=4 ny=2 (F = 0.98 Haar, Q = L L^T/nx, H ~ N(0, 1/nx), "
                        f"R = 0.1 I), B={B}, T={T}, FP32, d ell / d (F, L_Q): 32 parameters",
            "reverse_ms": ms_rev, "max_rel_err_vs_fd_fp64": float(np.max(rel)),
            "rel_err_definition": "|g - fd| / max(|fd|, 1e-3 max |fd|)"}


def rank_batch(S, batch_size, rank):
    """Rank ``rank``'s share of a weak-scaling run: its own B sequences (the same length draw,
    sequence i simulated from seed rank * B + i), independent of every other rank's."""
    lengths = S.data.ragged_lengths(batch_size, seed=0)
    batch = S.data.bearings_batch(lengths, qc=QC, qw=QW, sigma=SIGMA, dt=DT, seed0=rank * batch_size)
    return lengths, batch


def max_over_ranks(torch, dist, ms, device):
    """The slowest rank's step time: the job's step time."""
    if dist is None:
        return ms
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(world, sum_T, ms):
    """Whole-job timesteps/s: every rank processes its own sum_T steps per step time."""
    return world * sum_T / (ms * 1e-3)


def cv_section(torch, S, flush):
    """Constant-velocity linear model (nx = 4, ny = 2, dt = 0.1, q = 0.1, R = 0.5 I, m0 = 0,
    P0 = I), T = 1000 from seed 0, FP64: one parallel square-root filter + RTS smoother pass
    (the smoother at a given nominal, replayed as a CUDA graph).  Its agreement with the FP64
    oracle (1e-10) is checked in the GPU tests."""
    w = S.data.cv_workload(1000, seed=0)
    d = torch.float64
    tm = S.FunctionalModel(S.models.LinearModel(torch.as_tensor(w["F"])),
                           S.MVNSqrt(torch.zeros(4, dtype=d), torch.as_tensor(np.linalg.cholesky(w["Q"]))))
    om = S.FunctionalModel(S.models.LinearModel(torch.as_tensor(w["H"])),
                           S.MVNSqrt(torch.zeros(2, dtype=d), torch.as_tensor(np.linalg.cholesky(w["R"]))))
    x0 = S.MVNSqrt(torch.zeros(4, dtype=d), torch.eye(4, dtype=d))
    nom = S.MVNSqrt(torch.zeros(1001, 4, dtype=d), torch.eye(4, dtype=d).expand(1001, 4, 4).contiguous())
    plan = S.IteratedSmootherPlan(torch.as_tensor(w["ys"], dtype=d), x0, tm, om, S.linearization.extended, nom,
                                  criterion=S.FixedIterations(1), graph=True)
    ms, _ = time_plan(torch, plan, 10, 3, flush)
    return {"workload": "constant velocity nx=4 ny=2, T=1000, FP64, one filter+smoother pass",
            "ms": float(np.median(ms)), "timesteps_per_s": 1000 / (float(np.median(ms)) * 1e-3)}


def published_runtime_section(torch, S, flush):
    """The reference's own GPU runtime experiment (notebooks/experiment_bearing_only_GPU_runtime.ipynb):
    bearings-only CT with r = 0.5, qc = 0.01, qw = 0.1, dt = 0.01, prior m0 = (-4, -1, 2, 7, 3),
    P0 = I, 10 iterated-smoother calls from the nominal (-1, -1, 6, 4, 2) broadcast, FP64,
    one sequence of T = 4096, square-root parallel form; beside the reference's published times
    for T = 4096 (notebooks/new_outputs/rtx-GPU-all-methods.csv:11, GeForce RTX 3080 Ti:
    cubature 0.3751 s, extended 0.3012 s)."""
    T = 4096
    one = S.data.bearings_batch(np.array([T]), qc=0.01, qw=0.1, sigma=0.5, dt=0.01, seed0=50_000)
    Q, R = S.data.bearings_noise(0.01, 0.1, 0.5, 0.01)
    d = torch.float64
    tm = S.FunctionalModel(S.models.CoordinatedTurn(0.01),
                           S.MVNSqrt(torch.zeros(5, dtype=d), torch.as_tensor(np.linalg.cholesky(Q))))
    om = S.FunctionalModel(S.models.Bearings((-1.5, 0.5), (1.0, 1.0)),
                           S.MVNSqrt(torch.zeros(2, dtype=d), torch.as_tensor(np.linalg.cholesky(R))))
    m0 = torch.tensor([-4.0, -1.0, 2.0, 7.0, 3.0], dtype=d)
    x0 = S.MVNSqrt(m0, torch.eye(5, dtype=d))
    n0 = torch.tensor([-1.0, -1.0, 6.0, 4.0, 2.0], dtype=d)
    nom = S.MVNSqrt(n0.expand(T + 1, 5).contiguous(), torch.eye(5, dtype=d).expand(T + 1, 5, 5).contiguous())
    out = {"workload": "bearings CT r=0.5 qc=0.01 qw=0.1, T=4096, 10 calls from (-1,-1,6,4,2) broadcast, FP64, "
                       "sqrt parallel"}
    for name, meth in (("cubature", S.linearization.cubature), ("extended", S.linearization.extended)):
        plan = S.IteratedSmootherPlan(torch.as_tensor(one["ys"], dtype=d), x0, tm, om, meth, nom,
                                      criterion=S.FixedIterations(10), graph=True)
        ms, _ = time_plan(torch, plan, 10, 3, flush)
        out[name + "_s"] = float(np.median(ms)) * 1e-3
        del plan
    out["reference_published_s"] = {"cubature": 0.3751, "extended": 0.3012, "hardware": "GeForce RTX 3080 Ti"}
    out["speedup_vs_published"] = {k: out["reference_published_s"][k] / out[k + "_s"] for k in ("cubature", "extended")}
    return out


def population_section(torch, S, flush):
    """The reference's population experiment (notebooks/experiment-poisson.ipynb): a Ricker-map
    transition and Poisson counts as conditional-moments models, nx = ny = 1, T = 128, 100
    iterated-smoother calls, FP64 (the notebook enables x64), one CUDA graph.  Beside it, the
    reference's own published GPU times for the same setting
    (notebooks/outputs/GPU-population-model.csv, T = 128: parallel IEKS 0.1676 s, IPLS 0.1666 s
    per run, covariance form; this run uses the square-root form).  The notebook starts from a
    random nominal, from which undamped Gauss-Newton leaves the data's basin and overflows; this
    run starts from log((y + 1) / lam), so every one of the 100 calls does finite work."""
    T, lam, Q = 128, 10.0, np.array([[0.3 ** 2]])
    _, ys = S.data.population_data(T)
    mean_f, _, mean_h, _, chol_f, chol_h = S.models.population_parameters(lam, Q)
    f = S.ConditionalMomentsModel(mean_f, chol_f)
    h = S.ConditionalMomentsModel(mean_h, chol_h)
    d = torch.float64
    m0 = np.array([np.log(7.0)])
    x0 = S.MVNSqrt(torch.as_tensor(m0), torch.tensor([[0.5]], dtype=d))
    m_nom = np.concatenate([m0[None], np.log((ys + 1.0) / lam)], 0)
    nom = S.MVNSqrt(torch.as_tensor(m_nom), torch.full((T + 1, 1, 1), 0.5 ** 0.5, dtype=d))
    out = {"workload": "population (Ricker + Poisson conditional moments), T=128, 100 calls, FP64, one CUDA graph"}
    for name, meth in (("ieks", S.linearization.extended), ("ipls", S.linearization.cubature)):
        plan = S.IteratedSmootherPlan(torch.as_tensor(ys, dtype=d), x0, f, h, meth, nom,
                                      criterion=S.FixedIterations(100), graph=True)
        ms, _ = time_plan(torch, plan, 5, 3, flush)
        out[name + "_s"] = float(np.median(ms)) * 1e-3
        del plan
    out["reference_published_s"] = {"ieks_par": 0.16761423110961915, "ipls_par": 0.16656035900115967}
    out["speedup_vs_published"] = {"ieks": out["reference_published_s"]["ieks_par"] / out["ieks_s"],
                                   "ipls": out["reference_published_s"]["ipls_par"] / out["ipls_s"]}
    return out


def sampler_section(torch, S, flush, T=100_000):
    """Pathwise posterior sampling (parsmooth.sampling) of one draw of one bearings sequence of
    T = 1e5 steps, FP32, at the smoothed trajectory: the parallel-in-time sampler (with one
    walker, the per-walker kernel would be one thread stepping through all T steps).  Timed
    with CUDA events around the whole call (its linearisation, the smoothing elements and the
    draw), median of 5 after 2 warm-up calls."""
    one = S.data.bearings_batch(np.array([T]), qc=QC, qw=QW, sigma=SIGMA, dt=DT, seed0=40_000)
    dt = torch.float32
    tm, om = models(torch, S, dt)
    x0 = S.MVNSqrt(torch.as_tensor(PRIOR_M0, dtype=dt), torch.eye(5, dtype=dt))
    filt = S.filtering(torch.as_tensor(one["ys"], dtype=dt), x0, tm, om, S.linearization.cubature)
    nom = S.smoothing(tm, filt, S.linearization.cubature)
    eps = torch.randn((T + 1, 1, 5), dtype=dt, device="cuda", generator=torch.Generator("cuda").manual_seed(0))
    ms = []
    for k in range(7):
        flush.add_(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        xs = S.sampling(None, 1, tm, filt, S.linearization.cubature, nom, eps=eps)
        e1.record()
        torch.cuda.synchronize()
        if k >= 2:
            ms.append(e0.elapsed_time(e1))
    return {"T": T, "samples": 1, "dtype": "f32", "ms": float(np.median(ms)),
            "timesteps_per_s": T / (float(np.median(ms)) * 1e-3), "finite": bool(torch.isfinite(xs).all()),
            "path": "parallel in time (chunks of ~sqrt(T) steps)"}


def sweep_section(torch, S, flush):
    """Single-sequence bearings smoother (10 calls from the prior mean broadcast) for
    T = 1e2 .. 1e5, FP64 then FP32: timesteps/s and the FP32 position RMSE against FP64's."""
    out = []
    for k, T in enumerate((100, 1000, 10_000, 100_000)):
        one = S.data.bearings_batch(np.array([T]), qc=QC, qw=QW, sigma=SIGMA, dt=DT, seed0=30_000 + k)
        row = {"T": T}
        means = {}
        for name, dt in (("fp64", torch.float64), ("fp32", torch.float32)):
            plan = make_plan(torch, S, one["ys"], one["offsets"], dt)
            ms, _ = time_plan(torch, plan, 3, 3, flush)
            row[name] = {"ms": float(np.median(ms)), "timesteps_per_s": T / (float(np.median(ms)) * 1e-3)}
            means[name] = plan.mean.double().cpu().numpy()
            del plan
        xs = one["xs"].astype(np.float64)
        r64 = position_rmse(means["fp64"], xs, one["offsets"])[0]
        r32 = position_rmse(means["fp32"], xs, one["offsets"])[0]
        row["rmse_fp64"], row["rmse_fp32"] = float(r64), float(r32)
        row["rmse_rel_diff"] = float(abs(r32 - r64) / max(r64, 1e-12))
        out.append(row)
        torch.cuda.empty_cache()
    return out


# Algorithmic FP32 flops of the large-state kernels (nx = 32, ny = 16).  A Householder
# lower-triangularisation of an r x c matrix costs 4 sum_{p<r} (c - p)(r - p) flops.  The
# factor recursion (trias, factor products, triangular solves) is counted once per time step
# (shared by the batch in the shared-covariance mode the workload runs in), the vector work
# (means, g, residuals: products of B x nx rows with nx x nx matrices) once per sequence step.
def _tria_flops(r, c):
    return 4 * sum((c - p) * (r - p) for p in range(r))


_NX, _NY = 32, 16
LARGE_FLOPS_FACTOR = {
    "filter_walk": _tria_flops(2 * _NX, 2 * _NX) + _tria_flops(_NX + _NY, _NX + _NY) + _NX ** 3 + _NY * _NX ** 2
                   + _NX ** 3,
    "smoother_leaf": _tria_flops(_NX, 2 * _NX) + _NX ** 3 + 2 * _NX ** 3,
    "smoother_walk": _tria_flops(_NX, 2 * _NX) + _NX ** 3,
}
LARGE_FLOPS_VECTOR = {
    "filter_walk": 2 * (2 * _NX * _NX) + 2 * (2 * _NX * _NY) + _NY * _NY,
    "smoother_leaf": 2 * _NX * _NX,
    "smoother_walk": 2 * _NX * _NX,
}


def large_state_section(torch, S, flush, chunk=32, T=131_072, compare=True):
    """The large-state regime: random stable linear SSM nx = 32, ny = 16, B = 16 sequences of
    T = 131 072, FP32, 10 filter-smoother passes (the default-nominal pass and 9 counted calls;
    a linear model's passes are identical), one CUDA graph.  Errors of the smoothed means and
    covariances against the FP64 path (itself pinned to the FP64 oracle in the tests)."""
    from sqrt_parallel_smoothers_gb300 import _lib
    B, nx, ny = 16, 32, 16
    F, Q, H, R = S.data.large_state_model(nx, ny, 0)
    rng = np.random.RandomState(1)
    cQ, cR = np.linalg.cholesky(Q), np.linalg.cholesky(R)
    x = rng.randn(B, nx)
    ys = np.zeros((B, T, ny), np.float32)
    for t in range(T):
        x = x @ F.T + rng.randn(B, nx) @ cQ.T
        ys[:, t] = x @ H.T + rng.randn(B, ny) @ cR.T
    offsets = np.arange(B + 1) * T

    def setup(dt):
        tm = S.FunctionalModel(S.models.LinearModel(torch.as_tensor(F, dtype=dt)),
                               S.MVNSqrt(torch.zeros(nx, dtype=dt), torch.as_tensor(cQ, dtype=dt)))
        om = S.FunctionalModel(S.models.LinearModel(torch.as_tensor(H, dtype=dt)),
                               S.MVNSqrt(torch.zeros(ny, dtype=dt), torch.as_tensor(cR, dtype=dt)))
        return tm, om, S.MVNSqrt(torch.zeros(nx, dtype=dt), torch.eye(nx, dtype=dt))

    tm, om, x0 = setup(torch.float32)
    y32 = torch.as_tensor(ys.reshape(-1, ny))
    plan = S.IteratedSmootherPlan(y32, x0, tm, om, S.linearization.cubature, None, criterion=S.FixedIterations(9),
                                  offsets=offsets, chunk=chunk, group=8, graph=True)
    ms, _ = time_plan(torch, plan, 2, 1, flush)
    step_ms = float(np.median(ms))
    m32 = plan.mean.double().cpu()
    L32 = plan.chol.cpu()
    launches = plan.launches_per_run
    del plan
    torch.cuda.empty_cache()
    # the general batch: every sequence's factor recursion computed separately
    S.set_large_state_options(per_sequence_covariance=True)
    try:
        plan = S.IteratedSmootherPlan(y32, x0, tm, om, S.linearization.cubature, None,
                                      criterion=S.FixedIterations(9), offsets=offsets, chunk=chunk, group=8,
                                      graph=True)
        ms_ps, _ = time_plan(torch, plan, 2, 1, flush)
        del plan
        torch.cuda.empty_cache()
        pplan = S.IteratedSmootherPlan(y32, x0, tm, om, S.linearization.cubature, None,
                                       criterion=S.FixedIterations(9), offsets=offsets, chunk=chunk, group=8,
                                       graph=True, profile=True)
        pplan.run()
        torch.cuda.synchronize()
        prof_ps = _lib.profile_read()
        del pplan
        _lib.profile_reset()
    finally:
        S.set_large_state_options(per_sequence_covariance=False)
    torch.cuda.empty_cache()
    per_seq_ms = float(np.median(ms_ps))
    tot_ps = sum(v[1] for v in prof_ps.values()) or 1.0
    kern_ps = {k: {"launches": v[0], "total_ms": v[1], "share": v[1] / tot_ps} for k, v in prof_ps.items()}
    pplan = S.IteratedSmootherPlan(y32, x0, tm, om, S.linearization.cubature, None, criterion=S.FixedIterations(9),
                                   offsets=offsets, chunk=chunk, group=8, graph=True, profile=True)
    pplan.run()
    torch.cuda.synchronize()
    prof = _lib.profile_read()
    del pplan
    _lib.profile_reset()
    torch.cuda.empty_cache()
    tot = sum(v[1] for v in prof.values()) or 1.0
    kern = {k: {"launches": v[0], "total_ms": v[1], "share": v[1] / tot} for k, v in prof.items()}
    dom = max(kern, key=lambda k: kern[k]["total_ms"])
    roof = None
    if dom in LARGE_FLOPS_FACTOR:
        per_launch_ms = kern[dom]["total_ms"] / kern[dom]["launches"]
        flops = LARGE_FLOPS_FACTOR[dom] * T + LARGE_FLOPS_VECTOR[dom] * B * T
        ach = flops / (per_launch_ms * 1e-3) / 1e12
        peak = measure_fp32_peak(torch)
        roof = {"kernel": dom, "bound": "fp32", "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": ach / peak,
                "peak_source": "measured here: cuBLAS SGEMM 8192^3, TF32 off (the kernels' factor products run "
                               "on the tensor cores as 3xTF32 mma.sync, the Householder steps on the FP32 pipe)",
                "alg_flops_per_launch": flops,
                "flops_model": "factor recursion once per time step (shared covariance), vectors per sequence step"}
    out = {"workload": f"linear nx=32 ny=16 (F = 0.98 Haar, Q = L L^T/nx, H ~ N(0, 1/nx), R = 0.1 I), B=16, "
                       f"T={T}, FP32, 10 filter-smoother passes, chunk {chunk}, one CUDA graph",
           "mode": "shared covariance (one prior, equal lengths): factors once per time step, means per sequence",
           "ms_per_step": step_ms, "timesteps_per_s": B * T / (step_ms * 1e-3), "gpu_launches": launches,
           "per_sequence_covariance": {"ms_per_step": per_seq_ms, "timesteps_per_s": B * T / (per_seq_ms * 1e-3),
                                       "mode": "every sequence's factors computed separately (the general batch)",
                                       "kernels": kern_ps},
           "kernels": kern, "roofline": roof}
    if not compare:
        return out
    tm64, om64, x064 = setup(torch.float64)
    res64 = S.iterated_smoothing(torch.as_tensor(ys.reshape(-1, ny), dtype=torch.float64), x064, tm64, om64,
                                 S.linearization.cubature, None, criterion=S.FixedIterations(1), offsets=offsets,
                                 chunk=chunk)
    m64 = res64.mean.cpu()
    idx = torch.arange(0, m64.shape[0], 97)
    L64 = res64.chol[idx.to(res64.chol.device)].cpu()
    del res64
    torch.cuda.empty_cache()
    C32 = L32[idx].double() @ L32[idx].double().transpose(-1, -2)
    C64 = L64 @ L64.transpose(-1, -2)
    out["mean_err_rel_vs_fp64"] = float((m32 - m64).abs().max() / m64.abs().max())
    out["cov_err_rel_vs_fp64"] = float((C32 - C64).abs().max() / C64.abs().max())
    return out


def gpu_arm(args):
    import torch
    import sqrt_parallel_smoothers_gb300 as S
    from sqrt_parallel_smoothers_gb300 import _lib

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()

    if args.only_large:
        flush = torch.zeros(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
        if rank == 0:
            print(json.dumps(large_state_section(torch, S, flush, T=args.large_T, compare=False)), flush=True)
        return 0
    if args.only_adjoint:
        flush = torch.zeros(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
        if rank == 0:
            print(json.dumps(adjoint_section(torch, S, flush)), flush=True)
        return 0
    lengths, batch = rank_batch(S, args.batch, rank)
    offsets = batch["offsets"]
    tuning = None
    if args.chunk == 0 and not args.no_autotune:
        from sqrt_parallel_smoothers_gb300 import autotune
        key = autotune.signature(5, 2, "f32", lengths, "cubature") + ":streams"
        (args.chunk, args.group, args.streams), tuning = autotune.tune(
            lambda c, g, k: make_plan(torch, S, batch["ys"], offsets, torch.float32, c, g, streams=k), key=key)
    plan = make_plan(torch, S, batch["ys"], offsets, torch.float32, args.chunk, args.group, streams=args.streams)
    C = args.chunk or 16
    G = args.group or 8
    flush = torch.zeros(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MiB > L2
    sampler = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    step_ms, clocks = time_plan(torch, plan, args.steps, args.warmup, flush, sampler)
    torch.cuda.synchronize()
    barrier()
    ms = max_over_ranks(torch, dist, float(np.mean(step_ms)), "cuda")
    sum_T = int(lengths.sum())
    value = job_value(world, sum_T, ms)
    launches = plan.launches_per_run * args.steps

    # e2e: host observations in (pinned), the smoothed trajectory out (pinned), every step
    ys_host = torch.as_tensor(batch["ys"], dtype=torch.float32).pin_memory()
    m_host = torch.empty(plan.mean.shape, dtype=torch.float32).pin_memory()
    L_host = torch.empty(plan.chol.shape, dtype=torch.float32).pin_memory()
    for _ in range(max(args.warmup, 2)):
        plan.run_host(ys_host, m_host, L_host, pipelined=True)
    plan.sync_host()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        plan.run_host(ys_host, m_host, L_host, pipelined=True)
    plan.sync_host()                      # the last step's copy-out is inside the timed region
    e1.record()
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks(torch, dist, e0.elapsed_time(e1) / args.steps, "cuda")
    e2e = {"value": job_value(world, sum_T, e2e_ms), "unit": UNIT, "h2d_bytes_per_step": int(ys_host.nbytes),
           "d2h_bytes_per_step": int(m_host.nbytes + L_host.nbytes), "ms_per_step": e2e_ms,
           "path": "IteratedSmootherPlan.run_host(pipelined=True): pinned host copy-in, graph replay, "
                   "copy-out on a second stream overlapping the next step (two plans alternate)"}
    mean32 = m_host.numpy().astype(np.float64)

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded simulator of the reference's "
                                                       "bearings experiment)",
            "config": dict(workload_config(args.batch, lengths, C, G), streams=int(args.streams)), "e2e": e2e,
            "gpu_launches": int(launches),
            "clocks": clocks}
    if tuning is not None:
        line["config"]["autotune_ms"] = tuning

    # per-kernel device times from CUDA events captured in a second graph (roofline)
    pplan = make_plan(torch, S, batch["ys"], offsets, torch.float32, args.chunk, args.group, profile=True)
    totals = {}
    for _ in range(args.steps):
        flush.add_(1)
        pplan.run()
        torch.cuda.synchronize()
        for k, (n, t) in _lib.profile_read().items():
            a = totals.setdefault(k, [0, 0.0])
            a[0] += n
            a[1] += t
    del pplan
    torch.cuda.synchronize()
    _lib.profile_reset()
    kern = {k: {"launches": v[0], "total_ms": v[1], "avg_ms": v[1] / max(v[0], 1)} for k, v in totals.items()}
    tot = sum(v["total_ms"] for v in kern.values()) or 1.0
    for v in kern.values():
        v["share"] = v["total_ms"] / tot
    dom = max(kern, key=lambda k: kern[k]["total_ms"])
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    alg = ALG_BYTES_PER_STEP.get(dom)
    if alg is not None:
        achieved = alg * sum_T / (kern[dom]["avg_ms"] * 1e-3) / 1e9
        line["roofline"] = {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                            "frac": achieved / hbm_peak,
                            "traffic": TRAFFIC_BYTES_PER_STEP[dom] * sum_T if dom in TRAFFIC_BYTES_PER_STEP else None,
                            "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback",
                            "alg_bytes_per_launch": alg * sum_T}
    # the other side of the roofline: executed FP32 flops against the measured FP32 rate, per
    # kernel and for the whole pass; and the whole pass's HBM fraction on its own minimal bytes
    fp32_peak = measure_fp32_peak(torch)
    pass_gbs = PASS_ALG_BYTES_PER_STEP * sum_T * N_ITER / (ms * 1e-3) / 1e9
    line["roofline_pass"] = {
        "hbm": {"alg_bytes_per_step_call": PASS_ALG_BYTES_PER_STEP, "achieved_gbs": pass_gbs,
                "frac": pass_gbs / hbm_peak,
                "definition": "observation, nominal in, smoothed out, filtered hand-off written and read: "
                              "82 floats per timestep and call"},
        "fp32_peak_tflops": fp32_peak,
        "fp32_peak_source": "measured here: cuBLAS SGEMM 8192^3, TF32 off, best of 5"}
    if FP32_FLOPS_PER_STEP:
        fl = {}
        for k, f in FP32_FLOPS_PER_STEP.items():
            if k in kern:
                tf = f * sum_T / (kern[k]["avg_ms"] * 1e-3) / 1e12
                fl[k] = {"flops_per_step": f, "achieved_tflops": tf, "frac": tf / fp32_peak}
        tot_f = sum(FP32_FLOPS_PER_STEP.values())
        pass_tf = tot_f * sum_T * N_ITER / (ms * 1e-3) / 1e12
        line["roofline_pass"]["fp32"] = {"flops_per_step_call": tot_f, "achieved_tflops": pass_tf,
                                         "frac": pass_tf / fp32_peak, "kernels": fl,
                                         "source": "executed FP32 operations of the per-step kernels (ncu)"}
        if dom in fl:
            line["roofline_fp32"] = {"kernel": dom, "bound": "fp32", "achieved": fl[dom]["achieved_tflops"],
                                     "peak": fp32_peak, "unit": "TFLOP/s", "frac": fl[dom]["frac"]}
    line["kernels"] = kern
    if args.only_main:
        print(json.dumps(line), flush=True)
        return 0

    # FP64 plain: one sequence, T = 5000, FP64
    one = S.data.bearings_batch(np.array([FP64_PLAIN_T]), qc=QC, qw=QW, sigma=SIGMA, dt=DT, seed0=10_000)
    plan64 = make_plan(torch, S, one["ys"], one["offsets"], torch.float64)
    ms64, _ = time_plan(torch, plan64, max(3, min(args.steps, 5)), 1, flush)
    v64 = FP64_PLAIN_T / (float(np.mean(ms64)) * 1e-3)
    line["fp64_plain"] = {"value": v64, "unit": UNIT, "T": FP64_PLAIN_T, "ms_per_step": float(np.mean(ms64))}
    line["ratio_vs_fp64_plain"] = value / world / v64

    # accuracy: FP32 batched vs FP64 batched (same GPU path in FP64, checked against the FP64 oracle in
    # the tests) against the simulated truth.  "Converged" = the FP64 run meets the reference's default
    # test (mean squared change <= 1e-6) within the same 10 calls; the FP32 and FP64 RMSEs are compared
    # on those sequences (undamped Gauss-Newton diverges on some long, strongly manoeuvring tracks).
    plan_acc = make_plan(torch, S, batch["ys"], offsets, torch.float64, graph=False)
    plan_acc.run()
    torch.cuda.synchronize()
    mean64 = plan_acc.mean.cpu().numpy()
    del plan_acc
    plan_cv = make_plan(torch, S, batch["ys"], offsets, torch.float64, graph=False,
                        criterion=S.MeanSquaredChange(1e-6, N_ITER))
    plan_cv.run()
    torch.cuda.synchronize()
    conv = (plan_cv._outs[4].cpu().numpy() & 4) == 0
    del plan_cv
    r32 = position_rmse(mean32, batch["xs"].astype(np.float64), offsets)
    r64 = position_rmse(mean64, batch["xs"].astype(np.float64), offsets)
    rel = np.abs(r32 - r64) / np.maximum(r64, 1e-12)
    line["accuracy"] = {"frac_within_1pct_all": float(np.mean(rel <= 0.01)),
                        "frac_within_1pct_converged": float(np.mean(rel[conv] <= 0.01)),
                        "frac_within_1pct_not_converged": float(np.mean(rel[~conv] <= 0.01))
                        if (~conv).any() else None,
                        "converged_frac_fp64": float(np.mean(conv)),
                        "rmse_fp32_median_converged": float(np.median(r32[conv])),
                        "rmse_fp64_median_converged": float(np.median(r64[conv])),
                        "rmse_rel_diff_median_converged": float(np.median(rel[conv])),
                        "rmse_rel_diff_max_converged": float(np.max(rel[conv])),
                        "rmse": "position RMSE of smoothed means vs simulated truth, per sequence, "
                                "FP32 GPU vs FP64 GPU over the whole batch"}
    if rank == 0 and not args.no_cpu_baseline:
        line["accuracy"]["vs_oracle"] = oracle_accuracy_sample(batch, lengths, mean32, mean64, conv)

    line["adjoint"] = adjoint_section(torch, S, flush)
    if not args.no_extra:
        line["cv_fp64"] = cv_section(torch, S, flush)
        line["population"] = population_section(torch, S, flush)
        line["published_runtime"] = published_runtime_section(torch, S, flush)
        line["sweep_T"] = sweep_section(torch, S, flush)
        line["sampler"] = sampler_section(torch, S, flush)
        line["large_state"] = large_state_section(torch, S, flush)

    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        seqs, tot = cpu_sample(lengths, batch, budget_steps=6000)
        t_cpu = run_cpu(seqs, 1)
        line["cpu_baseline"] = {"value": tot / t_cpu, "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": f"first {len(seqs)} sequences of the batch (sum T = {tot}), "
                                          f"{N_ITER} calls, FP64 NumPy port, 1 process"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--batch", type=int, default=B_DEFAULT)
    ap.add_argument("--chunk", type=int, default=0)
    ap.add_argument("--group", type=int, default=0)
    ap.add_argument("--streams", type=int, default=1, help="concurrent sequence groups (tuned with --chunk 0)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--only-main", action="store_true", help="time the FP32 batched smoother and its kernels only")
    ap.add_argument("--no-autotune", action="store_true", help="use the default chunk/group (16, 8)")
    ap.add_argument("--no-extra", action="store_true", help="skip the T sweep and the large-state workload")
    ap.add_argument("--only-large", action="store_true", help="run the large-state workload only")
    ap.add_argument("--large-T", type=int, default=131_072, help="sequence length of the large-state workload")
    ap.add_argument("--only-adjoint", action="store_true",
                    help="run the gradient workloads only (reverse and tangent passes, p = 4 and p = 32)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return reference_arm(args)
    return gpu_arm(args)


if __name__ == "__main__":
    sys.exit(main())
