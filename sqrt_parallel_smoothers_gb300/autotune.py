"""Autotuner for the scan geometry (steps per chunk C, summaries per group G) and the
number of concurrent sequence groups S.

The chunk kernels are register-bound (one thread holds a chunk's square-root
summary), so C trades resident-thread waves on the 152 SMs against the work
left to the higher scan levels.  The tuner times each candidate on the real
workload (a captured CUDA graph of the whole iterated smoother, CUDA events,
median of a few replays) and caches the winner per workload signature in a
JSON file (``$SQRTSMOOTH_CACHE`` or ``~/.cache/sqrtsmooth/autotune.json``).
"""
import json
import os

import torch

# (steps per chunk C, summaries per group G, concurrent sequence groups S)
DEFAULT_CANDIDATES = ((8, 8, 1), (16, 4, 1), (32, 4, 1), (32, 4, 3), (16, 8, 4), (8, 8, 4), (12, 4, 2),
                      (12, 4, 4), (16, 4, 2), (16, 4, 3), (16, 4, 4), (20, 4, 2), (24, 4, 2), (24, 4, 4))


def cache_path():
    base = os.environ.get("SQRTSMOOTH_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "sqrtsmooth")
    return os.path.join(base, "autotune.json")


def signature(nx, ny, dtype, lengths, method):
    """Key of a workload: dims, dtype, method, batch size and a coarse length histogram."""
    import numpy as np
    lengths = np.asarray(lengths)
    hist = np.histogram(np.log2(np.maximum(lengths, 1)), bins=8, range=(0, 24))[0]
    return f"{nx}x{ny}:{dtype}:{method}:B{len(lengths)}:N{int(lengths.sum()) >> 14}:" + ",".join(map(str, hist))


def _load():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(table):
    path = cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as f:
            json.dump(table, f, indent=1, sort_keys=True)
    except OSError:
        pass


def time_plan(plan, reps=5):
    """Median device time (ms) of ``reps`` replays of a plan."""
    plan.run()
    torch.cuda.synchronize()
    times = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        plan.run()
        b.record()
        torch.cuda.synchronize()
        times.append(a.elapsed_time(b))
    times.sort()
    return times[len(times) // 2]


def tune(make_plan, key=None, candidates=DEFAULT_CANDIDATES, reps=5, use_cache=True):
    """Pick a geometry for ``make_plan(*candidate) -> IteratedSmootherPlan``.

    Candidates are tuples such as ``(chunk, group, streams)``.  Returns
    ``(best_candidate, {"C,G,S": ms})``; with a ``key`` the result is cached."""
    table = _load() if (use_cache and key) else {}
    if key and key in table:
        return tuple(table[key]["best"]), table[key]["ms"]
    results = {}
    for cand in candidates:
        plan = make_plan(*cand)
        results[",".join(str(v) for v in cand)] = time_plan(plan, reps)
        del plan
        torch.cuda.empty_cache()
    best = tuple(int(v) for v in min(results, key=results.get).split(","))
    if key:
        table = _load()
        table[key] = {"best": list(best), "ms": results}
        _store(table)
    return best, results
