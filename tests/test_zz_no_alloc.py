"""ss_iterated_noalloc: the iterated smoother for callers that cannot allocate
device memory (hosts that only hand over data pointers and a stream).  It must
give the same trajectory as ss_iterated with a caller workspace, call after
call, although every call reuses the library's one static scratch array.

Runs through the C ABI with ctypes; collected last so that a run stopping at
the first failure has already run every other test."""
import ctypes

import numpy as np
import pytest
import torch

from sqrt_parallel_smoothers_gb300 import _lib
import sqrt_parallel_smoothers_gb300 as S

pytestmark = pytest.mark.gpu

P = ctypes.c_void_p
NOALLOC_MAX = 64 * 1024 * 1024  # SS_NOALLOC_SCRATCH_BYTES in include/sqrtsmooth.h


def _bind():
    lib = _lib.load()
    lib.ss_iterated_noalloc.argtypes = [ctypes.POINTER(_lib.SSProblem), P, P, P, ctypes.c_int32, P, P,
                                        ctypes.c_int32, ctypes.c_double, P, P, P, P, P, P]
    lib.ss_iterated_noalloc.restype = ctypes.c_int
    return lib


def _bearings_problem(lengths, dtype, seed0=0):
    batch = S.data.bearings_batch(np.asarray(lengths), seed0=seed0)
    dev = torch.device("cuda", torch.cuda.current_device())
    Q, R = batch["Q"], batch["R"]
    t = dict(
        ys=torch.as_tensor(batch["ys"], dtype=dtype, device=dev),
        offsets=torch.as_tensor(batch["offsets"], dtype=torch.int64, device=dev),
        m0=torch.tensor([0.1, 0.2, 1.0, 0.0, 1.0], dtype=dtype, device=dev),
        L0=torch.eye(5, dtype=dtype, device=dev),
        tqm=torch.zeros(5, dtype=dtype, device=dev),
        tqL=torch.as_tensor(np.linalg.cholesky(Q), dtype=dtype, device=dev),
        oqm=torch.zeros(2, dtype=dtype, device=dev),
        oqL=torch.as_tensor(np.linalg.cholesky(R), dtype=dtype, device=dev))
    p = _lib.SSProblem()
    p.dtype = _lib.SS_F32 if dtype == torch.float32 else _lib.SS_F64
    p.nx, p.ny, p.lin_method, p.gh_order = 5, 2, _lib.SS_LIN_CUBATURE, 3
    p.ut_alpha, p.ut_kappa_default = 1.0, 1
    p.transition.kind = _lib.SS_MODEL_COORDINATED_TURN
    p.transition.params[0] = 0.01
    p.transition.noise_mean, p.transition.noise_chol = t["tqm"].data_ptr(), t["tqL"].data_ptr()
    p.observation.kind = _lib.SS_MODEL_BEARINGS
    for k, v in enumerate((-1.5, 0.5, 1.0, 1.0)):
        p.observation.params[k] = v
    p.observation.noise_mean, p.observation.noise_chol = t["oqm"].data_ptr(), t["oqL"].data_ptr()
    p.batch, p.total_steps, p.max_len = len(lengths), int(np.sum(lengths)), int(np.max(lengths))
    p.offsets = t["offsets"].data_ptr()
    return p, t


def _outputs(p, t):
    n_states = p.total_steps + p.batch
    return dict(m=torch.empty((n_states, 5), dtype=t["ys"].dtype, device=t["ys"].device),
                L=torch.empty((n_states, 5, 5), dtype=t["ys"].dtype, device=t["ys"].device),
                ell=torch.empty(p.batch, dtype=torch.float64, device=t["ys"].device),
                iters=torch.empty(p.batch, dtype=torch.int32, device=t["ys"].device),
                flags=torch.empty(p.batch, dtype=torch.int32, device=t["ys"].device))


def _run_with_workspace(lib, p, t, n_iter, tol=0.0):
    nbytes = ctypes.c_size_t(0)
    assert lib.ss_workspace_bytes(ctypes.byref(p), ctypes.byref(nbytes)) == _lib.SS_OK
    ws = torch.empty(nbytes.value, dtype=torch.uint8, device=t["ys"].device)
    o = _outputs(p, t)
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.ss_iterated(ctypes.byref(p), t["ys"].data_ptr(), t["m0"].data_ptr(), t["L0"].data_ptr(), 0, None,
                         None, n_iter, tol, o["m"].data_ptr(), o["L"].data_ptr(), o["ell"].data_ptr(),
                         o["iters"].data_ptr(), o["flags"].data_ptr(), ws.data_ptr(), nbytes.value, stream)
    assert rc == _lib.SS_OK
    torch.cuda.synchronize()
    return o


def _run_noalloc(lib, p, t, n_iter, tol=0.0):
    o = _outputs(p, t)
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.ss_iterated_noalloc(ctypes.byref(p), t["ys"].data_ptr(), t["m0"].data_ptr(), t["L0"].data_ptr(), 0,
                                 None, None, n_iter, tol, o["m"].data_ptr(), o["L"].data_ptr(),
                                 o["ell"].data_ptr(), o["iters"].data_ptr(), o["flags"].data_ptr(), stream)
    assert rc == _lib.SS_OK, _lib.load().ss_status_string(rc)
    torch.cuda.synchronize()
    return o


# Both entry points run the same kernels on the same inputs with the same
# layout inside their scratch, so the results must agree bit for bit.
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_noalloc_matches_workspace_entry_point(dtype):
    lib = _bind()
    for call, (lengths, seed0) in enumerate((([120, 7, 64, 300], 0), ([55, 260, 1, 90, 33], 100))):
        p, t = _bearings_problem(lengths, dtype, seed0)
        ref = _run_with_workspace(lib, p, t, 3)
        got = _run_noalloc(lib, p, t, 3)
        for key in ("m", "L", "ell", "iters", "flags"):
            assert torch.equal(got[key], ref[key]), (call, key)
        assert torch.isfinite(got["m"]).all()


# With a tolerance the smoother keeps per-sequence state (mean-squared change,
# active flags, call counts) in the shared scratch.  Two calls back to back
# check that each call starts that state afresh instead of inheriting the
# previous call's (the second problem converges differently from the first).
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_noalloc_tolerance_criterion_twice(dtype):
    lib = _bind()
    for call, (lengths, seed0) in enumerate((([200, 40, 500], 7), ([90, 350, 12, 260], 300))):
        p, t = _bearings_problem(lengths, dtype, seed0)
        ref = _run_with_workspace(lib, p, t, 20, 1e-6)
        got = _run_noalloc(lib, p, t, 20, 1e-6)
        for key in ("m", "L", "ell", "iters", "flags"):
            assert torch.equal(got[key], ref[key]), (call, key)
        assert int(got["iters"].min()) >= 1


def test_noalloc_rejects_problems_beyond_its_scratch():
    lib = _bind()
    p, t = _bearings_problem([50], torch.float32)
    p.total_steps = p.max_len = 400_000   # only the sizes are read before the rejection
    need = ctypes.c_size_t(0)
    assert lib.ss_workspace_bytes(ctypes.byref(p), ctypes.byref(need)) == _lib.SS_OK
    assert need.value > NOALLOC_MAX
    o = _outputs(_bearings_problem([50], torch.float32)[0], t)
    rc = lib.ss_iterated_noalloc(ctypes.byref(p), t["ys"].data_ptr(), t["m0"].data_ptr(), t["L0"].data_ptr(), 0,
                                 None, None, 3, 0.0, o["m"].data_ptr(), o["L"].data_ptr(), None, None, None,
                                 torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.SS_ERR_WORKSPACE
