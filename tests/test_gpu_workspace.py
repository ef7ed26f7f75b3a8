"""The library writes nothing outside the workspace it sized: ss_iterated with a workspace of
exactly ss_workspace_bytes, followed by a guard region, for every small state dimension (the
loop's intermediate nominals are packed state records, longer than nx * nx for nx <= 3)."""
import ctypes

import numpy as np
import pytest
import torch

from sqrt_parallel_smoothers_gb300 import _lib

pytestmark = pytest.mark.gpu

P = ctypes.c_void_p
GUARD = 1 << 16


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("nx,ny", [(1, 1), (2, 1), (3, 2), (4, 2), (5, 2)])
def test_iterated_stays_inside_its_workspace(nx, ny, dtype):
    dev = torch.device("cuda", torch.cuda.current_device())
    rng = np.random.RandomState(nx * 10 + ny)
    lengths = np.array([5, 1, 0, 3])
    offsets = np.concatenate([[0], np.cumsum(lengths)])
    N, B = int(offsets[-1]), len(lengths)
    A = np.eye(nx) * 0.9 + 0.05 * rng.randn(nx, nx)
    H = rng.randn(ny, nx)
    t = dict(ys=torch.as_tensor(rng.randn(N, ny), dtype=dtype, device=dev),
             offsets=torch.as_tensor(offsets, dtype=torch.int64, device=dev),
             m0=torch.zeros(nx, dtype=dtype, device=dev), L0=torch.eye(nx, dtype=dtype, device=dev),
             A=torch.as_tensor(A, dtype=dtype, device=dev), H=torch.as_tensor(H, dtype=dtype, device=dev),
             qm=torch.zeros(nx, dtype=dtype, device=dev), qL=0.3 * torch.eye(nx, dtype=dtype, device=dev),
             rm=torch.zeros(ny, dtype=dtype, device=dev), rL=0.5 * torch.eye(ny, dtype=dtype, device=dev))
    p = _lib.SSProblem()
    p.dtype = _lib.SS_F32 if dtype == torch.float32 else _lib.SS_F64
    p.nx, p.ny, p.lin_method, p.gh_order = nx, ny, _lib.SS_LIN_CUBATURE, 3
    p.ut_alpha, p.ut_kappa_default = 1.0, 1
    for mdl, mat, qm, qL in ((p.transition, t["A"], t["qm"], t["qL"]), (p.observation, t["H"], t["rm"], t["rL"])):
        mdl.kind = _lib.SS_MODEL_LINEAR
        mdl.matrix, mdl.noise_mean, mdl.noise_chol = mat.data_ptr(), qm.data_ptr(), qL.data_ptr()
    p.batch, p.total_steps, p.max_len = B, N, int(lengths.max())
    p.chunk, p.group = 2, 2
    p.offsets = t["offsets"].data_ptr()
    lib = _lib.load()
    nbytes = ctypes.c_size_t(0)
    assert lib.ss_workspace_bytes(ctypes.byref(p), ctypes.byref(nbytes)) == _lib.SS_OK
    n = int(nbytes.value)
    buf = torch.full((n + GUARD,), 0x5A, dtype=torch.uint8, device=dev)
    out_m = torch.empty((N + B, nx), dtype=dtype, device=dev)
    out_L = torch.empty((N + B, nx, nx), dtype=dtype, device=dev)
    rc = lib.ss_iterated(ctypes.byref(p), t["ys"].data_ptr(), t["m0"].data_ptr(), t["L0"].data_ptr(), 0, None, None,
                         4, 0.0, out_m.data_ptr(), out_L.data_ptr(), None, None, None, buf.data_ptr(), n,
                         torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.SS_OK
    torch.cuda.synchronize()
    assert torch.isfinite(out_m).all()
    assert bool((buf[n:] == 0x5A).all()), "the call wrote past its workspace"
