"""Host-side checks that need no GPU: the C ABI loads and exports every symbol
declared in include/*.h, struct layouts agree, argument validation maps to
the reference's exception types, and the batch/criterion host logic."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest
import torch

import sqrt_parallel_smoothers_gb300 as S
from sqrt_parallel_smoothers_gb300 import _lib, methods
from sqrt_parallel_smoothers_gb300.linearization import cubature, unscented, gauss_hermite, resolve

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        names |= set(re.findall(r"^\s*(?:int|const char\*|long long)\s+(ss_\w+)\s*\(", src, flags=re.M))
    return names


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    declared = _declared_symbols()
    assert declared, "no declarations found"
    for name in declared:
        assert hasattr(lib, name), name
    assert lib.ss_version() >= 10000


def test_struct_layout():
    assert ctypes.sizeof(_lib.SSModel) == 64
    assert ctypes.sizeof(_lib.SSProblem) == 224


def _problem(**kw):
    p = _lib.SSProblem()
    p.dtype, p.nx, p.ny, p.lin_method, p.batch = _lib.SS_F32, 5, 2, _lib.SS_LIN_CUBATURE, 1
    p.gh_order = 3
    dummy = ctypes.c_double(0)
    for m in (p.transition, p.observation):
        m.kind = _lib.SS_MODEL_LINEAR
        m.matrix = m.noise_mean = m.noise_chol = ctypes.addressof(dummy)
    p.offsets = ctypes.addressof(dummy)
    p.total_steps = p.max_len = 10
    for k, v in kw.items():
        setattr(p, k, v)
    return p, dummy


def test_workspace_query_and_validation():
    lib = _lib.load()
    p, keep = _problem()
    n = ctypes.c_size_t(0)
    assert lib.ss_workspace_bytes(ctypes.byref(p), ctypes.byref(n)) == 0
    assert n.value > 0
    p2, keep2 = _problem(nx=40)
    assert lib.ss_workspace_bytes(ctypes.byref(p2), ctypes.byref(n)) == _lib.SS_ERR_UNSUPPORTED
    p3, keep3 = _problem(dtype=7)
    assert lib.ss_workspace_bytes(ctypes.byref(p3), ctypes.byref(n)) == _lib.SS_ERR_INVALID
    with pytest.raises(NotImplementedError):
        _lib.check(_lib.SS_ERR_UNSUPPORTED)
    with pytest.raises(ValueError):
        _lib.check(_lib.SS_ERR_INVALID)
    # a bearings observation needs ny = 2: (nx=5, ny=3) with bearings is not built
    p4, keep4 = _problem(ny=3)
    p4.observation.kind = _lib.SS_MODEL_BEARINGS
    assert lib.ss_supported(ctypes.byref(p4)) == 0
    p4.observation.kind = _lib.SS_MODEL_LINEAR
    assert lib.ss_supported(ctypes.byref(p4)) == 1


def test_large_state_dims_are_linear_only():
    """The large-state kernels (nx = 8 and 32) take linear models only; their workspace
    holds one smoothing element per step, which dominates at the large-state workload."""
    lib = _lib.load()
    n = ctypes.c_size_t(0)
    for nx, ny in ((8, 4), (32, 16)):
        for dt in (_lib.SS_F32, _lib.SS_F64):
            p, keep = _problem(nx=nx, ny=ny, dtype=dt)
            assert lib.ss_supported(ctypes.byref(p)) == 1
            assert lib.ss_workspace_bytes(ctypes.byref(p), ctypes.byref(n)) == 0
            assert n.value > 0
            p.transition.kind = _lib.SS_MODEL_COORDINATED_TURN
            assert lib.ss_supported(ctypes.byref(p)) == 0
    p, keep = _problem(nx=32, ny=16, batch=16)
    p.total_steps, p.max_len = 16 * 131072, 131072
    assert lib.ss_workspace_bytes(ctypes.byref(p), ctypes.byref(n)) == 0
    per_step = (2 * 32 * 32 + 32) * 4
    assert per_step * p.total_steps <= n.value <= 4 * per_step * p.total_steps
    p2, keep2 = _problem(nx=16, ny=8)
    assert lib.ss_supported(ctypes.byref(p2)) == 0


def test_wide_dims_are_supported_and_nine_states_are_not():
    """ss_supported answers for the six- to eight-state pairs (a nonlinear model included)."""
    lib = _lib.load()
    dummy = ctypes.c_double(0)
    for nx, ny, ok in ((6, 2, 1), (7, 2, 1), (8, 2, 1), (8, 1, 1), (6, 3, 1), (9, 2, 0), (7, 3, 0)):
        p = _lib.SSProblem()
        p.dtype, p.nx, p.ny, p.lin_method, p.batch, p.gh_order = _lib.SS_F32, nx, ny, _lib.SS_LIN_CUBATURE, 1, 3
        p.transition.kind = _lib.SS_MODEL_RICKER
        p.observation.kind = _lib.SS_MODEL_BEARINGS if ny == 2 else _lib.SS_MODEL_LINEAR
        for mdl in (p.transition, p.observation):
            mdl.matrix = mdl.noise_mean = mdl.noise_chol = ctypes.addressof(dummy)
        p.offsets = ctypes.addressof(dummy)
        p.total_steps = p.max_len = 10
        assert lib.ss_supported(ctypes.byref(p)) == ok, (nx, ny)


def test_calls_without_workspace_fail_cleanly():
    lib = _lib.load()
    p, keep = _problem()
    buf = ctypes.c_double(0)
    a = ctypes.addressof(buf)
    # workspace too small: rejected on the host before any launch
    rc = lib.ss_filter(ctypes.byref(p), a, a, a, 0, None, None, a, a, None, a, 8, None)
    assert rc == _lib.SS_ERR_WORKSPACE


def test_criterion_schedule():
    assert methods._criterion_schedule(lambda i, *_: i < 10) == (10, 0.0)
    assert methods._criterion_schedule(lambda i, *_: i < 1) == (1, 0.0)
    assert methods._criterion_schedule(methods._default_criterion) == (100, 1e-6)
    assert methods._criterion_schedule(S.MeanSquaredChange(1e-8, 7)) == (7, 1e-8)
    with pytest.raises(NotImplementedError):
        methods._criterion_schedule(lambda i, a, b: float(np.mean(a.mean)) > 0)


def test_method_resolution():
    import functools
    assert resolve(cubature).code == _lib.SS_LIN_CUBATURE
    m = resolve(functools.partial(unscented, alpha=0.5))
    assert m.params["alpha"] == 0.5 and m.code == _lib.SS_LIN_UNSCENTED
    assert resolve(functools.partial(gauss_hermite, order=5)).params["order"] == 5
    with pytest.raises(NotImplementedError):
        resolve(lambda model, x: None)


def test_ragged_layout_roundtrip():
    lengths = np.array([3, 0, 5, 1])
    ys = torch.arange(4 * 5 * 2, dtype=torch.float32).reshape(4, 5, 2)
    lay = methods._Layout(ys, lengths, None, None, torch.device("cpu"))
    assert (lay.B, lay.N, lay.max_len) == (4, 9, 5)
    assert lay.offsets.tolist() == [0, 3, 3, 8, 9]
    np.testing.assert_array_equal(lay.ys[3:8].numpy(), ys[2, :5].numpy())
    traj = torch.randn(4, 6, 3)
    packed = lay.pack_states(traj, (3,))
    assert packed.shape == (9 + 4, 3)
    back = lay.unpack_states(packed, (3,))
    for i, T in enumerate(lengths):
        np.testing.assert_array_equal(back[i, :T + 1].numpy(), traj[i, :T + 1].numpy())


def test_non_device_models_are_rejected():
    with pytest.raises(NotImplementedError):
        S.models.as_device_model(lambda x: x)
    # parsmooth/linearization/_common.py:17-66 wraps a Python f(x, q): no device form
    with pytest.raises(NotImplementedError, match="device models"):
        S.linearization.get_conditional_model(lambda x, q: x + q, None, S.linearization.cubature)


def test_gh_roots_match_numpy():
    # the library computes Gauss-Hermite roots by bisection; check against numpy's
    from numpy.polynomial.hermite import hermgauss
    for p in range(1, 9):
        r, w = hermgauss(p)
        from oracle.linearization import gauss_hermite_weights
        wm, _, xi = gauss_hermite_weights(1, p)
        np.testing.assert_allclose(np.sort(xi[:, 0]), np.sqrt(2) * np.sort(r), atol=1e-10)


def test_group_cuts_cover_the_batch():
    """Concurrent sequence groups of IteratedSmootherPlan: contiguous, covering every sequence,
    at most k of them, each with at least one step, about equal in steps."""
    rng = np.random.RandomState(0)
    cases = [np.array([60, 3, 0, 140, 97, 1, 33, 250]), np.array([0, 0, 5, 0]), np.array([5, 0, 0, 0]),
             np.array([1, 1]), np.array([7]), rng.randint(0, 50, size=300)]
    for lengths in cases:
        off = np.concatenate([[0], np.cumsum(lengths)])
        for k in (1, 2, 3, 4, 6, 8):
            cuts = methods._group_cuts(lengths, k)
            assert cuts[0] == 0 and cuts[-1] == len(lengths)
            assert all(a < b for a, b in zip(cuts[:-1], cuts[1:]))
            assert len(cuts) - 1 <= k
            steps = [int(off[b] - off[a]) for a, b in zip(cuts[:-1], cuts[1:])]
            if off[-1] > 0:
                assert min(steps) >= 1
            if len(lengths) >= 100 and k > 1:
                assert max(steps) <= 2 * off[-1] / (len(cuts) - 1)


def test_layout_rejects_bad_shapes():
    """Shape errors are raised on the host, before any device work (ValueError, as the
    reference's own shape checks)."""
    ys = torch.zeros(3, 5, 2)
    with pytest.raises(ValueError):
        methods._Layout(ys, np.array([1, 2]), None, None, torch.device("cpu"))        # B mismatch
    with pytest.raises(ValueError):
        methods._Layout(ys, np.array([1, 6, 2]), None, None, torch.device("cpu"))     # T_i > T
    with pytest.raises(ValueError):
        methods._Layout(ys, np.array([1, -1, 2]), None, None, torch.device("cpu"))    # negative
    with pytest.raises(ValueError):
        methods._Layout(torch.zeros(3, 5, 2, 1), None, None, None, torch.device("cpu"))  # rank 4
    with pytest.raises(ValueError):
        methods._Layout(torch.zeros(10), None, [0, 4, 10], None, torch.device("cpu"))   # packed needs (N, ny)
    with pytest.raises(TypeError):
        methods._Layout(torch.zeros(4, 2, dtype=torch.int32), None, None, torch.int32, torch.device("cpu"))


def test_mixed_sqrt_and_covariance_inputs_raise_type_error():
    # parsmooth/_base.py:25-30 via parsmooth/linearization/_sigma_points.py:64: a covariance-form
    # noise or nominal beside square-root states is a TypeError, as in the reference
    A = torch.eye(2, dtype=torch.float64)
    model = S.FunctionalModel(S.models.LinearModel(A), S.MVNStandard(torch.zeros(2, dtype=torch.float64), A))
    with pytest.raises(TypeError, match="same type"):
        methods._model_tensors(model, 2, 2, torch.float64, torch.device("cpu"))
    with pytest.raises(TypeError, match="same type"):
        methods._nominal(S.MVNStandard(torch.zeros(3, 2), torch.eye(2).expand(3, 2, 2)), None, 2)
    # the plan and the gradients take square-root inputs only, and say which entry points convert
    with pytest.raises(NotImplementedError, match="iterated_smoothing also accept MVNStandard"):
        methods._check_common(S.MVNStandard(torch.zeros(2), torch.eye(2)), True, cubature)


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the behaviour without a CUDA device")
def test_no_cpu_fallback_without_a_gpu():
    # every public entry point needs the CUDA path; none computes on the host instead
    A = torch.eye(2, dtype=torch.float64)
    noise = S.MVNSqrt(torch.zeros(2, dtype=torch.float64), A)
    tm = om = S.FunctionalModel(S.models.LinearModel(A), noise)
    x0 = S.MVNSqrt(torch.zeros(2, dtype=torch.float64), A)
    ys = torch.zeros(4, 2, dtype=torch.float64)
    with pytest.raises(RuntimeError, match="CUDA device"):
        S.filtering(ys, x0, tm, om, cubature)
    with pytest.raises(RuntimeError, match="CUDA device"):
        S.iterated_smoothing(ys, x0, tm, om, cubature, criterion=lambda i, *_: i < 2)
    with pytest.raises(RuntimeError, match="CUDA device"):
        S.filtering(ys, S.MVNStandard(x0.mean, A), S.FunctionalModel(tm.function, S.MVNStandard(noise.mean, A)),
                    S.FunctionalModel(om.function, S.MVNStandard(noise.mean, A)), cubature)
