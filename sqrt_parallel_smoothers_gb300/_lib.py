"""ctypes binding of ``libsqrtsmooth.so`` (the C ABI declared in ``include/sqrtsmooth.h``).

The library is the only compute path: if it is missing or fails to load,
every entry point raises - there is no CPU fallback.
"""
import ctypes
import os
import threading

from ._build import LIB

SS_OK, SS_ERR_INVALID, SS_ERR_UNSUPPORTED, SS_ERR_CUDA, SS_ERR_WORKSPACE = 0, 1, 2, 3, 4
SS_F32, SS_F64 = 0, 1
SS_LIN_EXTENDED, SS_LIN_CUBATURE, SS_LIN_UNSCENTED, SS_LIN_GAUSS_HERMITE = 0, 1, 2, 3
SS_MODEL_LINEAR, SS_MODEL_COORDINATED_TURN, SS_MODEL_BEARINGS, SS_MODEL_RICKER, SS_MODEL_POISSON_EXP = 0, 1, 2, 3, 4
SS_MAX_GH_ORDER = 8
SS_MAX_TANGENTS = 4
SS_OPT_PER_SEQUENCE_COVARIANCE = 1
SS_OPT_COVARIANCE_FORM = 2

EXPORTED = ("ss_version", "ss_status_string", "ss_supported", "ss_workspace_bytes", "ss_linearize",
            "ss_filter", "ss_smooth", "ss_iterated", "ss_filter_grad", "ss_filter_grad_workspace_bytes",
            "ss_iterated_grad", "ss_iterated_grad_workspace_bytes", "ss_sample", "ss_filter_adjoint",
            "ss_filter_adjoint_workspace_bytes", "ss_launch_count", "ss_profile_enable", "ss_profile_read", "ss_profile_reset")


class SSModel(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("reserved", ctypes.c_int32), ("matrix", ctypes.c_void_p),
                ("params", ctypes.c_double * 4), ("noise_mean", ctypes.c_void_p),
                ("noise_chol", ctypes.c_void_p)]


class SSProblem(ctypes.Structure):
    _fields_ = [("dtype", ctypes.c_int32), ("nx", ctypes.c_int32), ("ny", ctypes.c_int32),
                ("lin_method", ctypes.c_int32), ("ut_alpha", ctypes.c_double), ("ut_beta", ctypes.c_double),
                ("ut_kappa", ctypes.c_double), ("ut_kappa_default", ctypes.c_int32),
                ("gh_order", ctypes.c_int32), ("slr_form", ctypes.c_int32), ("chunk", ctypes.c_int32),
                ("group", ctypes.c_int32), ("options", ctypes.c_int32), ("transition", SSModel),
                ("observation", SSModel), ("batch", ctypes.c_int64), ("total_steps", ctypes.c_int64),
                ("max_len", ctypes.c_int64), ("offsets", ctypes.c_void_p)]


class SSTangents(ctypes.Structure):
    _fields_ = [("n_dir", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("trans_params", (ctypes.c_double * 4) * SS_MAX_TANGENTS),
                ("obs_params", (ctypes.c_double * 4) * SS_MAX_TANGENTS),
                ("trans_matrix", ctypes.c_void_p), ("obs_matrix", ctypes.c_void_p),
                ("trans_noise_mean", ctypes.c_void_p), ("trans_noise_chol", ctypes.c_void_p),
                ("obs_noise_mean", ctypes.c_void_p), ("obs_noise_chol", ctypes.c_void_p)]


class SSAdjoints(ctypes.Structure):
    _fields_ = [(name, ctypes.c_void_p) for name in
                ("trans_matrix", "trans_noise_mean", "trans_noise_chol", "obs_matrix", "obs_noise_mean",
                 "obs_noise_chol", "trans_params", "obs_params", "m0", "L0")]


_lock = threading.Lock()
_handle = None

P = ctypes.c_void_p
PP = ctypes.POINTER(SSProblem)


def load():
    """Load the shared library once; raise ``RuntimeError`` if it is not built."""
    global _handle
    if _handle is not None:
        return _handle
    with _lock:
        if _handle is not None:
            return _handle
        if not os.path.exists(LIB):
            raise RuntimeError(f"sqrtsmooth CUDA library not found at {LIB}; build it with "
                               "`python -c 'import __graft_entry__ as g; g.build()'`")
        lib = ctypes.CDLL(LIB)
        lib.ss_version.restype = ctypes.c_int
        lib.ss_status_string.restype = ctypes.c_char_p
        lib.ss_status_string.argtypes = [ctypes.c_int]
        lib.ss_supported.argtypes = [PP]
        lib.ss_workspace_bytes.argtypes = [PP, ctypes.POINTER(ctypes.c_size_t)]
        lib.ss_linearize.argtypes = [PP, ctypes.c_int32, ctypes.c_int64, P, P, P, P, P, P]
        lib.ss_filter.argtypes = [PP, P, P, P, ctypes.c_int32, P, P, P, P, P, P, ctypes.c_size_t, P]
        lib.ss_smooth.argtypes = [PP, P, P, P, P, P, P, P, ctypes.c_size_t, P]
        lib.ss_iterated.argtypes = [PP, P, P, P, ctypes.c_int32, P, P, ctypes.c_int32, ctypes.c_double,
                                    P, P, P, P, P, P, ctypes.c_size_t, P]
        lib.ss_filter_grad_workspace_bytes.argtypes = [PP, ctypes.POINTER(ctypes.c_size_t)]
        lib.ss_filter_grad.argtypes = [PP, ctypes.POINTER(SSTangents), P, P, P, ctypes.c_int32, P, P, P, P, P,
                                       ctypes.c_size_t, P]
        lib.ss_iterated_grad_workspace_bytes.argtypes = [PP, ctypes.POINTER(ctypes.c_size_t)]
        lib.ss_iterated_grad.argtypes = [PP, ctypes.POINTER(SSTangents), P, P, P, ctypes.c_int32, P, P,
                                         ctypes.c_int32, P, P, P, ctypes.c_size_t, P]
        lib.ss_filter_adjoint_workspace_bytes.argtypes = [PP, ctypes.POINTER(ctypes.c_size_t)]
        lib.ss_filter_adjoint.argtypes = [PP, P, P, P, ctypes.c_int32, P, P, P, ctypes.POINTER(SSAdjoints), P,
                                          ctypes.c_size_t, P]
        lib.ss_sample.argtypes = [PP, P, P, P, P, ctypes.c_int32, P, P, P, ctypes.c_size_t, P]
        lib.ss_profile_enable.argtypes = [ctypes.c_int]
        lib.ss_profile_read.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
        for name in EXPORTED:
            getattr(lib, name).restype = ctypes.c_int
        lib.ss_status_string.restype = ctypes.c_char_p
        lib.ss_launch_count.restype = ctypes.c_longlong
        _handle = lib
        return lib


class SqrtSmoothError(RuntimeError):
    """A CUDA-side failure reported by the library."""


def check(status):
    """Map a status code to the reference's exception types (TypeError/NotImplementedError/...)."""
    if status == SS_OK:
        return
    msg = load().ss_status_string(status).decode()
    if status == SS_ERR_INVALID:
        raise ValueError(msg)
    if status == SS_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    raise SqrtSmoothError(msg)


def launch_count():
    """Kernels launched by the library in this process so far."""
    return int(load().ss_launch_count())


def profile_enable(on=True):
    load().ss_profile_enable(1 if on else 0)


def profile_read():
    """``{kernel: (launches, total_ms)}`` over the events recorded while profiling."""
    import json
    buf = ctypes.create_string_buffer(1 << 16)
    check(load().ss_profile_read(buf, len(buf)))
    return {k: (int(v[0]), float(v[1])) for k, v in json.loads(buf.value.decode()).items()}


def profile_reset():
    load().ss_profile_reset()
