"""Public entry points with the signatures of ``parsmooth.methods`` (parsmooth/methods.py:14-76).

Every call runs on the current CUDA device through the C ABI of
``libsqrtsmooth.so``; each entry point is registered as a torch custom op
(``torch.ops.sqrtsmooth.*``) so that it can be captured in CUDA graphs.

Extensions over the reference:

* batches of independent sequences - ``observations`` of shape ``(B, T, ny)``
  with optional ``lengths`` (ragged, zero-padded), or packed ``(sum T_i, ny)``
  with ``offsets``; trajectories then have ``T_i + 1`` states per sequence in
  the same layout (padded ``(B, T+1, ...)`` or packed ``(sum (T_i+1), ...)``);
* the dtype of ``observations`` (float32 or float64) selects the arithmetic;
  log-likelihoods are accumulated and returned in float64.

``parallel=False`` and Python callables that are not device models raise
``NotImplementedError``; a ``ConditionalMomentsModel`` must be built from the conditional
moments of a device model (``models.PoissonExp``, ``models.population_parameters``).
"""
from typing import List, Optional, Tuple

import numpy as np
import torch

from . import _lib
from ._base import MVNSqrt, MVNStandard, FunctionalModel, ConditionalMomentsModel, are_inputs_compatible
from .linearization import resolve
from .models import as_device_model

_DT = {torch.float32: _lib.SS_F32, torch.float64: _lib.SS_F64}

# ----------------------------------------------------------------------------- criteria


class FixedIterations:
    """Criterion ``i < n``: exactly ``n`` filter-smoother calls."""

    def __init__(self, n):
        self.n = int(n)

    def __call__(self, i, *_):
        return i < self.n


class MeanSquaredChange:
    """The reference default (parsmooth/methods.py:50-51): continue while the mean squared
    change of the means exceeds ``tol``; at most ``max_iter`` calls."""

    def __init__(self, tol=1e-6, max_iter=100):
        self.tol = float(tol)
        self.max_iter = int(max_iter)

    def __call__(self, _i, prev, cur):
        return float(torch.mean((torch.as_tensor(prev.mean) - torch.as_tensor(cur.mean)) ** 2)) > self.tol


def _default_criterion(_i, nominal_traj_prev, curr_nominal_traj):
    """parsmooth/methods.py:50-51."""
    return float(torch.mean((torch.as_tensor(nominal_traj_prev.mean) -
                             torch.as_tensor(curr_nominal_traj.mean)) ** 2)) > 1e-6


def _criterion_schedule(criterion):
    """``(n_calls, tol)`` for the device loop: a count criterion or the mean-squared-change test."""
    if criterion is _default_criterion:
        return 100, 1e-6
    if isinstance(criterion, MeanSquaredChange):
        return criterion.max_iter, criterion.tol
    if isinstance(criterion, FixedIterations):
        return max(criterion.n, 1), 0.0
    n = 1
    try:
        while criterion(n, None, None):
            n += 1
            if n > 1_000_000:
                raise NotImplementedError("criterion does not terminate as a function of the count")
    except (TypeError, AttributeError) as exc:
        raise NotImplementedError(
            "criterion must depend only on the iteration count (e.g. `lambda i, *_: i < N`), "
            "or be the default mean-squared-change test") from exc
    return n, 0.0


# ----------------------------------------------------------------------------- layout helpers


def _device():
    if not torch.cuda.is_available():
        raise RuntimeError("the square-root smoother runs on a CUDA device and none is available")
    return torch.device("cuda", torch.cuda.current_device())


def _as(x, dtype, device):
    return torch.as_tensor(np.asarray(x) if not isinstance(x, torch.Tensor) else x).to(
        device=device, dtype=dtype).contiguous()


def _lower(chol):
    """Lower-triangular square root with the same ``L L^T`` (QR of ``chol^T`` when needed)."""
    c = chol.detach().to("cpu", torch.float64)
    if torch.count_nonzero(torch.triu(c, 1)) == 0:
        return chol
    r = torch.linalg.qr(c.transpose(-1, -2), mode="r")[1]
    L = r.transpose(-1, -2)
    s = torch.where(torch.diagonal(L, dim1=-2, dim2=-1) < 0, -1.0, 1.0)
    return (L * s[..., None, :]).to(chol.dtype)


class _Layout:
    """Packed-batch geometry of one call and conversions to/from the user layout."""

    def __init__(self, observations, lengths, offsets, dtype, device):
        ys = observations if isinstance(observations, torch.Tensor) else torch.as_tensor(np.asarray(observations))
        if dtype is None:
            dtype = ys.dtype if ys.dtype in _DT else torch.float32
        if dtype not in _DT:
            raise TypeError(f"unsupported dtype {dtype}")
        self.dtype, self.device = dtype, device
        if offsets is not None:
            if ys.ndim != 2:
                raise ValueError("packed observations must be (sum T_i, ny)")
            off = torch.as_tensor(offsets, dtype=torch.int64).cpu()
            self.kind = "packed"
            self.lengths = (off[1:] - off[:-1]).numpy()
            self.ys = _as(ys, dtype, device)
        elif ys.ndim == 2:
            self.kind = "single"
            self.lengths = np.array([ys.shape[0]], dtype=np.int64)
            self.ys = _as(ys, dtype, device)
        elif ys.ndim == 3:
            self.kind = "padded"
            B, Tm, _ = ys.shape
            self.lengths = (np.full(B, Tm, dtype=np.int64) if lengths is None
                            else np.asarray(torch.as_tensor(lengths).cpu(), dtype=np.int64))
            if self.lengths.shape != (B,) or (self.lengths > Tm).any() or (self.lengths < 0).any():
                raise ValueError("lengths must be (B,) with 0 <= T_i <= T")
            self.Tmax = Tm
            y = _as(ys, dtype, device)
            self.step_idx = self._index(self.lengths, Tm, 0)
            self.ys = y.reshape(B * Tm, -1).index_select(0, self.step_idx).contiguous()
            self.state_idx = self._index(self.lengths, Tm + 1, 1)
        else:
            raise ValueError("observations must be (T, ny), (B, T, ny) or packed with offsets")
        if (self.lengths < 0).any():
            raise ValueError("negative sequence length")
        self.B = int(len(self.lengths))
        self.N = int(self.lengths.sum())
        self.max_len = int(self.lengths.max()) if self.B else 0
        self.ny = int(self.ys.shape[-1])
        self.offsets = torch.as_tensor(np.concatenate([[0], np.cumsum(self.lengths)]), dtype=torch.int64,
                                       device=device)

    def _index(self, lengths, width, extra):
        idx = [np.arange(i * width, i * width + T + extra) for i, T in enumerate(lengths)]
        return torch.as_tensor(np.concatenate(idx) if idx else np.zeros(0, np.int64), device=self.device)

    def pack_states(self, x, tail):
        """User-layout trajectory -> packed ``(N + B, *tail)``."""
        x = _as(x, self.dtype, self.device)
        if self.kind == "padded":
            return x.reshape((self.B * (self.Tmax + 1),) + tail).index_select(0, self.state_idx).contiguous()
        return x.reshape((self.N + self.B,) + tail)

    def unpack_states(self, x, tail):
        if self.kind == "padded":
            out = torch.zeros((self.B * (self.Tmax + 1),) + tail, dtype=x.dtype, device=x.device)
            out.index_copy_(0, self.state_idx, x)
            return out.reshape((self.B, self.Tmax + 1) + tail)
        return x

    def per_sequence(self, v):
        return v[0] if self.kind == "single" else v


def _prior(x0, lay, nx):
    m0 = _as(x0.mean, lay.dtype, lay.device)
    L0 = _lower(_as(x0.chol, lay.dtype, lay.device))
    if m0.ndim == 1:
        return m0.reshape(1, nx), L0.reshape(1, nx, nx).contiguous(), 0
    if m0.shape[0] != lay.B:
        raise ValueError("a per-sequence prior needs one mean per sequence")
    L0 = L0.expand(lay.B, nx, nx) if L0.ndim == 2 else L0
    return m0.contiguous(), L0.contiguous(), 1


def _model_tensors(model, d_in, d_out, dtype, device, sqrt=True):
    if isinstance(model, ConditionalMomentsModel):
        from .models import conditional_owner
        fn = conditional_owner(model)
        if fn.d_out != d_out or fn.d_in != d_in:
            raise ValueError(f"{fn!r} maps R^{fn.d_in} -> R^{fn.d_out}, expected R^{d_in} -> R^{d_out}")
        qm = torch.zeros(d_out, dtype=dtype, device=device)
        qL = _as(fn.noise_chol(), dtype, device).reshape(d_out, d_out).contiguous()
        return fn, None, qm, qL
    if not isinstance(model, FunctionalModel):
        raise TypeError(f"expected a FunctionalModel, got {type(model).__name__}")
    fn = as_device_model(model.function)
    if fn.d_out != d_out or fn.d_in != d_in:
        raise ValueError(f"{fn!r} maps R^{fn.d_in} -> R^{fn.d_out}, expected R^{d_in} -> R^{d_out}")
    q = model.mvn
    if isinstance(q, MVNStandard):
        # covariance-form inputs were converted as a whole before this point, so this noise
        # sits beside square-root inputs (parsmooth/linearization/_sigma_points.py:64 raises too)
        raise TypeError(f"All inputs should have the same type: an MVNStandard noise with MVNSqrt states "
                        f"({model!r})")
    qm = _as(q.mean, dtype, device).reshape(d_out)
    qL = _lower(_as(q.chol, dtype, device)).reshape(d_out, d_out).contiguous()
    mat = fn.matrix()
    mat = None if mat is None else _as(mat, dtype, device)
    return fn, mat, qm, qL


# Bit of the slr_form slot of the integer config that selects the covariance-form kernels
# (ss_problem.options SS_OPT_COVARIANCE_FORM); the slot's low bits keep the SLR form.
_COV_FLAG = 16


def _icfg(method, nx, ny, fn_t, fn_o, lay, chunk, group, slr_form, extra, cov=False):
    p = method.params
    kappa_default = 1 if p.get("kappa", None) is None else 0
    return [nx, ny, method.code, kappa_default, int(p.get("order", 3)), int(slr_form) | (_COV_FLAG if cov else 0),
            int(chunk), int(group), fn_t.kind, fn_o.kind, lay.B, lay.N, lay.max_len] + list(extra)


def _fcfg(method, fn_t, fn_o, extra=()):
    p = method.params
    kappa = p.get("kappa", None)
    return [float(p.get("alpha", 1.0)), float(p.get("beta", 0.0)), float(0.0 if kappa is None else kappa)] + \
        [float(v) for v in fn_t.params()] + [float(v) for v in fn_o.params()] + [float(v) for v in extra]


# ----------------------------------------------------------------------------- ctypes glue

_WS = {}


def _workspace(nbytes, device):
    if torch.cuda.is_current_stream_capturing():
        # a graph keeps its own workspace, allocated from the graph's private pool
        return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)
    key = (device.index, torch.cuda.current_stream(device).cuda_stream)
    buf = _WS.get(key)
    if buf is None or buf.numel() < nbytes:
        buf = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)
        _WS[key] = buf
    return buf


def _ptr(t):
    return None if t is None else t.data_ptr()


_OPTIONS = {"per_sequence_covariance": False}


def set_large_state_options(per_sequence_covariance=False):
    """Large-state path (linear models, nx > 5): by default a batch of equally long sequences
    with one shared prior computes its common covariance recursion once and the means per
    sequence; ``per_sequence_covariance=True`` computes every sequence separately."""
    _OPTIONS["per_sequence_covariance"] = bool(per_sequence_covariance)


def _problem(icfg, fcfg, dtype, offsets, t_mat, t_qm, t_qL, o_mat, o_qm, o_qL):
    (nx, ny, code, kdef, order, slr, chunk, group, tk, ok, B, N, maxlen) = icfg[:13]
    pr = _lib.SSProblem()
    pr.options = _lib.SS_OPT_PER_SEQUENCE_COVARIANCE if _OPTIONS["per_sequence_covariance"] else 0
    if slr & _COV_FLAG:
        pr.options |= _lib.SS_OPT_COVARIANCE_FORM
    pr.dtype = _DT[dtype]
    pr.nx, pr.ny, pr.lin_method = nx, ny, code
    pr.ut_alpha, pr.ut_beta, pr.ut_kappa = fcfg[0], fcfg[1], fcfg[2]
    pr.ut_kappa_default, pr.gh_order, pr.slr_form = kdef, order, slr & ~_COV_FLAG
    pr.chunk, pr.group = chunk, group
    for mdl, kind, mat, qm, qL, par in ((pr.transition, tk, t_mat, t_qm, t_qL, fcfg[3:7]),
                                        (pr.observation, ok, o_mat, o_qm, o_qL, fcfg[7:11])):
        mdl.kind = kind
        mdl.matrix = _ptr(mat)
        for k in range(4):
            mdl.params[k] = par[k]
        mdl.noise_mean = _ptr(qm)
        mdl.noise_chol = _ptr(qL)
    pr.batch, pr.total_steps, pr.max_len = B, N, maxlen
    pr.offsets = _ptr(offsets)
    return pr


def _ws_for(pr, device):
    lib = _lib.load()
    nbytes = _lib.ctypes.c_size_t(0)
    _lib.check(lib.ss_workspace_bytes(_lib.ctypes.byref(pr), _lib.ctypes.byref(nbytes)))
    return _workspace(nbytes.value, device), nbytes.value


def _stream(device):
    return torch.cuda.current_stream(device).cuda_stream


# ----------------------------------------------------------------------------- torch ops

@torch.library.custom_op("sqrtsmooth::filter", mutates_args=())
def _filter_op(ys: torch.Tensor, offsets: torch.Tensor, m0: torch.Tensor, L0: torch.Tensor,
               nom_m: Optional[torch.Tensor], nom_L: Optional[torch.Tensor], t_mat: Optional[torch.Tensor],
               t_qm: torch.Tensor, t_qL: torch.Tensor, o_mat: Optional[torch.Tensor], o_qm: torch.Tensor,
               o_qL: torch.Tensor, icfg: List[int], fcfg: List[float]
               ) -> Tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
    nx, B, N = icfg[0], icfg[10], icfg[11]
    prior_per_seq, want_ell = icfg[13], icfg[14]
    dev = ys.device
    pr = _problem(icfg, fcfg, ys.dtype, offsets, t_mat, t_qm, t_qL, o_mat, o_qm, o_qL)
    ws, nbytes = _ws_for(pr, dev)
    out_m = torch.empty((N + B, nx), dtype=ys.dtype, device=dev)
    out_L = torch.empty((N + B, nx, nx), dtype=ys.dtype, device=dev)
    ell = torch.empty((B if want_ell else 0,), dtype=torch.float64, device=dev)
    _lib.check(_lib.load().ss_filter(_lib.ctypes.byref(pr), _ptr(ys), _ptr(m0), _ptr(L0), prior_per_seq,
                                     _ptr(nom_m), _ptr(nom_L), _ptr(out_m), _ptr(out_L),
                                     _ptr(ell) if want_ell else None, _ptr(ws), nbytes, _stream(dev)))
    return out_m, out_L, ell


@_filter_op.register_fake
def _(ys, offsets, m0, L0, nom_m, nom_L, t_mat, t_qm, t_qL, o_mat, o_qm, o_qL, icfg, fcfg):
    nx, B, N = icfg[0], icfg[10], icfg[11]
    return (ys.new_empty((N + B, nx)), ys.new_empty((N + B, nx, nx)),
            ys.new_empty((B if icfg[14] else 0,), dtype=torch.float64))


@torch.library.custom_op("sqrtsmooth::smooth", mutates_args=())
def _smooth_op(filt_m: torch.Tensor, filt_L: torch.Tensor, offsets: torch.Tensor, nom_m: Optional[torch.Tensor],
               nom_L: Optional[torch.Tensor], t_mat: Optional[torch.Tensor], t_qm: torch.Tensor,
               t_qL: torch.Tensor, o_mat: Optional[torch.Tensor], o_qm: torch.Tensor, o_qL: torch.Tensor,
               icfg: List[int], fcfg: List[float]) -> Tuple[torch.Tensor, torch.Tensor]:
    dev = filt_m.device
    pr = _problem(icfg, fcfg, filt_m.dtype, offsets, t_mat, t_qm, t_qL, o_mat, o_qm, o_qL)
    ws, nbytes = _ws_for(pr, dev)
    out_m = torch.empty_like(filt_m)
    out_L = torch.empty_like(filt_L)
    _lib.check(_lib.load().ss_smooth(_lib.ctypes.byref(pr), _ptr(filt_m), _ptr(filt_L), _ptr(nom_m),
                                     _ptr(nom_L), _ptr(out_m), _ptr(out_L), _ptr(ws), nbytes, _stream(dev)))
    return out_m, out_L


@_smooth_op.register_fake
def _(filt_m, filt_L, offsets, nom_m, nom_L, t_mat, t_qm, t_qL, o_mat, o_qm, o_qL, icfg, fcfg):
    return torch.empty_like(filt_m), torch.empty_like(filt_L)


@torch.library.custom_op("sqrtsmooth::sample", mutates_args=())
def _sample_op(filt_m: torch.Tensor, filt_L: torch.Tensor, offsets: torch.Tensor, nom_m: Optional[torch.Tensor],
               nom_L: Optional[torch.Tensor], t_mat: Optional[torch.Tensor], t_qm: torch.Tensor,
               t_qL: torch.Tensor, o_mat: Optional[torch.Tensor], o_qm: torch.Tensor, o_qL: torch.Tensor,
               eps: torch.Tensor, icfg: List[int], fcfg: List[float]) -> torch.Tensor:
    dev = filt_m.device
    pr = _problem(icfg, fcfg, filt_m.dtype, offsets, t_mat, t_qm, t_qL, o_mat, o_qm, o_qL)
    ws, nbytes = _ws_for(pr, dev)
    out = torch.empty_like(eps)
    _lib.check(_lib.load().ss_sample(_lib.ctypes.byref(pr), _ptr(filt_m), _ptr(filt_L), _ptr(nom_m), _ptr(nom_L),
                                     int(eps.shape[1]), _ptr(eps), _ptr(out), _ptr(ws), nbytes, _stream(dev)))
    return out


@_sample_op.register_fake
def _(filt_m, filt_L, offsets, nom_m, nom_L, t_mat, t_qm, t_qL, o_mat, o_qm, o_qL, eps, icfg, fcfg):
    return torch.empty_like(eps)


@torch.library.custom_op("sqrtsmooth::iterated", mutates_args=())
def _iterated_op(ys: torch.Tensor, offsets: torch.Tensor, m0: torch.Tensor, L0: torch.Tensor,
                 init_m: Optional[torch.Tensor], init_L: Optional[torch.Tensor], t_mat: Optional[torch.Tensor],
                 t_qm: torch.Tensor, t_qL: torch.Tensor, o_mat: Optional[torch.Tensor], o_qm: torch.Tensor,
                 o_qL: torch.Tensor, icfg: List[int], fcfg: List[float]
                 ) -> Tuple[torch.Tensor, torch.Tensor, torch.Tensor, torch.Tensor, torch.Tensor]:
    nx, B, N = icfg[0], icfg[10], icfg[11]
    prior_per_seq, want_ell, n_iter = icfg[13], icfg[14], icfg[15]
    tol = fcfg[11]
    dev = ys.device
    pr = _problem(icfg, fcfg, ys.dtype, offsets, t_mat, t_qm, t_qL, o_mat, o_qm, o_qL)
    ws, nbytes = _ws_for(pr, dev)
    out_m = torch.empty((N + B, nx), dtype=ys.dtype, device=dev)
    out_L = torch.empty((N + B, nx, nx), dtype=ys.dtype, device=dev)
    ell = torch.empty((B if want_ell else 0,), dtype=torch.float64, device=dev)
    iters = torch.empty((B,), dtype=torch.int32, device=dev)
    flags = torch.empty((B,), dtype=torch.int32, device=dev)
    _lib.check(_lib.load().ss_iterated(_lib.ctypes.byref(pr), _ptr(ys), _ptr(m0), _ptr(L0), prior_per_seq,
                                       _ptr(init_m), _ptr(init_L), n_iter, tol, _ptr(out_m), _ptr(out_L),
                                       _ptr(ell) if want_ell else None, _ptr(iters), _ptr(flags), _ptr(ws),
                                       nbytes, _stream(dev)))
    return out_m, out_L, ell, iters, flags


@_iterated_op.register_fake
def _(ys, offsets, m0, L0, init_m, init_L, t_mat, t_qm, t_qL, o_mat, o_qm, o_qL, icfg, fcfg):
    nx, B, N = icfg[0], icfg[10], icfg[11]
    return (ys.new_empty((N + B, nx)), ys.new_empty((N + B, nx, nx)),
            ys.new_empty((B if icfg[14] else 0,), dtype=torch.float64),
            ys.new_empty((B,), dtype=torch.int32), ys.new_empty((B,), dtype=torch.int32))


@torch.library.custom_op("sqrtsmooth::linearize", mutates_args=())
def _linearize_op(m: torch.Tensor, L: torch.Tensor, offsets: torch.Tensor, t_mat: Optional[torch.Tensor],
                  t_qm: torch.Tensor, t_qL: torch.Tensor, o_mat: Optional[torch.Tensor], o_qm: torch.Tensor,
                  o_qL: torch.Tensor, icfg: List[int], fcfg: List[float], which: int
                  ) -> Tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
    nx, ny = icfg[0], icfg[1]
    d_out = nx if which == 0 else ny
    n = m.shape[0]
    dev = m.device
    pr = _problem(icfg, fcfg, m.dtype, offsets, t_mat, t_qm, t_qL, o_mat, o_qm, o_qL)
    F = torch.empty((n, d_out, nx), dtype=m.dtype, device=dev)
    chol = torch.empty((n, d_out, d_out), dtype=m.dtype, device=dev)
    b = torch.empty((n, d_out), dtype=m.dtype, device=dev)
    _lib.check(_lib.load().ss_linearize(_lib.ctypes.byref(pr), which, n, _ptr(m), _ptr(L), _ptr(F), _ptr(chol),
                                        _ptr(b), _stream(dev)))
    return F, chol, b


@_linearize_op.register_fake
def _(m, L, offsets, t_mat, t_qm, t_qL, o_mat, o_qm, o_qL, icfg, fcfg, which):
    nx, ny = icfg[0], icfg[1]
    d_out = nx if which == 0 else ny
    n = m.shape[0]
    return m.new_empty((n, d_out, nx)), m.new_empty((n, d_out, d_out)), m.new_empty((n, d_out))


@torch.library.custom_op("sqrtsmooth::filter_grad", mutates_args=())
def _filter_grad_op(ys: torch.Tensor, offsets: torch.Tensor, m0: torch.Tensor, L0: torch.Tensor,
                    nom_m: Optional[torch.Tensor], nom_L: Optional[torch.Tensor], t_mat: Optional[torch.Tensor],
                    t_qm: torch.Tensor, t_qL: torch.Tensor, o_mat: Optional[torch.Tensor], o_qm: torch.Tensor,
                    o_qL: torch.Tensor, d_tmat: Optional[torch.Tensor], d_omat: Optional[torch.Tensor],
                    d_tqm: Optional[torch.Tensor], d_tqL: Optional[torch.Tensor], d_oqm: Optional[torch.Tensor],
                    d_oqL: Optional[torch.Tensor], d_params: List[float], icfg: List[int], fcfg: List[float]
                    ) -> Tuple[torch.Tensor, torch.Tensor]:
    B, n_dir, per = icfg[10], icfg[14], icfg[13]
    n_iter = icfg[15] if len(icfg) > 15 else 0
    dev = ys.device
    pr = _problem(icfg, fcfg, ys.dtype, offsets, t_mat, t_qm, t_qL, o_mat, o_qm, o_qL)
    lib = _lib.load()
    nbytes = _lib.ctypes.c_size_t(0)
    ws_query = lib.ss_iterated_grad_workspace_bytes if n_iter > 0 else lib.ss_filter_grad_workspace_bytes
    _lib.check(ws_query(_lib.ctypes.byref(pr), _lib.ctypes.byref(nbytes)))
    ws = _workspace(nbytes.value, dev)
    tg = _lib.SSTangents()
    tg.n_dir = n_dir
    for d in range(n_dir):
        for k in range(4):
            tg.trans_params[d][k] = d_params[d * 8 + k]
            tg.obs_params[d][k] = d_params[d * 8 + 4 + k]
    tg.trans_matrix, tg.obs_matrix = _ptr(d_tmat), _ptr(d_omat)
    tg.trans_noise_mean, tg.trans_noise_chol = _ptr(d_tqm), _ptr(d_tqL)
    tg.obs_noise_mean, tg.obs_noise_chol = _ptr(d_oqm), _ptr(d_oqL)
    ell = torch.empty((B,), dtype=torch.float64, device=dev)
    grad = torch.empty((B, n_dir), dtype=torch.float64, device=dev)
    if n_iter > 0:
        _lib.check(lib.ss_iterated_grad(_lib.ctypes.byref(pr), _lib.ctypes.byref(tg), _ptr(ys), _ptr(m0), _ptr(L0),
                                        per, _ptr(nom_m), _ptr(nom_L), n_iter, _ptr(ell), _ptr(grad), _ptr(ws),
                                        nbytes.value, _stream(dev)))
    else:
        _lib.check(lib.ss_filter_grad(_lib.ctypes.byref(pr), _lib.ctypes.byref(tg), _ptr(ys), _ptr(m0), _ptr(L0),
                                      per, _ptr(nom_m), _ptr(nom_L), _ptr(ell), _ptr(grad), _ptr(ws), nbytes.value,
                                      _stream(dev)))
    return ell, grad


@_filter_grad_op.register_fake
def _(ys, offsets, m0, L0, nom_m, nom_L, t_mat, t_qm, t_qL, o_mat, o_qm, o_qL, d_tmat, d_omat, d_tqm, d_tqL,
      d_oqm, d_oqL, d_params, icfg, fcfg):
    B, n_dir = icfg[10], icfg[14]
    return ys.new_empty((B,), dtype=torch.float64), ys.new_empty((B, n_dir), dtype=torch.float64)


# Outputs of ss_filter_adjoint in ss_adjoints order, with their per-sequence shapes.
ADJOINT_KEYS = ("trans_matrix", "trans_noise_mean", "trans_noise_chol", "obs_matrix", "obs_noise_mean",
                "obs_noise_chol", "trans_params", "obs_params", "m0", "L0")


def _adjoint_shapes(nx, ny):
    return ((nx, nx), (nx,), (nx, nx), (ny, nx), (ny,), (ny, ny), (4,), (4,), (nx,), (nx, nx))


@torch.library.custom_op("sqrtsmooth::filter_adjoint", mutates_args=())
def _filter_adjoint_op(ys: torch.Tensor, offsets: torch.Tensor, m0: torch.Tensor, L0: torch.Tensor,
                       nom_m: Optional[torch.Tensor], nom_L: Optional[torch.Tensor], t_mat: Optional[torch.Tensor],
                       t_qm: torch.Tensor, t_qL: torch.Tensor, o_mat: Optional[torch.Tensor], o_qm: torch.Tensor,
                       o_qL: torch.Tensor, icfg: List[int], fcfg: List[float]) -> List[torch.Tensor]:
    nx, ny, B, per, want_params = icfg[0], icfg[1], icfg[10], icfg[13], icfg[14]
    dev = ys.device
    pr = _problem(icfg, fcfg, ys.dtype, offsets, t_mat, t_qm, t_qL, o_mat, o_qm, o_qL)
    lib = _lib.load()
    nbytes = _lib.ctypes.c_size_t(0)
    _lib.check(lib.ss_filter_adjoint_workspace_bytes(_lib.ctypes.byref(pr), _lib.ctypes.byref(nbytes)))
    ws = _workspace(nbytes.value, dev)
    ell = torch.empty((B,), dtype=torch.float64, device=dev)
    outs = [torch.zeros((B,) + s, dtype=torch.float64, device=dev) for s in _adjoint_shapes(nx, ny)]
    adj = _lib.SSAdjoints()
    for key, t in zip(ADJOINT_KEYS, outs):
        if key in ("trans_params", "obs_params") and not want_params:
            continue
        setattr(adj, key, _ptr(t))
    _lib.check(lib.ss_filter_adjoint(_lib.ctypes.byref(pr), _ptr(ys), _ptr(m0), _ptr(L0), per, _ptr(nom_m),
                                     _ptr(nom_L), _ptr(ell), _lib.ctypes.byref(adj), _ptr(ws), nbytes.value,
                                     _stream(dev)))
    return [ell] + outs


@_filter_adjoint_op.register_fake
def _(ys, offsets, m0, L0, nom_m, nom_L, t_mat, t_qm, t_qL, o_mat, o_qm, o_qL, icfg, fcfg):
    nx, ny, B = icfg[0], icfg[1], icfg[10]
    return [ys.new_empty((B,), dtype=torch.float64)] + \
        [ys.new_empty((B,) + s, dtype=torch.float64) for s in _adjoint_shapes(nx, ny)]


# ----------------------------------------------------------------------------- public API

def _factor(P):
    """Lower-triangular L with L L^T = P (batched), non-negative diagonal.  Cholesky where it
    succeeds; a positive semi-definite P whose Cholesky fails is factored through its
    eigendecomposition and a QR, i.e. tria(V sqrt(w))."""
    P = P if isinstance(P, torch.Tensor) else torch.as_tensor(P)
    L, info = torch.linalg.cholesky_ex(P)
    if bool((info != 0).any()):
        w, V = torch.linalg.eigh(0.5 * (P + P.transpose(-1, -2)))
        Sq = V * w.clamp_min(0).sqrt().unsqueeze(-2)
        L = torch.linalg.qr(Sq.transpose(-1, -2), mode="r").R.transpose(-1, -2)
        sg = torch.sign(torch.diagonal(L, dim1=-2, dim2=-1))
        L = L * torch.where(sg == 0, torch.ones_like(sg), sg).unsqueeze(-2)
    return L


def _std_to_sqrt(x):
    return None if x is None else MVNSqrt(x.mean, _factor(x.cov))


def _sqrt_to_std(x):
    L = x.chol
    return MVNStandard(x.mean, L @ L.transpose(-1, -2))


def _model_to_sqrt(model):
    if isinstance(model, FunctionalModel) and isinstance(model.mvn, MVNStandard):
        return FunctionalModel(model.function, _std_to_sqrt(model.mvn))
    return model


# Covariance-form ("standard") inputs: by default they run the reference's covariance-form
# operators on the GPU (csrc/ss_std.cuh); covariance_form="factored" factors them instead and runs
# the square-root kernels (results returned as covariances).
_COV_FORMS = ("operators", "factored")


def _cov_form(covariance_form):
    if covariance_form not in _COV_FORMS:
        raise ValueError(f"covariance_form must be one of {_COV_FORMS}, got {covariance_form!r}")
    return covariance_form == "operators"


def _model_tensors_std(model, d_in, d_out, dtype, device):
    """Device model with its noise mean and covariance (covariance-form kernels)."""
    if isinstance(model, ConditionalMomentsModel):
        # the device model's constant noise enters as its covariance (conditional observation
        # models compute theirs per point in the kernel and ignore it)
        fn, mat, qm, qL = _model_tensors(model, d_in, d_out, dtype, device)
        return fn, mat, qm, (qL @ qL.transpose(-1, -2)).contiguous()
    if not isinstance(model, FunctionalModel):
        raise TypeError(f"expected a FunctionalModel, got {type(model).__name__}")
    fn = as_device_model(model.function)
    if fn.d_out != d_out or fn.d_in != d_in:
        raise ValueError(f"{fn!r} maps R^{fn.d_in} -> R^{fn.d_out}, expected R^{d_in} -> R^{d_out}")
    q = model.mvn
    if not isinstance(q, MVNStandard):
        raise TypeError(f"All inputs should have the same type: an MVNSqrt noise with MVNStandard states ({model!r})")
    qm = _as(q.mean, dtype, device).reshape(d_out)
    Q = _as(q.cov, dtype, device).reshape(d_out, d_out).contiguous()
    mat = fn.matrix()
    mat = None if mat is None else _as(mat, dtype, device)
    return fn, mat, qm, Q


def _prior_std(x0, lay, nx):
    m0 = _as(x0.mean, lay.dtype, lay.device)
    P0 = _as(x0.cov, lay.dtype, lay.device)
    if m0.ndim == 1:
        return m0.reshape(1, nx), P0.reshape(1, nx, nx).contiguous(), 0
    if m0.shape[0] != lay.B:
        raise ValueError("a per-sequence prior needs one mean per sequence")
    P0 = P0.expand(lay.B, nx, nx) if P0.ndim == 2 else P0
    return m0.contiguous(), P0.contiguous(), 1


def _nominal_std(nominal, lay, nx):
    if nominal is None:
        return None, None
    if not isinstance(nominal, MVNStandard):
        raise TypeError("All inputs should have the same type: an MVNSqrt nominal trajectory with an "
                        "MVNStandard prior")
    return lay.pack_states(nominal.mean, (nx,)), lay.pack_states(nominal.cov, (nx, nx)).contiguous()


def _check_common(x0, parallel, method):
    if not parallel:
        raise NotImplementedError("only parallel=True is implemented on the GPU")
    if isinstance(x0, MVNStandard):
        raise NotImplementedError("this entry point takes square-root (MVNSqrt) inputs; filtering, smoothing, "
                                  "sampling and iterated_smoothing also accept MVNStandard")
    if not isinstance(x0, MVNSqrt):
        raise TypeError(f"x0 must be an MVNSqrt, got {type(x0).__name__}")
    return resolve(method)


def _nominal(nominal, lay, nx):
    if nominal is None:
        return None, None
    if isinstance(nominal, MVNStandard):
        raise TypeError("All inputs should have the same type: an MVNStandard nominal trajectory with an "
                        "MVNSqrt prior")
    m = lay.pack_states(nominal.mean, (nx,))
    L = lay.pack_states(nominal.chol, (nx, nx))
    return m, _lower_batched(L)


def _lower_batched(L):
    if torch.count_nonzero(torch.triu(L, 1)) == 0:
        return L.contiguous()
    return _lower(L).to(L.device).contiguous()


def _dummy_observation(nx, dtype, device, ny=1):
    from .models import LinearModel
    fn = LinearModel(torch.zeros(ny, nx))
    return fn, _as(fn.A, dtype, device), torch.zeros(ny, dtype=dtype, device=device), \
        torch.eye(ny, dtype=dtype, device=device)


def _dummy_ny(nx, fn=None):
    """Observation size of the placeholder model when a transition is linearised alone: 1,
    except for linear transitions at the large-state sizes, whose compiled kernels pair nx with
    ny = nx / 2."""
    linear = fn is None or getattr(fn, "kind", None) == _lib.SS_MODEL_LINEAR
    return nx // 2 if (linear and nx in (8, 32)) else 1


def filtering(observations, x0, transition_model, observation_model, linearization_method,
              nominal_trajectory=None, parallel=True, return_loglikelihood=False, *, lengths=None,
              offsets=None, chunk=0, group=0, slr_form=0, covariance_form="operators"):
    """Parallel square-root filter (parsmooth/methods.py:14-26 -> parsmooth/parallel/_filtering.py:13-61).

    Covariance-form inputs (``MVNStandard`` prior, nominal and model noises) run the reference's
    standard filter: its covariance-form linearisation, elements and combine
    (parsmooth/parallel/_filtering.py:64-97, parsmooth/parallel/_operators.py:7-40) in CUDA
    kernels.  ``covariance_form="factored"`` instead factors the covariances (torch, where the
    tensors live), runs the square-root kernels and returns covariances."""
    if isinstance(x0, MVNStandard):
        if nominal_trajectory is not None:
            are_inputs_compatible(x0, nominal_trajectory)
        if _cov_form(covariance_form):
            return _filtering_std(observations, x0, transition_model, observation_model, linearization_method,
                                  nominal_trajectory, parallel, return_loglikelihood, lengths, offsets, chunk, group)
        out = filtering(observations, _std_to_sqrt(x0), _model_to_sqrt(transition_model),
                        _model_to_sqrt(observation_model), linearization_method, _std_to_sqrt(nominal_trajectory),
                        parallel, return_loglikelihood, lengths=lengths, offsets=offsets, chunk=chunk, group=group,
                        slr_form=slr_form)
        if return_loglikelihood:
            return _sqrt_to_std(out[0]), out[1]
        return _sqrt_to_std(out)
    method = _check_common(x0, parallel, linearization_method)
    if nominal_trajectory is not None:
        are_inputs_compatible(x0, nominal_trajectory)
    dev = _device()
    lay = _Layout(observations, lengths, offsets, None, dev)
    nx = int(torch.as_tensor(x0.mean).shape[-1])
    fn_t, t_mat, t_qm, t_qL = _model_tensors(transition_model, nx, nx, lay.dtype, dev)
    fn_o, o_mat, o_qm, o_qL = _model_tensors(observation_model, nx, lay.ny, lay.dtype, dev)
    m0, L0, per = _prior(x0, lay, nx)
    nm, nL = _nominal(nominal_trajectory, lay, nx)
    icfg = _icfg(method, nx, lay.ny, fn_t, fn_o, lay, chunk, group, slr_form,
                 [per, int(bool(return_loglikelihood))])
    out_m, out_L, ell = torch.ops.sqrtsmooth.filter(lay.ys, lay.offsets, m0, L0, nm, nL, t_mat, t_qm, t_qL,
                                                    o_mat, o_qm, o_qL, icfg, _fcfg(method, fn_t, fn_o))
    res = MVNSqrt(lay.unpack_states(out_m, (nx,)), lay.unpack_states(out_L, (nx, nx)))
    if return_loglikelihood:
        return res, lay.per_sequence(ell)
    return res


def _filtering_std(observations, x0, transition_model, observation_model, linearization_method, nominal_trajectory,
                   parallel, return_loglikelihood, lengths, offsets, chunk, group):
    """The covariance-form filter on the GPU (ss_filter with SS_OPT_COVARIANCE_FORM)."""
    if not parallel:
        raise NotImplementedError("only parallel=True is implemented on the GPU")
    method = resolve(linearization_method)
    dev = _device()
    lay = _Layout(observations, lengths, offsets, None, dev)
    nx = int(torch.as_tensor(x0.mean).shape[-1])
    fn_t, t_mat, t_qm, t_Q = _model_tensors_std(transition_model, nx, nx, lay.dtype, dev)
    fn_o, o_mat, o_qm, o_Q = _model_tensors_std(observation_model, nx, lay.ny, lay.dtype, dev)
    m0, P0, per = _prior_std(x0, lay, nx)
    nm, nP = _nominal_std(nominal_trajectory, lay, nx)
    icfg = _icfg(method, nx, lay.ny, fn_t, fn_o, lay, chunk, group, 0, [per, int(bool(return_loglikelihood))],
                 cov=True)
    out_m, out_P, ell = torch.ops.sqrtsmooth.filter(lay.ys, lay.offsets, m0, P0, nm, nP, t_mat, t_qm, t_Q,
                                                    o_mat, o_qm, o_Q, icfg, _fcfg(method, fn_t, fn_o))
    res = MVNStandard(lay.unpack_states(out_m, (nx,)), lay.unpack_states(out_P, (nx, nx)))
    if return_loglikelihood:
        return res, lay.per_sequence(ell)
    return res


def _smooth_layout(fm, lengths, offsets, dtype, dev):
    """Batch geometry from a trajectory's shape (T+1 states per sequence)."""
    if offsets is not None:
        off = torch.as_tensor(offsets, dtype=torch.int64)
        return _Layout(torch.zeros((int(off[-1]), 1), dtype=dtype), None, off, dtype, dev)
    if fm.ndim == 2:
        return _Layout(torch.zeros((fm.shape[0] - 1, 1), dtype=dtype), None, None, dtype, dev)
    B, Tp1 = fm.shape[:2]
    return _Layout(torch.zeros((B, Tp1 - 1, 1), dtype=dtype), lengths, None, dtype, dev)


def _smoothing_std(transition_model, filter_trajectory, linearization_method, nominal_trajectory, parallel,
                   lengths, offsets, chunk, group):
    """The covariance-form smoother on the GPU (ss_smooth with SS_OPT_COVARIANCE_FORM)."""
    if not parallel:
        raise NotImplementedError("only parallel=True is implemented on the GPU")
    method = resolve(linearization_method)
    dev = _device()
    fm = filter_trajectory.mean if isinstance(filter_trajectory.mean, torch.Tensor) else \
        torch.as_tensor(filter_trajectory.mean)
    nx = int(fm.shape[-1])
    dtype = fm.dtype if fm.dtype in _DT else torch.float32
    lay = _smooth_layout(fm, lengths, offsets, dtype, dev)
    fn_t, t_mat, t_qm, t_Q = _model_tensors_std(transition_model, nx, nx, lay.dtype, dev)
    ny = _dummy_ny(nx, fn_t)
    fn_o, o_mat, o_qm, o_Q = _dummy_observation(nx, lay.dtype, dev, ny)
    fmp = lay.pack_states(filter_trajectory.mean, (nx,))
    fPp = lay.pack_states(filter_trajectory.cov, (nx, nx)).contiguous()
    nm, nP = _nominal_std(nominal_trajectory, lay, nx)
    icfg = _icfg(method, nx, ny, fn_t, fn_o, lay, chunk, group, 0, [0, 0], cov=True)
    out_m, out_P = torch.ops.sqrtsmooth.smooth(fmp, fPp, lay.offsets, nm, nP, t_mat, t_qm, t_Q, o_mat, o_qm,
                                               o_Q, icfg, _fcfg(method, fn_t, fn_o))
    return MVNStandard(lay.unpack_states(out_m, (nx,)), lay.unpack_states(out_P, (nx, nx)))


def smoothing(transition_model, filter_trajectory, linearization_method, nominal_trajectory=None,
              parallel=True, *, lengths=None, offsets=None, chunk=0, group=0, slr_form=0,
              covariance_form="operators"):
    """Parallel square-root RTS smoother (parsmooth/methods.py:29-35 -> parsmooth/parallel/_smoothing.py:14-44).

    For batches pass ``lengths`` (padded trajectories ``(B, T+1, ...)``) or
    ``offsets`` (packed trajectories, offsets of the steps).  A covariance-form filtered
    trajectory runs the reference's standard smoother (parsmooth/parallel/_smoothing.py:60-69,
    parsmooth/parallel/_operators.py:80-101) unless ``covariance_form="factored"``."""
    if isinstance(filter_trajectory, MVNStandard):
        if nominal_trajectory is not None:
            are_inputs_compatible(filter_trajectory, nominal_trajectory)
        if _cov_form(covariance_form):
            return _smoothing_std(transition_model, filter_trajectory, linearization_method, nominal_trajectory,
                                  parallel, lengths, offsets, chunk, group)
        return _sqrt_to_std(smoothing(_model_to_sqrt(transition_model), _std_to_sqrt(filter_trajectory),
                                      linearization_method, _std_to_sqrt(nominal_trajectory), parallel,
                                      lengths=lengths, offsets=offsets, chunk=chunk, group=group,
                                      slr_form=slr_form))
    method = _check_common(filter_trajectory, parallel, linearization_method)
    if nominal_trajectory is not None:
        are_inputs_compatible(filter_trajectory, nominal_trajectory)
    dev = _device()
    fm = torch.as_tensor(filter_trajectory.mean) if not isinstance(filter_trajectory.mean, torch.Tensor) \
        else filter_trajectory.mean
    nx = int(fm.shape[-1])
    dtype = fm.dtype if fm.dtype in _DT else torch.float32
    # geometry from the trajectory shape: T+1 states per sequence
    if offsets is not None:
        off = torch.as_tensor(offsets, dtype=torch.int64)
        n_steps = int(off[-1])
        fake = torch.zeros((n_steps, 1), dtype=dtype)
        lay = _Layout(fake, None, off, dtype, dev)
    elif fm.ndim == 2:
        lay = _Layout(torch.zeros((fm.shape[0] - 1, 1), dtype=dtype), None, None, dtype, dev)
    else:
        B, Tp1 = fm.shape[:2]
        lay = _Layout(torch.zeros((B, Tp1 - 1, 1), dtype=dtype), lengths, None, dtype, dev)
    fn_t, t_mat, t_qm, t_qL = _model_tensors(transition_model, nx, nx, lay.dtype, dev)
    ny = _dummy_ny(nx, fn_t)
    fn_o, o_mat, o_qm, o_qL = _dummy_observation(nx, lay.dtype, dev, ny)
    fmp = lay.pack_states(filter_trajectory.mean, (nx,))
    fLp = _lower_batched(lay.pack_states(filter_trajectory.chol, (nx, nx)))
    nm, nL = _nominal(nominal_trajectory, lay, nx)
    icfg = _icfg(method, nx, ny, fn_t, fn_o, lay, chunk, group, slr_form, [0, 0])
    out_m, out_L = torch.ops.sqrtsmooth.smooth(fmp, fLp, lay.offsets, nm, nL, t_mat, t_qm, t_qL, o_mat, o_qm,
                                               o_qL, icfg, _fcfg(method, fn_t, fn_o))
    return MVNSqrt(lay.unpack_states(out_m, (nx,)), lay.unpack_states(out_L, (nx, nx)))


def sampling(key, n_samples, transition_model, filter_trajectory, linearization_method, nominal_trajectory=None,
             parallel=True, *, lengths=None, offsets=None, eps=None, chunk=0, group=0, slr_form=0):
    """Pathwise posterior sampler (parsmooth/methods.py:79-91, parsmooth/_pathwise_sampler.py:13-127).

    Returns ``n_samples`` trajectories drawn from the smoothing posterior given the filtered
    trajectory: ``(T+1, n_samples, nx)`` (or ``(B, T+1, n_samples, nx)`` for padded batches,
    packed ``(sum (T_i+1), n_samples, nx)`` with ``offsets``).  ``key`` seeds the draws (an int
    or a ``torch.Generator``); ``eps`` may instead give the standard normals in the
    reference's order, shape ``(T+1, n_samples, nx)`` with ``eps[0]`` driving the last state
    and ``eps[1 + t]`` step t (per sequence for batches).  The default nominal is the smoothed
    trajectory, as in the reference.  The draws run on the GPU, one thread per (sequence,
    sample) walking its trajectory backwards; ``parallel`` selects nothing (both of the
    reference's forms give the same draws)."""
    if isinstance(filter_trajectory, MVNStandard):
        if nominal_trajectory is not None:
            are_inputs_compatible(filter_trajectory, nominal_trajectory)
        return sampling(key, n_samples, _model_to_sqrt(transition_model), _std_to_sqrt(filter_trajectory),
                        linearization_method, _std_to_sqrt(nominal_trajectory), parallel, lengths=lengths,
                        offsets=offsets, eps=eps, chunk=chunk, group=group, slr_form=slr_form)
    if nominal_trajectory is None:
        nominal_trajectory = smoothing(transition_model, filter_trajectory, linearization_method, None, parallel,
                                       lengths=lengths, offsets=offsets, chunk=chunk, group=group,
                                       slr_form=slr_form)
    method = _check_common(filter_trajectory, True, linearization_method)
    are_inputs_compatible(filter_trajectory, nominal_trajectory)
    fm = filter_trajectory.mean if isinstance(filter_trajectory.mean, torch.Tensor) else \
        torch.as_tensor(filter_trajectory.mean)
    dtype = fm.dtype if fm.dtype in _DT else torch.float32
    dev = _device()
    nx = int(fm.shape[-1])
    if offsets is not None:
        off = torch.as_tensor(offsets, dtype=torch.int64)
        lay = _Layout(torch.zeros((int(off[-1]), 1), dtype=dtype), None, off, dtype, dev)
    elif fm.ndim == 2:
        lay = _Layout(torch.zeros((fm.shape[0] - 1, 1), dtype=dtype), None, None, dtype, dev)
    else:
        B, Tp1 = fm.shape[:2]
        lay = _Layout(torch.zeros((B, Tp1 - 1, 1), dtype=dtype), lengths, None, dtype, dev)
    fn_t, t_mat, t_qm, t_qL = _model_tensors(transition_model, nx, nx, lay.dtype, dev)
    ny = _dummy_ny(nx, fn_t)
    fn_o, o_mat, o_qm, o_qL = _dummy_observation(nx, lay.dtype, dev, ny)
    fmp = lay.pack_states(filter_trajectory.mean, (nx,))
    fLp = _lower_batched(lay.pack_states(filter_trajectory.chol, (nx, nx)))
    nm, nL = _nominal(nominal_trajectory, lay, nx)
    n_samples = int(n_samples)
    if eps is None:
        gen = key if isinstance(key, torch.Generator) else torch.Generator(device=dev).manual_seed(int(key))
        e = torch.randn((fmp.shape[0], n_samples, nx), generator=gen, dtype=lay.dtype, device=dev)
    else:
        # reference order per sequence (eps[0] last state, eps[1 + t] step t) -> state order
        # (eps[t] step t, eps[T] last): state t of sequence i takes entry (t + 1) mod (T_i + 1)
        e = lay.pack_states(torch.as_tensor(eps), (n_samples, nx))
        off = lay.offsets.to(dev)
        n_st = off[1:] - off[:-1] + 1
        s0 = off[:-1] + torch.arange(off.shape[0] - 1, device=dev)
        seq = torch.repeat_interleave(torch.arange(n_st.shape[0], device=dev), n_st)
        t_in = torch.arange(e.shape[0], device=dev) - s0[seq]
        e = e.index_select(0, s0[seq] + (t_in + 1) % n_st[seq]).contiguous()
    icfg = _icfg(method, nx, ny, fn_t, fn_o, lay, chunk, group, slr_form, [0, 0])
    out = torch.ops.sqrtsmooth.sample(fmp, fLp, lay.offsets, nm, nL, t_mat, t_qm, t_qL, o_mat, o_qm, o_qL, e,
                                      icfg, _fcfg(method, fn_t, fn_o))
    return lay.unpack_states(out, (n_samples, nx))


def filter_smoother(observations, x0, transition_model, observation_model, linearization_method,
                    nominal_trajectory=None, parallel=True, **kw):
    """parsmooth/methods.py:38-47."""
    filt = filtering(observations, x0, transition_model, observation_model, linearization_method,
                     nominal_trajectory, parallel, **kw)
    kw = {k: v for k, v in kw.items() if k in ("lengths", "offsets", "chunk", "group", "slr_form",
                                               "covariance_form")}
    return smoothing(transition_model, filt, linearization_method, nominal_trajectory, parallel, **kw)


def iterated_smoothing(observations, x0, transition_model, observation_model, linearization_method,
                       init_nominal_trajectory=None, parallel=True, criterion=_default_criterion,
                       return_loglikelihood=False, *, lengths=None, offsets=None, chunk=0, group=0,
                       slr_form=0, return_info=False, covariance_form="operators"):
    """Iterated square-root smoother (parsmooth/methods.py:54-76), the whole loop on the device.

    ``criterion`` may be a count test such as ``lambda i, *_: i < N`` (exactly
    ``N`` filter-smoother calls), the default mean-squared-change test, or
    :class:`MeanSquaredChange` / :class:`FixedIterations`.  With
    ``return_info=True`` a dict with per-sequence ``iterations`` and status
    ``flags`` (1 non-finite output, 2 non-finite log-likelihood, 4 not
    converged) is returned last.  Covariance-form inputs run the reference's covariance-form
    filter and smoother in every call, or (``covariance_form="factored"``) are factored and the
    result returned as covariances (see :func:`filtering`)."""
    if isinstance(x0, MVNStandard):
        if init_nominal_trajectory is not None:
            are_inputs_compatible(x0, init_nominal_trajectory)
        if _cov_form(covariance_form):
            return _iterated_std(observations, x0, transition_model, observation_model, linearization_method,
                                 init_nominal_trajectory, parallel, criterion, return_loglikelihood, lengths,
                                 offsets, chunk, group, return_info)
        out = iterated_smoothing(observations, _std_to_sqrt(x0), _model_to_sqrt(transition_model),
                                 _model_to_sqrt(observation_model), linearization_method,
                                 _std_to_sqrt(init_nominal_trajectory), parallel, criterion, return_loglikelihood,
                                 lengths=lengths, offsets=offsets, chunk=chunk, group=group, slr_form=slr_form,
                                 return_info=return_info)
        if isinstance(out, MVNSqrt):   # MVNSqrt is itself a tuple: test it first
            return _sqrt_to_std(out)
        return (_sqrt_to_std(out[0]),) + tuple(out[1:])
    method = _check_common(x0, parallel, linearization_method)
    if init_nominal_trajectory is not None:
        are_inputs_compatible(x0, init_nominal_trajectory)
    n_calls, tol = _criterion_schedule(criterion)
    dev = _device()
    lay = _Layout(observations, lengths, offsets, None, dev)
    nx = int(torch.as_tensor(x0.mean).shape[-1])
    fn_t, t_mat, t_qm, t_qL = _model_tensors(transition_model, nx, nx, lay.dtype, dev)
    fn_o, o_mat, o_qm, o_qL = _model_tensors(observation_model, nx, lay.ny, lay.dtype, dev)
    m0, L0, per = _prior(x0, lay, nx)
    im, iL = _nominal(init_nominal_trajectory, lay, nx)
    icfg = _icfg(method, nx, lay.ny, fn_t, fn_o, lay, chunk, group, slr_form,
                 [per, int(bool(return_loglikelihood)), n_calls])
    fcfg = _fcfg(method, fn_t, fn_o, [tol])
    out_m, out_L, ell, iters, flags = torch.ops.sqrtsmooth.iterated(lay.ys, lay.offsets, m0, L0, im, iL, t_mat,
                                                                    t_qm, t_qL, o_mat, o_qm, o_qL, icfg, fcfg)
    res = MVNSqrt(lay.unpack_states(out_m, (nx,)), lay.unpack_states(out_L, (nx, nx)))
    out = (res,)
    if return_loglikelihood:
        out += (lay.per_sequence(ell),)
    if return_info:
        out += ({"iterations": lay.per_sequence(iters), "flags": lay.per_sequence(flags)},)
    return out[0] if len(out) == 1 else out


def _iterated_std(observations, x0, transition_model, observation_model, linearization_method,
                  init_nominal_trajectory, parallel, criterion, return_loglikelihood, lengths, offsets, chunk,
                  group, return_info):
    """The covariance-form iterated smoother on the GPU (ss_iterated with SS_OPT_COVARIANCE_FORM)."""
    if not parallel:
        raise NotImplementedError("only parallel=True is implemented on the GPU")
    method = resolve(linearization_method)
    n_calls, tol = _criterion_schedule(criterion)
    dev = _device()
    lay = _Layout(observations, lengths, offsets, None, dev)
    nx = int(torch.as_tensor(x0.mean).shape[-1])
    fn_t, t_mat, t_qm, t_Q = _model_tensors_std(transition_model, nx, nx, lay.dtype, dev)
    fn_o, o_mat, o_qm, o_Q = _model_tensors_std(observation_model, nx, lay.ny, lay.dtype, dev)
    m0, P0, per = _prior_std(x0, lay, nx)
    im, iP = _nominal_std(init_nominal_trajectory, lay, nx)
    icfg = _icfg(method, nx, lay.ny, fn_t, fn_o, lay, chunk, group, 0,
                 [per, int(bool(return_loglikelihood)), n_calls], cov=True)
    fcfg = _fcfg(method, fn_t, fn_o, [tol])
    out_m, out_P, ell, iters, flags = torch.ops.sqrtsmooth.iterated(lay.ys, lay.offsets, m0, P0, im, iP, t_mat,
                                                                    t_qm, t_Q, o_mat, o_qm, o_Q, icfg, fcfg)
    out = (MVNStandard(lay.unpack_states(out_m, (nx,)), lay.unpack_states(out_P, (nx, nx))),)
    if return_loglikelihood:
        out += (lay.per_sequence(ell),)
    if return_info:
        out += ({"iterations": lay.per_sequence(iters), "flags": lay.per_sequence(flags)},)
    return out[0] if len(out) == 1 else out


def linearize(model, x, method, *, covariance_form="operators"):
    """Linearise ``model`` at ``x`` (one point or a batch) with ``method`` on the GPU.

    Equivalent of ``method(model, x)`` in parsmooth/linearization/*.py.  For a covariance-form
    ``x`` (``MVNStandard``) the result is ``(F, Q, b)`` with ``Q`` a covariance: the reference's
    covariance-form regression (parsmooth/linearization/_sigma_points.py:39-60, 81-86) in a
    CUDA kernel, or (``covariance_form="factored"``) the square-root regression squared."""
    if isinstance(x, MVNStandard):
        if not _cov_form(covariance_form):
            F, L, b = linearize(_model_to_sqrt(model), _std_to_sqrt(x), method)
            return F, L @ L.transpose(-1, -2), b
        return _linearize_std(model, x, method)
    method = resolve(method)
    dev = _device()
    m = torch.as_tensor(x.mean) if not isinstance(x.mean, torch.Tensor) else x.mean
    dtype = m.dtype if m.dtype in _DT else torch.float32
    single = m.ndim == 1
    nx = int(m.shape[-1])
    mm = _as(m, dtype, dev).reshape(-1, nx)
    LL = _lower_batched(_as(x.chol, dtype, dev).reshape(-1, nx, nx))
    if isinstance(model, ConditionalMomentsModel):
        from .models import conditional_owner
        fn = conditional_owner(model)
    else:
        fn = as_device_model(model.function)
    d_out = fn.d_out
    is_obs = not (d_out == nx and fn.kind not in (_lib.SS_MODEL_BEARINGS, _lib.SS_MODEL_POISSON_EXP))
    fnm, mat, qm, qL = _model_tensors(model, nx, d_out, dtype, dev)
    if is_obs:
        fn_t, t_mat, t_qm, t_qL = _dummy_transition(nx, dtype, dev)
        o = (fnm, mat, qm, qL)
        ny = d_out
    else:
        fn_t, t_mat, t_qm, t_qL = fnm, mat, qm, qL
        ny = _dummy_ny(nx, fnm)
        o = _dummy_observation(nx, dtype, dev, ny)
    lay_off = torch.zeros(2, dtype=torch.int64, device=dev)

    class _L:
        B, N, max_len = 1, 0, 0

    icfg = _icfg(method, nx, ny, fn_t, o[0], _L, 0, 0, 0, [])
    F, chol, b = torch.ops.sqrtsmooth.linearize(mm, LL, lay_off, t_mat, t_qm, t_qL, o[1], o[2], o[3], icfg,
                                                _fcfg(method, fn_t, o[0]), 1 if is_obs else 0)
    if single:
        return F[0], chol[0], b[0]
    return F.reshape(m.shape[:-1] + F.shape[1:]), chol.reshape(m.shape[:-1] + chol.shape[1:]), \
        b.reshape(m.shape[:-1] + b.shape[1:])


def _linearize_std(model, x, method):
    """Covariance-form linearisation on the GPU (ss_linearize with SS_OPT_COVARIANCE_FORM)."""
    method = resolve(method)
    dev = _device()
    m = torch.as_tensor(x.mean) if not isinstance(x.mean, torch.Tensor) else x.mean
    dtype = m.dtype if m.dtype in _DT else torch.float32
    single = m.ndim == 1
    nx = int(m.shape[-1])
    mm = _as(m, dtype, dev).reshape(-1, nx)
    PP = _as(x.cov, dtype, dev).reshape(-1, nx, nx).contiguous()
    if isinstance(model, ConditionalMomentsModel):
        from .models import conditional_owner
        fn = conditional_owner(model)
    else:
        fn = as_device_model(model.function)
    d_out = fn.d_out
    is_obs = not (d_out == nx and fn.kind not in (_lib.SS_MODEL_BEARINGS, _lib.SS_MODEL_POISSON_EXP))
    fnm, mat, qm, Q = _model_tensors_std(model, nx, d_out, dtype, dev)
    if is_obs:
        fn_t, t_mat, t_qm, t_Q = _dummy_transition(nx, dtype, dev)
        o = (fnm, mat, qm, Q)
        ny = d_out
    else:
        fn_t, t_mat, t_qm, t_Q = fnm, mat, qm, Q
        ny = _dummy_ny(nx, fnm)
        o = _dummy_observation(nx, dtype, dev, ny)
    lay_off = torch.zeros(2, dtype=torch.int64, device=dev)

    class _L:
        B, N, max_len = 1, 0, 0

    icfg = _icfg(method, nx, ny, fn_t, o[0], _L, 0, 0, 0, [], cov=True)
    F, cov_out, b = torch.ops.sqrtsmooth.linearize(mm, PP, lay_off, t_mat, t_qm, t_Q, o[1], o[2], o[3], icfg,
                                                   _fcfg(method, fn_t, o[0]), 1 if is_obs else 0)
    if single:
        return F[0], cov_out[0], b[0]
    return F.reshape(m.shape[:-1] + F.shape[1:]), cov_out.reshape(m.shape[:-1] + cov_out.shape[1:]), \
        b.reshape(m.shape[:-1] + b.shape[1:])


def _dummy_transition(nx, dtype, device):
    from .models import LinearModel
    fn = LinearModel(torch.eye(nx))
    return fn, _as(fn.A, dtype, device), torch.zeros(nx, dtype=dtype, device=device), \
        torch.eye(nx, dtype=dtype, device=device)


# ----------------------------------------------------------------------------- graph-replayed plans

def _group_cuts(lengths, k):
    """Sequence boundaries [0 = c_0 < c_1 < ... = B] of at most k contiguous groups with about
    equal numbers of steps, every group holding at least one step (when any sequence has one)."""
    lengths = np.asarray(lengths, dtype=np.int64)
    B = len(lengths)
    off = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64)
    k = max(1, min(int(k), B))
    cuts = [0]
    for g in range(1, k):
        c = int(np.searchsorted(off, g * off[-1] / k))
        cuts.append(max(cuts[-1] + 1, min(c, B - (k - g))))
    cuts.append(B)
    cuts = [c for i, c in enumerate(cuts) if i == 0 or off[c] > off[cuts[i - 1]] or c == B]
    if len(cuts) > 2 and off[cuts[-1]] == off[cuts[-2]]:
        del cuts[-2]
    return cuts


class IteratedSmootherPlan:
    """An iterated smoother staged once and replayed as a CUDA graph.

    Arguments are those of :func:`iterated_smoothing`.  Construction packs
    and uploads every input, runs the smoother once (workspace allocation,
    warm-up) and captures the whole N-iteration loop - every kernel of every
    iteration - into one CUDA graph.  :meth:`run` replays it on the current
    stream; :meth:`set_observations` refreshes the observations in place (same
    shapes) and :meth:`run_host` does copy-in, replay and copy-out from and to
    host buffers.  Results live in :attr:`mean` / :attr:`chol` (packed
    ``(sum (T_i+1), nx)`` layout) and :attr:`ell` (when requested).  With
    ``profile=True`` every captured kernel is bracketed by CUDA events that
    each replay re-records; ``_lib.profile_read()`` returns the last replay's
    per-kernel times (call ``_lib.profile_reset()`` only after the plan is gone).

    ``streams=k`` (k > 1, with ``graph=True``) cuts the batch into k contiguous
    groups of sequences with about equal step counts and captures each group's
    loop on its own stream of the same graph: the groups are independent, so
    one group's per-step kernels fill the GPU while another is in its scan
    levels (a few hundred threads each).  Each group has its own workspace and
    writes its slice of the shared outputs."""

    def __init__(self, observations, x0, transition_model, observation_model, linearization_method,
                 init_nominal_trajectory=None, criterion=_default_criterion, return_loglikelihood=False, *,
                 lengths=None, offsets=None, chunk=0, group=0, slr_form=0, graph=True, profile=False,
                 streams=1):
        self._ctor = ((observations, x0, transition_model, observation_model, linearization_method,
                       init_nominal_trajectory, criterion, return_loglikelihood),
                      dict(lengths=lengths, offsets=offsets, chunk=chunk, group=group, slr_form=slr_form,
                           graph=graph, profile=False, streams=streams))
        self._twin_plan, self._copy_stream, self._flip = None, None, 0
        method = _check_common(x0, True, linearization_method)
        if init_nominal_trajectory is not None:
            are_inputs_compatible(x0, init_nominal_trajectory)
        n_calls, tol = _criterion_schedule(criterion)
        dev = _device()
        lay = _Layout(observations, lengths, offsets, None, dev)
        nx = int(torch.as_tensor(x0.mean).shape[-1])
        fn_t, t_mat, t_qm, t_qL = _model_tensors(transition_model, nx, nx, lay.dtype, dev)
        fn_o, o_mat, o_qm, o_qL = _model_tensors(observation_model, nx, lay.ny, lay.dtype, dev)
        m0, L0, per = _prior(x0, lay, nx)
        im, iL = _nominal(init_nominal_trajectory, lay, nx)
        icfg = _icfg(method, nx, lay.ny, fn_t, fn_o, lay, chunk, group, slr_form,
                     [per, int(bool(return_loglikelihood)), n_calls])
        fcfg = _fcfg(method, fn_t, fn_o, [tol])
        self.layout, self.nx = lay, nx
        self._args = (lay.ys, lay.offsets, m0, L0, im, iL, t_mat, t_qm, t_qL, o_mat, o_qm, o_qL, icfg, fcfg)
        self.steps = lay.N
        self.graph = None
        if graph and streams > 1 and lay.B > 1:
            self._build_grouped(int(streams), profile)
            return
        stream = torch.cuda.Stream(dev)
        stream.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(stream):
            self._outs = _iterated_op(*self._args)      # warm-up, allocates the cached workspace
            if graph:
                n0 = _lib.launch_count()
                self._outs = _iterated_op(*self._args)
                self.launches_per_run = _lib.launch_count() - n0
                g = torch.cuda.CUDAGraph()
                if profile:
                    # per-kernel CUDA events recorded by every replay (read with _lib.profile_read)
                    _lib.profile_reset()
                    _lib.profile_enable(True)
                try:
                    with torch.cuda.graph(g, stream=stream):
                        self._outs = _iterated_op(*self._args)
                finally:
                    if profile:
                        _lib.profile_enable(False)
                self.graph = g
        torch.cuda.current_stream(dev).wait_stream(stream)
        torch.cuda.synchronize(dev)

    def _build_grouped(self, k, profile):
        """Concurrent sequence groups (see the class docstring)."""
        (ys, offsets, m0, L0, im, iL, t_mat, t_qm, t_qL, o_mat, o_qm, o_qL, icfg, fcfg) = self._args
        lay, nx, dev = self.layout, self.nx, ys.device
        off = np.concatenate([[0], np.cumsum(lay.lengths)]).astype(np.int64)
        cuts = _group_cuts(lay.lengths, k)
        per, want_ell, n_iter, tol = icfg[13], icfg[14], icfg[15], fcfg[11]
        N, B = lay.N, lay.B
        out_m = torch.empty((N + B, nx), dtype=ys.dtype, device=dev)
        out_L = torch.empty((N + B, nx, nx), dtype=ys.dtype, device=dev)
        ell = torch.empty((B if want_ell else 0,), dtype=torch.float64, device=dev)
        iters = torch.empty((B,), dtype=torch.int32, device=dev)
        flags = torch.empty((B,), dtype=torch.int32, device=dev)
        self._outs = (out_m, out_L, ell, iters, flags)
        lib = _lib.load()
        calls = []
        for a, b in zip(cuts[:-1], cuts[1:]):
            s0, s1 = int(off[a]) + a, int(off[b]) + b          # state rows of the group
            lens = lay.lengths[a:b]
            og = torch.as_tensor(off[a:b + 1] - off[a], dtype=torch.int64, device=dev)
            cfg = list(icfg)
            cfg[10], cfg[11], cfg[12] = b - a, int(lens.sum()), int(lens.max())
            pr = _problem(cfg, fcfg, ys.dtype, og, t_mat, t_qm, t_qL, o_mat, o_qm, o_qL)
            nbytes = _lib.ctypes.c_size_t(0)
            _lib.check(lib.ss_workspace_bytes(_lib.ctypes.byref(pr), _lib.ctypes.byref(nbytes)))
            ws = torch.empty(max(int(nbytes.value), 256), dtype=torch.uint8, device=dev)
            gm0, gL0 = (m0[a:b], L0[a:b]) if per else (m0, L0)
            gim, giL = (im[s0:s1], iL[s0:s1]) if im is not None else (None, None)
            calls.append(dict(pr=pr, og=og, ws=ws, nbytes=nbytes.value, ys=ys[int(off[a]):int(off[b])],
                              m0=gm0, L0=gL0, im=gim, iL=giL, m=out_m[s0:s1], L=out_L[s0:s1],
                              ell=ell[a:b] if want_ell else None, iters=iters[a:b], flags=flags[a:b],
                              stream=torch.cuda.Stream(dev)))
        self._groups = calls

        def launch(main):
            for c in calls:
                c["stream"].wait_stream(main)
                _lib.check(lib.ss_iterated(_lib.ctypes.byref(c["pr"]), _ptr(c["ys"]), _ptr(c["m0"]), _ptr(c["L0"]),
                                           per, _ptr(c["im"]), _ptr(c["iL"]), n_iter, tol, _ptr(c["m"]),
                                           _ptr(c["L"]), _ptr(c["ell"]), _ptr(c["iters"]), _ptr(c["flags"]),
                                           _ptr(c["ws"]), c["nbytes"], c["stream"].cuda_stream))
            for c in calls:
                main.wait_stream(c["stream"])

        stream = torch.cuda.Stream(dev)
        stream.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(stream):
            launch(stream)                      # warm-up
            n0 = _lib.launch_count()
            launch(stream)
            self.launches_per_run = _lib.launch_count() - n0
            g = torch.cuda.CUDAGraph()
            if profile:
                _lib.profile_reset()
                _lib.profile_enable(True)
            try:
                with torch.cuda.graph(g, stream=stream):
                    launch(stream)
            finally:
                if profile:
                    _lib.profile_enable(False)
            self.graph = g
        torch.cuda.current_stream(dev).wait_stream(stream)
        torch.cuda.synchronize(dev)

    @property
    def mean(self):
        return self._outs[0]

    @property
    def chol(self):
        return self._outs[1]

    @property
    def ell(self):
        return self._outs[2]

    def run(self):
        """Replay the captured loop (or run it directly when built with ``graph=False``)."""
        if self.graph is not None:
            self.graph.replay()
        else:
            self._outs = _iterated_op(*self._args)
        return self._outs

    def set_observations(self, ys_packed, non_blocking=True):
        """Copy new packed observations ``(sum T_i, ny)`` into the staged buffer."""
        self._args[0].copy_(ys_packed, non_blocking=non_blocking)

    def run_host(self, ys_host, out_mean_host, out_chol_host=None, pipelined=False):
        """Host -> device copy of ``ys_host``, replay, device -> host copy of the results.

        With ``pipelined=True`` calls alternate between this plan and a twin
        (its own outputs and workspace, built at the first such call) and the
        copy-out runs on a separate stream, so one call's device-to-host copy
        overlaps the next call's smoother.  The host buffers are complete once
        :meth:`sync_host` has been called (or the copy stream synchronised).
        Pipelined results are delivered only to the host buffers: :attr:`mean`
        and :attr:`chol` hold this plan's own last replay, not the twin's."""
        if not pipelined:
            self.set_observations(ys_host)
            self.run()
            out_mean_host.copy_(self.mean, non_blocking=True)
            if out_chol_host is not None:
                out_chol_host.copy_(self.chol, non_blocking=True)
            return out_mean_host, out_chol_host
        dev = self._args[0].device
        if self._copy_stream is None:
            self._copy_stream = torch.cuda.Stream(dev)
            self._events = [(torch.cuda.Event(), torch.cuda.Event()) for _ in range(2)]
        if self._flip == 1 and self._twin_plan is None:
            args, kw = self._ctor
            self._twin_plan = IteratedSmootherPlan(*args, **kw)
        plan = self if self._flip == 0 else self._twin_plan
        done, copied = self._events[self._flip]
        main = torch.cuda.current_stream(dev)
        main.wait_event(copied)          # this plan's outputs of two calls ago have been read
        plan.set_observations(ys_host)
        plan.run()
        done.record(main)
        self._copy_stream.wait_event(done)
        with torch.cuda.stream(self._copy_stream):
            out_mean_host.copy_(plan.mean, non_blocking=True)
            if out_chol_host is not None:
                out_chol_host.copy_(plan.chol, non_blocking=True)
        copied.record(self._copy_stream)
        self._flip ^= 1
        return out_mean_host, out_chol_host

    def sync_host(self):
        """Make the current stream wait for the pipelined copy-outs."""
        if self._copy_stream is not None:
            torch.cuda.current_stream(self._args[0].device).wait_stream(self._copy_stream)

    def result(self):
        """The smoothed trajectory in the caller's layout."""
        lay, nx = self.layout, self.nx
        return MVNSqrt(lay.unpack_states(self.mean, (nx,)), lay.unpack_states(self.chol, (nx, nx)))


# ----------------------------------------------------------------------------- gradients

class ModelTangent:
    """Derivative of one model's scalars with respect to one parameter direction.

    ``params``: d(model params)/dtheta (``dt`` of CoordinatedTurn, ``(s1x, s1y, s2x, s2y)`` of
    Bearings); ``matrix``: d A/dtheta of a LinearModel; ``noise_mean`` / ``noise_chol``: derivative
    of the noise mean and (lower) square root.  Missing entries are zero."""

    def __init__(self, params=None, matrix=None, noise_mean=None, noise_chol=None):
        self.params = list(params) if params is not None else [0.0] * 4
        self.params += [0.0] * (4 - len(self.params))
        self.matrix, self.noise_mean, self.noise_chol = matrix, noise_mean, noise_chol


def filter_loglikelihood_grad(observations, x0, transition_model, observation_model, linearization_method,
                              nominal_trajectory, directions, *, lengths=None, offsets=None, chunk=0, group=0,
                              slr_form=0, n_iter=0):
    """Log-likelihood of the parallel filter and its derivatives along parameter directions.

    ``directions``: list (at most 4) of ``(transition ModelTangent, observation ModelTangent)``.
    The filter (parsmooth/parallel/_filtering.py:13-61, return_loglikelihood) runs in
    tangent-linear arithmetic, one pass per direction, on the GPU.  Returns ``(ell, grad)``
    (FP64), ``grad[..., k] = d ell / d theta_k``; per sequence for batches.

    With ``n_iter > 0`` the function is instead the log-likelihood of the iterated smoother
    (``iterated_smoothing(..., init_nominal_trajectory=nominal_trajectory, criterion=i < n_iter,
    return_loglikelihood=True)``, parsmooth/methods.py:54-76): the whole loop runs in
    tangent-linear arithmetic, so the nominal's dependence on the parameters is included (the
    derivative parameter estimation takes through the fixed point, parsmooth/_utils.py:113-133)."""
    method = _check_common(x0, True, linearization_method)
    if nominal_trajectory is not None:
        are_inputs_compatible(x0, nominal_trajectory)
    n_dir = len(directions)
    if not 1 <= n_dir <= _lib.SS_MAX_TANGENTS:
        raise ValueError(f"1..{_lib.SS_MAX_TANGENTS} directions are supported")
    dev = _device()
    lay = _Layout(observations, lengths, offsets, None, dev)
    nx = int(torch.as_tensor(x0.mean).shape[-1])
    fn_t, t_mat, t_qm, t_qL = _model_tensors(transition_model, nx, nx, lay.dtype, dev)
    fn_o, o_mat, o_qm, o_qL = _model_tensors(observation_model, nx, lay.ny, lay.dtype, dev)
    m0, L0, per = _prior(x0, lay, nx)
    nm, nL = _nominal(nominal_trajectory, lay, nx)

    def stack(get, shape):
        vals = [get(d) for d in directions]
        if all(v is None for v in vals):
            return None
        return torch.stack([torch.zeros(shape, dtype=lay.dtype, device=dev) if v is None
                            else _as(v, lay.dtype, dev).reshape(shape) for v in vals]).contiguous()

    ny = lay.ny
    d_tmat = stack(lambda d: d[0].matrix, (nx, nx))
    d_omat = stack(lambda d: d[1].matrix, (ny, nx))
    d_tqm = stack(lambda d: d[0].noise_mean, (nx,))
    d_tqL = stack(lambda d: d[0].noise_chol, (nx, nx))
    d_oqm = stack(lambda d: d[1].noise_mean, (ny,))
    d_oqL = stack(lambda d: d[1].noise_chol, (ny, ny))
    d_params = []
    for d in directions:
        d_params += [float(v) for v in d[0].params] + [float(v) for v in d[1].params]
    icfg = _icfg(method, nx, ny, fn_t, fn_o, lay, chunk, group, slr_form, [per, n_dir, int(n_iter)])
    ell, grad = torch.ops.sqrtsmooth.filter_grad(lay.ys, lay.offsets, m0, L0, nm, nL, t_mat, t_qm, t_qL, o_mat,
                                                 o_qm, o_qL, d_tmat, d_omat, d_tqm, d_tqL, d_oqm, d_oqL, d_params,
                                                 icfg, _fcfg(method, fn_t, fn_o))
    return lay.per_sequence(ell), lay.per_sequence(grad)


class BearingsLogLikelihood(torch.autograd.Function):
    """Pseudo-log-likelihood of the bearings model as a differentiable function of
    ``theta = (s1x, s1y, log q, log sigma)``.

    ``Q(q) = q * Q1`` (``Q1`` the coordinated-turn noise at q = 1) and ``R = sigma^2 I``; the
    second sensor, the prior and the nominal trajectory are fixed.  The forward pass runs the
    GPU filter in tangent-linear arithmetic and keeps ``d ell / d theta``; backward is the
    vector-Jacobian product.  ``ell`` is summed over the batch.  With ``n_iter > 0`` the
    log-likelihood is the iterated smoother's after ``n_iter`` calls from ``nominal`` (the
    pseudo-log-likelihood of the reference's parameter estimation), differentiated through
    the iterations.  ``mode="reverse"`` (``n_iter = 0`` only) takes the gradient from one
    reverse pass instead (:func:`filter_loglikelihood_adjoint`)."""

    @staticmethod
    def forward(ctx, theta, observations, x0, nominal, Q1, dt, s2, method, lengths, offsets, n_iter=0,
                mode="tangent"):
        from .models import Bearings, CoordinatedTurn
        th = theta.detach().double().cpu()
        s1 = (float(th[0]), float(th[1]))
        q, sigma = float(torch.exp(th[2])), float(torch.exp(th[3]))
        cQ = torch.linalg.cholesky(torch.as_tensor(Q1, dtype=torch.float64) * q)
        cR = sigma * torch.eye(2, dtype=torch.float64)
        tm = FunctionalModel(CoordinatedTurn(dt), MVNSqrt(torch.zeros(5, dtype=torch.float64), cQ))
        om = FunctionalModel(Bearings(s1, s2), MVNSqrt(torch.zeros(2, dtype=torch.float64), cR))
        if mode == "reverse":
            if n_iter:
                raise ValueError("the reverse pass differentiates the filter at a fixed nominal (n_iter = 0)")
            ell, adj = filter_loglikelihood_adjoint(observations, x0, tm, om, method, nominal, lengths=lengths,
                                                    offsets=offsets)
            dev = adj["obs_params"].device
            op = adj["obs_params"].reshape(-1, 4).sum(0)
            gq = (adj["trans_noise_chol"].reshape(-1, 5, 5).sum(0) * (0.5 * cQ).to(dev)).sum()
            gr = (adj["obs_noise_chol"].reshape(-1, 2, 2).sum(0) * cR.to(dev)).sum()
            grad = torch.stack([op[0], op[1], gq, gr])
        elif mode == "tangent":
            dirs = [(ModelTangent(), ModelTangent(params=[1, 0, 0, 0])),
                    (ModelTangent(), ModelTangent(params=[0, 1, 0, 0])),
                    (ModelTangent(noise_chol=0.5 * cQ), ModelTangent()),
                    (ModelTangent(), ModelTangent(noise_chol=cR))]
            ell, grad = filter_loglikelihood_grad(observations, x0, tm, om, method, nominal, dirs, lengths=lengths,
                                                  offsets=offsets, n_iter=n_iter)
            grad = grad.reshape(-1, 4).sum(0)
        else:
            raise ValueError(f"mode must be 'tangent' or 'reverse', got {mode!r}")
        ctx.save_for_backward(grad.to(device=theta.device, dtype=theta.dtype))
        return ell.sum().to(device=theta.device, dtype=theta.dtype)

    @staticmethod
    def backward(ctx, grad_out):
        (g,) = ctx.saved_tensors
        return (grad_out * g.to(grad_out.device),) + (None,) * 11


def filter_loglikelihood_adjoint(observations, x0, transition_model, observation_model, linearization_method,
                                 nominal_trajectory=None, *, lengths=None, offsets=None, chunk=0, group=0,
                                 slr_form=0, model_params=None):
    """Log-likelihood of the parallel filter and its gradient with respect to every input, from
    one reverse pass (``ss_filter_adjoint``).

    The reference obtains these by ``jax.grad`` through its parallel filter
    (parsmooth/parallel/_filtering.py:13-61 with ``return_loglikelihood``).  Here the filter and
    the smoother's backward scan run once at the given nominal, and the gradient comes from the
    smoothed moments of the linearised model (Fisher's identity), so the cost does not depend
    on how many parameters are differentiated.  Returns ``(ell, adj)``: ``adj`` maps each of
    ``ADJOINT_KEYS`` to ``d ell / d (that input)`` in FP64, per sequence for batches:
    ``trans_matrix`` / ``obs_matrix`` (linear models), the noise means, the noise square roots
    (lower triangles, as the library reads them), ``trans_params`` / ``obs_params`` (the device
    models' scalars: coordinated-turn ``dt``, bearings sensor coordinates, Ricker ``a``), and the
    prior's ``m0`` / ``L0`` (with a shared prior each sequence's share).  ``model_params``:
    compute the model-scalar gradients (default: unless the method is Gauss-Hermite, which the
    dual-number chain does not cover)."""
    method = _check_common(x0, True, linearization_method)
    if nominal_trajectory is not None:
        are_inputs_compatible(x0, nominal_trajectory)
    if model_params is None:
        model_params = method.code != _lib.SS_LIN_GAUSS_HERMITE
    dev = _device()
    lay = _Layout(observations, lengths, offsets, None, dev)
    nx = int(torch.as_tensor(x0.mean).shape[-1])
    fn_t, t_mat, t_qm, t_qL = _model_tensors(transition_model, nx, nx, lay.dtype, dev)
    fn_o, o_mat, o_qm, o_qL = _model_tensors(observation_model, nx, lay.ny, lay.dtype, dev)
    m0, L0, per = _prior(x0, lay, nx)
    nm, nL = _nominal(nominal_trajectory, lay, nx)
    icfg = _icfg(method, nx, lay.ny, fn_t, fn_o, lay, chunk, group, slr_form, [per, int(bool(model_params))])
    res = torch.ops.sqrtsmooth.filter_adjoint(lay.ys, lay.offsets, m0, L0, nm, nL, t_mat, t_qm, t_qL, o_mat, o_qm,
                                              o_qL, icfg, _fcfg(method, fn_t, fn_o))
    adj = {k: lay.per_sequence(v) for k, v in zip(ADJOINT_KEYS, res[1:])}
    if not model_params:
        del adj["trans_params"], adj["obs_params"]
    return lay.per_sequence(res[0]), adj


class LinearGaussianLogLikelihood(torch.autograd.Function):
    """Log-likelihood of the parallel square-root filter for a linear-Gaussian model,
    ``ell(F, L_Q, b, H, L_R, c, m0, L0)`` summed over the batch, differentiable in all eight
    arrays at once: the forward pass runs :func:`filter_loglikelihood_adjoint` (one filter,
    one smoother scan, one contraction) and backward scales the stored gradients.

    ``x_t = F x_{t-1} + b + N(0, L_Q L_Q^T)``, ``y_t = H x_t + c + N(0, L_R L_R^T)``,
    ``x_0 ~ N(m0, L0 L0^T)`` (``m0`` (nx,) shared or (B, nx) per sequence); the square roots are
    read as lower triangles.  ``observations``, ``lengths``, ``offsets`` as in
    :func:`filtering`."""

    @staticmethod
    def forward(ctx, F, Lq, b, H, Lr, c, m0, L0, observations, lengths=None, offsets=None):
        from .models import LinearModel
        from .linearization import extended
        d = lambda t: t.detach()
        tm = FunctionalModel(LinearModel(d(F)), MVNSqrt(d(b), d(Lq)))
        om = FunctionalModel(LinearModel(d(H)), MVNSqrt(d(c), d(Lr)))
        ell, adj = filter_loglikelihood_adjoint(observations, MVNSqrt(d(m0), d(L0)), tm, om, extended, None,
                                                lengths=lengths, offsets=offsets, model_params=False)
        batched = ell.ndim == 1

        def total(key, like):
            g = adj[key]
            if batched and g.ndim == like.ndim + 1:
                g = g.sum(0)
            return g.to(device=like.device, dtype=like.dtype).reshape(like.shape)

        grads = [total("trans_matrix", F), total("trans_noise_chol", Lq), total("trans_noise_mean", b),
                 total("obs_matrix", H), total("obs_noise_chol", Lr), total("obs_noise_mean", c),
                 total("m0", m0), total("L0", L0)]
        ctx.save_for_backward(*grads)
        return ell.sum().to(device=F.device, dtype=F.dtype)

    @staticmethod
    def backward(ctx, grad_out):
        return tuple(grad_out.to(g.device) * g for g in ctx.saved_tensors) + (None,) * 3
