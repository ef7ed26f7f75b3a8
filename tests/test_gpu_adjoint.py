"""Reverse-mode gradient of the filter log-likelihood (ss_filter_adjoint) on the GPU, against
the oracle's restatement (smoothed moments contracted per step, FP64; itself checked against
central differences of the oracle's log-likelihood in test_oracle_adjoint.py), against the
tangent-linear path, and through the torch.autograd.Function interfaces.

Tolerances: FP64 1e-9 relative to the largest entry (the same arithmetic in another order),
widened to 4 cond(c)^2 eps where a random noise or prior factor c is ill-conditioned (every
contraction solves with c twice), and 1e-8 on the bearings model (its process noise factor has
entries of 1e-4, so rounding differences of the two linearisations are amplified by Q^-1);
FP32 5e-3 on short sequences and 1e-2 on the config of the reference's parameter-estimation
study at B = 64, T = 5000, against FP64 finite differences."""
import numpy as np
import pytest
import torch

import oracle as O
from oracle import adjoint as OA
from oracle import models as OM
import sqrt_parallel_smoothers_gb300 as S
from sqrt_parallel_smoothers_gb300 import models as GM
from tests._parity import assert_rel, linear_pair, np_
from tests._systems import lgssm

pytestmark = pytest.mark.gpu

DIMS = [(1, 1), (2, 1), (2, 2), (3, 3), (4, 2), (5, 2), (5, 3)]


def _linear_case(nx, ny, T, seed):
    s = lgssm(nx, ny, T, seed=seed)
    return s, s["ys"].astype(np.float64)


@pytest.mark.parametrize("nx,ny", DIMS)
def test_linear_adjoints_fp64_vs_oracle(nx, ny):
    s, ys = _linear_case(nx, ny, 30, seed=3 * nx + ny)
    ot, gt = linear_pair(s["F"], s["b"], s["cholQ"])
    oo, go = linear_pair(s["H"], s["c"], s["cholR"])
    x0o = O.MVNSqrt(s["chol_x0"].mean, s["chol_x0"].chol)
    ell_ref, adj = OA.filter_adjoint(ys, x0o, ot, oo, O.linearization.extended)
    ref = OA.linear_model_adjoints(adj, s["cholQ"], s["cholR"])
    x0 = S.MVNSqrt(torch.as_tensor(x0o.mean), torch.as_tensor(x0o.chol))
    ell, got = S.filter_loglikelihood_adjoint(torch.as_tensor(ys), x0, gt, go, S.linearization.extended)
    assert abs(float(ell) - ell_ref) <= 1e-10 * max(1.0, abs(ell_ref))
    cond = max(np.linalg.cond(c) for c in (s["cholQ"], s["cholR"], s["chol_x0"].chol))
    tol = max(1e-9, 4 * cond ** 2 * np.finfo(float).eps)
    for key in ("trans_matrix", "trans_noise_mean", "trans_noise_chol", "obs_matrix", "obs_noise_mean",
                "obs_noise_chol", "m0", "L0"):
        assert_rel(got[key], ref[key], tol, key)
    assert np.all(np_(got["trans_params"]) == 0) and np.all(np_(got["obs_params"]) == 0)


@pytest.mark.parametrize("method", ["cubature", "unscented", "gauss_hermite"])
def test_linear_adjoints_do_not_depend_on_the_linearisation(method):
    """A linear model linearises to itself with every rule: the same gradient at any nominal."""
    s, ys = _linear_case(3, 2, 25, seed=11)
    _, gt = linear_pair(s["F"], s["b"], s["cholQ"])
    _, go = linear_pair(s["H"], s["c"], s["cholR"])
    x0 = S.MVNSqrt(torch.as_tensor(s["chol_x0"].mean), torch.as_tensor(s["chol_x0"].chol))
    nom = S.MVNSqrt(torch.as_tensor(s["m_nominal"][:26]), torch.eye(3, dtype=torch.float64).expand(26, 3, 3))
    _, a1 = S.filter_loglikelihood_adjoint(torch.as_tensor(ys), x0, gt, go, S.linearization.extended)
    _, a2 = S.filter_loglikelihood_adjoint(torch.as_tensor(ys), x0, gt, go, getattr(S.linearization, method), nom)
    for key in ("trans_matrix", "trans_noise_chol", "obs_matrix", "obs_noise_chol", "m0", "L0"):
        assert_rel(a2[key], a1[key], 1e-9, key)


def test_ragged_batch_per_sequence_prior_vs_oracle():
    """Packed batch with an empty sequence and one prior per sequence: each row is that sequence's
    gradient (the empty sequence's is zero)."""
    nx, ny = 4, 2
    lengths = [17, 0, 40, 1, 23]
    rng = np.random.RandomState(4)
    s, _ = _linear_case(nx, ny, 5, seed=9)
    ot, gt = linear_pair(s["F"], s["b"], s["cholQ"])
    oo, go = linear_pair(s["H"], s["c"], s["cholR"])
    from sqrt_parallel_smoothers_gb300.data import lgssm_data
    ys_all, m0s, L0s, refs = [], [], [], []
    for i, T in enumerate(lengths):
        m0 = rng.randn(nx)
        L0 = np.tril(rng.rand(nx, nx)) + np.eye(nx)
        _, y = lgssm_data(m0, s["F"], s["H"], s["R"], s["Q"], s["b"], s["c"], max(T, 1), random_state=i)
        y = y[:T].astype(np.float64)
        ys_all.append(y.reshape(T, ny))
        m0s.append(m0)
        L0s.append(L0)
        if T == 0:
            refs.append(None)
            continue
        _, adj = OA.filter_adjoint(y, O.MVNSqrt(m0, L0), ot, oo, O.linearization.extended)
        refs.append(OA.linear_model_adjoints(adj, s["cholQ"], s["cholR"]))
    ys = torch.as_tensor(np.concatenate(ys_all))
    offsets = np.concatenate([[0], np.cumsum(lengths)])
    x0 = S.MVNSqrt(torch.as_tensor(np.stack(m0s)), torch.as_tensor(np.stack(L0s)))
    _, got = S.filter_loglikelihood_adjoint(ys, x0, gt, go, S.linearization.extended, offsets=offsets)
    for i, ref in enumerate(refs):
        for key in ("trans_matrix", "trans_noise_chol", "obs_matrix", "obs_noise_chol", "m0", "L0"):
            g = np_(got[key])[i]
            if ref is None:
                assert np.all(g == 0), (i, key)
            else:
                assert_rel(g, ref[key], 1e-9, f"{key}[{i}]")


def _bearings_models_np(theta, Q1, dt=0.01, s2=(1.0, 1.0)):
    q, sigma = np.exp(theta[2]), np.exp(theta[3])
    tm = O.FunctionalModel(OM.CoordinatedTurn(dt), O.MVNSqrt(np.zeros(5), np.linalg.cholesky(q * Q1)))
    om = O.FunctionalModel(OM.Bearings((theta[0], theta[1]), s2), O.MVNSqrt(np.zeros(2), sigma * np.eye(2)))
    return tm, om


def _bearings_problem(T, seed):
    w = S.data.bearings_workload(T, seed=seed)
    ys = w["ys"].astype(np.float64)
    Q1, _ = OM.bearings_noise(1.0, 5.0, 0.05, 0.01)
    m0 = np.array([0.1, 0.2, 1.0, 0.0, 1.0])
    rng = np.random.RandomState(seed)
    nom = O.MVNSqrt(np.repeat(m0[None], T + 1, 0) + 0.05 * rng.randn(T + 1, 5),
                    np.repeat(0.3 * np.eye(5)[None], T + 1, 0))
    theta = np.array([-1.5, 0.5, np.log(0.1), np.log(0.05)])
    return ys, m0, nom, Q1, theta


@pytest.mark.parametrize("method", ["cubature", "extended", "unscented"])
def test_bearings_model_params_fp64_vs_oracle(method):
    T = 50
    ys, m0, nom, Q1, theta = _bearings_problem(T, seed=2)
    lin = getattr(O.linearization, method)
    tm, om = _bearings_models_np(theta, Q1)
    x0o = O.MVNSqrt(m0, np.eye(5))
    ell_ref, adj = OA.filter_adjoint(ys, x0o, tm, om, lin, nom)
    n_next = O.MVNSqrt(nom.mean[1:], nom.chol[1:])
    h = 1e-6
    ref_params = []
    for j in range(4):
        sens = [theta[0], theta[1], 1.0, 1.0]
        sp, sm = list(sens), list(sens)
        sp[j] += h
        sm[j] -= h
        mk = lambda s_: O.FunctionalModel(OM.Bearings((s_[0], s_[1]), (s_[2], s_[3])), om.mvn)
        ref_params.append(OA.param_adjoint(adj, 1, lin(mk(sp), n_next), lin(mk(sm), n_next), h))
    gt = S.FunctionalModel(GM.CoordinatedTurn(0.01), S.MVNSqrt(torch.zeros(5, dtype=torch.float64),
                                                                torch.as_tensor(tm.mvn.chol)))
    go = S.FunctionalModel(GM.Bearings((theta[0], theta[1]), (1.0, 1.0)),
                           S.MVNSqrt(torch.zeros(2, dtype=torch.float64), torch.as_tensor(om.mvn.chol)))
    x0 = S.MVNSqrt(torch.as_tensor(m0), torch.eye(5, dtype=torch.float64))
    nomg = S.MVNSqrt(torch.as_tensor(nom.mean), torch.as_tensor(nom.chol))
    ell, got = S.filter_loglikelihood_adjoint(torch.as_tensor(ys), x0, gt, go, getattr(S.linearization, method),
                                              nomg)
    assert abs(float(ell) - ell_ref) <= 1e-10 * abs(ell_ref)
    # the oracle's parameter chain differentiates the local linearisation numerically (h = 1e-6)
    assert_rel(got["obs_params"], np.array(ref_params), 1e-6, "obs_params")
    assert_rel(got["trans_noise_chol"], OA.noise_chol_adjoint(adj["A_q"], adj["lin"][1], tm.mvn.chol), 1e-8,
               "trans_noise_chol")
    assert_rel(got["obs_noise_chol"], OA.noise_chol_adjoint(adj["A_r"], adj["lin"][4], om.mvn.chol), 1e-8,
               "obs_noise_chol")
    assert_rel(got["trans_noise_mean"], adj["b"].sum(0), 1e-8, "trans_noise_mean")
    assert_rel(got["m0"], adj["m0"], 1e-8, "m0")


@pytest.mark.parametrize("dtype,tol,ell_tol", [(torch.float64, 1e-8, 1e-9), (torch.float32, 5e-3, 1e-5)])
def test_reverse_matches_tangent_path_bearings(dtype, tol, ell_tol):
    """The reverse pass and the tangent-linear pass give the same four derivatives."""
    T = 200
    ys, m0, nom, Q1, theta = _bearings_problem(T, seed=5)
    th = torch.tensor(theta)
    x0 = S.MVNSqrt(torch.as_tensor(m0), torch.eye(5, dtype=torch.float64))
    nomg = S.MVNSqrt(torch.as_tensor(nom.mean), torch.as_tensor(nom.chol))
    out = {}
    for mode in ("tangent", "reverse"):
        t = th.clone().requires_grad_(True)
        ell = S.BearingsLogLikelihood.apply(t, torch.as_tensor(ys, dtype=dtype), x0, nomg, Q1, 0.01, (1.0, 1.0),
                                            S.linearization.cubature, None, None, 0, mode)
        ell.backward()
        out[mode] = (float(ell.detach()), t.grad.numpy().copy())
    # the FP32 tangent pass runs the dual-number kernels, the reverse pass the primal ones
    assert abs(out["tangent"][0] - out["reverse"][0]) <= ell_tol * abs(out["tangent"][0])
    g_t, g_r = out["tangent"][1], out["reverse"][1]
    assert np.all(np.abs(g_r - g_t) <= tol * np.maximum(1.0, np.abs(g_t))), (g_r, g_t)


def test_config3_reverse_fp32_vs_fd_fp64():
    """The reference's parameter-estimation configuration (bearings, B = 64, T = 5000, four
    parameters, FP32) from the reverse pass, against central differences (h = 1e-3) of the FP64
    filter log-likelihood, as the bench reports it."""
    B, T = 64, 5000
    batch = S.data.bearings_batch(np.full(B, T), qc=0.1, qw=0.5, sigma=0.05, dt=0.01, seed0=20_000)
    Q1, _ = S.data.bearings_noise(1.0, 5.0, 0.05, 0.01)
    m0 = torch.tensor([-4.0, -1.0, 2.0, 7.0, 3.0], dtype=torch.float64)
    x0 = S.MVNSqrt(m0, torch.eye(5, dtype=torch.float64))
    n_states = B * (T + 1)
    nom = S.MVNSqrt(m0.expand(n_states, 5).contiguous(), torch.eye(5, dtype=torch.float64).expand(n_states, 5, 5))
    theta0 = np.array([-1.5, 0.5, np.log(0.1), np.log(0.05)])

    def ell_grad(theta, dtype, mode):
        t = torch.tensor(theta, requires_grad=True)
        ell = S.BearingsLogLikelihood.apply(t, torch.as_tensor(batch["ys"], dtype=dtype), x0, nom, Q1, 0.01,
                                            (1.0, 1.0), S.linearization.cubature, None, batch["offsets"], 0, mode)
        ell.backward()
        return float(ell), t.grad.numpy()

    _, g = ell_grad(theta0, torch.float32, "reverse")
    h = 1e-3
    fd = np.array([(ell_grad(theta0 + h * e, torch.float64, "tangent")[0] -
                    ell_grad(theta0 - h * e, torch.float64, "tangent")[0]) / (2 * h) for e in np.eye(4)])
    rel = np.abs(g - fd) / np.abs(fd)
    assert np.all(rel < 1e-2), (g, fd, rel)


def test_linear_gaussian_autograd_function():
    """LinearGaussianLogLikelihood: torch.autograd over all eight arrays of a linear model,
    against the oracle restatement (FP64)."""
    s, ys = _linear_case(4, 2, 40, seed=21)
    leaves = [torch.tensor(np.asarray(v, float), requires_grad=True) for v in
              (s["F"], s["cholQ"], s["b"], s["H"], s["cholR"], s["c"], s["chol_x0"].mean, s["chol_x0"].chol)]
    ell = S.LinearGaussianLogLikelihood.apply(*leaves, torch.as_tensor(ys))
    (2.0 * ell).backward()
    ot, _ = linear_pair(s["F"], s["b"], s["cholQ"])
    oo, _ = linear_pair(s["H"], s["c"], s["cholR"])
    ell_ref, adj = OA.filter_adjoint(ys, O.MVNSqrt(s["chol_x0"].mean, s["chol_x0"].chol), ot, oo,
                                     O.linearization.extended)
    ref = OA.linear_model_adjoints(adj, s["cholQ"], s["cholR"])
    assert abs(float(ell) - ell_ref) <= 1e-10 * abs(ell_ref)
    keys = ("trans_matrix", "trans_noise_chol", "trans_noise_mean", "obs_matrix", "obs_noise_chol",
            "obs_noise_mean", "m0", "L0")
    for leaf, key in zip(leaves, keys):
        assert_rel(leaf.grad, 2.0 * ref[key], 1e-9, key)


def test_unsupported_combinations_raise():
    """A conditional-moments observation (its noise arguments are ignored) and the covariance
    form are rejected, and Gauss-Hermite gives no model-scalar gradients."""
    s, ys = _linear_case(2, 2, 10, seed=1)
    _, gt = linear_pair(s["F"], s["b"], s["cholQ"])
    h = GM.PoissonExp(1.0, d_in=2, d_out=2)
    x0 = S.MVNSqrt(torch.zeros(2, dtype=torch.float64), torch.eye(2, dtype=torch.float64))
    with pytest.raises(NotImplementedError):
        S.filter_loglikelihood_adjoint(torch.as_tensor(ys), x0, gt,
                                       S.ConditionalMomentsModel(h.conditional_mean, h.conditional_chol),
                                       S.linearization.extended)
    _, go = linear_pair(s["H"], s["c"], s["cholR"])
    _, adj = S.filter_loglikelihood_adjoint(torch.as_tensor(ys), x0, gt, go, S.linearization.gauss_hermite)
    assert "obs_params" not in adj and "trans_matrix" in adj
