// Reverse-mode gradient of the filter's log-likelihood (ss_filter_adjoint).
//
// The reference differentiates its parallel filter with jax.grad
// (parsmooth/parallel/_filtering.py:13-61 with return_loglikelihood, the sum of
// :149-154).  At a fixed nominal trajectory that log-likelihood is the exact
// marginal log-likelihood of the linearised Gaussian model the filter runs,
//   x_0 ~ N(m0, L0 L0^T),  x_t = F_t x_{t-1} + b_t + N(0, cQ_t cQ_t^T),
//   y_t = H_t x_t + c_t + N(0, cR_t cR_t^T),
// so its gradient with respect to every per-step parameter is the posterior
// expectation of the complete-data score (Fisher's identity), which needs only
// the smoothed moments.  The reverse pass is therefore the smoother's own
// backward associative scan, run once whatever the number of parameters, plus
// one per-step contraction of the filtered, predicted and smoothed moments:
//   transition (adjoint_transition): with d = ms_t - mp_t (smoothed minus
//     predicted mean), [Y, y] = Lp^-1 [Ls_t, d] (Lp the predicted factor) and
//     N = Y Y^T - I + y y^T:  dl/dQ = Lp^-T N Lp^-1 / 2, dl/db = Lp^-T y,
//     dl/dF = Lp^-T ((Y Y^T - I) (E Lp)^T + y ms_{t-1}^T); for a factor L of an
//     additive part of Q, dl/dL = Lp^-T N Lp^-1 L;
//   observation (adjoint_observation): Z = cR^-1 [H Ls_t, y_t - H ms_t - c],
//     A = Z Z^T - I: dl/dR = cR^-T A cR^-1 / 2, dl/dH = cR^-T (z_r ms_t^T - Z_1 Ls_t^T),
//     dl/dc = cR^-T z_r;
//   prior (adjoint_prior_kernel): the observation's form with L0 and ms_0 - m0.
// Model parameters that enter a nonlinear model's linearisation are chained
// per step through a one-direction dual-number linearisation (at most four per
// model): tr(Fbar^T dF) + bbar . db + tr(Qbar d(c c^T)).
//
// Work decomposition: one thread per level-1 chunk (the scan's geometry)
// accumulates its steps' contributions in FP64 (a per-thread column of shared
// memory), a per-(sequence, component) kernel sums the chunks, and one thread
// per sequence forms the prior's adjoint.
#pragma once
#include "ss_run.cuh"

namespace ss {

// Components of the per-chunk partial sums.
template <int NX, int NY>
struct AdjK {
  static constexpr int F = 0, B = NX * NX, LQ = B + NX, H = LQ + NX * NX, C = H + NY * NX, LR = C + NY,
                       TP = LR + NY * NY, OP = TP + 4, K = OP + 4;
};

constexpr int ADJ_BLOCK = 64;

template <typename R, int NX, int NY>
struct AdjTrans {
  R Fbar[NX][NX], bbar[NX];
  R N[NX][NX];    // dl/dQ = Lp^-T N Lp^-1 / 2
  R Lp[NX][NX];   // the filter's predicted factor
};
template <typename R, int NX, int NY>
struct AdjObs {
  R Hbar[NY][NX], cbar[NY], A[NY][NY];
};

// Transition part of step t (x_{t-1} -> x_t), in the predicted-moment
// (disturbance-smoother) form.  With the filter's predicted moments of x_t
// (mean mp = F mf + b; factor Lp from tria([[F Lf, cQ], [Lf, 0]]), whose
// lower-left block is Phi21 = E Lp for the smoothing gain E) and the smoothed
// x_t ~ N(ms, Ls Ls^T), the residual e = x_t - F x_{t-1} - b has E e = Q P^-1 d
// and Q^-1 Cov(e) Q^-1 - Q^-1 = P^-1 (Ps - P) P^-1, d = ms - mp.  So with
// [Y, y] = Lp^-1 [Ls, d] and N = Y Y^T - I + y y^T:
//   dl/dQ = Lp^-T N Lp^-1 / 2,   dl/db = Lp^-T y,
//   dl/dF = Lp^-T ((Y Y^T - I) Phi21^T + y ms_{t-1}^T).
// Nothing subtracts two states to form the O(sqrt Q) residual itself: FP32
// smoothed means carry errors far above sqrt Q when the process noise is small
// against the state, and Q^-1 would amplify them.  f = filtered x_{t-1},
// msp = smoothed mean of x_{t-1}, sn = smoothed x_t.
template <typename R, int NX, int NY>
SS_DEV void adjoint_transition(const Lin<R, NX, NY>& l, const State<R, NX>& f, const R (&msp)[NX],
                               const State<R, NX>& sn, AdjTrans<R, NX, NY>& o) {
  R X[2 * NX][2 * NX], mp[NX];
  SElem<R, NX> se;
  smoother_element<R, NX>(l.F, l.cQ, l.bq, f, se, X, mp);
  R Y[NX][NX + 1];
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) Y[i][j] = sn.L[i][j];
    Y[i][NX] = sn.m[i] - mp[i];
  }
  solve_lower<R, NX, NX + 1>(X, Y);
  R Ap[NX][NX];
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) {
      R q = (i == j) ? R(-1) : R(0);
      SS_UNROLL
      for (int k = 0; k < NX; ++k) q += Y[i][k] * Y[j][k];
      Ap[i][j] = q;
      o.N[i][j] = q + Y[i][NX] * Y[j][NX];
      o.Lp[i][j] = (j <= i) ? X[i][j] : R(0);
    }
  }
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) {
      R q = Y[i][NX] * msp[j];
      SS_UNROLL
      for (int k = 0; k < NX; ++k) q += Ap[i][k] * X[NX + j][k];
      o.Fbar[i][j] = q;
    }
  }
  solve_lower_T<R, NX, NX>(X, o.Fbar);
  R zb[NX][1];
  SS_UNROLL
  for (int i = 0; i < NX; ++i) zb[i][0] = Y[i][NX];
  solve_lower_T<R, NX, 1>(X, zb);
  SS_UNROLL
  for (int i = 0; i < NX; ++i) o.bbar[i] = zb[i][0];
}

// Observation part of step t (y_t, smoothed x_t).
template <typename R, int NX, int NY>
SS_DEV void adjoint_observation(const Lin<R, NX, NY>& l, const R (&y)[NY], const State<R, NX>& sn,
                                AdjObs<R, NX, NY>& o) {
  R Z[NY][NX + 1];
  SS_UNROLL
  for (int r = 0; r < NY; ++r) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) {
      R q = R(0);
      SS_UNROLL
      for (int k = j; k < NX; ++k) q += l.H[r][k] * sn.L[k][j];
      Z[r][j] = q;
    }
    R e = y[r] - l.c[r];
    SS_UNROLL
    for (int k = 0; k < NX; ++k) e -= l.H[r][k] * sn.m[k];
    Z[r][NX] = e;
  }
  solve_lower<R, NY, NX + 1>(l.cR, Z);
  SS_UNROLL
  for (int i = 0; i < NY; ++i) {
    SS_UNROLL
    for (int j = 0; j < NY; ++j) {
      R q = (i == j) ? R(-1) : R(0);
      SS_UNROLL
      for (int k = 0; k <= NX; ++k) q += Z[i][k] * Z[j][k];
      o.A[i][j] = q;
    }
  }
  SS_UNROLL
  for (int r = 0; r < NY; ++r) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) {
      R q = Z[r][NX] * sn.m[j];
      SS_UNROLL
      for (int k = 0; k <= j; ++k) q -= Z[r][k] * sn.L[j][k];
      o.Hbar[r][j] = q;
    }
  }
  solve_lower_T<R, NY, NX>(l.cR, o.Hbar);
  R zc[NY][1];
  SS_UNROLL
  for (int r = 0; r < NY; ++r) zc[r][0] = Z[r][NX];
  solve_lower_T<R, NY, 1>(l.cR, zc);
  SS_UNROLL
  for (int r = 0; r < NY; ++r) o.cbar[r] = zc[r][0];
}

// tril(c^-T A c^-1 L) for the factor L of an additive part of c c^T.
template <typename R, int D>
SS_DEV void noise_factor_adjoint(const R (&c)[D][D], const R (&A)[D][D], const R (&L)[D][D], R (&out)[D][D]) {
  R Y[D][D];
  SS_UNROLL
  for (int i = 0; i < D; ++i) {
    SS_UNROLL
    for (int j = 0; j < D; ++j) Y[i][j] = L[i][j];
  }
  solve_lower<R, D, D>(c, Y);
  SS_UNROLL
  for (int i = 0; i < D; ++i) {
    SS_UNROLL
    for (int j = 0; j < D; ++j) {
      R q = R(0);
      SS_UNROLL
      for (int k = 0; k < D; ++k) q += A[i][k] * Y[k][j];
      out[i][j] = q;
    }
  }
  solve_lower_T<R, D, D>(c, out);
  SS_UNROLL
  for (int i = 0; i < D; ++i) {
    SS_UNROLL
    for (int j = i + 1; j < D; ++j) out[i][j] = R(0);
  }
}

template <typename R>
struct AdjArgs {
  const R* fm;      // filtered trajectory (caller layout)
  const R* fL;
  const R* sm;      // smoothed trajectory (caller layout)
  const R* sL;
  const R* nom_m;   // the nominal (null: zero means, identity factors)
  const R* nom_L;
  const R* tq_L;    // the models' own noise factors
  const R* oq_L;
  double* part;     // (level-1 items, K) partial sums
};

template <typename R, int NX, int NY>
SS_DEV void load_step(const ScanArgs<R>& a, const AdjArgs<R>& b, int64_t i, int64_t base, int64_t t,
                      Lin<R, NX, NY>& l, R (&y)[NY], State<R, NX>& sn) {
  typedef Rec<R, NX, NY> Q;
  load_lin<R, NX, NY>(a.lin + (base + t) * Q::LIN_P, l);
  SS_UNROLL
  for (int k = 0; k < NY; ++k) y[k] = a.ys[(base + t) * NY + k];
  load_traj<R, NX>(b.sm, b.sL, base + i + t + 1, sn);
}

// A lower factor (its lower entries; the kernels read no other part).
template <typename R, int D>
SS_DEV void load_factor(const R* L, R (&out)[D][D]) {
  SS_UNROLL
  for (int i = 0; i < D; ++i) {
    SS_UNROLL
    for (int j = 0; j < D; ++j) out[i][j] = (j <= i) ? ldg(L + i * D + j) : R(0);
  }
}

template <typename R, int NX>
SS_DEV void load_prev_mean(const AdjArgs<R>& b, int64_t s, R (&mp)[NX]) {
  SS_UNROLL
  for (int k = 0; k < NX; ++k) mp[k] = b.sm[s * NX + k];
}

// The model-independent components of one chunk: the linearised-model adjoints
// reduced to the linear models' arrays and both noise factors.
template <typename R, int NX, int NY>
__global__ void __launch_bounds__(ADJ_BLOCK) adjoint_chunk_kernel(ScanArgs<R> a, AdjArgs<R> b) {
  typedef AdjK<NX, NY> K;
  extern __shared__ double adj_acc[];
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.g.lvl[1][a.g.B]) return;
  auto acc = [&](int k) -> double& { return adj_acc[k * ADJ_BLOCK + threadIdx.x]; };
  for (int k = 0; k < K::TP; ++k) acc(k) = 0.0;
  int64_t i, t0, t1;
  chunk_of(a.g, j, i, t0, t1);
  const int64_t base = a.g.off[i];
  R Lq[NX][NX], Lr[NY][NY];
  load_factor<R, NX>(b.tq_L, Lq);
  load_factor<R, NY>(b.oq_L, Lr);
  for (int64_t t = t0; t < t1; ++t) {
    Lin<R, NX, NY> l;
    R y[NY];
    State<R, NX> sn;
    load_step<R, NX, NY>(a, b, i, base, t, l, y, sn);
    State<R, NX> f;
    load_traj<R, NX>(b.fm, b.fL, base + i + t, f);
    R msp[NX];
    load_prev_mean<R, NX>(b, base + i + t, msp);
    {
      AdjTrans<R, NX, NY> tr;
      adjoint_transition<R, NX, NY>(l, f, msp, sn, tr);
      SS_UNROLL
      for (int r = 0; r < NX; ++r) {
        SS_UNROLL
        for (int c = 0; c < NX; ++c) acc(K::F + r * NX + c) += (double)tr.Fbar[r][c];
        acc(K::B + r) += (double)tr.bbar[r];
      }
      R G[NX][NX];
      noise_factor_adjoint<R, NX>(tr.Lp, tr.N, Lq, G);
      SS_UNROLL
      for (int r = 0; r < NX; ++r) {
        SS_UNROLL
        for (int c = 0; c <= r; ++c) acc(K::LQ + r * NX + c) += (double)G[r][c];
      }
    }
    {
      AdjObs<R, NX, NY> ob;
      adjoint_observation<R, NX, NY>(l, y, sn, ob);
      SS_UNROLL
      for (int r = 0; r < NY; ++r) {
        SS_UNROLL
        for (int c = 0; c < NX; ++c) acc(K::H + r * NX + c) += (double)ob.Hbar[r][c];
        acc(K::C + r) += (double)ob.cbar[r];
      }
      R G[NY][NY];
      noise_factor_adjoint<R, NY>(l.cR, ob.A, Lr, G);
      SS_UNROLL
      for (int r = 0; r < NY; ++r) {
        SS_UNROLL
        for (int c = 0; c <= r; ++c) acc(K::LR + r * NY + c) += (double)G[r][c];
      }
    }
  }
  for (int k = 0; k < K::TP; ++k) b.part[j * K::K + k] = acc(k);
  for (int k = K::TP; k < K::K; ++k) b.part[j * K::K + k] = 0.0;
}

// Model parameters of one nonlinear model (WHICH 0 transition, 1 observation):
// per step and parameter direction d in mask, the dual-number linearisation at
// the nominal gives (dF, dc, db) and the contribution
// tr(Fbar^T dF) + bbar . db + tr(A c^-1 dc).
template <typename R, int NX, int NY, int WHICH, template <typename, int, int> class Fn, int METHOD>
__global__ void __launch_bounds__(ADJ_BLOCK) adjoint_param_kernel(ScanArgs<R> a, AdjArgs<R> b, LinArgs<R> la,
                                                                  int mask) {
  typedef AdjK<NX, NY> K;
  typedef Dual<R, 1> D;
  constexpr int DOUT = WHICH == 0 ? NX : NY;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.g.lvl[1][a.g.B]) return;
  int64_t i, t0, t1;
  chunk_of(a.g, j, i, t0, t1);
  const int64_t base = a.g.off[i];
  double g[4] = {0.0, 0.0, 0.0, 0.0};
  for (int64_t t = t0; t < t1; ++t) {
    Lin<R, NX, NY> l;
    R y[NY];
    State<R, NX> sn;
    load_step<R, NX, NY>(a, b, i, base, t, l, y, sn);
    // the step's adjoints and its noise-covariance adjoint as W^-T Cq W^-1 / 2 (W the
    // whitening factor: the predicted factor for the transition, the observation's
    // noise factor itself; Cq the core matrix), with the factor c of the linearised noise
    R Fbar[DOUT][NX], bbar[DOUT], Cq[DOUT][DOUT], W[DOUT][DOUT], c[DOUT][DOUT];
    if constexpr (WHICH == 0) {
      State<R, NX> f;
      load_traj<R, NX>(b.fm, b.fL, base + i + t, f);
      R msp[NX];
      load_prev_mean<R, NX>(b, base + i + t, msp);
      AdjTrans<R, NX, NY> tr;
      adjoint_transition<R, NX, NY>(l, f, msp, sn, tr);
      SS_UNROLL
      for (int r = 0; r < NX; ++r) {
        bbar[r] = tr.bbar[r];
        SS_UNROLL
        for (int q = 0; q < NX; ++q) {
          Fbar[r][q] = tr.Fbar[r][q];
          Cq[r][q] = tr.N[r][q];
          W[r][q] = tr.Lp[r][q];
          c[r][q] = l.cQ[r][q];
        }
      }
    } else {
      AdjObs<R, NX, NY> ob;
      adjoint_observation<R, NX, NY>(l, y, sn, ob);
      SS_UNROLL
      for (int r = 0; r < NY; ++r) {
        bbar[r] = ob.cbar[r];
        SS_UNROLL
        for (int q = 0; q < NX; ++q) Fbar[r][q] = ob.Hbar[r][q];
        SS_UNROLL
        for (int q = 0; q < NY; ++q) {
          Cq[r][q] = ob.A[r][q];
          W[r][q] = l.cR[r][q];
          c[r][q] = l.cR[r][q];
        }
      }
    }
    // tr(Qbar d(c c^T)) = tr(Cq U V^T), U = W^-1 dc, V = W^-1 c
    R V[DOUT][DOUT];
    SS_UNROLL
    for (int r = 0; r < DOUT; ++r) {
      SS_UNROLL
      for (int q = 0; q < DOUT; ++q) V[r][q] = c[r][q];
    }
    solve_lower<R, DOUT, DOUT>(W, V);
    // the nominal at t - 1 (transition) or t (observation), the model noise
    R m[NX], C[NX][NX], qm[DOUT], qL[DOUT][DOUT];
    load_nominal<R, NX>(b.nom_m, b.nom_L, base + i + t + WHICH, m, C);
    load_noise<R, DOUT>(WHICH == 0 ? la.tq_m : la.oq_m, WHICH == 0 ? la.tq_L : la.oq_L, qm, qL);
    D dm[NX], dC[NX][NX], dqm[DOUT], dqL[DOUT][DOUT];
    SS_UNROLL
    for (int r = 0; r < NX; ++r) {
      dm[r] = D(m[r]);
      SS_UNROLL
      for (int q = 0; q < NX; ++q) dC[r][q] = D(C[r][q]);
    }
    SS_UNROLL
    for (int r = 0; r < DOUT; ++r) {
      dqm[r] = D(qm[r]);
      SS_UNROLL
      for (int q = 0; q < DOUT; ++q) dqL[r][q] = D(qL[r][q]);
    }
    const ModelArgs<R>& mar = WHICH == 0 ? la.tm : la.om;
    for (int d = 0; d < 4; ++d) {
      if (!((mask >> d) & 1)) continue;
      ModelArgs<D> ma;
      ma.mat = nullptr;
      SS_UNROLL
      for (int k = 0; k < 4; ++k) {
        ma.p[k] = D(mar.p[k]);
        ma.p[k].d[0] = (k == d) ? R(1) : R(0);
      }
      Fn<D, NX, DOUT> f;
      f.init(ma);
      D dF[DOUT][NX], dc[DOUT][DOUT], db[DOUT];
      linearize<D, NX, DOUT, Fn<D, NX, DOUT>, METHOD>(f, dm, dC, dqm, dqL, la.rule, la.slr_form, dF, dc, db);
      R U[DOUT][DOUT];
      SS_UNROLL
      for (int r = 0; r < DOUT; ++r) {
        SS_UNROLL
        for (int q = 0; q < DOUT; ++q) U[r][q] = dc[r][q].d[0];
      }
      solve_lower<R, DOUT, DOUT>(W, U);
      R s = R(0);
      SS_UNROLL
      for (int r = 0; r < DOUT; ++r) {
        s += bbar[r] * db[r].d[0];
        SS_UNROLL
        for (int q = 0; q < NX; ++q) s += Fbar[r][q] * dF[r][q].d[0];
        SS_UNROLL
        for (int q = 0; q < DOUT; ++q) {
          R cu = R(0);
          SS_UNROLL
          for (int k = 0; k < DOUT; ++k) cu += Cq[r][k] * U[k][q];
          s += cu * V[r][q];
        }
      }
      g[d] += (double)s;
    }
  }
  const int col = WHICH == 0 ? K::TP : K::OP;
  for (int d = 0; d < 4; ++d) b.part[j * K::K + col + d] = g[d];
}

// Output arrays of ss_filter_adjoint, with the partial-sum component each entry comes from.
struct AdjOut {
  double* p[8];   // trans_matrix, trans_noise_mean, trans_noise_chol, obs_matrix, obs_noise_mean,
                  // obs_noise_chol, trans_params, obs_params
  int begin[9];   // component ranges
};

// Per (sequence, component): the sum over the sequence's chunks.
static __global__ void adjoint_reduce_kernel(Geo g, int K, const double* __restrict__ part, AdjOut out) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= g.B * K) return;
  const int64_t i = q / K;
  const int k = (int)(q - i * K);
  int w = 0;
  while (w < 7 && k >= out.begin[w + 1]) ++w;
  if (out.p[w] == nullptr) return;
  double s = 0.0;
  for (int64_t j = g.lvl[1][i]; j < g.lvl[1][i + 1]; ++j) s += part[j * K + k];
  const int n = out.begin[w + 1] - out.begin[w];
  out.p[w][i * n + (k - out.begin[w])] = s;
}

// The prior's adjoint per sequence: d0 = ms_0 - m0, Z0 = L0^-1 [Ls_0, d0],
// dl/dm0 = L0^-T z_d, dl/dL0 = tril(L0^-T (Z0 Z0^T - I)); zero for empty sequences.
template <typename R, int NX>
__global__ void __launch_bounds__(128) adjoint_prior_kernel(ScanArgs<R> a, AdjArgs<R> b, double* __restrict__ m0bar,
                                                            double* __restrict__ L0bar) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.g.B) return;
  const int64_t T = a.g.off[i + 1] - a.g.off[i];
  R Z[NX][NX + 1], A[NX][NX], v[NX][1];
  R L0[NX][NX];
  {
    const int64_t ps = i * a.prior_stride;
    State<R, NX> s;
    load_traj<R, NX>(b.sm, b.sL, a.g.off[i] + i, s);
    SS_UNROLL
    for (int r = 0; r < NX; ++r) {
      SS_UNROLL
      for (int c = 0; c < NX; ++c) {
        L0[r][c] = (c <= r) ? a.L0[(ps * NX + r) * NX + c] : R(0);
        Z[r][c] = s.L[r][c];
      }
      Z[r][NX] = s.m[r] - a.m0[ps * NX + r];
    }
  }
  solve_lower<R, NX, NX + 1>(L0, Z);
  SS_UNROLL
  for (int r = 0; r < NX; ++r) {
    v[r][0] = Z[r][NX];
    SS_UNROLL
    for (int c = 0; c < NX; ++c) {
      R q = (r == c) ? R(-1) : R(0);
      SS_UNROLL
      for (int k = 0; k <= NX; ++k) q += Z[r][k] * Z[c][k];
      A[r][c] = q;
    }
  }
  solve_lower_T<R, NX, 1>(L0, v);
  solve_lower_T<R, NX, NX>(L0, A);
  const bool empty = (T == 0);
  if (m0bar != nullptr) {
    SS_UNROLL
    for (int r = 0; r < NX; ++r) m0bar[i * NX + r] = empty ? 0.0 : (double)v[r][0];
  }
  if (L0bar != nullptr) {
    SS_UNROLL
    for (int r = 0; r < NX; ++r) {
      SS_UNROLL
      for (int c = 0; c < NX; ++c) L0bar[(i * NX + r) * NX + c] = (empty || c > r) ? 0.0 : (double)A[r][c];
    }
  }
}

// Parameter masks: the model parameters each device model reads.
inline int param_mask(int kind) {
  switch (kind) {
    case SS_MODEL_COORDINATED_TURN: return 1;    // dt
    case SS_MODEL_BEARINGS: return 15;           // both sensors
    case SS_MODEL_RICKER: return 1;              // a
    case SS_MODEL_POISSON_EXP: return 1;         // lam
    default: return 0;
  }
}

struct AdjLayout {
  Layout inner;
  size_t part, fm, fL, bytes;
};

// The scan's workspace, then the partial sums and the filtered trajectory (the
// smoothed one goes to the scan's nominal buffers, which this call does not use).
template <typename R, int NX, int NY>
inline int make_adj_layout(const ss_problem& p, AdjLayout& y) {
  int rc = make_layout<R, NX, NY>(p, y.inner);
  if (rc) return rc;
  const size_t S = (size_t)(p.total_steps + p.batch);
  y.part = y.inner.bytes;
  y.fm = y.part + align_up(sizeof(double) * (size_t)y.inner.items[1] * AdjK<NX, NY>::K);
  y.fL = y.fm + align_up(sizeof(R) * S * NX);
  y.bytes = y.fL + align_up(sizeof(R) * S * NX * NX);
  return SS_OK;
}

template <typename R, int NX, int NY, int WHICH, template <typename, int, int> class Fn>
inline int launch_param_method(const Runner<R, NX, NY>& rn, const AdjArgs<R>& b, unsigned grid, int mask) {
  const auto& a = rn.sa;
  const auto& la = rn.la;
  cudaStream_t st = rn.st;
  switch (rn.p.lin_method) {
    case SS_LIN_EXTENDED:
      SS_LAUNCH("adjoint_param", st, adjoint_param_kernel<R, NX, NY, WHICH, Fn, SS_LIN_EXTENDED><<<grid, ADJ_BLOCK, 0, st>>>(a, b, la, mask));
      return SS_OK;
    case SS_LIN_CUBATURE:
      SS_LAUNCH("adjoint_param", st, adjoint_param_kernel<R, NX, NY, WHICH, Fn, SS_LIN_CUBATURE><<<grid, ADJ_BLOCK, 0, st>>>(a, b, la, mask));
      return SS_OK;
    case SS_LIN_UNSCENTED:
      SS_LAUNCH("adjoint_param", st, adjoint_param_kernel<R, NX, NY, WHICH, Fn, SS_LIN_UNSCENTED><<<grid, ADJ_BLOCK, 0, st>>>(a, b, la, mask));
      return SS_OK;
    default:
      return SS_ERR_UNSUPPORTED;   // Gauss-Hermite: not differentiated
  }
}

template <typename R, int NX, int NY>
inline int launch_params(const Runner<R, NX, NY>& rn, const AdjArgs<R>& b, unsigned grid, bool trans, bool obs) {
  const ss_problem& p = rn.p;
  int rc = SS_OK;
  if (trans && param_mask(p.transition.kind) != 0) {
    const int mask = param_mask(p.transition.kind);
    if constexpr (ct_ok<NX>()) {
      if (p.transition.kind == SS_MODEL_COORDINATED_TURN)
        rc = launch_param_method<R, NX, NY, 0, CoordinatedTurnFn>(rn, b, grid, mask);
    }
    if (p.transition.kind == SS_MODEL_RICKER) rc = launch_param_method<R, NX, NY, 0, RickerFn>(rn, b, grid, mask);
    if (rc) return rc;
  }
  if (obs && param_mask(p.observation.kind) != 0) {
    const int mask = param_mask(p.observation.kind);
    if constexpr (bearings_ok<NX, NY>()) {
      if (p.observation.kind == SS_MODEL_BEARINGS) rc = launch_param_method<R, NX, NY, 1, BearingsFn>(rn, b, grid, mask);
    }
    if (p.observation.kind == SS_MODEL_POISSON_EXP) return SS_ERR_UNSUPPORTED;
    if (rc) return rc;
  }
  return SS_OK;
}

template <typename R, int NX, int NY>
int run_adjoint(const Call& c) {
  typedef AdjK<NX, NY> K;
  const ss_problem& p = *c.p;
  if (!models_supported<R, NX, NY>(p.transition.kind, p.observation.kind)) return SS_ERR_UNSUPPORTED;
  // the conditional-moments observation ignores its noise arguments, which the
  // contraction reads: not differentiated
  if (p.observation.kind == SS_MODEL_POISSON_EXP) return SS_ERR_UNSUPPORTED;
  AdjLayout y;
  int rc = make_adj_layout<R, NX, NY>(p, y);
  if (rc) return rc;
  if (c.op == OP_WORKSPACE) {
    *c.ws_bytes_out = y.bytes;
    return SS_OK;
  }
  if (c.ws == nullptr || c.ws_bytes < y.bytes) return SS_ERR_WORKSPACE;
  const ss_adjoints* out = c.adjoints;
  Runner<R, NX, NY> rn(c);
  if ((rc = rn.prepare())) return rc;
  cudaStream_t st = rn.st;
  const R* nm = static_cast<const R*>(c.nom_m);
  const R* nL = static_cast<const R*>(c.nom_L);
  if ((rc = rn.lin(nm, nL, nullptr, false))) return rc;
  R* sm = rn.template at<R>(rn.y.nomA_m);
  R* sL = rn.template at<R>(rn.y.nomA_L);
  double* part = rn.template at<double>(y.part);
  // filter with the smoothing elements, the filtered trajectory and the log-likelihood partial sums
  R* fm = rn.template at<R>(y.fm);
  R* fL = rn.template at<R>(y.fL);
  rn.sa.filt_m = fm;
  rn.sa.filt_L = fL;
  rn.sa.ll_chunk = rn.template at<double>(rn.y.ll);
  if ((rc = rn.filter_pass(true))) return rc;
  if (c.out_ell != nullptr)
    SS_LAUNCH("ll_reduce", st, ll_reduce_kernel<<<grid_for(p.batch, 128), 128, 0, st>>>(rn.geo, NY, 1, rn.template at<double>(rn.y.ll), c.out_ell, nullptr, 0, 0, nullptr));
  // the smoother's backward scan: smoothed trajectory into the workspace
  rn.sa.out_m = sm;
  rn.sa.out_L = sL;
  rn.sa.out_rec = nullptr;
  rn.sa.prev_m = nullptr;
  rn.sa.prev_L = nullptr;
  rn.sa.prev_rec = nullptr;
  rn.sa.mse = nullptr;
  rn.sa.flags = nullptr;
  if ((rc = rn.smoother_scan_and_walk())) return rc;
  rn.sa.filt_m = nullptr;
  rn.sa.filt_L = nullptr;
  AdjArgs<R> b;
  b.fm = fm;
  b.fL = fL;
  b.sm = sm;
  b.sL = sL;
  b.nom_m = nm;
  b.nom_L = nL;
  b.tq_L = static_cast<const R*>(p.transition.noise_chol);
  b.oq_L = static_cast<const R*>(p.observation.noise_chol);
  b.part = part;
  const int64_t items = rn.y.items[1];
  const unsigned grid = grid_for(items, ADJ_BLOCK);
  if (p.total_steps > 0) {
    constexpr int smem = (int)(sizeof(double) * K::TP * ADJ_BLOCK);
    cudaFuncSetAttribute(adjoint_chunk_kernel<R, NX, NY>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    SS_LAUNCH("adjoint_chunk", st, adjoint_chunk_kernel<R, NX, NY><<<grid, ADJ_BLOCK, smem, st>>>(rn.sa, b));
    if ((rc = launch_params<R, NX, NY>(rn, b, grid, out->trans_params != nullptr, out->obs_params != nullptr)))
      return rc;
  }
  AdjOut o;
  o.p[0] = p.transition.kind == SS_MODEL_LINEAR ? out->trans_matrix : nullptr;
  o.p[1] = out->trans_noise_mean;
  o.p[2] = out->trans_noise_chol;
  o.p[3] = p.observation.kind == SS_MODEL_LINEAR ? out->obs_matrix : nullptr;
  o.p[4] = out->obs_noise_mean;
  o.p[5] = out->obs_noise_chol;
  o.p[6] = out->trans_params;
  o.p[7] = out->obs_params;
  const int begins[9] = {K::F, K::B, K::LQ, K::H, K::C, K::LR, K::TP, K::OP, K::K};
  for (int k = 0; k < 9; ++k) o.begin[k] = begins[k];
  SS_LAUNCH("adjoint_reduce", st, adjoint_reduce_kernel<<<grid_for(p.batch * K::K, 128), 128, 0, st>>>(rn.geo, K::K, part, o));
  if (out->m0 != nullptr || out->L0 != nullptr) {
    SS_LAUNCH("adjoint_prior", st, adjoint_prior_kernel<R, NX><<<grid_for(p.batch, 128), 128, 0, st>>>(rn.sa, b, out->m0, out->L0));
  }
  return SS_OK;
}

}  // namespace ss

#define SS_INST_ADJ(R, TAG, NX, NY) \
  namespace ss {                    \
  int adj_##TAG##_##NX##_##NY(const Call& c) { return run_adjoint<R, NX, NY>(c); } \
  }
