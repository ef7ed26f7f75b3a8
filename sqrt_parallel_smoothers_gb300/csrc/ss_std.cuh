// Covariance-form ("standard") parallel filter and smoother: the reference's
// non-square-root elements, operators and linearisation
// (parsmooth/parallel/_operators.py:7-40 and 80-101,
// parsmooth/parallel/_filtering.py:64-97 and 157-163,
// parsmooth/parallel/_smoothing.py:60-69,
// parsmooth/linearization/_sigma_points.py:39-60 and 81-86,
// parsmooth/linearization/_extended.py).
//
// These run when the caller passes covariances (MVNStandard) and asks for the
// reference's covariance-form arithmetic.  They keep that arithmetic - full
// covariance matrices, Cholesky solves where the reference solves with a
// positive-definite matrix, LU with partial pivoting where it calls a general
// solve - in the given precision, without symmetrising or clamping beyond what
// the reference does.  The scan is the square-root path's (chunks, groups, top
// walk, down-sweep, state-form walks): the state form of the filtering combine
// keeps only the prefix's (b, C) = (mean, cov), and that of the smoothing
// combine is one RTS step.
#pragma once
#include "ss_pipeline.cuh"

namespace ss {

// Record sizes (elements; _P: padded to whole 16-byte units).  Covariances are
// stored as full matrices.
template <typename R, int NX, int NY>
struct SRec {
  static constexpr int LIN = 2 * NX * NX + NX + NY * NX + NY * NY + NY;  // F, Q, b, H, R, c
  static constexpr int LIN_P = Padded<R, LIN>::n;
  static constexpr int FE = 3 * NX * NX + 2 * NX;                        // A, b, C, eta, J
  static constexpr int FE_P = Padded<R, FE>::n;
  static constexpr int SE = NX + 2 * NX * NX;                            // g, E, L
  static constexpr int SE_P = Padded<R, SE>::n;
  static constexpr int ST = NX + NX * NX;                                // m, P
  static constexpr int ST_P = Padded<R, ST>::n;
};

// Linearised model at one step: x' = F x + b + N(0, Q), y = H x' + c + N(0, Rm).
template <typename R, int NX, int NY>
struct SLin {
  R F[NX][NX];
  R Q[NX][NX];
  R b[NX];
  R H[NY][NX];
  R Rm[NY][NY];
  R c[NY];
};

// Filtering element (A, b, C, eta, J) of parsmooth/parallel/_filtering.py:72-97.
template <typename R, int NX>
struct SFElem {
  R A[NX][NX];
  R b[NX];
  R C[NX][NX];
  R eta[NX];
  R J[NX][NX];
};

// Smoothing element (g, E, L) of parsmooth/parallel/_smoothing.py:60-69.
template <typename R, int NX>
struct SSElem {
  R g[NX];
  R E[NX][NX];
  R L[NX][NX];
};

template <typename R, int NX>
struct SState {
  R m[NX];
  R P[NX][NX];
};

// ----------------------------------------------------------------------------- records

template <typename R, int NX, int NY>
SS_DEV void load_slin(const R* p, SLin<R, NX, NY>& l) {
  typedef SRec<R, NX, NY> Q;
  R r[Q::LIN_P];
  load_rec<R, Q::LIN>(p, r);
  int o = 0;
  unpack<R, NX, NX>(r, o, l.F); o += NX * NX;
  unpack<R, NX, NX>(r, o, l.Q); o += NX * NX;
  unpack_vec<R, NX>(r, o, l.b); o += NX;
  unpack<R, NY, NX>(r, o, l.H); o += NY * NX;
  unpack<R, NY, NY>(r, o, l.Rm); o += NY * NY;
  unpack_vec<R, NY>(r, o, l.c);
}
template <typename R, int NX, int NY>
SS_DEV void store_slin(R* p, const SLin<R, NX, NY>& l) {
  typedef SRec<R, NX, NY> Q;
  R r[Q::LIN_P];
  SS_UNROLL
  for (int q = Q::LIN; q < Q::LIN_P; ++q) r[q] = R(0);
  int o = 0;
  pack<R, NX, NX>(r, o, l.F); o += NX * NX;
  pack<R, NX, NX>(r, o, l.Q); o += NX * NX;
  pack_vec<R, NX>(r, o, l.b); o += NX;
  pack<R, NY, NX>(r, o, l.H); o += NY * NX;
  pack<R, NY, NY>(r, o, l.Rm); o += NY * NY;
  pack_vec<R, NY>(r, o, l.c);
  store_rec<R, Q::LIN>(p, r);
}
template <typename R, int NX>
SS_DEV void load_sfe(const R* p, SFElem<R, NX>& e) {
  typedef SRec<R, NX, 1> Q;
  R r[Q::FE_P];
  load_rec<R, Q::FE>(p, r);
  int o = 0;
  unpack<R, NX, NX>(r, o, e.A); o += NX * NX;
  unpack_vec<R, NX>(r, o, e.b); o += NX;
  unpack<R, NX, NX>(r, o, e.C); o += NX * NX;
  unpack_vec<R, NX>(r, o, e.eta); o += NX;
  unpack<R, NX, NX>(r, o, e.J);
}
template <typename R, int NX>
SS_DEV void store_sfe(R* p, const SFElem<R, NX>& e) {
  typedef SRec<R, NX, 1> Q;
  R r[Q::FE_P];
  SS_UNROLL
  for (int q = Q::FE; q < Q::FE_P; ++q) r[q] = R(0);
  int o = 0;
  pack<R, NX, NX>(r, o, e.A); o += NX * NX;
  pack_vec<R, NX>(r, o, e.b); o += NX;
  pack<R, NX, NX>(r, o, e.C); o += NX * NX;
  pack_vec<R, NX>(r, o, e.eta); o += NX;
  pack<R, NX, NX>(r, o, e.J);
  store_rec<R, Q::FE>(p, r);
}
template <typename R, int NX>
SS_DEV void load_sse(const R* p, SSElem<R, NX>& e) {
  typedef SRec<R, NX, 1> Q;
  R r[Q::SE_P];
  load_rec<R, Q::SE>(p, r);
  unpack_vec<R, NX>(r, 0, e.g);
  unpack<R, NX, NX>(r, NX, e.E);
  unpack<R, NX, NX>(r, NX + NX * NX, e.L);
}
template <typename R, int NX>
SS_DEV void store_sse(R* p, const SSElem<R, NX>& e) {
  typedef SRec<R, NX, 1> Q;
  R r[Q::SE_P];
  SS_UNROLL
  for (int q = Q::SE; q < Q::SE_P; ++q) r[q] = R(0);
  pack_vec<R, NX>(r, 0, e.g);
  pack<R, NX, NX>(r, NX, e.E);
  pack<R, NX, NX>(r, NX + NX * NX, e.L);
  store_rec<R, Q::SE>(p, r);
}
template <typename R, int NX>
SS_DEV void load_sst(const R* p, SState<R, NX>& s) {
  typedef SRec<R, NX, 1> Q;
  R r[Q::ST_P];
  load_rec<R, Q::ST>(p, r);
  unpack_vec<R, NX>(r, 0, s.m);
  unpack<R, NX, NX>(r, NX, s.P);
}
template <typename R, int NX>
SS_DEV void store_sst(R* p, const SState<R, NX>& s) {
  typedef SRec<R, NX, 1> Q;
  R r[Q::ST_P];
  SS_UNROLL
  for (int q = Q::ST; q < Q::ST_P; ++q) r[q] = R(0);
  pack_vec<R, NX>(r, 0, s.m);
  pack<R, NX, NX>(r, NX, s.P);
  store_rec<R, Q::ST>(p, r);
}
// A state of a trajectory in the caller's layout: means (N, NX), covariances (N, NX, NX).
template <typename R, int NX>
SS_DEV void load_straj(const R* __restrict__ m, const R* __restrict__ P, int64_t s, SState<R, NX>& st) {
  SS_UNROLL
  for (int r = 0; r < NX; ++r) {
    st.m[r] = m[s * NX + r];
    SS_UNROLL
    for (int c = 0; c < NX; ++c) st.P[r][c] = P[(s * NX + r) * NX + c];
  }
}
template <typename R, int NX>
SS_DEV void store_straj(R* __restrict__ m, R* __restrict__ P, int64_t s, const SState<R, NX>& st) {
  SS_UNROLL
  for (int r = 0; r < NX; ++r) {
    m[s * NX + r] = st.m[r];
    SS_UNROLL
    for (int c = 0; c < NX; ++c) P[(s * NX + r) * NX + c] = st.P[r][c];
  }
}

// ----------------------------------------------------------------------------- dense algebra

// Lower Cholesky factor of a symmetric matrix (its lower triangle is read).  A
// matrix that is not positive definite gives non-finite entries, as the
// reference's jnp.linalg.cholesky returns NaN.
template <typename R, int N>
SS_DEV void cholesky(const R (&A)[N][N], R (&L)[N][N]) {
  SS_UNROLL
  for (int j = 0; j < N; ++j) {
    R s = A[j][j];
    SS_UNROLL
    for (int k = 0; k < j; ++k) s -= L[j][k] * L[j][k];
    const R d = ss_sqrt(s);
    L[j][j] = d;
    SS_UNROLL
    for (int i = j + 1; i < N; ++i) {
      R t = A[i][j];
      SS_UNROLL
      for (int k = 0; k < j; ++k) t -= L[i][k] * L[j][k];
      L[i][j] = t / d;
    }
    SS_UNROLL
    for (int i = 0; i < j; ++i) L[i][j] = R(0);
  }
}

// B <- S^{-1} B for a symmetric positive-definite S (jax.scipy.linalg.solve
// with assume_a="pos": Cholesky, then two triangular solves).
template <typename R, int N, int K>
SS_DEV void solve_pos(const R (&S)[N][N], R (&B)[N][K]) {
  R L[N][N];
  cholesky<R, N>(S, L);
  SS_UNROLL
  for (int i = 0; i < N; ++i) {
    SS_UNROLL
    for (int k = 0; k < K; ++k) {
      R s = B[i][k];
      SS_UNROLL
      for (int j = 0; j < i; ++j) s -= L[i][j] * B[j][k];
      B[i][k] = s / L[i][i];
    }
  }
  SS_UNROLL
  for (int i = N - 1; i >= 0; --i) {
    SS_UNROLL
    for (int k = 0; k < K; ++k) {
      R s = B[i][k];
      SS_UNROLL
      for (int j = i + 1; j < N; ++j) s -= L[j][i] * B[j][k];
      B[i][k] = s / L[i][i];
    }
  }
}

// B <- M^{-1} B for a general M (jnp.linalg.solve: LU with partial pivoting).
// M is overwritten.  Rows are exchanged by unrolled selects, so everything
// stays in registers.
template <typename R, int N, int K>
SS_DEV void solve_lu(R (&M)[N][N], R (&B)[N][K]) {
  SS_UNROLL
  for (int c = 0; c < N; ++c) {
    int p = c;
    R best = ss_abs(M[c][c]);
    SS_UNROLL
    for (int r = c + 1; r < N; ++r) {
      const R v = ss_abs(M[r][c]);
      if (v > best) { best = v; p = r; }
    }
    SS_UNROLL
    for (int r = c + 1; r < N; ++r) {
      if (r == p) {
        SS_UNROLL
        for (int j = 0; j < N; ++j) { const R t = M[c][j]; M[c][j] = M[r][j]; M[r][j] = t; }
        SS_UNROLL
        for (int k = 0; k < K; ++k) { const R t = B[c][k]; B[c][k] = B[r][k]; B[r][k] = t; }
      }
    }
    SS_UNROLL
    for (int r = c + 1; r < N; ++r) {
      const R f = M[r][c] / M[c][c];
      SS_UNROLL
      for (int j = c + 1; j < N; ++j) M[r][j] -= f * M[c][j];
      SS_UNROLL
      for (int k = 0; k < K; ++k) B[r][k] -= f * B[c][k];
    }
  }
  SS_UNROLL
  for (int i = N - 1; i >= 0; --i) {
    SS_UNROLL
    for (int k = 0; k < K; ++k) {
      R s = B[i][k];
      SS_UNROLL
      for (int j = i + 1; j < N; ++j) s -= M[i][j] * B[j][k];
      B[i][k] = s / M[i][i];
    }
  }
}

// C = A B^T   (A: M x K, B: N x K)
template <typename R, int M, int K, int N>
SS_DEV void matmul_nt(const R (&A)[M][K], const R (&B)[N][K], R (&C)[M][N]) {
  SS_UNROLL
  for (int i = 0; i < M; ++i) {
    SS_UNROLL
    for (int j = 0; j < N; ++j) {
      R s = R(0);
      SS_UNROLL
      for (int k = 0; k < K; ++k) s += A[i][k] * B[j][k];
      C[i][j] = s;
    }
  }
}

// F P F^T
template <typename R, int M, int N>
SS_DEV void sandwich(const R (&F)[M][N], const R (&P)[N][N], R (&out)[M][M]) {
  R FP[M][N];
  matmul<R, M, N, N>(F, P, FP);
  matmul_nt<R, M, N, M>(FP, F, out);
}

// ----------------------------------------------------------------------------- linearisation

// Unit sigma point k of the method chosen at run time.
template <typename R, int DIN>
SS_DEV void sigma_point_rt(const RuleArgs& ru, int method, int k, R (&xi)[DIN], R& wm, R& wc) {
  if (method == SS_LIN_CUBATURE) sigma_point<R, DIN, SS_LIN_CUBATURE>(ru, k, xi, wm, wc);
  else if (method == SS_LIN_UNSCENTED) sigma_point<R, DIN, SS_LIN_UNSCENTED>(ru, k, xi, wm, wc);
  else sigma_point<R, DIN, SS_LIN_GAUSS_HERMITE>(ru, k, xi, wm, wc);
}
template <int DIN>
SS_DEV int num_points_rt(const RuleArgs& ru, int method) {
  if (method == SS_LIN_CUBATURE) return num_points<DIN, SS_LIN_CUBATURE>(ru);
  if (method == SS_LIN_UNSCENTED) return num_points<DIN, SS_LIN_UNSCENTED>(ru);
  return num_points<DIN, SS_LIN_GAUSS_HERMITE>(ru);
}

// Covariance-form linearisation of f at x ~ N(m, P) with additive noise
// N(qm, Qn): (F, Q, b) with f(x') + q ~= F x' + b + N(0, Q).
// Sigma-point rules follow parsmooth/linearization/_sigma_points.py:81-86 and
// 88-100: chol = cholesky(P), points m + chol xi_k, F = cho_solve(chol,
// Psi_x)^T, Q = Phi - F P F^T + Qn symmetrised, b = m_f - F m + qm; for
// conditional-moments models (:39-60) Qn is the weighted sum of the points'
// conditional covariances and b = m_f - F m.  Extended (_extended.py): F the
// Jacobian at m, b = f(m) - F m + qm, Q = Qn (the conditional covariance at m).
template <typename R, int DIN, int DOUT, class Fn>
SS_DEV void linearize_cov(const Fn& f, int method, const R (&m)[DIN], const R (&P)[DIN][DIN], const R (&qm)[DOUT],
                          const R (&Qn)[DOUT][DOUT], const RuleArgs& ru, R (&F)[DOUT][DIN], R (&Q)[DOUT][DOUT],
                          R (&b)[DOUT]) {
  constexpr bool COND = IsConditional<Fn>::value;
  if (method == SS_LIN_EXTENDED) {
    f.jac(m, F);
    R fm[DOUT];
    f.eval(m, fm);
    R cm[DOUT][DOUT];
    if constexpr (COND) {
      R cc[DOUT][DOUT];
      f.cond_chol(m, cc);
      matmul_nt<R, DOUT, DOUT, DOUT>(cc, cc, cm);
    }
    SS_UNROLL
    for (int i = 0; i < DOUT; ++i) {
      R s = COND ? fm[i] : fm[i] + qm[i];
      SS_UNROLL
      for (int j = 0; j < DIN; ++j) s -= F[i][j] * m[j];
      b[i] = s;
      SS_UNROLL
      for (int j = 0; j < DOUT; ++j) Q[i][j] = COND ? cm[i][j] : Qn[i][j];
    }
    return;
  }
  R C[DIN][DIN];
  cholesky<R, DIN>(P, C);
  const int np = num_points_rt<DIN>(ru, method);
  R mf[DOUT];
  SS_UNROLL
  for (int i = 0; i < DOUT; ++i) mf[i] = R(0);
#pragma unroll 1
  for (int k = 0; k < np; ++k) {
    R xi[DIN], x[DIN], fx[DOUT], wm, wc;
    sigma_point_rt<R, DIN>(ru, method, k, xi, wm, wc);
    SS_UNROLL
    for (int i = 0; i < DIN; ++i) {
      R s = m[i];
      SS_UNROLL
      for (int j = 0; j <= i; ++j) s += C[i][j] * xi[j];
      x[i] = s;
    }
    f.eval(x, fx);
    SS_UNROLL
    for (int i = 0; i < DOUT; ++i) mf[i] += wm * fx[i];
  }
  // Psi_x = sum wc (x_k - m)(f_k - m_f)^T, Phi = sum wc (f_k - m_f)(f_k - m_f)^T
  R Psi[DIN][DOUT], Phi[DOUT][DOUT], V[DOUT][DOUT];
  SS_UNROLL
  for (int i = 0; i < DOUT; ++i) {
    SS_UNROLL
    for (int j = 0; j < DIN; ++j) Psi[j][i] = R(0);
    SS_UNROLL
    for (int j = 0; j < DOUT; ++j) { Phi[i][j] = R(0); V[i][j] = R(0); }
  }
#pragma unroll 1
  for (int k = 0; k < np; ++k) {
    R xi[DIN], x[DIN], dx[DIN], fx[DOUT], wm, wc;
    sigma_point_rt<R, DIN>(ru, method, k, xi, wm, wc);
    SS_UNROLL
    for (int i = 0; i < DIN; ++i) {
      R s = R(0);
      SS_UNROLL
      for (int j = 0; j <= i; ++j) s += C[i][j] * xi[j];
      x[i] = m[i] + s;
      dx[i] = x[i] - m[i];     // the reference subtracts the mean from the points
    }
    f.eval(x, fx);
    SS_UNROLL
    for (int i = 0; i < DOUT; ++i) fx[i] -= mf[i];
    SS_UNROLL
    for (int j = 0; j < DIN; ++j) {
      SS_UNROLL
      for (int i = 0; i < DOUT; ++i) Psi[j][i] += wc * dx[j] * fx[i];
    }
    SS_UNROLL
    for (int i = 0; i < DOUT; ++i) {
      SS_UNROLL
      for (int j = 0; j < DOUT; ++j) Phi[i][j] += wc * fx[i] * fx[j];
    }
    if constexpr (COND) {
      R cc[DOUT][DOUT], cv[DOUT][DOUT];
      f.cond_chol(x, cc);
      matmul_nt<R, DOUT, DOUT, DOUT>(cc, cc, cv);
      SS_UNROLL
      for (int i = 0; i < DOUT; ++i) {
        SS_UNROLL
        for (int j = 0; j < DOUT; ++j) V[i][j] += wc * cv[i][j];
      }
    }
  }
  // F^T = cho_solve(C, Psi_x): C^{-T} C^{-1} Psi_x
  SS_UNROLL
  for (int i = 0; i < DIN; ++i) {
    SS_UNROLL
    for (int k = 0; k < DOUT; ++k) {
      R s = Psi[i][k];
      SS_UNROLL
      for (int j = 0; j < i; ++j) s -= C[i][j] * Psi[j][k];
      Psi[i][k] = s / C[i][i];
    }
  }
  SS_UNROLL
  for (int i = DIN - 1; i >= 0; --i) {
    SS_UNROLL
    for (int k = 0; k < DOUT; ++k) {
      R s = Psi[i][k];
      SS_UNROLL
      for (int j = i + 1; j < DIN; ++j) s -= C[j][i] * Psi[j][k];
      Psi[i][k] = s / C[i][i];
    }
  }
  SS_UNROLL
  for (int i = 0; i < DOUT; ++i) {
    SS_UNROLL
    for (int j = 0; j < DIN; ++j) F[i][j] = Psi[j][i];
  }
  R FPF[DOUT][DOUT];
  sandwich<R, DOUT, DIN>(F, P, FPF);
  SS_UNROLL
  for (int i = 0; i < DOUT; ++i) {
    SS_UNROLL
    for (int j = 0; j < DOUT; ++j) {
      const R lij = Phi[i][j] - FPF[i][j] + (COND ? V[i][j] : Qn[i][j]);
      const R lji = Phi[j][i] - FPF[j][i] + (COND ? V[j][i] : Qn[j][i]);
      Q[i][j] = COND ? lij : R(0.5) * (lij + lji);
    }
  }
  SS_UNROLL
  for (int i = 0; i < DOUT; ++i) {
    R s = COND ? mf[i] : mf[i] + qm[i];
    SS_UNROLL
    for (int j = 0; j < DIN; ++j) s -= F[i][j] * m[j];
    b[i] = s;
  }
}

// ----------------------------------------------------------------------------- elements and operators

// Filtering element of one step with a zero prior (the true prior is the
// scan's initial state): parsmooth/parallel/_filtering.py:72-97 with m = 0,
// P = 0 before the prediction.  eta uses y - H b - c with the transition
// offset b, as the reference does (:94).
template <typename R, int NX, int NY>
SS_DEV void std_filter_element(const SLin<R, NX, NY>& l, const R (&y)[NY], SFElem<R, NX>& e) {
  // m = b, P = Q;  S = H P H^T + R
  R S[NY][NY];
  sandwich<R, NY, NX>(l.H, l.Q, S);
  SS_UNROLL
  for (int i = 0; i < NY; ++i) {
    SS_UNROLL
    for (int j = 0; j < NY; ++j) S[i][j] += l.Rm[i][j];
  }
  // S^{-1} H
  R SiH[NY][NX];
  SS_UNROLL
  for (int i = 0; i < NY; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) SiH[i][j] = l.H[i][j];
  }
  solve_pos<R, NY, NX>(S, SiH);
  // K = (S^{-1} H P)^T = P H^T S^{-1}
  R K[NX][NY];
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NY; ++j) {
      R s = R(0);
      SS_UNROLL
      for (int k = 0; k < NX; ++k) s += SiH[j][k] * l.Q[k][i];
      K[i][j] = s;
    }
  }
  // A = F - K H F
  R HF[NY][NX];
  matmul<R, NY, NX, NX>(l.H, l.F, HF);
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) {
      R s = l.F[i][j];
      SS_UNROLL
      for (int k = 0; k < NY; ++k) s -= K[i][k] * HF[k][j];
      e.A[i][j] = s;
    }
  }
  // b_std = m + K (y - H m - c), m = b
  R r[NY];
  SS_UNROLL
  for (int i = 0; i < NY; ++i) {
    R s = y[i] - l.c[i];
    SS_UNROLL
    for (int k = 0; k < NX; ++k) s -= l.H[i][k] * l.b[k];
    r[i] = s;
  }
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    R s = l.b[i];
    SS_UNROLL
    for (int k = 0; k < NY; ++k) s += K[i][k] * r[k];
    e.b[i] = s;
  }
  // C = P - K S K^T
  R KS[NX][NY];
  matmul<R, NX, NY, NY>(K, S, KS);
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) {
      R s = l.Q[i][j];
      SS_UNROLL
      for (int k = 0; k < NY; ++k) s -= KS[i][k] * K[j][k];
      e.C[i][j] = s;
    }
  }
  // temp = (S^{-1} H F)^T; eta = temp (y - H b - c); J = temp H F
  R SiHF[NY][NX];
  matmul<R, NY, NX, NX>(SiH, l.F, SiHF);
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    R s = R(0);
    SS_UNROLL
    for (int k = 0; k < NY; ++k) s += SiHF[k][i] * r[k];
    e.eta[i] = s;
    SS_UNROLL
    for (int j = 0; j < NX; ++j) {
      R t = R(0);
      SS_UNROLL
      for (int k = 0; k < NY; ++k) t += SiHF[k][i] * HF[k][j];
      e.J[i][j] = t;
    }
  }
}

// a <- combine(a, e) with a earlier: parsmooth/parallel/_operators.py:7-40.
template <typename R, int NX>
SS_DEV void std_filter_combine(SFElem<R, NX>& a, const SFElem<R, NX>& e) {
  // X = (A2 (I + C1 J2)^{-1})^T = solve((I + C1 J2)^T, A2^T)
  R M[NX][NX], X[NX][NX];
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) {
      R s = (i == j) ? R(1) : R(0);   // (I + C1 J2)^T [i][j] = (I + C1 J2)[j][i]
      SS_UNROLL
      for (int k = 0; k < NX; ++k) s += a.C[j][k] * e.J[k][i];
      M[i][j] = s;
      X[i][j] = e.A[j][i];
    }
  }
  solve_lu<R, NX, NX>(M, X);
  // Y = (A1^T (I + J2 C1)^{-1})^T = solve((I + J2 C1)^T, A1)
  R N[NX][NX], Y[NX][NX];
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) {
      R s = (i == j) ? R(1) : R(0);
      SS_UNROLL
      for (int k = 0; k < NX; ++k) s += e.J[j][k] * a.C[k][i];
      N[i][j] = s;
      Y[i][j] = a.A[i][j];
    }
  }
  solve_lu<R, NX, NX>(N, Y);
  // b = X^T (b1 + C1 eta2) + b2;  eta = Y^T (eta2 - J2 b1) + eta1
  R v[NX], w[NX];
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    R s = a.b[i];
    SS_UNROLL
    for (int k = 0; k < NX; ++k) s += a.C[i][k] * e.eta[k];
    v[i] = s;
    R t = e.eta[i];
    SS_UNROLL
    for (int k = 0; k < NX; ++k) t -= e.J[i][k] * a.b[k];
    w[i] = t;
  }
  R nb[NX], neta[NX];
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    R s = e.b[i], t = a.eta[i];
    SS_UNROLL
    for (int k = 0; k < NX; ++k) { s += X[k][i] * v[k]; t += Y[k][i] * w[k]; }
    nb[i] = s;
    neta[i] = t;
  }
  // A = X^T A1;  C = X^T C1 A2^T + C2;  J = Y^T J2 A1 + J1
  R CA[NX][NX], JA[NX][NX];
  matmul_nt<R, NX, NX, NX>(a.C, e.A, CA);
  matmul<R, NX, NX, NX>(e.J, a.A, JA);
  R nA[NX][NX], nC[NX][NX], nJ[NX][NX];
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) {
      R sa = R(0), sc = e.C[i][j], sj = a.J[i][j];
      SS_UNROLL
      for (int k = 0; k < NX; ++k) {
        sa += X[k][i] * a.A[k][j];
        sc += X[k][i] * CA[k][j];
        sj += Y[k][i] * JA[k][j];
      }
      nA[i][j] = sa;
      nC[i][j] = sc;
      nJ[i][j] = sj;
    }
  }
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    a.b[i] = nb[i];
    a.eta[i] = neta[i];
    SS_UNROLL
    for (int j = 0; j < NX; ++j) {
      a.A[i][j] = nA[i][j];
      a.C[i][j] = nC[i][j];
      a.J[i][j] = nJ[i][j];
    }
  }
}

// State form of the filtering combine: a prefix (mean m, covariance P) as elem1
// contributes only its (b, C), so the combined (b, C) is
// b = A2 (I + P J2)^{-1} (m + P eta2) + b2, C = A2 (I + P J2)^{-1} P A2^T + C2.
template <typename R, int NX>
SS_DEV void std_filter_apply(SState<R, NX>& s, const SFElem<R, NX>& e) {
  R M[NX][NX], X[NX][NX];
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) {
      R t = (i == j) ? R(1) : R(0);
      SS_UNROLL
      for (int k = 0; k < NX; ++k) t += s.P[j][k] * e.J[k][i];
      M[i][j] = t;
      X[i][j] = e.A[j][i];
    }
  }
  solve_lu<R, NX, NX>(M, X);
  R v[NX];
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    R t = s.m[i];
    SS_UNROLL
    for (int k = 0; k < NX; ++k) t += s.P[i][k] * e.eta[k];
    v[i] = t;
  }
  R PA[NX][NX];
  matmul_nt<R, NX, NX, NX>(s.P, e.A, PA);
  R nm[NX], nP[NX][NX];
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    R t = e.b[i];
    SS_UNROLL
    for (int k = 0; k < NX; ++k) t += X[k][i] * v[k];
    nm[i] = t;
    SS_UNROLL
    for (int j = 0; j < NX; ++j) {
      R u = e.C[i][j];
      SS_UNROLL
      for (int k = 0; k < NX; ++k) u += X[k][i] * PA[k][j];
      nP[i][j] = u;
    }
  }
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    s.m[i] = nm[i];
    SS_UNROLL
    for (int j = 0; j < NX; ++j) s.P[i][j] = nP[i][j];
  }
}

// Smoothing element at a filtered state (m, P) with the transition linearised
// there: parsmooth/parallel/_smoothing.py:60-69.
template <typename R, int NX>
SS_DEV void std_smoother_element(const R (&F)[NX][NX], const R (&Q)[NX][NX], const R (&b)[NX],
                                 const SState<R, NX>& s, SSElem<R, NX>& e) {
  R Pp[NX][NX];
  sandwich<R, NX, NX>(F, s.P, Pp);
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) Pp[i][j] += Q[i][j];
  }
  // E = solve(Pp, F P, pos)^T
  R FP[NX][NX];
  matmul<R, NX, NX, NX>(F, s.P, FP);
  solve_pos<R, NX, NX>(Pp, FP);
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) e.E[i][j] = FP[j][i];
  }
  // g = m - E (F m + b)
  R mp[NX];
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    R t = b[i];
    SS_UNROLL
    for (int k = 0; k < NX; ++k) t += F[i][k] * s.m[k];
    mp[i] = t;
  }
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    R t = s.m[i];
    SS_UNROLL
    for (int k = 0; k < NX; ++k) t -= e.E[i][k] * mp[k];
    e.g[i] = t;
  }
  // L = P - E Pp E^T
  R EPp[NX][NX];
  matmul<R, NX, NX, NX>(e.E, Pp, EPp);
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) {
      R t = s.P[i][j];
      SS_UNROLL
      for (int k = 0; k < NX; ++k) t -= EPp[i][k] * e.E[j][k];
      e.L[i][j] = t;
    }
  }
}

// acc <- combine(later = e, earlier = acc) of parsmooth/parallel/_operators.py:80-101
// (the reverse scan passes the later partial first): g = E_acc g_e + g_acc,
// E = E_acc E_e, L = E_acc L_e E_acc^T + L_acc.
template <typename R, int NX>
SS_DEV void std_smoother_fold(SSElem<R, NX>& acc, const SSElem<R, NX>& e) {
  R ng[NX], nE[NX][NX], EL[NX][NX], nL[NX][NX];
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    R t = acc.g[i];
    SS_UNROLL
    for (int k = 0; k < NX; ++k) t += acc.E[i][k] * e.g[k];
    ng[i] = t;
  }
  matmul<R, NX, NX, NX>(acc.E, e.E, nE);
  matmul<R, NX, NX, NX>(acc.E, e.L, EL);
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) {
      R t = acc.L[i][j];
      SS_UNROLL
      for (int k = 0; k < NX; ++k) t += EL[i][k] * acc.E[j][k];
      nL[i][j] = t;
    }
  }
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    acc.g[i] = ng[i];
    SS_UNROLL
    for (int j = 0; j < NX; ++j) {
      acc.E[i][j] = nE[i][j];
      acc.L[i][j] = nL[i][j];
    }
  }
}

// State form of the smoothing combine (one RTS step): m <- E m + g, P <- E P E^T + L.
template <typename R, int NX>
SS_DEV void std_smoother_apply(SState<R, NX>& s, const SSElem<R, NX>& e) {
  R nm[NX], EP[NX][NX], nP[NX][NX];
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    R t = e.g[i];
    SS_UNROLL
    for (int k = 0; k < NX; ++k) t += e.E[i][k] * s.m[k];
    nm[i] = t;
  }
  matmul<R, NX, NX, NX>(e.E, s.P, EP);
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) {
      R t = e.L[i][j];
      SS_UNROLL
      for (int k = 0; k < NX; ++k) t += EP[i][k] * e.E[j][k];
      nP[i][j] = t;
    }
  }
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    s.m[i] = nm[i];
    SS_UNROLL
    for (int j = 0; j < NX; ++j) s.P[i][j] = nP[i][j];
  }
}

// Log-density term of one step without the -ny/2 log(2 pi) constant:
// parsmooth/parallel/_filtering.py:157-163 with parsmooth/_utils.py:152-160 at
// the filtered state before the step.
template <typename R, int NX, int NY>
SS_DEV R std_loglik(const SLin<R, NX, NY>& l, const SState<R, NX>& s, const R (&y)[NY]) {
  R mp[NX], Pp[NX][NX];
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    R t = l.b[i];
    SS_UNROLL
    for (int k = 0; k < NX; ++k) t += l.F[i][k] * s.m[k];
    mp[i] = t;
  }
  sandwich<R, NX, NX>(l.F, s.P, Pp);
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) Pp[i][j] += l.Q[i][j];
  }
  R S[NY][NY], L[NY][NY], r[NY];
  sandwich<R, NY, NX>(l.H, Pp, S);
  SS_UNROLL
  for (int i = 0; i < NY; ++i) {
    R t = y[i] - l.c[i];
    SS_UNROLL
    for (int k = 0; k < NX; ++k) t -= l.H[i][k] * mp[k];
    r[i] = t;
    SS_UNROLL
    for (int j = 0; j < NY; ++j) S[i][j] += l.Rm[i][j];
  }
  cholesky<R, NY>(S, L);
  R q = R(0), logdet = R(0);
  SS_UNROLL
  for (int i = 0; i < NY; ++i) {
    R t = r[i];
    SS_UNROLL
    for (int k = 0; k < i; ++k) t -= L[i][k] * r[k];
    r[i] = t / L[i][i];
    q += r[i] * r[i];
    logdet += ss_log(ss_abs(L[i][i]));
  }
  return R(-0.5) * q - logdet;
}

// ----------------------------------------------------------------------------- kernels

template <typename R, int NX>
SS_DEV void load_nominal_cov(const R* nm, const R* nP, int64_t s, R (&m)[NX], R (&P)[NX][NX]) {
  if (nm == nullptr) {
    // the reference's default nominal: zero means, identity covariances (_filtering.py:25-28)
    SS_UNROLL
    for (int r = 0; r < NX; ++r) {
      m[r] = R(0);
      SS_UNROLL
      for (int c = 0; c < NX; ++c) P[r][c] = (r == c) ? R(1) : R(0);
    }
  } else {
    SS_UNROLL
    for (int r = 0; r < NX; ++r) {
      m[r] = nm[s * NX + r];
      SS_UNROLL
      for (int c = 0; c < NX; ++c) P[r][c] = nP[(s * NX + r) * NX + c];
    }
  }
}

// Per-step covariance-form linearisation (transition at nominal[t], observation
// at nominal[t + 1]); LinArgs carries covariances in nom_L, tq_L and oq_L.
template <typename R, int NX, int NY, class TF, class OF>
__global__ void __launch_bounds__(128) std_lin_kernel(LinArgs<R> a) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.total) return;
  const int64_t i = find_seq(a.off, a.B, k);
  if (a.active != nullptr && a.active[i] == 0) return;
  const int64_t t = k - a.off[i];
  const int64_t s = a.off[i] + i + t;
  SLin<R, NX, NY> l;
  {
    TF f;
    f.init(a.tm);
    R m[NX], P[NX][NX], qm[NX], Qn[NX][NX];
    load_nominal_cov<R, NX>(a.nom_m, a.nom_L, s, m, P);
    SS_UNROLL
    for (int r = 0; r < NX; ++r) {
      qm[r] = ldg(a.tq_m + r);
      SS_UNROLL
      for (int c = 0; c < NX; ++c) Qn[r][c] = ldg(a.tq_L + r * NX + c);
    }
    linearize_cov<R, NX, NX, TF>(f, a.rule.method, m, P, qm, Qn, a.rule, l.F, l.Q, l.b);
  }
  if (a.trans_only) {
    SS_UNROLL
    for (int r = 0; r < NY; ++r) {
      l.c[r] = R(0);
      SS_UNROLL
      for (int j = 0; j < NX; ++j) l.H[r][j] = R(0);
      SS_UNROLL
      for (int j = 0; j < NY; ++j) l.Rm[r][j] = R(0);
    }
  } else {
    OF h;
    h.init(a.om);
    R m[NX], P[NX][NX], qm[NY], Rn[NY][NY];
    load_nominal_cov<R, NX>(a.nom_m, a.nom_L, s + 1, m, P);
    SS_UNROLL
    for (int r = 0; r < NY; ++r) {
      qm[r] = ldg(a.oq_m + r);
      SS_UNROLL
      for (int c = 0; c < NY; ++c) Rn[r][c] = ldg(a.oq_L + r * NY + c);
    }
    linearize_cov<R, NX, NY, OF>(h, a.rule.method, m, P, qm, Rn, a.rule, l.H, l.Rm, l.c);
  }
  store_slin<R, NX, NY>(a.out + k * SRec<R, NX, NY>::LIN_P, l);
}

// Linearise one model at n independent points (ss_linearize, covariance form).
template <typename R, int DIN, int DOUT, class Fn>
__global__ void __launch_bounds__(128) std_lin_points_kernel(PointArgs<R> a) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.n) return;
  Fn f;
  f.init(a.model);
  R m[DIN], P[DIN][DIN], qm[DOUT], Qn[DOUT][DOUT];
  SS_UNROLL
  for (int r = 0; r < DIN; ++r) {
    m[r] = a.m[k * DIN + r];
    SS_UNROLL
    for (int c = 0; c < DIN; ++c) P[r][c] = a.L[(k * DIN + r) * DIN + c];
  }
  SS_UNROLL
  for (int r = 0; r < DOUT; ++r) {
    qm[r] = a.q_m[r];
    SS_UNROLL
    for (int c = 0; c < DOUT; ++c) Qn[r][c] = a.q_L[r * DOUT + c];
  }
  R F[DOUT][DIN], Q[DOUT][DOUT], b[DOUT];
  linearize_cov<R, DIN, DOUT, Fn>(f, a.rule.method, m, P, qm, Qn, a.rule, F, Q, b);
  SS_UNROLL
  for (int r = 0; r < DOUT; ++r) {
    a.b[k * DOUT + r] = b[r];
    SS_UNROLL
    for (int c = 0; c < DIN; ++c) a.F[(k * DOUT + r) * DIN + c] = F[r][c];
    SS_UNROLL
    for (int c = 0; c < DOUT; ++c) a.chol[(k * DOUT + r) * DOUT + c] = Q[r][c];
  }
}

template <typename R, int NX, int NY>
__global__ void __launch_bounds__(128) std_filter_leaf_kernel(ScanArgs<R> a) {
  typedef SRec<R, NX, NY> Q;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.g.lvl[1][a.g.B]) return;
  int64_t i, t0, t1;
  chunk_of(a.g, j, i, t0, t1);
  if (seq_inactive(a.active, i)) return;
  const int64_t base = a.g.off[i];
  SFElem<R, NX> acc;
  for (int64_t t = t0; t < t1; ++t) {
    SLin<R, NX, NY> l;
    load_slin<R, NX, NY>(a.lin + (base + t) * Q::LIN_P, l);
    R y[NY];
    SS_UNROLL
    for (int k = 0; k < NY; ++k) y[k] = a.ys[(base + t) * NY + k];
    if (t == t0) {
      std_filter_element<R, NX, NY>(l, y, acc);
    } else {
      SFElem<R, NX> e;
      std_filter_element<R, NX, NY>(l, y, e);
      std_filter_combine<R, NX>(acc, e);
    }
  }
  store_sfe<R, NX>(a.fsum[1] + j * Q::FE_P, acc);
}

template <typename R, int NX>
__global__ void __launch_bounds__(128) std_filter_up_kernel(ScanArgs<R> a, int l) {
  typedef SRec<R, NX, 1> Q;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.g.lvl[l + 1][a.g.B]) return;
  int64_t i, m0, m1;
  group_of(a.g, l, j, i, m0, m1);
  if (seq_inactive(a.active, i)) return;
  SFElem<R, NX> acc;
  load_sfe<R, NX>(a.fsum[l] + m0 * Q::FE_P, acc);
  for (int64_t m = m0 + 1; m < m1; ++m) {
    SFElem<R, NX> e;
    load_sfe<R, NX>(a.fsum[l] + m * Q::FE_P, e);
    std_filter_combine<R, NX>(acc, e);
  }
  store_sfe<R, NX>(a.fsum[l + 1] + j * Q::FE_P, acc);
}

template <typename R, int NX>
SS_DEV void load_std_prior(const ScanArgs<R>& a, int64_t i, SState<R, NX>& s) {
  const int64_t p = i * a.prior_stride;
  SS_UNROLL
  for (int r = 0; r < NX; ++r) {
    s.m[r] = a.m0[p * NX + r];
    SS_UNROLL
    for (int c = 0; c < NX; ++c) s.P[r][c] = a.L0[(p * NX + r) * NX + c];
  }
}

template <typename R, int NX>
__global__ void __launch_bounds__(128) std_filter_top_kernel(ScanArgs<R> a) {
  typedef SRec<R, NX, 1> Q;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.g.B) return;
  if (seq_inactive(a.active, i)) return;
  SState<R, NX> s;
  load_std_prior<R, NX>(a, i, s);
  if (a.filt_m != nullptr) store_straj<R, NX>(a.filt_m, a.filt_L, a.g.off[i] + i, s);
  const int L = a.g.L;
  const int64_t b = a.g.lvl[L][i], e = a.g.lvl[L][i + 1];
  if (b == e) {
    store_sst<R, NX>(a.fT + i * Q::ST_P, s);
    return;
  }
  for (int64_t m = b; m < e; ++m) {
    store_sst<R, NX>(a.fst[L] + m * Q::ST_P, s);
    if (m + 1 < e) {
      SFElem<R, NX> el;
      load_sfe<R, NX>(a.fsum[L] + m * Q::FE_P, el);
      std_filter_apply<R, NX>(s, el);
    }
  }
}

template <typename R, int NX>
__global__ void __launch_bounds__(128) std_filter_down_kernel(ScanArgs<R> a, int l) {
  typedef SRec<R, NX, 1> Q;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.g.lvl[l + 1][a.g.B]) return;
  int64_t i, m0, m1;
  group_of(a.g, l, j, i, m0, m1);
  if (seq_inactive(a.active, i)) return;
  SState<R, NX> s;
  load_sst<R, NX>(a.fst[l + 1] + j * Q::ST_P, s);
  for (int64_t m = m0; m < m1; ++m) {
    store_sst<R, NX>(a.fst[l] + m * Q::ST_P, s);
    if (m + 1 < m1) {
      SFElem<R, NX> el;
      load_sfe<R, NX>(a.fsum[l] + m * Q::FE_P, el);
      std_filter_apply<R, NX>(s, el);
    }
  }
}

// One chunk from its entry state: per step the smoothing element of the state
// before the step (emitted and folded into the chunk's smoothing summary), the
// log-likelihood term, then the step's filtering element applied in state form.
template <typename R, int NX, int NY>
__global__ void __launch_bounds__(128) std_filter_walk_kernel(ScanArgs<R> a) {
  typedef SRec<R, NX, NY> Q;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.g.lvl[1][a.g.B]) return;
  int64_t i, t0, t1;
  chunk_of(a.g, j, i, t0, t1);
  if (seq_inactive(a.active, i)) return;
  const int64_t base = a.g.off[i];
  SState<R, NX> s;
  load_sst<R, NX>(a.fst[1] + j * Q::ST_P, s);
  SSElem<R, NX> acc;
  double ll = 0.0;
  for (int64_t t = t0; t < t1; ++t) {
    SLin<R, NX, NY> l;
    load_slin<R, NX, NY>(a.lin + (base + t) * Q::LIN_P, l);
    R y[NY];
    SS_UNROLL
    for (int k = 0; k < NY; ++k) y[k] = a.ys[(base + t) * NY + k];
    if (a.emit_smoother) {
      SSElem<R, NX> se;
      std_smoother_element<R, NX>(l.F, l.Q, l.b, s, se);
      store_sse<R, NX>(a.selem + (base + t) * Q::SE_P, se);
      if (t == t0) acc = se; else std_smoother_fold<R, NX>(acc, se);
    }
    if (a.ll_chunk != nullptr) ll += (double)std_loglik<R, NX, NY>(l, s, y);
    SFElem<R, NX> e;
    std_filter_element<R, NX, NY>(l, y, e);
    std_filter_apply<R, NX>(s, e);
    if (a.filt_m != nullptr) store_straj<R, NX>(a.filt_m, a.filt_L, base + i + t + 1, s);
  }
  if (a.emit_smoother) store_sse<R, NX>(a.ssum[1] + j * Q::SE_P, acc);
  if (a.ll_chunk != nullptr) a.ll_chunk[j] = ll;
  if (t1 == a.g.off[i + 1] - base) store_sst<R, NX>(a.fT + i * Q::ST_P, s);
}

// Smoothing elements of a given filtered trajectory (standalone smoothing).
template <typename R, int NX, int NY>
__global__ void __launch_bounds__(128) std_smoother_leaf_kernel(ScanArgs<R> a) {
  typedef SRec<R, NX, NY> Q;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.g.lvl[1][a.g.B]) return;
  int64_t i, t0, t1;
  chunk_of(a.g, j, i, t0, t1);
  const int64_t base = a.g.off[i];
  SSElem<R, NX> acc;
  for (int64_t t = t0; t < t1; ++t) {
    SLin<R, NX, NY> l;
    load_slin<R, NX, NY>(a.lin + (base + t) * Q::LIN_P, l);
    SState<R, NX> s;
    load_straj<R, NX>(a.in_m, a.in_L, base + i + t, s);
    SSElem<R, NX> se;
    std_smoother_element<R, NX>(l.F, l.Q, l.b, s, se);
    store_sse<R, NX>(a.selem + (base + t) * Q::SE_P, se);
    if (t == t0) acc = se; else std_smoother_fold<R, NX>(acc, se);
  }
  store_sse<R, NX>(a.ssum[1] + j * Q::SE_P, acc);
}

template <typename R, int NX>
__global__ void __launch_bounds__(128) std_last_state_kernel(ScanArgs<R> a) {
  typedef SRec<R, NX, 1> Q;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.g.B) return;
  SState<R, NX> s;
  load_straj<R, NX>(a.in_m, a.in_L, a.g.off[i + 1] + i, s);
  store_sst<R, NX>(a.fT + i * Q::ST_P, s);
}

template <typename R, int NX>
__global__ void __launch_bounds__(128) std_smoother_up_kernel(ScanArgs<R> a, int l) {
  typedef SRec<R, NX, 1> Q;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.g.lvl[l + 1][a.g.B]) return;
  int64_t i, m0, m1;
  group_of(a.g, l, j, i, m0, m1);
  if (seq_inactive(a.active, i)) return;
  SSElem<R, NX> acc;
  load_sse<R, NX>(a.ssum[l] + m0 * Q::SE_P, acc);
  for (int64_t m = m0 + 1; m < m1; ++m) {
    SSElem<R, NX> e;
    load_sse<R, NX>(a.ssum[l] + m * Q::SE_P, e);
    std_smoother_fold<R, NX>(acc, e);
  }
  store_sse<R, NX>(a.ssum[l + 1] + j * Q::SE_P, acc);
}

// Convergence bookkeeping of one smoothed state (as accumulate_change).
template <typename R, int NX>
SS_DEV void std_accumulate_change(const ScanArgs<R>& a, int64_t i, int64_t s, const SState<R, NX>& st) {
  if (a.mse != nullptr) {
    double d2 = 0.0;
    SS_UNROLL
    for (int r = 0; r < NX; ++r) {
      const double d = (double)st.m[r] - (double)a.prev_m[s * NX + r];
      d2 += d * d;
    }
    atomicAdd(a.mse + i, d2);
  }
  if (a.flags != nullptr) {
    bool ok = true;
    SS_UNROLL
    for (int r = 0; r < NX; ++r) ok = ok && ss_isfinite(st.m[r]);
    if (!ok) atomicOr(a.flags + i, 1u);
  }
}

template <typename R, int NX>
SS_DEV void std_copy_state(const ScanArgs<R>& a, int64_t s) {
  SState<R, NX> st;
  load_straj<R, NX>(a.prev_m, a.prev_L, s, st);
  store_straj<R, NX>(a.out_m, a.out_L, s, st);
}

template <typename R, int NX>
__global__ void __launch_bounds__(128) std_smoother_top_kernel(ScanArgs<R> a) {
  typedef SRec<R, NX, 1> Q;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.g.B) return;
  const int64_t T = a.g.off[i + 1] - a.g.off[i];
  const int64_t sT = a.g.off[i] + i + T;
  if (seq_inactive(a.active, i)) {
    std_copy_state<R, NX>(a, sT);
    return;
  }
  SState<R, NX> s;
  load_sst<R, NX>(a.fT + i * Q::ST_P, s);
  store_straj<R, NX>(a.out_m, a.out_L, sT, s);
  std_accumulate_change<R, NX>(a, i, sT, s);
  const int L = a.g.L;
  const int64_t b = a.g.lvl[L][i], e = a.g.lvl[L][i + 1];
  for (int64_t m = e - 1; m >= b; --m) {
    store_sst<R, NX>(a.sst[L] + m * Q::ST_P, s);
    if (m > b) {
      SSElem<R, NX> el;
      load_sse<R, NX>(a.ssum[L] + m * Q::SE_P, el);
      std_smoother_apply<R, NX>(s, el);
    }
  }
}

template <typename R, int NX>
__global__ void __launch_bounds__(128) std_smoother_down_kernel(ScanArgs<R> a, int l) {
  typedef SRec<R, NX, 1> Q;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.g.lvl[l + 1][a.g.B]) return;
  int64_t i, m0, m1;
  group_of(a.g, l, j, i, m0, m1);
  if (seq_inactive(a.active, i)) return;
  SState<R, NX> s;
  load_sst<R, NX>(a.sst[l + 1] + j * Q::ST_P, s);
  for (int64_t m = m1 - 1; m >= m0; --m) {
    store_sst<R, NX>(a.sst[l] + m * Q::ST_P, s);
    if (m > m0) {
      SSElem<R, NX> el;
      load_sse<R, NX>(a.ssum[l] + m * Q::SE_P, el);
      std_smoother_apply<R, NX>(s, el);
    }
  }
}

template <typename R, int NX>
__global__ void __launch_bounds__(128) std_smoother_walk_kernel(ScanArgs<R> a) {
  typedef SRec<R, NX, 1> Q;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.g.lvl[1][a.g.B]) return;
  int64_t i, t0, t1;
  chunk_of(a.g, j, i, t0, t1);
  const int64_t base = a.g.off[i];
  if (seq_inactive(a.active, i)) {
    for (int64_t t = t0; t < t1; ++t) std_copy_state<R, NX>(a, base + i + t);
    return;
  }
  SState<R, NX> s;
  load_sst<R, NX>(a.sst[1] + j * Q::ST_P, s);
  for (int64_t t = t1 - 1; t >= t0; --t) {
    SSElem<R, NX> e;
    load_sse<R, NX>(a.selem + (base + t) * Q::SE_P, e);
    std_smoother_apply<R, NX>(s, e);
    store_straj<R, NX>(a.out_m, a.out_L, base + i + t, s);
    std_accumulate_change<R, NX>(a, i, base + i + t, s);
  }
}

}  // namespace ss
