// Square-root filter/smoother element algebra for one thread.
//
// Scan design.  The reference forms one filtering element per time step and
// runs jax.lax.associative_scan over all of them.  Here each sequence is cut
// into chunks: a chunk's elements are folded into one summary with the same
// associative combine (parsmooth/parallel/_operators.py:43-77 and 104-125),
// summaries are scanned level by level, and each chunk then walks its steps
// forward from the state that enters it.  The walk uses the state form of the
// combine: a prefix enters only through its (mean, chol) pair, so applying a
// filtering element to a state is one predict+update Kalman step, and applying
// a smoothing element is one RTS step.  Results equal the reference's up to
// floating-point association.
#pragma once
#include "ss_la.cuh"

namespace ss {

template <typename R, int NX>
struct State {
  R m[NX];
  R L[NX][NX];
};

// Filtering element / summary (A, b, U, eta, Z): p(x_end | x_start, y) =
// N(A x_start + b, U U^T) and the information eta, Z Z^T that the
// observations carry about x_start.
template <typename R, int NX>
struct FElem {
  R A[NX][NX];
  R b[NX];
  R U[NX][NX];
  R eta[NX];
  R Z[NX][NX];
};

// Smoothing element / summary (g, E, D): x_start = E x_end + g + N(0, D D^T).
template <typename R, int NX>
struct SElem {
  R g[NX];
  R E[NX][NX];
  R D[NX][NX];
};

// Linearised model at one step: x' = F x + bq + N(0, cQ cQ^T),
// y = H x' + c + N(0, cR cR^T).
template <typename R, int NX, int NY>
struct Lin {
  R F[NX][NX];
  R cQ[NX][NX];
  R bq[NX];
  R H[NY][NX];
  R cR[NY][NY];
  R c[NY];
};

// ---------------------------------------------------------------------------
// Filtering element of one step with a zero prior; the true prior enters as
// the initial state of the scan.  parsmooth/parallel/_filtering.py:115-146
// with m0 = 0, L0 = 0 (so m1 = bq and N1 = cQ).
template <typename R, int NX, int NY>
SS_DEV void filter_element(const Lin<R, NX, NY>& l, const R (&y)[NY], FElem<R, NX>& e) {
  constexpr int P = NX + NY;
  R M[P][P];
  // Psi = [[H cQ, cR], [cQ, 0]]
  SS_UNROLL
  for (int r = 0; r < NY; ++r) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) {
      R s = R(0);
      SS_UNROLL
      for (int k = j; k < NX; ++k) s += l.H[r][k] * l.cQ[k][j];
      M[r][j] = s;
    }
    SS_UNROLL
    for (int j = 0; j < NY; ++j) M[r][NX + j] = l.cR[r][j];
  }
  SS_UNROLL
  for (int r = 0; r < NX; ++r) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) M[NY + r][j] = l.cQ[r][j];
    SS_UNROLL
    for (int j = 0; j < NY; ++j) M[NY + r][NX + j] = R(0);
  }
  tria_sp<R, P, P, PatBlocks<NY, NX>>(M);
  // Psi11 = M[0:NY, 0:NY], Psi21 = M[NY:, 0:NY], U = M[NY:, NY:]
  R W[NY][NX];  // Psi11^{-1} H F
  matmul<R, NY, NX, NX>(l.H, l.F, W);
  solve_lower<R, NY, NX>(M, W);
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) {
      R s = l.F[i][j];
      SS_UNROLL
      for (int k = 0; k < NY; ++k) s -= M[NY + i][k] * W[k][j];
      e.A[i][j] = s;                       // A = F - K H F, K = Psi21 Psi11^{-1}
    }
  }
  R r[NY];  // Psi11^{-1} (y - H bq - c)
  SS_UNROLL
  for (int k = 0; k < NY; ++k) {
    R s = y[k] - l.c[k];
    SS_UNROLL
    for (int j = 0; j < NX; ++j) s -= l.H[k][j] * l.bq[j];
    r[k] = s;
  }
  solve_lower_vec<R, NY>(M, r);
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    R s = l.bq[i];
    SS_UNROLL
    for (int k = 0; k < NY; ++k) s += M[NY + i][k] * r[k];
    e.b[i] = s;                            // b = m1 + K (y - H m1 - c)
    R t = R(0);
    SS_UNROLL
    for (int k = 0; k < NY; ++k) t += W[k][i] * r[k];
    e.eta[i] = t;                          // eta = Z Psi11^{-1} (y - H b - c), Z = W^T
    SS_UNROLL
    for (int j = 0; j < NX; ++j) e.U[i][j] = (j <= i) ? M[NY + i][NY + j] : R(0);
  }
  if constexpr (NX > NY) {
    SS_UNROLL
    for (int i = 0; i < NX; ++i) {
      SS_UNROLL
      for (int j = 0; j < NX; ++j) e.Z[i][j] = (j < NY) ? W[j][i] : R(0);
    }
  } else {
    R Zt[NX][NY];
    SS_UNROLL
    for (int i = 0; i < NX; ++i) {
      SS_UNROLL
      for (int j = 0; j < NY; ++j) Zt[i][j] = W[j][i];
    }
    tria<R, NX, NY>(Zt);
    SS_UNROLL
    for (int i = 0; i < NX; ++i) {
      SS_UNROLL
      for (int j = 0; j < NX; ++j) e.Z[i][j] = Zt[i][j];
    }
  }
}

// Zero pattern of xi_core's input [[L^T Z2, I], [Z2, 0]] when only the first
// ZC columns of Z2 can be non-zero.
template <int NX, int ZC>
struct XiPat {
  __host__ __device__ static constexpr bool nz(int r, int c) {
    if (r < NX) return c < ZC || c - NX == r;
    return c < ZC;
  }
};

// Zero patterns of a filtering element's Z (filter_element): with NX > NY only
// its first NY columns are non-zero, otherwise it is lower triangular.  Every
// combined summary has a lower-triangular Z.  ZK: leading full columns of a Z
// that is otherwise lower triangular; ZC: columns that can be non-zero.
template <int NX, int NY>
struct ElemZ {
  static constexpr int ZK = NX > NY ? NY : 0;
  static constexpr int ZC = NX > NY ? NY : NX;
};

// Xi = tria([[L^T Z2, I], [Z2, 0]]) and V = Xi11^{-1} L^T, the common core of
// the filtering combine and of its state form.  Columns >= ZC of Z2 are zero.
template <typename R, int NX, int ZC = NX>
SS_DEV void xi_core(const R (&L)[NX][NX], const R (&Z2)[NX][NX], R (&X)[2 * NX][2 * NX],
                    R (&V)[NX][NX]) {
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) {
      R s = R(0);
      if (j < ZC) {
        SS_UNROLL
        for (int k = i; k < NX; ++k) s += L[k][i] * Z2[k][j];   // L lower: L[k][i] = 0 for k < i
      }
      X[i][j] = s;
      X[i][NX + j] = (i == j) ? R(1) : R(0);
      X[NX + i][j] = (j < ZC) ? Z2[i][j] : R(0);
      X[NX + i][NX + j] = R(0);
    }
  }
  tria_sp<R, 2 * NX, 2 * NX, XiPat<NX, ZC>>(X);
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) V[i][j] = L[j][i];
  }
  solve_lower<R, NX, NX>(X, V);
}

// a <- a (x) e, a earlier, e later.  parsmooth/parallel/_operators.py:43-77,
// rewritten with V = Xi11^{-1} U1^T and N = (I - V^T Xi21^T) A1:
//   A = A2 N, b = A2 (I - V^T Xi21^T)(b1 + U1 U1^T eta2) + b2,
//   eta = N^T (eta2 - Z2 Z2^T b1) + eta1, U = tria([A2 V^T, U2]),
//   Z = tria([A1^T Xi22, Z1]).
// AZK: a.Z is lower triangular apart from its first AZK columns; EZC: only the
// first EZC columns of e.Z can be non-zero (ElemZ gives both for elements).
template <typename R, int NX, int AZK = NX, int EZC = NX>
SS_DEV void filter_combine(FElem<R, NX>& a, const FElem<R, NX>& e) {
  R X[2 * NX][2 * NX];
  R V[NX][NX];
  xi_core<R, NX, EZC>(a.U, e.Z, X, V);
  // Z = tria([A1^T Xi22, Z1])
  {
    R W[NX][2 * NX];
    SS_UNROLL
    for (int i = 0; i < NX; ++i) {
      SS_UNROLL
      for (int j = 0; j < NX; ++j) {
        R s = R(0);
        SS_UNROLL
        for (int k = j; k < NX; ++k) s += a.A[k][i] * X[NX + k][NX + j];
        W[i][j] = s;
        W[i][NX + j] = a.Z[i][j];
      }
    }
    tria_sp<R, NX, 2 * NX, PatBlocks<NX, NX, AZK>>(W);
    SS_UNROLL
    for (int i = 0; i < NX; ++i) {
      SS_UNROLL
      for (int j = 0; j < NX; ++j) a.Z[i][j] = W[i][j];
    }
  }
  // v = b1 + U1 (U1^T eta2); w = v - V^T (Xi21^T v);  u = eta2 - Z2 (Z2^T b1)
  R v[NX], u[NX];
  {
    R t[NX], z[NX];
    matvec_t<R, NX, NX>(a.U, e.eta, t);
    matvec_t<R, NX, NX>(e.Z, a.b, z);
    SS_UNROLL
    for (int i = 0; i < NX; ++i) {
      R s = a.b[i], q = e.eta[i];
      SS_UNROLL
      for (int k = 0; k <= i; ++k) s += a.U[i][k] * t[k];
      SS_UNROLL
      for (int k = 0; k < NX; ++k) q -= e.Z[i][k] * z[k];
      v[i] = s;
      u[i] = q;
    }
    R x[NX];
    SS_UNROLL
    for (int j = 0; j < NX; ++j) {
      R s = R(0);
      SS_UNROLL
      for (int k = 0; k < NX; ++k) s += X[NX + k][j] * v[k];
      x[j] = s;                                 // Xi21^T v (Xi21 is a full block)
    }
    SS_UNROLL
    for (int i = 0; i < NX; ++i) {
      R s = v[i];
      SS_UNROLL
      for (int k = 0; k < NX; ++k) s -= V[k][i] * x[k];
      t[i] = s;                                 // w
    }
    matvec<R, NX, NX>(e.A, t, z);
    SS_UNROLL
    for (int i = 0; i < NX; ++i) a.b[i] = z[i] + e.b[i];
  }
  // N = A1 - V^T (Xi21^T A1)
  R N[NX][NX];
  {
    R T[NX][NX];
    SS_UNROLL
    for (int i = 0; i < NX; ++i) {
      SS_UNROLL
      for (int j = 0; j < NX; ++j) {
        R s = R(0);
        SS_UNROLL
        for (int k = 0; k < NX; ++k) s += X[NX + k][i] * a.A[k][j];
        T[i][j] = s;
      }
    }
    SS_UNROLL
    for (int i = 0; i < NX; ++i) {
      SS_UNROLL
      for (int j = 0; j < NX; ++j) {
        R s = a.A[i][j];
        SS_UNROLL
        for (int k = 0; k < NX; ++k) s -= V[k][i] * T[k][j];
        N[i][j] = s;
      }
    }
  }
  // eta = N^T u + eta1
  SS_UNROLL
  for (int j = 0; j < NX; ++j) {
    R s = a.eta[j];
    SS_UNROLL
    for (int i = 0; i < NX; ++i) s += N[i][j] * u[i];
    a.eta[j] = s;
  }
  // U = tria([A2 V^T, U2])
  {
    R W[NX][2 * NX];
    SS_UNROLL
    for (int i = 0; i < NX; ++i) {
      SS_UNROLL
      for (int j = 0; j < NX; ++j) {
        R s = R(0);
        SS_UNROLL
        for (int k = 0; k < NX; ++k) s += e.A[i][k] * V[j][k];
        W[i][j] = s;
        W[i][NX + j] = e.U[i][j];
      }
    }
    tria_sp<R, NX, 2 * NX, PatBlocks<NX, NX>>(W);
    SS_UNROLL
    for (int i = 0; i < NX; ++i) {
      SS_UNROLL
      for (int j = 0; j < NX; ++j) a.U[i][j] = (j <= i) ? W[i][j] : R(0);
    }
  }
  // A = A2 N
  matmul<R, NX, NX, NX>(e.A, N, a.A);
}

// Zero pattern of [Z, W^T] in filter_extend: Z lower triangular apart from its
// first ZK columns, W^T (NX x NY) full.
template <int NX, int ZK>
struct ZExtPat {
  __host__ __device__ static constexpr bool nz(int r, int c) { return c >= NX || c <= r || c < ZK; }
};

// a <- a (x) filter_element(l, y), computed without the element: the summary
// of a chunk's steps, x_t | x_s ~ N(A x_s + b, U U^T) with information
// (eta, Z Z^T) on the state x_s before the chunk, extended by one Kalman step
// in conditional form.  Predict: Ap = F A, bp = F b + bq, Up = tria([F U, cQ]);
// update with y = H x + c + N(0, cR cR^T): tria([[H Up, cR], [Up, 0]]) gives
// Psi11 (innovation factor), Psi21 and U' = Psi22, and with
// W = Psi11^{-1} H Ap and r = Psi11^{-1} (y - H bp - c):
//   A' = Ap - Psi21 W,  b' = bp + Psi21 r,  eta' = eta + W^T r,
//   Z' = tria([Z, W^T]).
// The result is the associative combine of parsmooth/parallel/_operators.py:43-77
// applied to the element of parsmooth/parallel/_filtering.py:115-146 (the same
// conditional distribution and information), at about half its arithmetic.
// AZK: a.Z is lower triangular apart from its first AZK columns.
template <typename R, int NX, int NY, int AZK = NX>
SS_DEV void filter_extend(FElem<R, NX>& a, const Lin<R, NX, NY>& l, const R (&y)[NY]) {
  constexpr int P = NX + NY;
  R M[P][P];
  {
    R X[NX][2 * NX];
    SS_UNROLL
    for (int i = 0; i < NX; ++i) {
      SS_UNROLL
      for (int j = 0; j < NX; ++j) {
        R q = R(0);
        SS_UNROLL
        for (int k = j; k < NX; ++k) q += l.F[i][k] * a.U[k][j];
        X[i][j] = q;
        X[i][NX + j] = l.cQ[i][j];
      }
    }
    tria_sp<R, NX, 2 * NX, PatBlocks<NX, NX>>(X);
    SS_UNROLL
    for (int r = 0; r < NY; ++r) {
      SS_UNROLL
      for (int j = 0; j < NX; ++j) {
        R q = R(0);
        SS_UNROLL
        for (int k = j; k < NX; ++k) q += l.H[r][k] * X[k][j];
        M[r][j] = q;
      }
      SS_UNROLL
      for (int j = 0; j < NY; ++j) M[r][NX + j] = l.cR[r][j];
    }
    SS_UNROLL
    for (int r = 0; r < NX; ++r) {
      SS_UNROLL
      for (int j = 0; j < NX; ++j) M[NY + r][j] = X[r][j];
      SS_UNROLL
      for (int j = 0; j < NY; ++j) M[NY + r][NX + j] = R(0);
    }
  }
  tria_sp<R, P, P, PatBlocks<NY, NX>>(M);
  R Ap[NX][NX], bp[NX];
  matmul<R, NX, NX, NX>(l.F, a.A, Ap);
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    R q = l.bq[i];
    SS_UNROLL
    for (int k = 0; k < NX; ++k) q += l.F[i][k] * a.b[k];
    bp[i] = q;
  }
  R W[NY][NX], r[NY];
  matmul<R, NY, NX, NX>(l.H, Ap, W);
  solve_lower<R, NY, NX>(M, W);
  SS_UNROLL
  for (int k = 0; k < NY; ++k) {
    R q = y[k] - l.c[k];
    SS_UNROLL
    for (int j = 0; j < NX; ++j) q -= l.H[k][j] * bp[j];
    r[k] = q;
  }
  solve_lower_vec<R, NY>(M, r);
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    R q = bp[i], e = a.eta[i];
    SS_UNROLL
    for (int k = 0; k < NY; ++k) {
      q += M[NY + i][k] * r[k];
      e += W[k][i] * r[k];
    }
    a.b[i] = q;
    a.eta[i] = e;
    SS_UNROLL
    for (int j = 0; j < NX; ++j) {
      R s = Ap[i][j];
      SS_UNROLL
      for (int k = 0; k < NY; ++k) s -= M[NY + i][k] * W[k][j];
      a.A[i][j] = s;
      a.U[i][j] = (j <= i) ? M[NY + i][NY + j] : R(0);
    }
  }
  R Zx[NX][NX + NY];
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) Zx[i][j] = a.Z[i][j];
    SS_UNROLL
    for (int k = 0; k < NY; ++k) Zx[i][NX + k] = W[k][i];
  }
  // The one FP32 range-guarded tria of the pass (ss_la.cuh): W carries the chunk's product
  // of linearised transitions (Ap = F A), which a divergent Gauss-Newton iterate can grow
  // past FP32's range for squares; the other trias of the pass see bounded entries.
  tria_sp<R, NX, NX + NY, ZExtPat<NX, AZK>, true>(Zx);
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) a.Z[i][j] = (j <= i) ? Zx[i][j] : R(0);
  }
}

// State form of the filtering combine: (m, L) <- combine((., m, L, ., .), e)
// restricted to its (b, U) outputs.
template <typename R, int NX>
SS_DEV void filter_apply(State<R, NX>& s, const FElem<R, NX>& e) {
  R X[2 * NX][2 * NX];
  R V[NX][NX];
  xi_core<R, NX>(s.L, e.Z, X, V);
  R v[NX], t[NX], x[NX], w[NX];
  matvec_t<R, NX, NX>(s.L, e.eta, t);
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    R q = s.m[i];
    SS_UNROLL
    for (int k = 0; k <= i; ++k) q += s.L[i][k] * t[k];
    v[i] = q;
  }
  SS_UNROLL
  for (int j = 0; j < NX; ++j) {
    R q = R(0);
    SS_UNROLL
    for (int k = 0; k < NX; ++k) q += X[NX + k][j] * v[k];
    x[j] = q;
  }
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    R q = v[i];
    SS_UNROLL
    for (int k = 0; k < NX; ++k) q -= V[k][i] * x[k];
    w[i] = q;
  }
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    R q = e.b[i];
    SS_UNROLL
    for (int k = 0; k < NX; ++k) q += e.A[i][k] * w[k];
    s.m[i] = q;
  }
  R W[NX][2 * NX];
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) {
      R q = R(0);
      SS_UNROLL
      for (int k = 0; k < NX; ++k) q += e.A[i][k] * V[j][k];
      W[i][j] = q;
      W[i][NX + j] = e.U[i][j];
    }
  }
  tria_sp<R, NX, 2 * NX, PatBlocks<NX, NX>>(W);
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) s.L[i][j] = (j <= i) ? W[i][j] : R(0);
  }
}

// ---------------------------------------------------------------------------
// Smoothing element of step t from the filtered state (m, L) at t and the
// transition linearised at nominal[t] (parsmooth/parallel/_smoothing.py:72-85):
// Phi = tria([[F L, cQ], [L, 0]]), E = Phi21 Phi11^{-1}, g = m - E (F m + bq),
// D = Phi22.  Phi is left in X: Phi11 is also the predicted square root.
template <typename R, int NX>
SS_DEV void smoother_element(const R (&F)[NX][NX], const R (&cQ)[NX][NX], const R (&bq)[NX],
                             const State<R, NX>& s, SElem<R, NX>& se, R (&X)[2 * NX][2 * NX],
                             R (&mp)[NX]) {
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) {
      R q = R(0);
      SS_UNROLL
      for (int k = j; k < NX; ++k) q += F[i][k] * s.L[k][j];
      X[i][j] = q;
      X[i][NX + j] = cQ[i][j];
      X[NX + i][j] = s.L[i][j];
      X[NX + i][NX + j] = R(0);
    }
  }
  tria_sp<R, 2 * NX, 2 * NX, PatBlocks<NX, NX>>(X);
  // E^T = Phi11^{-T} Phi21^T
  R Et[NX][NX];
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) Et[i][j] = X[NX + j][i];
  }
  solve_lower_T<R, NX, NX>(X, Et);
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    R q = bq[i];
    SS_UNROLL
    for (int k = 0; k < NX; ++k) q += F[i][k] * s.m[k];
    mp[i] = q;
  }
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    R q = s.m[i];
    SS_UNROLL
    for (int k = 0; k < NX; ++k) q -= Et[k][i] * mp[k];
    se.g[i] = q;
    SS_UNROLL
    for (int j = 0; j < NX; ++j) {
      se.E[i][j] = Et[j][i];
      se.D[i][j] = (j <= i) ? X[NX + i][NX + j] : R(0);
    }
  }
}

// One filter step from the filtered state at t to t+1 using the predicted
// moments (mp, Phi11) of smoother_element: the square-root update of
// parsmooth/sequential/_filtering.py:89-108.  Returns the step's predictive
// log-likelihood (the same quantity as parsmooth/parallel/_filtering.py:149-154).
template <typename R, int NX, int NY>
SS_DEV R filter_update(State<R, NX>& s, const Lin<R, NX, NY>& l, const R (&y)[NY],
                       const R (&X)[2 * NX][2 * NX], const R (&mp)[NX]) {
  constexpr int P = NX + NY;
  R M[P][P];
  SS_UNROLL
  for (int r = 0; r < NY; ++r) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) {
      R q = R(0);
      SS_UNROLL
      for (int k = j; k < NX; ++k) q += l.H[r][k] * X[k][j];
      M[r][j] = q;
    }
    SS_UNROLL
    for (int j = 0; j < NY; ++j) M[r][NX + j] = l.cR[r][j];
  }
  SS_UNROLL
  for (int r = 0; r < NX; ++r) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) M[NY + r][j] = X[r][j];
    SS_UNROLL
    for (int j = 0; j < NY; ++j) M[NY + r][NX + j] = R(0);
  }
  tria_sp<R, P, P, PatBlocks<NY, NX>>(M);
  R r[NY];
  SS_UNROLL
  for (int k = 0; k < NY; ++k) {
    R q = y[k] - l.c[k];
    SS_UNROLL
    for (int j = 0; j < NX; ++j) q -= l.H[k][j] * mp[j];
    r[k] = q;
  }
  solve_lower_vec<R, NY>(M, r);
  R ll = R(0);
  SS_UNROLL
  for (int k = 0; k < NY; ++k) ll += r[k] * r[k] + R(2) * ss_log(ss_abs(M[k][k]));
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    R q = mp[i];
    SS_UNROLL
    for (int k = 0; k < NY; ++k) q += M[NY + i][k] * r[k];
    s.m[i] = q;
    SS_UNROLL
    for (int j = 0; j < NX; ++j) s.L[i][j] = (j <= i) ? M[NY + i][NY + j] : R(0);
  }
  return R(-0.5) * ll;   // the -NY/2 log(2 pi) constant is added by the caller in FP64
}

// acc <- e (x) acc for the reverse scan: acc covers earlier steps, e is the
// next (later) element.  parsmooth/parallel/_operators.py:104-125 with
// elem1 = e, elem2 = acc: g = E_acc g_e + g_acc, E = E_acc E_e,
// D = tria([E_acc D_e, D_acc]).
template <typename R, int NX>
SS_DEV void smoother_fold(SElem<R, NX>& a, const SElem<R, NX>& e) {
  R W[NX][2 * NX];
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) {
      R q = R(0);
      SS_UNROLL
      for (int k = j; k < NX; ++k) q += a.E[i][k] * e.D[k][j];
      W[i][j] = q;
      W[i][NX + j] = a.D[i][j];
    }
  }
  tria_sp<R, NX, 2 * NX, PatBlocks<NX, NX>>(W);
  R g[NX];
  matvec<R, NX, NX>(a.E, e.g, g);
  R E[NX][NX];
  matmul<R, NX, NX, NX>(a.E, e.E, E);
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    a.g[i] += g[i];
    SS_UNROLL
    for (int j = 0; j < NX; ++j) {
      a.E[i][j] = E[i][j];
      a.D[i][j] = (j <= i) ? W[i][j] : R(0);
    }
  }
}

// State form of the smoothing combine: smoothed (m, L) at the end of the
// element's range -> at its start: m <- E m + g, L <- tria([E L, D])
// (parsmooth/sequential/_smoothing.py:60-77 in element form).
template <typename R, int NX>
SS_DEV void smoother_apply(State<R, NX>& s, const SElem<R, NX>& e) {
  R W[NX][2 * NX];
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) {
      R q = R(0);
      SS_UNROLL
      for (int k = j; k < NX; ++k) q += e.E[i][k] * s.L[k][j];
      W[i][j] = q;
      W[i][NX + j] = e.D[i][j];
    }
  }
  tria_sp<R, NX, 2 * NX, PatBlocks<NX, NX>>(W);
  R m[NX];
  matvec<R, NX, NX>(e.E, s.m, m);
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    s.m[i] = m[i] + e.g[i];
    SS_UNROLL
    for (int j = 0; j < NX; ++j) s.L[i][j] = (j <= i) ? W[i][j] : R(0);
  }
}

}  // namespace ss
