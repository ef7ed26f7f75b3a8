// Large-state ("dense") square-root filter and smoother for linear models.
//
// Beyond nx = 5 one thread cannot hold a chunk's square-root summary, so this
// path gives every scan item (a chunk of C steps, a group of G summaries, a
// sequence at the top level) to one warp, with the matrices in the warp's
// shared memory and the warp-cooperative algebra of ss_dense_la.cuh.  The
// scan (levels, chunk and group geometry, state form of the walks, per-step
// smoothing elements, log-likelihood and convergence bookkeeping) is the one
// of the register path (ss_pipeline.cuh); the operators restate
// parsmooth/parallel/_operators.py:43-77 and 104-125 and the elements
// parsmooth/parallel/_filtering.py:115-146 and _smoothing.py:72-85.
//
// Linear models only (the registry has no nonlinear model with nx > 5).  The
// statistical linear regression of x -> A x + N(qm, qc qc^T) is exact for
// every rule (F = A, chol = qc, b = qm), so there is no per-step
// linearisation, and every filtering element has the same matrix part
// (A, U, Z) because elements carry a zero prior.  The leaf therefore folds a
// chunk with precomputed per-position coefficients: folding j elements with
// element j+1 maps the vectors linearly,
//   b' = M_j b + B_j r + bq,   eta' = eta + C_j r - D_j b,
// r = Psi11^{-1} (y - c - H bq), with M_j = A2 G, G = I - Vt Xi21^T,
// N_j = G A1, B_j = M_j U1 U1^T W^T + Psi21, C_j = N_j^T W^T,
// D_j = N_j^T Z2 Z2^T (the combine's own algebra regrouped), and the fold's
// matrix part after j elements is read from the same table.
#pragma once
#include "ss_dense_la.cuh"
#include "ss_run.cuh"

namespace ss {
namespace dense {

template <typename R, int NX, int NY>
struct DS {
  static_assert(NX % 4 == 0 && NY % 4 == 0, "dense dimensions are multiples of 4");
  static_assert(NX <= 32 && NY <= 32, "dense dimensions are at most 32");
  static constexpr int W = Vec<R>::n;
  static constexpr int LDN = Pad<R, NX>::ld;
  static constexpr int LDY = Pad<R, NY>::ld;
  static constexpr int LD2 = Pad<R, 2 * NX>::ld;
  static constexpr int LDP = Pad<R, NX + NY>::ld;
  static constexpr int VN = Pad<R, NX>::n;
  static constexpr int VY = Pad<R, NY>::n;
  static constexpr int VB = tria_scratch<R, (2 * NX > NX + NY ? 2 * NX : NX + NY)>();
  static constexpr int MN = NX * LDN;            // NX x NX
  static constexpr int MY = NX * LDY;            // NX x NY
  static constexpr int M2 = 2 * NX * LD2;        // 2NX x 2NX
  static constexpr int MW = NX * LD2;            // NX x 2NX
  static constexpr int MP = (NX + NY) * LDP;     // (NX+NY) x (NX+NY)
  static constexpr int MPHI = M2 > MP ? M2 : MP; // Phi, then Psi, in one region
  // global records (row-major, no padding): filtering summary, smoothing
  // element, state
  static constexpr int FE = 3 * NX * NX + 2 * NX;
  static constexpr int SE = 2 * NX * NX + NX;
  static constexpr int ST = NX * NX + NX;
  // fold table: constants, then per-position matrix parts (1..C), then
  // per-position coefficients (1..C-1, stored transposed)
  static constexpr int TC = (NY * NY + 2 * NX * NY + NY + 3) / 4 * 4;
  static constexpr int TS = 3 * NX * NX;
  static constexpr int TK = 2 * NX * NX + 2 * NX * NY;
  static size_t table_elems(int C) { return (size_t)TC + (size_t)C * TS + (size_t)(C > 1 ? C - 1 : 0) * TK; }
  static SS_DEV size_t summ_off(int j) { return (size_t)TC + (size_t)(j - 1) * TS; }
  static SS_DEV size_t coef_off(int C, int j) { return (size_t)TC + (size_t)C * TS + (size_t)(j - 1) * TK; }
};

template <typename R>
struct DenseArgs {
  ScanArgs<R> s;
  const R* F;   // transition matrix (NX x NX)
  const R* qm;  // transition noise mean
  const R* qc;  // transition noise chol
  const R* H;   // observation matrix (NY x NX)
  const R* rm;  // observation noise mean
  const R* rc;  // observation noise chol
  R* tab;       // fold table
  int C;
};

// Shared views of one filtering summary / smoothing element.
template <typename R>
struct FB {
  R *A, *U, *Z, *b, *eta;
};
template <typename R>
struct SB {
  R *E, *D, *g;
};

template <typename R, int NX, int NY>
SS_DEV FB<R> carve_fb(R*& p) {
  typedef DS<R, NX, NY> S;
  FB<R> f;
  f.A = p; p += S::MN;
  f.U = p; p += S::MN;
  f.Z = p; p += S::MN;
  f.b = p; p += S::VN;
  f.eta = p; p += S::VN;
  return f;
}
template <typename R, int NX, int NY>
SS_DEV SB<R> carve_sb(R*& p) {
  typedef DS<R, NX, NY> S;
  SB<R> f;
  f.E = p; p += S::MN;
  f.D = p; p += S::MN;
  f.g = p; p += S::VN;
  return f;
}
template <typename R, int NX, int NY>
__host__ __device__ constexpr int fb_elems() { return 3 * DS<R, NX, NY>::MN + 2 * DS<R, NX, NY>::VN; }
template <typename R, int NX, int NY>
__host__ __device__ constexpr int sb_elems() { return 2 * DS<R, NX, NY>::MN + DS<R, NX, NY>::VN; }

// ----------------------------------------------------------------------------- record I/O

template <typename R, int NX, int NY>
SS_DEV void load_fb(FB<R> f, const R* g) {
  typedef DS<R, NX, NY> S;
  g2s<R, NX, NX, S::LDN>(f.A, g);
  g2s<R, NX, NX, S::LDN>(f.U, g + NX * NX);
  g2s<R, NX, NX, S::LDN>(f.Z, g + 2 * NX * NX);
  const int l = lane_id();
  if (l < NX) {
    f.b[l] = g[3 * NX * NX + l];
    f.eta[l] = g[3 * NX * NX + NX + l];
  }
  __syncwarp();
}
template <typename R, int NX, int NY>
SS_DEV void store_fb(R* g, FB<R> f) {
  typedef DS<R, NX, NY> S;
  s2g<R, NX, NX, S::LDN>(g, f.A);
  s2g<R, NX, NX, S::LDN>(g + NX * NX, f.U);
  s2g<R, NX, NX, S::LDN>(g + 2 * NX * NX, f.Z);
  const int l = lane_id();
  if (l < NX) {
    g[3 * NX * NX + l] = f.b[l];
    g[3 * NX * NX + NX + l] = f.eta[l];
  }
  __syncwarp();
}
template <typename R, int NX, int NY>
SS_DEV void load_sb(SB<R> f, const R* g) {
  typedef DS<R, NX, NY> S;
  g2s<R, NX, NX, S::LDN>(f.E, g);
  g2s<R, NX, NX, S::LDN>(f.D, g + NX * NX);
  const int l = lane_id();
  if (l < NX) f.g[l] = g[2 * NX * NX + l];
  __syncwarp();
}
template <typename R, int NX, int NY>
SS_DEV void store_sb(R* g, SB<R> f) {
  typedef DS<R, NX, NY> S;
  s2g<R, NX, NX, S::LDN>(g, f.E);
  s2g<R, NX, NX, S::LDN>(g + NX * NX, f.D);
  const int l = lane_id();
  if (l < NX) g[2 * NX * NX + l] = f.g[l];
  __syncwarp();
}
// state record: L then m
template <typename R, int NX, int NY>
SS_DEV void load_st(R* L, R* m, const R* g) {
  g2s<R, NX, NX, DS<R, NX, NY>::LDN>(L, g);
  const int l = lane_id();
  if (l < NX) m[l] = g[NX * NX + l];
  __syncwarp();
}
template <typename R, int NX, int NY>
SS_DEV void store_st(R* g, const R* L, const R* m) {
  s2g<R, NX, NX, DS<R, NX, NY>::LDN>(g, L);
  const int l = lane_id();
  if (l < NX) g[NX * NX + l] = m[l];
  __syncwarp();
}
// state s of a user trajectory (means (N, NX), factors (N, NX, NX))
template <typename R, int NX, int NY>
SS_DEV void load_traj(R* L, R* m, const R* tm, const R* tL, int64_t s) {
  g2s<R, NX, NX, DS<R, NX, NY>::LDN>(L, tL + s * NX * NX);
  const int l = lane_id();
  if (l < NX) m[l] = tm[s * NX + l];
  __syncwarp();
}
template <typename R, int NX, int NY>
SS_DEV void store_traj(R* tm, R* tL, int64_t s, const R* L, const R* m) {
  s2g<R, NX, NX, DS<R, NX, NY>::LDN>(tL + s * NX * NX, L);
  const int l = lane_id();
  if (l < NX) tm[s * NX + l] = m[l];
  __syncwarp();
}

// ----------------------------------------------------------------------------- operators

// Scratch of the filtering combine and its state form.
template <typename R>
struct FS {
  R *Xi, *Wm, *Vt, *T, *N, *v1, *v2, *v3, *v4, *vb;
};
template <typename R, int NX, int NY>
SS_DEV FS<R> carve_fs(R*& p) {
  typedef DS<R, NX, NY> S;
  FS<R> f;
  f.Xi = p; p += S::M2;
  f.Wm = p; p += S::MW;
  f.Vt = p; p += S::MN;
  f.T = p; p += S::MN;
  f.N = p; p += S::MN;
  f.v1 = p; p += S::VN;
  f.v2 = p; p += S::VN;
  f.v3 = p; p += S::VN;
  f.v4 = p; p += S::VN;
  f.vb = p; p += S::VB;
  return f;
}
template <typename R, int NX, int NY>
__host__ __device__ constexpr int fs_elems() {
  typedef DS<R, NX, NY> S;
  return S::M2 + S::MW + 3 * S::MN + 4 * S::VN + S::VB;
}

// Xi = tria([[U^T Z2, I], [Z2, 0]]) and Vt = U Xi11^{-T} (V^T of the register path).
template <typename R, int NX, int NY>
SS_DEV void xi_core(const R* U, const R* Z2, FS<R> s) {
  typedef DS<R, NX, NY> S;
  mm<R, NX, NX, NX, true, false, S::LDN, S::LDN, S::LD2>(s.Xi, U, Z2);
  fill_diag<R, NX, NX, S::LD2>(s.Xi + NX, R(1));
  copy<R, NX, NX, false, S::LD2, S::LDN>(s.Xi + NX * S::LD2, Z2);
  fill_diag<R, NX, NX, S::LD2>(s.Xi + NX * S::LD2 + NX, R(0));
  tria<R, 2 * NX, 2 * NX, S::LD2>(s.Xi, s.vb);
  copy<R, NX, NX, false, S::LDN, S::LDN>(s.Vt, U);
  trsm_rlt<R, NX, NX, S::LDN, S::LD2>(s.Vt, s.Xi);
}

// a <- a (x) e, a earlier (parsmooth/parallel/_operators.py:43-77), with
// V = Xi11^{-1} U1^T and N = (I - V^T Xi21^T) A1 as in the register path.
template <typename R, int NX, int NY>
SS_DEV void combine(FB<R> a, FB<R> e, FS<R> s) {
  typedef DS<R, NX, NY> S;
  const int l = lane_id();
  xi_core<R, NX, NY>(a.U, e.Z, s);
  const R* X21 = s.Xi + NX * S::LD2;
  const R* X22 = X21 + NX;
  // v = b1 + U1 U1^T eta2, u = eta2 - Z2 Z2^T b1, w = v - Vt Xi21^T v
  const R t1 = rowdot<R, NX, NX, true, S::LDN>(a.U, e.eta, l);
  const R t2 = rowdot<R, NX, NX, true, S::LDN>(e.Z, a.b, l);
  if (l < NX) {
    s.v1[l] = t1;
    s.v2[l] = t2;
  }
  __syncwarp();
  const R v = (l < NX ? a.b[l] : R(0)) + rowdot<R, NX, NX, false, S::LDN>(a.U, s.v1, l);
  const R u = (l < NX ? e.eta[l] : R(0)) - rowdot<R, NX, NX, false, S::LDN>(e.Z, s.v2, l);
  __syncwarp();
  if (l < NX) {
    s.v3[l] = v;
    s.v4[l] = u;
  }
  __syncwarp();
  const R x = rowdot<R, NX, NX, true, S::LD2>(X21, s.v3, l);
  if (l < NX) s.v1[l] = x;
  __syncwarp();
  const R w = v - rowdot<R, NX, NX, false, S::LDN>(s.Vt, s.v1, l);
  if (l < NX) s.v2[l] = w;
  __syncwarp();
  const R bnew = rowdot<R, NX, NX, false, S::LDN>(e.A, s.v2, l) + (l < NX ? e.b[l] : R(0));
  // N = A1 - Vt (Xi21^T A1)
  mm<R, NX, NX, NX, true, false, S::LD2, S::LDN, S::LDN>(s.T, X21, a.A);
  copy<R, NX, NX, false, S::LDN, S::LDN>(s.N, a.A);
  mm<R, NX, NX, NX, false, false, S::LDN, S::LDN, S::LDN>(s.N, s.Vt, s.T, R(-1), true);
  const R enew = rowdot<R, NX, NX, true, S::LDN>(s.N, s.v4, l) + (l < NX ? a.eta[l] : R(0));
  // Z = tria([A1^T Xi22, Z1])
  mm<R, NX, NX, NX, true, false, S::LDN, S::LD2, S::LD2>(s.Wm, a.A, X22);
  copy<R, NX, NX, false, S::LD2, S::LDN>(s.Wm + NX, a.Z);
  tria<R, NX, 2 * NX, S::LD2>(s.Wm, s.vb);
  copy<R, NX, NX, false, S::LDN, S::LD2>(a.Z, s.Wm);
  // U = tria([A2 Vt, U2])
  mm<R, NX, NX, NX, false, false, S::LDN, S::LDN, S::LD2>(s.Wm, e.A, s.Vt);
  copy<R, NX, NX, false, S::LD2, S::LDN>(s.Wm + NX, e.U);
  tria<R, NX, 2 * NX, S::LD2>(s.Wm, s.vb);
  copy<R, NX, NX, false, S::LDN, S::LD2>(a.U, s.Wm);
  // A = A2 N
  mm<R, NX, NX, NX, false, false, S::LDN, S::LDN, S::LDN>(a.A, e.A, s.N);
  if (l < NX) {
    a.b[l] = bnew;
    a.eta[l] = enew;
  }
  __syncwarp();
}

// State form: (m, L) <- combine((., m, L, ., .), e) restricted to (b, U).
template <typename R, int NX, int NY>
SS_DEV void apply(R* L, R* m, FB<R> e, FS<R> s) {
  typedef DS<R, NX, NY> S;
  const int l = lane_id();
  xi_core<R, NX, NY>(L, e.Z, s);
  const R* X21 = s.Xi + NX * S::LD2;
  const R t1 = rowdot<R, NX, NX, true, S::LDN>(L, e.eta, l);
  if (l < NX) s.v1[l] = t1;
  __syncwarp();
  const R v = (l < NX ? m[l] : R(0)) + rowdot<R, NX, NX, false, S::LDN>(L, s.v1, l);
  if (l < NX) s.v3[l] = v;
  __syncwarp();
  const R x = rowdot<R, NX, NX, true, S::LD2>(X21, s.v3, l);
  if (l < NX) s.v1[l] = x;
  __syncwarp();
  const R w = v - rowdot<R, NX, NX, false, S::LDN>(s.Vt, s.v1, l);
  if (l < NX) s.v2[l] = w;
  __syncwarp();
  const R mnew = rowdot<R, NX, NX, false, S::LDN>(e.A, s.v2, l) + (l < NX ? e.b[l] : R(0));
  mm<R, NX, NX, NX, false, false, S::LDN, S::LDN, S::LD2>(s.Wm, e.A, s.Vt);
  copy<R, NX, NX, false, S::LD2, S::LDN>(s.Wm + NX, e.U);
  tria<R, NX, 2 * NX, S::LD2>(s.Wm, s.vb);
  copy<R, NX, NX, false, S::LDN, S::LD2>(L, s.Wm);
  if (l < NX) m[l] = mnew;
  __syncwarp();
}

// a <- e (x) a for the reverse scan (a earlier, e later):
// parsmooth/parallel/_operators.py:104-125 with elem1 = e, elem2 = a.
template <typename R, int NX, int NY>
SS_DEV void sfold(SB<R> a, SB<R> e, R* Wm, R* T, R* vb) {
  typedef DS<R, NX, NY> S;
  const int l = lane_id();
  mm<R, NX, NX, NX, false, false, S::LDN, S::LDN, S::LD2, true>(Wm, a.E, e.D);
  copy<R, NX, NX, false, S::LD2, S::LDN>(Wm + NX, a.D);
  tria<R, NX, 2 * NX, S::LD2>(Wm, vb);
  const R g = rowdot<R, NX, NX, false, S::LDN>(a.E, e.g, l) + (l < NX ? a.g[l] : R(0));
  mm<R, NX, NX, NX, false, false, S::LDN, S::LDN, S::LDN>(T, a.E, e.E);
  copy<R, NX, NX, false, S::LDN, S::LDN>(a.E, T);
  copy<R, NX, NX, false, S::LDN, S::LD2>(a.D, Wm);
  if (l < NX) a.g[l] = g;
  __syncwarp();
}

// Smoothed state at the end of e's range -> at its start: m <- E m + g,
// L <- tria([E L, D]).
template <typename R, int NX, int NY>
SS_DEV void sapply(R* L, R* m, SB<R> e, R* Wm, R* vb) {
  typedef DS<R, NX, NY> S;
  const int l = lane_id();
  mm<R, NX, NX, NX, false, false, S::LDN, S::LDN, S::LD2, true>(Wm, e.E, L);
  copy<R, NX, NX, false, S::LD2, S::LDN>(Wm + NX, e.D);
  tria<R, NX, 2 * NX, S::LD2>(Wm, vb);
  const R mn = rowdot<R, NX, NX, false, S::LDN>(e.E, m, l) + (l < NX ? e.g[l] : R(0));
  __syncwarp();
  copy<R, NX, NX, false, S::LDN, S::LD2>(L, Wm);
  if (l < NX) m[l] = mn;
  __syncwarp();
}

// Model constants of the walks, in the block's shared memory.
template <typename R>
struct MC {
  R *F, *cQ, *H, *cR, *bq, *c;
};
template <typename R, int NX, int NY>
__host__ __device__ constexpr int mc_elems() {
  typedef DS<R, NX, NY> S;
  return 2 * S::MN + NY * S::LDN + NY * S::LDY + S::VN + S::VY;
}
template <typename R, int NX, int NY>
SS_DEV MC<R> carve_mc(R*& p) {
  typedef DS<R, NX, NY> S;
  MC<R> c;
  c.F = p; p += S::MN;
  c.cQ = p; p += S::MN;
  c.H = p; p += NY * S::LDN;
  c.cR = p; p += NY * S::LDY;
  c.bq = p; p += S::VN;
  c.c = p; p += S::VY;
  return c;
}
// Loaded by warp 0 of the block (element-wise: model arrays have no alignment
// guarantee); the caller synchronises the block.
template <typename R, int NX, int NY>
SS_DEV void load_mc(MC<R> c, const DenseArgs<R>& a) {
  typedef DS<R, NX, NY> S;
  g2s_any<R, NX, NX, S::LDN>(c.F, a.F);
  g2s_any<R, NX, NX, S::LDN>(c.cQ, a.qc);
  g2s_any<R, NY, NX, S::LDN>(c.H, a.H);
  g2s_any<R, NY, NY, S::LDY>(c.cR, a.rc);
  g2s_any<R, 1, NX, S::VN>(c.bq, a.qm);
  g2s_any<R, 1, NY, S::VY>(c.c, a.rm);
}

// Smoothing element of the filtered state (L, m) (parsmooth/parallel/
// _smoothing.py:72-85): Phi = tria([[F L, cQ], [L, 0]]) in Phi, E = Phi21
// Phi11^{-1} in place of Phi21, D = Phi22; mp = F m + bq into mpv, g into gv.
template <typename R, int NX, int NY>
SS_DEV void selem(MC<R> c, const R* L, const R* m, R* Phi, R* mpv, R* gv, R* vb) {
  typedef DS<R, NX, NY> S;
  const int l = lane_id();
  mm<R, NX, NX, NX, false, false, S::LDN, S::LDN, S::LD2, true>(Phi, c.F, L);
  copy<R, NX, NX, false, S::LD2, S::LDN>(Phi + NX, c.cQ);
  copy<R, NX, NX, false, S::LD2, S::LDN>(Phi + NX * S::LD2, L);
  fill_diag<R, NX, NX, S::LD2>(Phi + NX * S::LD2 + NX, R(0));
  tria<R, 2 * NX, 2 * NX, S::LD2>(Phi, vb);
  const R mp = rowdot<R, NX, NX, false, S::LDN>(c.F, m, l) + (l < NX ? c.bq[l] : R(0));
  if (l < NX) mpv[l] = mp;
  trsm_rl<R, NX, NX, S::LD2, S::LD2>(Phi + NX * S::LD2, Phi);
  const R g = (l < NX ? m[l] : R(0)) - rowdot<R, NX, NX, false, S::LD2>(Phi + NX * S::LD2, mpv, l);
  if (l < NX) gv[l] = g;
  __syncwarp();
}

// ----------------------------------------------------------------------------- setup

template <typename R, int NX, int NY>
__host__ __device__ constexpr int setup_elems() {
  typedef DS<R, NX, NY> S;
  return mc_elems<R, NX, NY>() + S::MP + NY * S::LDN + S::MY + 6 * S::MN + S::M2 + S::MW + 6 * S::MN +
         S::VY + S::VB;
}

// Store the rows of a shared (ROWS x COLS) matrix transposed: g[k * ROWS + i] = S[i][k].
template <typename R, int ROWS, int COLS, int LD>
SS_DEV void s2g_t(R* g, const R* S) {
  const int l = lane_id();
  if (l < ROWS) {
    SS_UNROLL
    for (int k = 0; k < COLS; ++k) g[k * ROWS + l] = S[l * LD + k];
  }
  __syncwarp();
}

// One warp: element constants and the fold table for chunk length C.
template <typename R, int NX, int NY>
__global__ void __launch_bounds__(32) setup_kernel(DenseArgs<R> a) {
  typedef DS<R, NX, NY> S;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* p = reinterpret_cast<R*>(smem_raw);
  zero(p, setup_elems<R, NX, NY>());
  MC<R> c = carve_mc<R, NX, NY>(p);
  R* Psi = p; p += S::MP;
  R* HF = p; p += NY * S::LDN;
  R* Wt = p; p += S::MY;
  R* A2 = p; p += S::MN;
  R* U2 = p; p += S::MN;
  R* Z2 = p; p += S::MN;
  R* A1 = p; p += S::MN;
  R* U1 = p; p += S::MN;
  R* Z1 = p; p += S::MN;
  FS<R> s;
  s.Xi = p; p += S::M2;
  s.Wm = p; p += S::MW;
  s.Vt = p; p += S::MN;
  R* G = p; p += S::MN;
  R* Mm = p; p += S::MN;
  R* N = p; p += S::MN;
  R* T1 = p; p += S::MN;
  R* T2 = p; p += S::MN;
  R* hb = p; p += S::VY;
  s.vb = p;
  load_mc<R, NX, NY>(c, a);
  const int l = lane_id();
  R* tab = a.tab;
  // Psi = tria([[H cQ, cR], [cQ, 0]]) (parsmooth/parallel/_filtering.py:127-133 with a zero prior)
  mm<R, NY, NX, NX, false, false, S::LDN, S::LDN, S::LDP>(Psi, c.H, c.cQ);
  copy<R, NY, NY, false, S::LDP, S::LDY>(Psi + NX, c.cR);
  copy<R, NX, NX, false, S::LDP, S::LDN>(Psi + NY * S::LDP, c.cQ);
  tria<R, NX + NY, NX + NY, S::LDP>(Psi, s.vb);
  const R* P21 = Psi + NY * S::LDP;
  copy<R, NX, NX, false, S::LDN, S::LDP>(U2, P21 + NY);
  // W^T = (Psi11^{-1} H F)^T, A = F - Psi21 W, Z = W^T zero-padded (nx > ny) or tria(W^T)
  mm<R, NY, NX, NX, false, false, S::LDN, S::LDN, S::LDN>(HF, c.H, c.F);
  copy<R, NX, NY, true, S::LDY, S::LDN>(Wt, HF);
  trsm_rlt<R, NX, NY, S::LDY, S::LDP>(Wt, Psi);
  copy<R, NX, NX, false, S::LDN, S::LDN>(A2, c.F);
  mm<R, NX, NY, NX, false, true, S::LDP, S::LDY, S::LDN>(A2, P21, Wt, R(-1), true);
  if constexpr (NX > NY) {
    copy<R, NX, NY, false, S::LDN, S::LDY>(Z2, Wt);
  } else {
    copy<R, NX, NY, false, S::LDY, S::LDY>(T1, Wt);
    tria<R, NX, NY, S::LDY>(T1, s.vb);
    copy<R, NX, NX, false, S::LDN, S::LDY>(Z2, T1);
  }
  const R h = rowdot<R, NY, NX, false, S::LDN>(c.H, c.bq, l) + (l < NY ? c.c[l] : R(0));
  if (l < NY) hb[l] = h;
  __syncwarp();
  // constants: Psi11, Psi21, W^T, c + H bq
  s2g<R, NY, NY, S::LDP>(tab, Psi);
  s2g<R, NX, NY, S::LDP>(tab + NY * NY, P21);
  s2g<R, NX, NY, S::LDY>(tab + NY * NY + NX * NY, Wt);
  if (l < NY) tab[NY * NY + 2 * NX * NY + l] = hb[l];
  // position 1: the element itself
  s2g<R, NX, NX, S::LDN>(tab + S::summ_off(1), A2);
  s2g<R, NX, NX, S::LDN>(tab + S::summ_off(1) + NX * NX, U2);
  s2g<R, NX, NX, S::LDN>(tab + S::summ_off(1) + 2 * NX * NX, Z2);
  copy<R, NX, NX, false, S::LDN, S::LDN>(A1, A2);
  copy<R, NX, NX, false, S::LDN, S::LDN>(U1, U2);
  copy<R, NX, NX, false, S::LDN, S::LDN>(Z1, Z2);
  for (int j = 1; j < a.C; ++j) {
    xi_core<R, NX, NY>(U1, Z2, s);
    const R* X21 = s.Xi + NX * S::LD2;
    const R* X22 = X21 + NX;
    fill_diag<R, NX, NX, S::LDN>(G, R(1));
    mm<R, NX, NX, NX, false, true, S::LDN, S::LD2, S::LDN>(G, s.Vt, X21, R(-1), true);
    mm<R, NX, NX, NX, false, false, S::LDN, S::LDN, S::LDN>(Mm, A2, G);
    mm<R, NX, NX, NX, false, false, S::LDN, S::LDN, S::LDN>(N, G, A1);
    R* co = tab + S::coef_off(a.C, j);
    s2g_t<R, NX, NX, S::LDN>(co, Mm);
    // B = M U1 U1^T W^T + Psi21
    mm<R, NX, NX, NX, false, false, S::LDN, S::LDN, S::LDN>(T1, Mm, U1);
    mm<R, NX, NX, NX, false, true, S::LDN, S::LDN, S::LDN>(T2, T1, U1);
    copy<R, NX, NY, false, S::LDN, S::LDP>(T1, P21);
    mm<R, NX, NX, NY, false, false, S::LDN, S::LDY, S::LDN>(T1, T2, Wt, R(1), true);
    s2g_t<R, NX, NY, S::LDN>(co + NX * NX, T1);
    // C = N^T W^T
    mm<R, NX, NX, NY, true, false, S::LDN, S::LDY, S::LDN>(T2, N, Wt);
    s2g_t<R, NX, NY, S::LDN>(co + NX * NX + NX * NY, T2);
    // D = N^T Z2 Z2^T
    mm<R, NX, NX, NX, true, false, S::LDN, S::LDN, S::LDN>(T1, N, Z2);
    mm<R, NX, NX, NX, false, true, S::LDN, S::LDN, S::LDN>(T2, T1, Z2);
    s2g_t<R, NX, NX, S::LDN>(co + NX * NX + 2 * NX * NY, T2);
    // matrix part of the fold of j + 1 elements
    mm<R, NX, NX, NX, true, false, S::LDN, S::LD2, S::LD2>(s.Wm, A1, X22);
    copy<R, NX, NX, false, S::LD2, S::LDN>(s.Wm + NX, Z1);
    tria<R, NX, 2 * NX, S::LD2>(s.Wm, s.vb);
    copy<R, NX, NX, false, S::LDN, S::LD2>(Z1, s.Wm);
    mm<R, NX, NX, NX, false, false, S::LDN, S::LDN, S::LD2>(s.Wm, A2, s.Vt);
    copy<R, NX, NX, false, S::LD2, S::LDN>(s.Wm + NX, U2);
    tria<R, NX, 2 * NX, S::LD2>(s.Wm, s.vb);
    copy<R, NX, NX, false, S::LDN, S::LD2>(U1, s.Wm);
    mm<R, NX, NX, NX, false, false, S::LDN, S::LDN, S::LDN>(T1, A2, N);
    copy<R, NX, NX, false, S::LDN, S::LDN>(A1, T1);
    R* sm = tab + S::summ_off(j + 1);
    s2g<R, NX, NX, S::LDN>(sm, A1);
    s2g<R, NX, NX, S::LDN>(sm + NX * NX, U1);
    s2g<R, NX, NX, S::LDN>(sm + 2 * NX * NX, Z1);
  }
}

// ----------------------------------------------------------------------------- filter scan

constexpr int LEAF_WARPS = 4;

template <typename R, int NX, int NY>
__host__ __device__ constexpr int leaf_cta_elems() {
  typedef DS<R, NX, NY> S;
  return NY * S::LDY + 2 * S::MY + S::VY + S::VN;
}
template <typename R, int NX, int NY>
__host__ __device__ constexpr int leaf_elems() {
  return leaf_cta_elems<R, NX, NY>() + LEAF_WARPS * DS<R, NX, NY>::VN;
}

// r = Psi11^{-1} (y - c - H bq), every lane the whole vector.
template <typename R, int NY, int LDY>
SS_DEV void obs_residual(const R* y, const R* P11, const R* hb, R (&z)[NY]) {
  SS_UNROLL
  for (int k = 0; k < NY; ++k) {
    R t = y[k] - hb[k];
    SS_UNROLL
    for (int j = 0; j < k; ++j) t -= P11[k * LDY + j] * z[j];
    z[k] = t / P11[k * LDY + k];
  }
}

// Level-1 summaries by the per-position vector recursion (see the top of the file).
template <typename R, int NX, int NY>
__global__ void __launch_bounds__(32 * LEAF_WARPS) leaf_kernel(DenseArgs<R> a) {
  typedef DS<R, NX, NY> S;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* sm = reinterpret_cast<R*>(smem_raw);
  R* P11 = sm;
  R* P21 = P11 + NY * S::LDY;
  R* Wt = P21 + S::MY;
  R* hb = Wt + S::MY;
  R* bq = hb + S::VY;
  const int warp = threadIdx.x >> 5, l = lane_id();
  R* bv = sm + leaf_cta_elems<R, NX, NY>() + warp * S::VN;
  if (warp == 0) {
    zero(sm, leaf_elems<R, NX, NY>());
    g2s<R, NY, NY, S::LDY>(P11, a.tab);
    g2s<R, NX, NY, S::LDY>(P21, a.tab + NY * NY);
    g2s<R, NX, NY, S::LDY>(Wt, a.tab + NY * NY + NX * NY);
    if (l < NY) hb[l] = a.tab[NY * NY + 2 * NX * NY + l];
    g2s_any<R, 1, NX, S::VN>(bq, a.qm);
  }
  __syncthreads();
  const ScanArgs<R>& sa = a.s;
  const int64_t j = (int64_t)blockIdx.x * LEAF_WARPS + warp;
  if (j >= sa.g.lvl[1][sa.g.B]) return;
  int64_t i, t0, t1;
  chunk_of(sa.g, j, i, t0, t1);
  if (seq_inactive(sa.active, i)) return;
  const int64_t base = sa.g.off[i];
  const int n = (int)(t1 - t0);
  R z[NY];
  obs_residual<R, NY, S::LDY>(sa.ys + (base + t0) * NY, P11, hb, z);
  const int il = l < NX ? l : NX - 1;
  R b = bq[il], eta = R(0);
  SS_UNROLL
  for (int k = 0; k < NY; ++k) {
    b += P21[il * S::LDY + k] * z[k];
    eta += Wt[il * S::LDY + k] * z[k];
  }
  for (int q = 1; q < n; ++q) {
    obs_residual<R, NY, S::LDY>(sa.ys + (base + t0 + q) * NY, P11, hb, z);
    if (l < NX) bv[l] = b;
    __syncwarp();
    const R* co = a.tab + S::coef_off(a.C, q);
    R nb = bq[il], ne = eta;
    SS_UNROLL
    for (int k = 0; k < NX; ++k) {
      const R bk = bv[k];
      nb += co[k * NX + il] * bk;
      ne -= co[NX * NX + 2 * NX * NY + k * NX + il] * bk;
    }
    SS_UNROLL
    for (int k = 0; k < NY; ++k) {
      nb += co[NX * NX + k * NX + il] * z[k];
      ne += co[NX * NX + NX * NY + k * NX + il] * z[k];
    }
    __syncwarp();
    b = nb;
    eta = ne;
  }
  R* out = sa.fsum[1] + j * S::FE;
  g2g<R>(out, a.tab + S::summ_off(n), 3 * NX * NX);
  if (l < NX) {
    out[3 * NX * NX + l] = b;
    out[3 * NX * NX + NX + l] = eta;
  }
}

template <typename R, int NX, int NY>
__host__ __device__ constexpr int up_elems() {
  return 2 * fb_elems<R, NX, NY>() + fs_elems<R, NX, NY>();
}

// Level l -> l+1 filtering summaries (fold of G summaries), one warp per block.
template <typename R, int NX, int NY>
__global__ void __launch_bounds__(32) up_kernel(DenseArgs<R> a, int lv) {
  typedef DS<R, NX, NY> S;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* p = reinterpret_cast<R*>(smem_raw);
  const ScanArgs<R>& sa = a.s;
  const int64_t j = blockIdx.x;
  if (j >= sa.g.lvl[lv + 1][sa.g.B]) return;
  int64_t i, m0, m1;
  group_of(sa.g, lv, j, i, m0, m1);
  if (seq_inactive(sa.active, i)) return;
  zero(p, up_elems<R, NX, NY>());
  FB<R> acc = carve_fb<R, NX, NY>(p);
  FB<R> e = carve_fb<R, NX, NY>(p);
  FS<R> s = carve_fs<R, NX, NY>(p);
  load_fb<R, NX, NY>(acc, sa.fsum[lv] + m0 * S::FE);
  for (int64_t m = m0 + 1; m < m1; ++m) {
    load_fb<R, NX, NY>(e, sa.fsum[lv] + m * S::FE);
    combine<R, NX, NY>(acc, e, s);
  }
  store_fb<R, NX, NY>(sa.fsum[lv + 1] + j * S::FE, acc);
}

template <typename R, int NX, int NY>
__host__ __device__ constexpr int apply_elems() {
  return DS<R, NX, NY>::MN + DS<R, NX, NY>::VN + fb_elems<R, NX, NY>() + fs_elems<R, NX, NY>();
}

// Top level, one warp per sequence: walk the top items from the prior.
template <typename R, int NX, int NY>
__global__ void __launch_bounds__(32) top_kernel(DenseArgs<R> a) {
  typedef DS<R, NX, NY> S;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* p = reinterpret_cast<R*>(smem_raw);
  const ScanArgs<R>& sa = a.s;
  const int64_t i = blockIdx.x;
  if (i >= sa.g.B) return;
  if (seq_inactive(sa.active, i)) return;
  zero(p, apply_elems<R, NX, NY>());
  R* L = p; p += S::MN;
  R* m = p; p += S::VN;
  FB<R> e = carve_fb<R, NX, NY>(p);
  FS<R> s = carve_fs<R, NX, NY>(p);
  const int l = lane_id();
  const int64_t pr = i * sa.prior_stride;
  g2s_any<R, NX, NX, S::LDN>(L, sa.L0 + pr * NX * NX);
  if (l < NX) {
    SS_UNROLL
    for (int k = 0; k < NX; ++k)
      if (k > l) L[l * S::LDN + k] = R(0);   // the prior factor's strict upper part is ignored
    m[l] = sa.m0[pr * NX + l];
  }
  __syncwarp();
  if (sa.filt_m != nullptr) store_traj<R, NX, NY>(sa.filt_m, sa.filt_L, sa.g.off[i] + i, L, m);
  const int Lv = sa.g.L;
  const int64_t b = sa.g.lvl[Lv][i], en = sa.g.lvl[Lv][i + 1];
  if (b == en) {
    store_st<R, NX, NY>(sa.fT + i * S::ST, L, m);
    return;
  }
  for (int64_t q = b; q < en; ++q) {
    store_st<R, NX, NY>(sa.fst[Lv] + q * S::ST, L, m);
    if (q + 1 < en) {
      load_fb<R, NX, NY>(e, sa.fsum[Lv] + q * S::FE);
      apply<R, NX, NY>(L, m, e, s);
    }
  }
}

// Level l+1 -> l entry states, one warp per group.
template <typename R, int NX, int NY>
__global__ void __launch_bounds__(32) down_kernel(DenseArgs<R> a, int lv) {
  typedef DS<R, NX, NY> S;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* p = reinterpret_cast<R*>(smem_raw);
  const ScanArgs<R>& sa = a.s;
  const int64_t j = blockIdx.x;
  if (j >= sa.g.lvl[lv + 1][sa.g.B]) return;
  int64_t i, m0, m1;
  group_of(sa.g, lv, j, i, m0, m1);
  if (seq_inactive(sa.active, i)) return;
  zero(p, apply_elems<R, NX, NY>());
  R* L = p; p += S::MN;
  R* m = p; p += S::VN;
  FB<R> e = carve_fb<R, NX, NY>(p);
  FS<R> s = carve_fs<R, NX, NY>(p);
  load_st<R, NX, NY>(L, m, sa.fst[lv + 1] + j * S::ST);
  for (int64_t q = m0; q < m1; ++q) {
    store_st<R, NX, NY>(sa.fst[lv] + q * S::ST, L, m);
    if (q + 1 < m1) {
      load_fb<R, NX, NY>(e, sa.fsum[lv] + q * S::FE);
      apply<R, NX, NY>(L, m, e, s);
    }
  }
}

// ----------------------------------------------------------------------------- filter walk

template <typename R, int NX, int NY>
__host__ __device__ constexpr int walk_warp_elems() {
  typedef DS<R, NX, NY> S;
  return S::MN + S::MPHI + 3 * S::VN + S::VY + S::VB;
}
template <typename R, int NX, int NY>
__host__ __device__ constexpr int walk_warps() {
  constexpr int budget = 200 * 1024 / (int)sizeof(R);
  constexpr int w = (budget - mc_elems<R, NX, NY>()) / walk_warp_elems<R, NX, NY>();
  return w < 1 ? 1 : (w > 8 ? 8 : w);
}
template <typename R, int NX, int NY>
__host__ __device__ constexpr int walk_elems() {
  return mc_elems<R, NX, NY>() + walk_warps<R, NX, NY>() * walk_warp_elems<R, NX, NY>();
}

// Kalman steps of one chunk from its entry state; emits the smoothing elements.
// Phi and then Psi share one shared-memory region: Phi11 (the predicted factor)
// moves to the state buffer, whose old content Phi has consumed.  The FP64
// walk; FP32 runs walk_r_kernel (ss_dense_shared.cuh), which keeps Phi and Psi
// in registers.
template <typename R, int NX, int NY>
__global__ void __launch_bounds__(32 * walk_warps<R, NX, NY>()) walk_kernel(DenseArgs<R> a) {
  typedef DS<R, NX, NY> S;
  constexpr int WARPS = walk_warps<R, NX, NY>();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* p = reinterpret_cast<R*>(smem_raw);
  const int warp = threadIdx.x >> 5, l = lane_id();
  MC<R> c = carve_mc<R, NX, NY>(p);
  p += warp * walk_warp_elems<R, NX, NY>();
  zero(p, walk_warp_elems<R, NX, NY>());
  if (warp == 0) load_mc<R, NX, NY>(c, a);
  __syncthreads();
  R* L = p; p += S::MN;
  R* Phi = p; p += S::MPHI;
  R* Psi = Phi;
  R* m = p; p += S::VN;
  R* mp = p; p += S::VN;
  R* g = p; p += S::VN;
  R* rv = p; p += S::VY;
  R* vb = p;
  const ScanArgs<R>& sa = a.s;
  const int64_t j = (int64_t)blockIdx.x * WARPS + warp;
  if (j >= sa.g.lvl[1][sa.g.B]) return;
  int64_t i, t0, t1;
  chunk_of(sa.g, j, i, t0, t1);
  if (seq_inactive(sa.active, i)) return;
  const int64_t base = sa.g.off[i];
  load_st<R, NX, NY>(L, m, sa.fst[1] + j * S::ST);
  double ll = 0.0;
  for (int64_t t = t0; t < t1; ++t) {
    selem<R, NX, NY>(c, L, m, Phi, mp, g, vb);
    if (sa.emit_smoother) {
      R* rec = sa.selem + (base + t) * S::SE;
      s2g<R, NX, NX, S::LD2>(rec, Phi + NX * S::LD2);
      s2g<R, NX, NX, S::LD2>(rec + NX * NX, Phi + NX * S::LD2 + NX);
      if (l < NX) rec[2 * NX * NX + l] = g[l];
    }
    copy<R, NX, NX, false, S::LDN, S::LD2>(L, Phi);   // predicted factor N1 = Phi11
    // update: Psi = tria([[H N1, cR], [N1, 0]]) (parsmooth/sequential/_filtering.py:89-108)
    mm<R, NY, NX, NX, false, false, S::LDN, S::LDN, S::LDP, true>(Psi, c.H, L);
    copy<R, NY, NY, false, S::LDP, S::LDY>(Psi + NX, c.cR);
    copy<R, NX, NX, false, S::LDP, S::LDN>(Psi + NY * S::LDP, L);
    fill_diag<R, NX, NY, S::LDP>(Psi + NY * S::LDP + NX, R(0));
    tria<R, NX + NY, NX + NY, S::LDP>(Psi, vb);
    const R res = (l < NY ? sa.ys[(base + t) * NY + l] - c.c[l] : R(0)) - rowdot<R, NY, NX, false, S::LDN>(c.H, mp, l);
    if (l < NY) rv[l] = res;
    __syncwarp();
    R z[NY];
    R q = R(0), ld = R(0);
    SS_UNROLL
    for (int k = 0; k < NY; ++k) {
      R t2 = rv[k];
      SS_UNROLL
      for (int jj = 0; jj < k; ++jj) t2 -= Psi[k * S::LDP + jj] * z[jj];
      const R dk = Psi[k * S::LDP + k];
      z[k] = t2 / dk;
      q += z[k] * z[k];
      ld += ss_log(ss_abs(dk));
    }
    ll += -0.5 * ((double)q + 2.0 * (double)ld);
    const int il = l < NX ? l : NX - 1;
    R mn = mp[il];
    SS_UNROLL
    for (int k = 0; k < NY; ++k) mn += Psi[(NY + il) * S::LDP + k] * z[k];
    __syncwarp();
    copy<R, NX, NX, false, S::LDN, S::LDP>(L, Psi + NY * S::LDP + NY);
    if (l < NX) m[l] = mn;
    __syncwarp();
    if (sa.filt_m != nullptr) store_traj<R, NX, NY>(sa.filt_m, sa.filt_L, base + i + t + 1, L, m);
  }
  if (sa.ll_chunk != nullptr && l == 0) sa.ll_chunk[j] = ll;
  if (t1 == sa.g.off[i + 1] - base) store_st<R, NX, NY>(sa.fT + i * S::ST, L, m);
}

// ----------------------------------------------------------------------------- smoother

template <typename R, int NX, int NY>
__host__ __device__ constexpr int sfold_warp_elems() {
  typedef DS<R, NX, NY> S;
  return 2 * sb_elems<R, NX, NY>() + S::MW + S::MN + S::VB;
}
constexpr int SFOLD_WARPS = 2;

// Level-1 smoothing summaries: fold of the chunk's per-step elements.
template <typename R, int NX, int NY>
__global__ void __launch_bounds__(32 * SFOLD_WARPS) sleaf_kernel(DenseArgs<R> a) {
  typedef DS<R, NX, NY> S;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5;
  R* p = reinterpret_cast<R*>(smem_raw) + warp * sfold_warp_elems<R, NX, NY>();
  const ScanArgs<R>& sa = a.s;
  const int64_t j = (int64_t)blockIdx.x * SFOLD_WARPS + warp;
  if (j >= sa.g.lvl[1][sa.g.B]) return;
  int64_t i, t0, t1;
  chunk_of(sa.g, j, i, t0, t1);
  if (seq_inactive(sa.active, i)) return;
  zero(p, sfold_warp_elems<R, NX, NY>());
  SB<R> acc = carve_sb<R, NX, NY>(p);
  SB<R> e = carve_sb<R, NX, NY>(p);
  R* Wm = p; p += S::MW;
  R* T = p; p += S::MN;
  R* vb = p;
  const int64_t base = sa.g.off[i];
  load_sb<R, NX, NY>(acc, sa.selem + (base + t0) * S::SE);
  for (int64_t t = t0 + 1; t < t1; ++t) {
    load_sb<R, NX, NY>(e, sa.selem + (base + t) * S::SE);
    sfold<R, NX, NY>(acc, e, Wm, T, vb);
  }
  store_sb<R, NX, NY>(sa.ssum[1] + j * S::SE, acc);
}

template <typename R, int NX, int NY>
__global__ void __launch_bounds__(32 * SFOLD_WARPS) sup_kernel(DenseArgs<R> a, int lv) {
  typedef DS<R, NX, NY> S;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5;
  R* p = reinterpret_cast<R*>(smem_raw) + warp * sfold_warp_elems<R, NX, NY>();
  const ScanArgs<R>& sa = a.s;
  const int64_t j = (int64_t)blockIdx.x * SFOLD_WARPS + warp;
  if (j >= sa.g.lvl[lv + 1][sa.g.B]) return;
  int64_t i, m0, m1;
  group_of(sa.g, lv, j, i, m0, m1);
  if (seq_inactive(sa.active, i)) return;
  zero(p, sfold_warp_elems<R, NX, NY>());
  SB<R> acc = carve_sb<R, NX, NY>(p);
  SB<R> e = carve_sb<R, NX, NY>(p);
  R* Wm = p; p += S::MW;
  R* T = p; p += S::MN;
  R* vb = p;
  load_sb<R, NX, NY>(acc, sa.ssum[lv] + m0 * S::SE);
  for (int64_t q = m0 + 1; q < m1; ++q) {
    load_sb<R, NX, NY>(e, sa.ssum[lv] + q * S::SE);
    sfold<R, NX, NY>(acc, e, Wm, T, vb);
  }
  store_sb<R, NX, NY>(sa.ssum[lv + 1] + j * S::SE, acc);
}

template <typename R, int NX, int NY>
__host__ __device__ constexpr int sapply_warp_elems() {
  typedef DS<R, NX, NY> S;
  return S::MN + S::VN + sb_elems<R, NX, NY>() + S::MW + S::VB;
}

template <typename R, int NX, int NY>
SS_DEV void accumulate_change(const ScanArgs<R>& sa, int64_t i, int64_t s, const R* m) {
  const int l = lane_id();
  if (sa.mse != nullptr) {
    double d = 0.0;
    if (l < NX) {
      const double e = (double)m[l] - (double)sa.prev_m[s * NX + l];
      d = e * e;
    }
    d = warp_sum(d);
    if (l == 0) atomicAdd(sa.mse + i, d);
  }
  if (sa.flags != nullptr) {
    const bool bad = (l < NX) && !ss_isfinite(m[l]);
    if (__any_sync(0xffffffffu, bad) && l == 0) atomicOr(sa.flags + i, 1u);
  }
}

template <typename R, int NX, int NY>
SS_DEV void copy_state(const ScanArgs<R>& sa, int64_t s) {
  g2g<R>(sa.out_L + s * NX * NX, sa.prev_L + s * NX * NX, NX * NX);
  g2g<R>(sa.out_m + s * NX, sa.prev_m + s * NX, NX);
}

template <typename R, int NX, int NY>
__global__ void __launch_bounds__(32) stop_kernel(DenseArgs<R> a) {
  typedef DS<R, NX, NY> S;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* p = reinterpret_cast<R*>(smem_raw);
  const ScanArgs<R>& sa = a.s;
  const int64_t i = blockIdx.x;
  if (i >= sa.g.B) return;
  const int64_t T = sa.g.off[i + 1] - sa.g.off[i];
  const int64_t sT = sa.g.off[i] + i + T;
  if (seq_inactive(sa.active, i)) {
    copy_state<R, NX, NY>(sa, sT);
    return;
  }
  zero(p, sapply_warp_elems<R, NX, NY>());
  R* L = p; p += S::MN;
  R* m = p; p += S::VN;
  SB<R> e = carve_sb<R, NX, NY>(p);
  R* Wm = p; p += S::MW;
  R* vb = p;
  load_st<R, NX, NY>(L, m, sa.fT + i * S::ST);
  store_traj<R, NX, NY>(sa.out_m, sa.out_L, sT, L, m);
  accumulate_change<R, NX, NY>(sa, i, sT, m);
  const int Lv = sa.g.L;
  const int64_t b = sa.g.lvl[Lv][i], en = sa.g.lvl[Lv][i + 1];
  for (int64_t q = en - 1; q >= b; --q) {
    store_st<R, NX, NY>(sa.sst[Lv] + q * S::ST, L, m);
    if (q > b) {
      load_sb<R, NX, NY>(e, sa.ssum[Lv] + q * S::SE);
      sapply<R, NX, NY>(L, m, e, Wm, vb);
    }
  }
}

template <typename R, int NX, int NY>
__global__ void __launch_bounds__(32) sdown_kernel(DenseArgs<R> a, int lv) {
  typedef DS<R, NX, NY> S;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* p = reinterpret_cast<R*>(smem_raw);
  const ScanArgs<R>& sa = a.s;
  const int64_t j = blockIdx.x;
  if (j >= sa.g.lvl[lv + 1][sa.g.B]) return;
  int64_t i, m0, m1;
  group_of(sa.g, lv, j, i, m0, m1);
  if (seq_inactive(sa.active, i)) return;
  zero(p, sapply_warp_elems<R, NX, NY>());
  R* L = p; p += S::MN;
  R* m = p; p += S::VN;
  SB<R> e = carve_sb<R, NX, NY>(p);
  R* Wm = p; p += S::MW;
  R* vb = p;
  load_st<R, NX, NY>(L, m, sa.sst[lv + 1] + j * S::ST);
  for (int64_t q = m1 - 1; q >= m0; --q) {
    store_st<R, NX, NY>(sa.sst[lv] + q * S::ST, L, m);
    if (q > m0) {
      load_sb<R, NX, NY>(e, sa.ssum[lv] + q * S::SE);
      sapply<R, NX, NY>(L, m, e, Wm, vb);
    }
  }
}

constexpr int SWALK_WARPS = 4;

// RTS steps of one chunk from the smoothed state at its end.
template <typename R, int NX, int NY>
__global__ void __launch_bounds__(32 * SWALK_WARPS) swalk_kernel(DenseArgs<R> a) {
  typedef DS<R, NX, NY> S;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5;
  R* p = reinterpret_cast<R*>(smem_raw) + warp * sapply_warp_elems<R, NX, NY>();
  const ScanArgs<R>& sa = a.s;
  const int64_t j = (int64_t)blockIdx.x * SWALK_WARPS + warp;
  if (j >= sa.g.lvl[1][sa.g.B]) return;
  int64_t i, t0, t1;
  chunk_of(sa.g, j, i, t0, t1);
  const int64_t base = sa.g.off[i];
  if (seq_inactive(sa.active, i)) {
    for (int64_t t = t0; t < t1; ++t) copy_state<R, NX, NY>(sa, base + i + t);
    return;
  }
  zero(p, sapply_warp_elems<R, NX, NY>());
  R* L = p; p += S::MN;
  R* m = p; p += S::VN;
  SB<R> e = carve_sb<R, NX, NY>(p);
  R* Wm = p; p += S::MW;
  R* vb = p;
  load_st<R, NX, NY>(L, m, sa.sst[1] + j * S::ST);
  for (int64_t t = t1 - 1; t >= t0; --t) {
    load_sb<R, NX, NY>(e, sa.selem + (base + t) * S::SE);
    sapply<R, NX, NY>(L, m, e, Wm, vb);
    store_traj<R, NX, NY>(sa.out_m, sa.out_L, base + i + t, L, m);
    accumulate_change<R, NX, NY>(sa, i, base + i + t, m);
  }
}

template <typename R, int NX, int NY>
__host__ __device__ constexpr int selem_warp_elems() {
  typedef DS<R, NX, NY> S;
  return S::MN + S::M2 + 3 * S::VN + S::VB;
}
constexpr int SELEM_WARPS = 2;

// Smoothing elements of a given filtered trajectory (standalone smoothing).
template <typename R, int NX, int NY>
__global__ void __launch_bounds__(32 * SELEM_WARPS) selem_kernel(DenseArgs<R> a) {
  typedef DS<R, NX, NY> S;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* p = reinterpret_cast<R*>(smem_raw);
  const int warp = threadIdx.x >> 5, l = lane_id();
  MC<R> c = carve_mc<R, NX, NY>(p);
  p += warp * selem_warp_elems<R, NX, NY>();
  zero(p, selem_warp_elems<R, NX, NY>());
  if (warp == 0) load_mc<R, NX, NY>(c, a);
  __syncthreads();
  R* L = p; p += S::MN;
  R* Phi = p; p += S::M2;
  R* m = p; p += S::VN;
  R* mp = p; p += S::VN;
  R* g = p; p += S::VN;
  R* vb = p;
  const ScanArgs<R>& sa = a.s;
  const int64_t j = (int64_t)blockIdx.x * SELEM_WARPS + warp;
  if (j >= sa.g.lvl[1][sa.g.B]) return;
  int64_t i, t0, t1;
  chunk_of(sa.g, j, i, t0, t1);
  const int64_t base = sa.g.off[i];
  for (int64_t t = t0; t < t1; ++t) {
    load_traj<R, NX, NY>(L, m, sa.in_m, sa.in_L, base + i + t);
    selem<R, NX, NY>(c, L, m, Phi, mp, g, vb);
    R* rec = sa.selem + (base + t) * S::SE;
    s2g<R, NX, NX, S::LD2>(rec, Phi + NX * S::LD2);
    s2g<R, NX, NX, S::LD2>(rec + NX * NX, Phi + NX * S::LD2 + NX);
    if (l < NX) rec[2 * NX * NX + l] = g[l];
    __syncwarp();
  }
  if (t1 == sa.g.off[i + 1] - base) {
    load_traj<R, NX, NY>(L, m, sa.in_m, sa.in_L, base + i + t1);
    store_st<R, NX, NY>(sa.fT + i * S::ST, L, m);
  }
}

// The last state of each sequence of a given trajectory into fT (standalone
// smoothing; also for sequences without steps).  One warp per sequence.
template <typename R, int NX, int NY>
__global__ void __launch_bounds__(32) last_state_kernel(DenseArgs<R> a) {
  typedef DS<R, NX, NY> S;
  const ScanArgs<R>& sa = a.s;
  const int64_t i = blockIdx.x;
  if (i >= sa.g.B) return;
  const int64_t s = sa.g.off[i + 1] + i;
  g2g<R>(sa.fT + i * S::ST, sa.in_L + s * NX * NX, NX * NX);
  g2g<R>(sa.fT + i * S::ST + NX * NX, sa.in_m + s * NX, NX);
}

// Exact linearisation of a linear model at n points (ss_linearize): F = A,
// chol = qc (extended) or tria(qc) (the sigma-point rules' residual
// covariance is zero), b = qm.  One warp per point.
template <typename R, int NX, int DOUT>
__global__ void __launch_bounds__(32) lin_points_kernel(int64_t n, const R* A, const R* qm, const R* qc, int tria_chol,
                                                        R* F, R* chol, R* b) {
  constexpr int LD = Pad<R, DOUT>::ld;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* M = reinterpret_cast<R*>(smem_raw);
  R* vb = M + DOUT * LD;
  const int64_t pt = blockIdx.x;
  if (pt >= n) return;
  zero(M, DOUT * LD + tria_scratch<R, DOUT>());
  g2s_any<R, DOUT, DOUT, LD>(M, qc);
  if (tria_chol) tria<R, DOUT, DOUT, LD>(M, vb);
  for (int q = lane_id(); q < DOUT * DOUT; q += 32) {
    const int r = q / DOUT, cc = q - r * DOUT;
    chol[pt * DOUT * DOUT + q] = M[r * LD + cc];
  }
  for (int q = lane_id(); q < DOUT * NX; q += 32) F[pt * DOUT * NX + q] = A[q];
  for (int q = lane_id(); q < DOUT; q += 32) b[pt * DOUT + q] = qm[q];
}

}  // namespace dense
}  // namespace ss

