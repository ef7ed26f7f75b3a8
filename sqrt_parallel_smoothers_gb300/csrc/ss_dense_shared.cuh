// Shared-covariance mode of the large-state path.
//
// For a linear time-invariant model, a batch of B equally long sequences that
// share one prior has one covariance recursion: every filtering summary, entry
// state, smoothing element and smoothed factor has the same matrix part in all
// sequences; only the vectors (b, eta, means, g) depend on the observations.
// This mode gives each scan item index (a chunk, a group, the top level) to
// one warp that computes the matrix part once and carries the B sequences'
// vectors as the rows of a B x nx matrix (lane i = sequence i, B <= 32), so
// the vector algebra of parsmooth/parallel/_operators.py:43-77 and 104-125
// becomes small products with the shared matrices.  Results equal the
// per-sequence computation's up to floating-point association.
//
// Records keep the per-sequence layout of the large-state path: the matrix
// parts live in sequence 0's records only, the vectors in every sequence's.
#pragma once
#include "ss_dense.cuh"

namespace ss {
namespace dense {

constexpr int SB_ROWS = 32;  // batch rows (lanes)

template <typename R, int NX, int NY>
struct DSS {
  typedef DS<R, NX, NY> S;
  static constexpr int MB = SB_ROWS * S::LDN;   // B x NX batch matrix
  static constexpr int MBY = SB_ROWS * S::LDY;  // B x NY batch matrix
};

// Rows of a batch matrix from per-sequence records: row i < B is
// g[i * stride + off .. + NX); rows >= B are zero.
template <typename R, int NX, int NY>
SS_DEV void load_rows(R* Mb, const R* g, int64_t stride, int off, int B) {
  typedef DS<R, NX, NY> S;
  const int l = lane_id();
  R x[S::VN];
  if (l < B) {
    const R* src = g + (int64_t)l * stride + off;
    SS_UNROLL
    for (int j = 0; j < S::VN; j += S::W) {
      const Vec<R> v = ld16(src + j);
      SS_UNROLL
      for (int u = 0; u < S::W; ++u) x[j + u] = v.v[u];
    }
  } else {
    SS_UNROLL
    for (int j = 0; j < S::VN; ++j) x[j] = R(0);
  }
  store_row<R, NX, S::LDN>(Mb, l, x);
  __syncwarp();
}

template <typename R, int NX, int NY>
SS_DEV void store_rows(R* g, int64_t stride, int off, const R* Mb, int B) {
  typedef DS<R, NX, NY> S;
  const int l = lane_id();
  if (l < B) {
    R* dst = g + (int64_t)l * stride + off;
    SS_UNROLL
    for (int j = 0; j < S::VN; j += S::W) st16(dst + j, ld16(Mb + l * S::LDN + j));
  }
  __syncwarp();
}

// Scratch batch matrices of the shared operators.
template <typename R>
struct BT {
  R *T1, *V, *U, *X;
};
template <typename R, int NX, int NY>
SS_DEV BT<R> carve_bt(R*& p) {
  BT<R> b;
  b.T1 = p; p += DSS<R, NX, NY>::MB;
  b.V = p; p += DSS<R, NX, NY>::MB;
  b.U = p; p += DSS<R, NX, NY>::MB;
  b.X = p; p += DSS<R, NX, NY>::MB;
  return b;
}

// a <- a (x) e with shared matrix parts (as in combine()) and batch vectors:
// rows of Ba, Ea are b1, eta1; of Be, Ee are b2, eta2.
//   V = B1 + (E2 U1) U1^T, U = E2 - (B1 Z2) Z2^T, X = V Xi21, W = V - X Vt^T,
//   B' = W A2^T + B2, E' = U N + E1.
template <typename R, int NX, int NY>
SS_DEV void combine_b(FB<R> a, R* Ba, R* Ea, FB<R> e, const R* Be, const R* Ee, FS<R> s, BT<R> t) {
  typedef DS<R, NX, NY> S;
  constexpr int BR = SB_ROWS;
  xi_core<R, NX, NY>(a.U, e.Z, s);
  const R* X21 = s.Xi + NX * S::LD2;
  const R* X22 = X21 + NX;
  mm<R, BR, NX, NX, false, false, S::LDN, S::LDN, S::LDN>(t.T1, Ee, a.U);
  copy<R, BR, NX, false, S::LDN, S::LDN>(t.V, Ba);
  mm<R, BR, NX, NX, false, true, S::LDN, S::LDN, S::LDN>(t.V, t.T1, a.U, R(1), true);
  mm<R, BR, NX, NX, false, false, S::LDN, S::LDN, S::LDN>(t.T1, Ba, e.Z);
  copy<R, BR, NX, false, S::LDN, S::LDN>(t.U, Ee);
  mm<R, BR, NX, NX, false, true, S::LDN, S::LDN, S::LDN>(t.U, t.T1, e.Z, R(-1), true);
  mm<R, BR, NX, NX, false, false, S::LDN, S::LD2, S::LDN>(t.X, t.V, X21);
  copy<R, BR, NX, false, S::LDN, S::LDN>(t.T1, t.V);
  mm<R, BR, NX, NX, false, true, S::LDN, S::LDN, S::LDN>(t.T1, t.X, s.Vt, R(-1), true);
  copy<R, BR, NX, false, S::LDN, S::LDN>(Ba, Be);
  mm<R, BR, NX, NX, false, true, S::LDN, S::LDN, S::LDN>(Ba, t.T1, e.A, R(1), true);
  // N = A1 - Vt (Xi21^T A1)
  mm<R, NX, NX, NX, true, false, S::LD2, S::LDN, S::LDN>(s.T, X21, a.A);
  copy<R, NX, NX, false, S::LDN, S::LDN>(s.N, a.A);
  mm<R, NX, NX, NX, false, false, S::LDN, S::LDN, S::LDN>(s.N, s.Vt, s.T, R(-1), true);
  mm<R, BR, NX, NX, false, false, S::LDN, S::LDN, S::LDN>(Ea, t.U, s.N, R(1), true);
  mm<R, NX, NX, NX, true, false, S::LDN, S::LD2, S::LD2>(s.Wm, a.A, X22);
  copy<R, NX, NX, false, S::LD2, S::LDN>(s.Wm + NX, a.Z);
  tria<R, NX, 2 * NX, S::LD2>(s.Wm, s.vb);
  copy<R, NX, NX, false, S::LDN, S::LD2>(a.Z, s.Wm);
  mm<R, NX, NX, NX, false, false, S::LDN, S::LDN, S::LD2>(s.Wm, e.A, s.Vt);
  copy<R, NX, NX, false, S::LD2, S::LDN>(s.Wm + NX, e.U);
  tria<R, NX, 2 * NX, S::LD2>(s.Wm, s.vb);
  copy<R, NX, NX, false, S::LDN, S::LD2>(a.U, s.Wm);
  mm<R, NX, NX, NX, false, false, S::LDN, S::LDN, S::LDN>(a.A, e.A, s.N);
}

// State form with a shared factor L and batch means Mv:
//   V = Mv + (E2 L) L^T, X = V Xi21, W = V - X Vt^T, Mv' = W A2^T + B2, L' = tria([A2 Vt, U2]).
template <typename R, int NX, int NY>
SS_DEV void apply_b(R* L, R* Mv, FB<R> e, const R* Be, const R* Ee, FS<R> s, BT<R> t) {
  typedef DS<R, NX, NY> S;
  constexpr int BR = SB_ROWS;
  xi_core<R, NX, NY>(L, e.Z, s);
  const R* X21 = s.Xi + NX * S::LD2;
  mm<R, BR, NX, NX, false, false, S::LDN, S::LDN, S::LDN>(t.T1, Ee, L);
  copy<R, BR, NX, false, S::LDN, S::LDN>(t.V, Mv);
  mm<R, BR, NX, NX, false, true, S::LDN, S::LDN, S::LDN>(t.V, t.T1, L, R(1), true);
  mm<R, BR, NX, NX, false, false, S::LDN, S::LD2, S::LDN>(t.X, t.V, X21);
  copy<R, BR, NX, false, S::LDN, S::LDN>(t.T1, t.V);
  mm<R, BR, NX, NX, false, true, S::LDN, S::LDN, S::LDN>(t.T1, t.X, s.Vt, R(-1), true);
  copy<R, BR, NX, false, S::LDN, S::LDN>(Mv, Be);
  mm<R, BR, NX, NX, false, true, S::LDN, S::LDN, S::LDN>(Mv, t.T1, e.A, R(1), true);
  mm<R, NX, NX, NX, false, false, S::LDN, S::LDN, S::LD2>(s.Wm, e.A, s.Vt);
  copy<R, NX, NX, false, S::LD2, S::LDN>(s.Wm + NX, e.U);
  tria<R, NX, 2 * NX, S::LD2>(s.Wm, s.vb);
  copy<R, NX, NX, false, S::LDN, S::LD2>(L, s.Wm);
}

// Reverse-scan fold with shared (E, D) and batch g: a <- e (x) a, a earlier.
template <typename R, int NX, int NY>
SS_DEV void sfold_b(SB<R> a, R* Ga, SB<R> e, const R* Ge, R* Wm, R* T, R* vb) {
  typedef DS<R, NX, NY> S;
  mm<R, NX, NX, NX, false, false, S::LDN, S::LDN, S::LD2, true>(Wm, a.E, e.D);
  copy<R, NX, NX, false, S::LD2, S::LDN>(Wm + NX, a.D);
  tria<R, NX, 2 * NX, S::LD2>(Wm, vb);
  mm<R, SB_ROWS, NX, NX, false, true, S::LDN, S::LDN, S::LDN>(Ga, Ge, a.E, R(1), true);
  mm<R, NX, NX, NX, false, false, S::LDN, S::LDN, S::LDN>(T, a.E, e.E);
  copy<R, NX, NX, false, S::LDN, S::LDN>(a.E, T);
  copy<R, NX, NX, false, S::LDN, S::LD2>(a.D, Wm);
}

// Smoothed (L, Mv) at the end of e's range -> its start: Mv <- Mv E^T + G, L <- tria([E L, D]).
template <typename R, int NX, int NY>
SS_DEV void sapply_b(R* L, R* Mv, SB<R> e, const R* Ge, R* Wm, R* T, R* vb) {
  typedef DS<R, NX, NY> S;
  mm<R, NX, NX, NX, false, false, S::LDN, S::LDN, S::LD2, true>(Wm, e.E, L);
  copy<R, NX, NX, false, S::LD2, S::LDN>(Wm + NX, e.D);
  tria<R, NX, 2 * NX, S::LD2>(Wm, vb);
  copy<R, NX, NX, false, S::LDN, S::LD2>(L, Wm);
  copy<R, SB_ROWS, NX, false, S::LDN, S::LDN>(T, Ge);
  mm<R, SB_ROWS, NX, NX, false, true, S::LDN, S::LDN, S::LDN>(T, Mv, e.E, R(1), true);
  copy<R, SB_ROWS, NX, false, S::LDN, S::LDN>(Mv, T);
}

// Per-sequence bookkeeping of a smoothed batch state at step index t of every sequence.
template <typename R, int NX, int NY>
SS_DEV void out_rows(const ScanArgs<R>& sa, int B, int64_t Tp1, int64_t t, const R* L, const R* Mv) {
  typedef DS<R, NX, NY> S;
  const int l = lane_id();
  for (int i = 0; i < B; ++i) s2g<R, NX, NX, S::LDN>(sa.out_L + ((int64_t)i * Tp1 + t) * NX * NX, L);
  store_rows<R, NX, NY>(sa.out_m + t * NX, Tp1 * NX, 0, Mv, B);
  if (sa.mse != nullptr || sa.flags != nullptr) {
    double d = 0.0;
    bool bad = false;
    if (l < B) {
      const int64_t s = (int64_t)l * Tp1 + t;
      SS_UNROLL
      for (int k = 0; k < NX; ++k) {
        const R v = Mv[l * S::LDN + k];
        bad = bad || !ss_isfinite(v);
        if (sa.mse != nullptr) {
          const double e = (double)v - (double)sa.prev_m[s * NX + k];
          d += e * e;
        }
      }
      if (sa.mse != nullptr) atomicAdd(sa.mse + l, d);
      if (sa.flags != nullptr && bad) atomicOr(sa.flags + l, 1u);
    }
  }
  __syncwarp();
}

// ----------------------------------------------------------------------------- filter levels

template <typename R, int NX, int NY>
__host__ __device__ constexpr int up_b_elems() {
  return 2 * (3 * DS<R, NX, NY>::MN + 2 * DSS<R, NX, NY>::MB) + fs_elems<R, NX, NY>() + 4 * DSS<R, NX, NY>::MB;
}

// Level lv -> lv+1: warp per group index q (per sequence), members [q G, min(q G + G, n)).
template <typename R, int NX, int NY>
__global__ void __launch_bounds__(32) up_b_kernel(DenseArgs<R> a, int lv, int B, int64_t n_lo, int64_t n_hi) {
  typedef DS<R, NX, NY> S;
  typedef DSS<R, NX, NY> SS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* p = reinterpret_cast<R*>(smem_raw);
  const ScanArgs<R>& sa = a.s;
  const int64_t q = blockIdx.x;
  if (q >= n_hi) return;
  const int64_t m0 = q * sa.g.G, m1 = min(m0 + (int64_t)sa.g.G, n_lo);
  zero(p, up_b_elems<R, NX, NY>());
  FB<R> acc, e;
  acc.A = p; p += S::MN; acc.U = p; p += S::MN; acc.Z = p; p += S::MN;
  R* Ba = p; p += SS::MB;
  R* Ea = p; p += SS::MB;
  e.A = p; p += S::MN; e.U = p; p += S::MN; e.Z = p; p += S::MN;
  R* Be = p; p += SS::MB;
  R* Ee = p; p += SS::MB;
  FS<R> s = carve_fs<R, NX, NY>(p);
  BT<R> t = carve_bt<R, NX, NY>(p);
  const R* lo = sa.fsum[lv];
  const int64_t st_lo = n_lo * S::FE;
  g2s<R, NX, NX, S::LDN>(acc.A, lo + m0 * S::FE);
  g2s<R, NX, NX, S::LDN>(acc.U, lo + m0 * S::FE + NX * NX);
  g2s<R, NX, NX, S::LDN>(acc.Z, lo + m0 * S::FE + 2 * NX * NX);
  load_rows<R, NX, NY>(Ba, lo + m0 * S::FE, st_lo, 3 * NX * NX, B);
  load_rows<R, NX, NY>(Ea, lo + m0 * S::FE, st_lo, 3 * NX * NX + NX, B);
  for (int64_t m = m0 + 1; m < m1; ++m) {
    g2s<R, NX, NX, S::LDN>(e.A, lo + m * S::FE);
    g2s<R, NX, NX, S::LDN>(e.U, lo + m * S::FE + NX * NX);
    g2s<R, NX, NX, S::LDN>(e.Z, lo + m * S::FE + 2 * NX * NX);
    load_rows<R, NX, NY>(Be, lo + m * S::FE, st_lo, 3 * NX * NX, B);
    load_rows<R, NX, NY>(Ee, lo + m * S::FE, st_lo, 3 * NX * NX + NX, B);
    combine_b<R, NX, NY>(acc, Ba, Ea, e, Be, Ee, s, t);
  }
  R* hi = sa.fsum[lv + 1] + q * S::FE;
  s2g<R, NX, NX, S::LDN>(hi, acc.A);
  s2g<R, NX, NX, S::LDN>(hi + NX * NX, acc.U);
  s2g<R, NX, NX, S::LDN>(hi + 2 * NX * NX, acc.Z);
  store_rows<R, NX, NY>(hi, n_hi * S::FE, 3 * NX * NX, Ba, B);
  store_rows<R, NX, NY>(hi, n_hi * S::FE, 3 * NX * NX + NX, Ea, B);
}

template <typename R, int NX, int NY>
__host__ __device__ constexpr int apply_b_elems() {
  return DS<R, NX, NY>::MN + DSS<R, NX, NY>::MB + 3 * DS<R, NX, NY>::MN + 2 * DSS<R, NX, NY>::MB +
         fs_elems<R, NX, NY>() + 4 * DSS<R, NX, NY>::MB;
}

// Shared entry factor and batch entry means of the items [m0, m1) at level lv,
// starting from (L, Mv); stores each item's entry state and applies the items.
template <typename R, int NX, int NY>
SS_DEV void walk_items_b(const ScanArgs<R>& sa, int lv, int B, int64_t n, int64_t m0, int64_t m1, R* L, R* Mv,
                         FB<R> e, R* Be, R* Ee, FS<R> s, BT<R> t) {
  typedef DS<R, NX, NY> S;
  for (int64_t m = m0; m < m1; ++m) {
    R* st = sa.fst[lv] + m * S::ST;
    s2g<R, NX, NX, S::LDN>(st, L);
    store_rows<R, NX, NY>(st, n * S::ST, NX * NX, Mv, B);
    if (m + 1 < m1) {
      const R* f = sa.fsum[lv] + m * S::FE;
      g2s<R, NX, NX, S::LDN>(e.A, f);
      g2s<R, NX, NX, S::LDN>(e.U, f + NX * NX);
      g2s<R, NX, NX, S::LDN>(e.Z, f + 2 * NX * NX);
      load_rows<R, NX, NY>(Be, f, n * S::FE, 3 * NX * NX, B);
      load_rows<R, NX, NY>(Ee, f, n * S::FE, 3 * NX * NX + NX, B);
      apply_b<R, NX, NY>(L, Mv, e, Be, Ee, s, t);
    }
  }
}

// Top level (one warp): from the shared prior through the n top items.
template <typename R, int NX, int NY>
__global__ void __launch_bounds__(32) top_b_kernel(DenseArgs<R> a, int B, int64_t n, int64_t T) {
  typedef DS<R, NX, NY> S;
  typedef DSS<R, NX, NY> SS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* p = reinterpret_cast<R*>(smem_raw);
  const ScanArgs<R>& sa = a.s;
  zero(p, apply_b_elems<R, NX, NY>());
  R* L = p; p += S::MN;
  R* Mv = p; p += SS::MB;
  FB<R> e;
  e.A = p; p += S::MN; e.U = p; p += S::MN; e.Z = p; p += S::MN;
  R* Be = p; p += SS::MB;
  R* Ee = p; p += SS::MB;
  FS<R> s = carve_fs<R, NX, NY>(p);
  BT<R> t = carve_bt<R, NX, NY>(p);
  const int l = lane_id();
  g2s_any<R, NX, NX, S::LDN>(L, sa.L0);
  if (l < NX) {
    SS_UNROLL
    for (int k = 0; k < NX; ++k)
      if (k > l) L[l * S::LDN + k] = R(0);
  }
  if (l < B) {
    SS_UNROLL
    for (int k = 0; k < NX; ++k) Mv[l * S::LDN + k] = sa.m0[k];
  }
  __syncwarp();
  if (sa.filt_m != nullptr) {
    for (int i = 0; i < B; ++i) s2g<R, NX, NX, S::LDN>(sa.filt_L + (int64_t)i * (T + 1) * NX * NX, L);
    store_rows<R, NX, NY>(sa.filt_m, (T + 1) * NX, 0, Mv, B);
  }
  walk_items_b<R, NX, NY>(sa, sa.g.L, B, n, 0, n, L, Mv, e, Be, Ee, s, t);
}

template <typename R, int NX, int NY>
__global__ void __launch_bounds__(32) down_b_kernel(DenseArgs<R> a, int lv, int B, int64_t n_lo, int64_t n_hi) {
  typedef DS<R, NX, NY> S;
  typedef DSS<R, NX, NY> SS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* p = reinterpret_cast<R*>(smem_raw);
  const ScanArgs<R>& sa = a.s;
  const int64_t q = blockIdx.x;
  if (q >= n_hi) return;
  zero(p, apply_b_elems<R, NX, NY>());
  R* L = p; p += S::MN;
  R* Mv = p; p += SS::MB;
  FB<R> e;
  e.A = p; p += S::MN; e.U = p; p += S::MN; e.Z = p; p += S::MN;
  R* Be = p; p += SS::MB;
  R* Ee = p; p += SS::MB;
  FS<R> s = carve_fs<R, NX, NY>(p);
  BT<R> t = carve_bt<R, NX, NY>(p);
  const R* st = sa.fst[lv + 1] + q * S::ST;
  g2s<R, NX, NX, S::LDN>(L, st);
  load_rows<R, NX, NY>(Mv, st, n_hi * S::ST, NX * NX, B);
  const int64_t m0 = q * sa.g.G, m1 = min(m0 + (int64_t)sa.g.G, n_lo);
  walk_items_b<R, NX, NY>(sa, lv, B, n_lo, m0, m1, L, Mv, e, Be, Ee, s, t);
}

// ----------------------------------------------------------------------------- filter walk

template <typename R, int NX, int NY>
__host__ __device__ constexpr int walk_b_warp_elems() {
  typedef DS<R, NX, NY> S;
  typedef DSS<R, NX, NY> SS;
  return 2 * S::MN + (NY + NX) * S::LDY + 3 * SS::MB + 2 * SS::MBY + S::VB;
}
template <typename R, int NX, int NY>
__host__ __device__ constexpr int walk_b_warps() {
  constexpr int budget = 200 * 1024 / (int)sizeof(R);
  constexpr int w = (budget - mc_elems<R, NX, NY>()) / walk_b_warp_elems<R, NX, NY>();
  return w < 1 ? 1 : (w > 8 ? 8 : w);
}
template <typename R, int NX, int NY>
__host__ __device__ constexpr int walk_b_elems() {
  return mc_elems<R, NX, NY>() + walk_b_warps<R, NX, NY>() * walk_b_warp_elems<R, NX, NY>();
}

// Row r of Phi = [[F L, cQ], [L, 0]] (L lower, in shared memory) into registers,
// row r in lane r % 32, slot r / 32.
template <typename R, int NX, int NY>
SS_DEV void phi_rows(MC<R> c, const R* L, R (&row)[(2 * NX + 31) / 32][Pad<R, 2 * NX>::n]) {
  typedef DS<R, NX, NY> S;
  constexpr int W = S::W, CP = Pad<R, 2 * NX>::n;
  const int l = lane_id();
  SS_UNROLL
  for (int s = 0; s < (2 * NX + 31) / 32; ++s) {
    const int r = l + 32 * s;
    SS_UNROLL
    for (int j = 0; j < CP; ++j) row[s][j] = R(0);
    if (r < NX) {
      R f[S::VN];
      load_row<R, NX, S::LDN>(c.F, r, f);
      SS_UNROLL
      for (int k = 0; k < NX; ++k) {
        SS_UNROLL
        for (int j = 0; j <= k; j += W) {
          const Vec<R> b = ld16(L + k * S::LDN + j);
          SS_UNROLL
          for (int u = 0; u < W; ++u) row[s][j + u] += f[k] * b.v[u];
        }
      }
      SS_UNROLL
      for (int j = 0; j < NX; j += W) {
        const Vec<R> q = ld16(c.cQ + r * S::LDN + j);
        SS_UNROLL
        for (int u = 0; u < W; ++u) row[s][NX + j + u] = q.v[u];
      }
    } else if (r < 2 * NX) {
      SS_UNROLL
      for (int j = 0; j < NX; j += W) {
        const Vec<R> q = ld16(L + (r - NX) * S::LDN + j);
        SS_UNROLL
        for (int u = 0; u < W; ++u) row[s][j + u] = q.v[u];
      }
    }
  }
}

// Row r of Psi = [[H N1, cR], [N1, 0]] (N1 lower, in shared memory) into registers.
template <typename R, int NX, int NY>
SS_DEV void psi_rows(MC<R> c, const R* N1, R (&row)[(NX + NY + 31) / 32][Pad<R, NX + NY>::n]) {
  typedef DS<R, NX, NY> S;
  constexpr int W = S::W, CP = Pad<R, NX + NY>::n;
  const int l = lane_id();
  SS_UNROLL
  for (int s = 0; s < (NX + NY + 31) / 32; ++s) {
    const int r = l + 32 * s;
    SS_UNROLL
    for (int j = 0; j < CP; ++j) row[s][j] = R(0);
    if (r < NY) {
      R h[S::VN];
      load_row<R, NX, S::LDN>(c.H, r, h);
      SS_UNROLL
      for (int k = 0; k < NX; ++k) {
        SS_UNROLL
        for (int j = 0; j <= k; j += W) {
          const Vec<R> b = ld16(N1 + k * S::LDN + j);
          SS_UNROLL
          for (int u = 0; u < W; ++u) row[s][j + u] += h[k] * b.v[u];
        }
      }
      SS_UNROLL
      for (int j = 0; j < NY; j += W) {
        const Vec<R> q = ld16(c.cR + r * S::LDY + j);
        SS_UNROLL
        for (int u = 0; u < W; ++u) row[s][NX + j + u] = q.v[u];
      }
    } else if (r < NY + NX) {
      SS_UNROLL
      for (int j = 0; j < NX; j += W) {
        const Vec<R> q = ld16(N1 + (r - NY) * S::LDN + j);
        SS_UNROLL
        for (int u = 0; u < W; ++u) row[s][j + u] = q.v[u];
      }
    }
  }
}

// Kalman steps of chunk c of every sequence: the factor recursion once, the
// means as B rows.  Phi and Psi are built and triangularised in registers;
// only Phi11 (= the predicted factor N1), E and Psi's blocks go through
// shared memory.  Emits E, D (sequence 0's records) and g (every sequence's).
template <typename R, int NX, int NY>
__global__ void __launch_bounds__(32 * walk_b_warps<R, NX, NY>())
    walk_b_kernel(DenseArgs<R> a, int B, int64_t n_chunks, int64_t T) {
  typedef DS<R, NX, NY> S;
  typedef DSS<R, NX, NY> SS;
  constexpr int WARPS = walk_b_warps<R, NX, NY>();
  constexpr int BR = SB_ROWS;
  constexpr int W = S::W;
  constexpr int NSF = (2 * NX + 31) / 32, CPF = Pad<R, 2 * NX>::n;
  constexpr int NSP = (NX + NY + 31) / 32, CPP = Pad<R, NX + NY>::n;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* p = reinterpret_cast<R*>(smem_raw);
  const int warp = threadIdx.x >> 5, l = lane_id();
  MC<R> c = carve_mc<R, NX, NY>(p);
  p += warp * walk_b_warp_elems<R, NX, NY>();
  zero(p, walk_b_warp_elems<R, NX, NY>());
  if (warp == 0) load_mc<R, NX, NY>(c, a);
  __syncthreads();
  R* L = p; p += S::MN;
  R* Eb = p; p += S::MN;
  R* P11 = p; p += NY * S::LDY;
  R* P21 = p; p += NX * S::LDY;
  R* Mv = p; p += SS::MB;
  R* MP = p; p += SS::MB;
  R* Gv = p; p += SS::MB;
  R* Rv = p; p += SS::MBY;
  R* Zv = p; p += SS::MBY;
  R* vb = p;
  const ScanArgs<R>& sa = a.s;
  const int64_t j = (int64_t)blockIdx.x * WARPS + warp;
  if (j >= n_chunks) return;
  const int64_t t0 = j * sa.g.C, t1 = min(t0 + (int64_t)sa.g.C, T);
  const R* st = sa.fst[1] + j * S::ST;
  g2s<R, NX, NX, S::LDN>(L, st);
  load_rows<R, NX, NY>(Mv, st, n_chunks * S::ST, NX * NX, B);
  double ll = 0.0;
  for (int64_t t = t0; t < t1; ++t) {
    R* rec = sa.selem + t * S::SE;
    {
      // Phi = tria([[F L, cQ], [L, 0]]): Phi11 -> L (= N1), E = Phi21 Phi11^{-1} -> Eb, D -> record
      R row[NSF][CPF];
      phi_rows<R, NX, NY>(c, L, row);
      __syncwarp();
      Tria<R, 2 * NX, 2 * NX, CPF, false>::run_regs(row, vb);
      SS_UNROLL
      for (int s = 0; s < NSF; ++s) {
        const int r = l + 32 * s;
        if (r < NX) store_part<R, NX, S::LDN, 0>(L, r, row[s]);
      }
      __syncwarp();
      SS_UNROLL
      for (int s = 0; s < NSF; ++s) {
        const int r = l + 32 * s;
        if (r >= NX && r < 2 * NX) {
          SS_UNROLL
          for (int k = NX - 1; k >= 0; --k) {
            row[s][k] = row[s][k] * ss_rcp(L[k * S::LDN + k]);
            SS_UNROLL
            for (int jj = 0; jj < k; jj += W) {
              const Vec<R> lv = ld16(L + k * S::LDN + jj);
              SS_UNROLL
              for (int u = 0; u < W; ++u)
                if (jj + u < k) row[s][jj + u] -= row[s][k] * lv.v[u];
            }
          }
          store_part<R, NX, S::LDN, 0>(Eb, r - NX, row[s]);
          if (sa.emit_smoother) {
            R* dst = rec + NX * NX + (r - NX) * NX;
            SS_UNROLL
            for (int jj = 0; jj < NX; jj += W) {
              Vec<R> o;
              SS_UNROLL
              for (int u = 0; u < W; ++u) o.v[u] = row[s][NX + jj + u];
              st16(dst + jj, o);
            }
          }
        }
      }
      __syncwarp();
    }
    // MP = Mv F^T + bq, G = Mv - MP E^T (rows = sequences)
    mm<R, BR, NX, NX, false, true, S::LDN, S::LDN, S::LDN>(MP, Mv, c.F);
    if (l < B) {
      SS_UNROLL
      for (int k = 0; k < NX; ++k) MP[l * S::LDN + k] += c.bq[k];
    }
    __syncwarp();
    copy<R, BR, NX, false, S::LDN, S::LDN>(Gv, Mv);
    mm<R, BR, NX, NX, false, true, S::LDN, S::LDN, S::LDN>(Gv, MP, Eb, R(-1), true);
    if (sa.emit_smoother) {
      s2g<R, NX, NX, S::LDN>(rec, Eb);
      store_rows<R, NX, NY>(rec, T * S::SE, 2 * NX * NX, Gv, B);
    }
    {
      // Psi = tria([[H N1, cR], [N1, 0]]): Psi11 -> P11, Psi21 -> P21, Psi22 -> L
      R row[NSP][CPP];
      psi_rows<R, NX, NY>(c, L, row);
      __syncwarp();
      Tria<R, NX + NY, NX + NY, CPP, false>::run_regs(row, vb);
      SS_UNROLL
      for (int s = 0; s < NSP; ++s) {
        const int r = l + 32 * s;
        if (r < NY) {
          store_part<R, NY, S::LDY, 0>(P11, r, row[s]);
        } else if (r < NY + NX) {
          store_part<R, NY, S::LDY, 0>(P21, r - NY, row[s]);
          store_part<R, NX, S::LDN, NY>(L, r - NY, row[s]);
        }
      }
      __syncwarp();
    }
    // residual rows r_i = y_i - c - H mp_i, z_i = Psi11^{-1} r_i
    mm<R, BR, NX, NY, false, true, S::LDN, S::LDN, S::LDY>(Rv, MP, c.H);
    if (l < B) {
      const R* y = sa.ys + ((int64_t)l * T + t) * NY;
      SS_UNROLL
      for (int k = 0; k < NY; ++k) Rv[l * S::LDY + k] = y[k] - c.c[k] - Rv[l * S::LDY + k];
    }
    __syncwarp();
    copy<R, BR, NY, false, S::LDY, S::LDY>(Zv, Rv);
    trsm_rlt<R, BR, NY, S::LDY, S::LDY>(Zv, P11);
    if (l < B) {
      R q = R(0), ld = R(0);
      SS_UNROLL
      for (int k = 0; k < NY; ++k) {
        const R z = Zv[l * S::LDY + k];
        q += z * z;
        ld += ss_log(ss_abs(P11[k * S::LDY + k]));
      }
      ll += -0.5 * ((double)q + 2.0 * (double)ld);
    }
    // Mv = MP + Z Psi21^T
    copy<R, BR, NX, false, S::LDN, S::LDN>(Mv, MP);
    mm<R, BR, NY, NX, false, true, S::LDY, S::LDY, S::LDN>(Mv, Zv, P21, R(1), true);
    if (sa.filt_m != nullptr) {
      for (int i = 0; i < B; ++i) s2g<R, NX, NX, S::LDN>(sa.filt_L + ((int64_t)i * (T + 1) + t + 1) * NX * NX, L);
      store_rows<R, NX, NY>(sa.filt_m + (t + 1) * NX, (T + 1) * NX, 0, Mv, B);
    }
  }
  if (sa.ll_chunk != nullptr && l < B) sa.ll_chunk[(int64_t)l * n_chunks + j] = ll;
  if (t1 == T) {
    for (int i = 0; i < B; ++i) s2g<R, NX, NX, S::LDN>(sa.fT + (int64_t)i * S::ST, L);
    store_rows<R, NX, NY>(sa.fT, S::ST, NX * NX, Mv, B);
  }
}

// ----------------------------------------------------------------------------- per-sequence walk, register rows

// The per-sequence Kalman walk (walk_kernel's results, up to rounding) with Phi
// and Psi built and triangularised in registers as walk_b_kernel does: only the
// factor, Psi's blocks and the vectors go through shared memory, about 9 KB per
// warp against walk_kernel's 23 KB (whose Phi region alone is 17 KB), so the
// SM holds more warps.  FP32 (the rows of an FP64 Phi would not fit the
// register file).
template <typename R, int NX, int NY>
__host__ __device__ constexpr int walk_r_warp_elems() {
  typedef DS<R, NX, NY> S;
  return S::MN + (NY + NX) * S::LDY + 2 * S::VN + S::VY +
         2 * (Pad<R, (2 * NX > NX + NY ? 2 * NX : NX + NY)>::n + Vec<R>::n);
}
constexpr int WALK_R_WARPS = 2;
// Minimum resident blocks requested from the register allocator: one (229-242
// registers, 4 blocks = 8 warps per SM); a cap of 168 registers for five blocks
// spilled 644 bytes per thread.
#ifndef SS_DENSE_WALK_MINB
#define SS_DENSE_WALK_MINB 1
#endif
template <typename R, int NX, int NY>
__host__ __device__ constexpr int walk_r_elems() {
  return mc_elems<R, NX, NY>() + WALK_R_WARPS * walk_r_warp_elems<R, NX, NY>();
}

template <typename R, int NX, int NY>
__global__ void __launch_bounds__(32 * WALK_R_WARPS, SS_DENSE_WALK_MINB) walk_r_kernel(DenseArgs<R> a) {
  typedef DS<R, NX, NY> S;
  constexpr int W = S::W;
  constexpr int NSF = (2 * NX + 31) / 32, CPF = Pad<R, 2 * NX>::n;
  constexpr int NSP = (NX + NY + 31) / 32, CPP = Pad<R, NX + NY>::n;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* p = reinterpret_cast<R*>(smem_raw);
  const int warp = threadIdx.x >> 5, l = lane_id();
  MC<R> c = carve_mc<R, NX, NY>(p);
  p += warp * walk_r_warp_elems<R, NX, NY>();
  zero(p, walk_r_warp_elems<R, NX, NY>());
  if (warp == 0) load_mc<R, NX, NY>(c, a);
  __syncthreads();
  R* L = p; p += S::MN;
  R* P11 = p; p += NY * S::LDY;
  R* P21 = p; p += NX * S::LDY;
  R* m = p; p += S::VN;
  R* mp = p; p += S::VN;
  R* rv = p; p += S::VY;
  R* vb = p;
  const ScanArgs<R>& sa = a.s;
  const int64_t j = (int64_t)blockIdx.x * WALK_R_WARPS + warp;
  if (j >= sa.g.lvl[1][sa.g.B]) return;
  int64_t i, t0, t1;
  chunk_of(sa.g, j, i, t0, t1);
  if (seq_inactive(sa.active, i)) return;
  const int64_t base = sa.g.off[i];
  load_st<R, NX, NY>(L, m, sa.fst[1] + j * S::ST);
  double ll = 0.0;
  for (int64_t t = t0; t < t1; ++t) {
    R* rec = sa.selem + (base + t) * S::SE;
    {
      // Phi = tria([[F L, cQ], [L, 0]]): Phi11 -> L (the predicted factor N1), and
      // per row of Phi21 E = Phi21 Phi11^{-1}, D = Phi22 and g = m - E mp into the record
      R row[NSF][CPF];
      phi_rows<R, NX, NY>(c, L, row);
      const R mpl = rowdot<R, NX, NX, false, S::LDN>(c.F, m, l) + (l < NX ? c.bq[l] : R(0));
      __syncwarp();
      Tria<R, 2 * NX, 2 * NX, CPF>::run_regs(row, vb);
      if (l < NX) mp[l] = mpl;
      SS_UNROLL
      for (int s = 0; s < NSF; ++s) {
        const int r = l + 32 * s;
        if (r < NX) store_part<R, NX, S::LDN, 0>(L, r, row[s]);
      }
      __syncwarp();
      SS_UNROLL
      for (int s = 0; s < NSF; ++s) {
        const int r = l + 32 * s;
        if (r >= NX && r < 2 * NX && sa.emit_smoother) {
          SS_UNROLL
          for (int k = NX - 1; k >= 0; --k) {
            row[s][k] = row[s][k] * ss_rcp(L[k * S::LDN + k]);
            SS_UNROLL
            for (int jj = 0; jj < k; jj += W) {
              const Vec<R> lv = ld16(L + k * S::LDN + jj);
              SS_UNROLL
              for (int u = 0; u < W; ++u)
                if (jj + u < k) row[s][jj + u] -= row[s][k] * lv.v[u];
            }
          }
          R g = m[r - NX];
          SS_UNROLL
          for (int k = 0; k < NX; ++k) g -= row[s][k] * mp[k];
          R* de = rec + (r - NX) * NX;
          R* dd = rec + NX * NX + (r - NX) * NX;
          SS_UNROLL
          for (int jj = 0; jj < NX; jj += W) {
            Vec<R> oe, od;
            SS_UNROLL
            for (int u = 0; u < W; ++u) {
              oe.v[u] = row[s][jj + u];
              od.v[u] = row[s][NX + jj + u];
            }
            st16(de + jj, oe);
            st16(dd + jj, od);
          }
          rec[2 * NX * NX + r - NX] = g;
        }
      }
      __syncwarp();
    }
    {
      // update: Psi = tria([[H N1, cR], [N1, 0]]): Psi11 -> P11, Psi21 -> P21, Psi22 -> L
      R row[NSP][CPP];
      psi_rows<R, NX, NY>(c, L, row);
      __syncwarp();
      Tria<R, NX + NY, NX + NY, CPP>::run_regs(row, vb);
      SS_UNROLL
      for (int s = 0; s < NSP; ++s) {
        const int r = l + 32 * s;
        if (r < NY) {
          store_part<R, NY, S::LDY, 0>(P11, r, row[s]);
        } else if (r < NY + NX) {
          store_part<R, NY, S::LDY, 0>(P21, r - NY, row[s]);
          store_part<R, NX, S::LDN, NY>(L, r - NY, row[s]);
        }
      }
      __syncwarp();
    }
    const R res = (l < NY ? sa.ys[(base + t) * NY + l] - c.c[l] : R(0)) - rowdot<R, NY, NX, false, S::LDN>(c.H, mp, l);
    if (l < NY) rv[l] = res;
    __syncwarp();
    R z[NY];
    R q = R(0), ld = R(0);
    SS_UNROLL
    for (int k = 0; k < NY; ++k) {
      R t2 = rv[k];
      SS_UNROLL
      for (int jj = 0; jj < k; ++jj) t2 -= P11[k * S::LDY + jj] * z[jj];
      const R dk = P11[k * S::LDY + k];
      z[k] = t2 / dk;
      q += z[k] * z[k];
      ld += ss_log(ss_abs(dk));
    }
    ll += -0.5 * ((double)q + 2.0 * (double)ld);
    const int il = l < NX ? l : NX - 1;
    R mn = mp[il];
    SS_UNROLL
    for (int k = 0; k < NY; ++k) mn += P21[il * S::LDY + k] * z[k];
    __syncwarp();
    if (l < NX) m[l] = mn;
    __syncwarp();
    if (sa.filt_m != nullptr) store_traj<R, NX, NY>(sa.filt_m, sa.filt_L, base + i + t + 1, L, m);
  }
  if (sa.ll_chunk != nullptr && l == 0) sa.ll_chunk[j] = ll;
  if (t1 == sa.g.off[i + 1] - base) store_st<R, NX, NY>(sa.fT + i * S::ST, L, m);
}

// ----------------------------------------------------------------------------- smoother

template <typename R, int NX, int NY>
__host__ __device__ constexpr int sfold_b_warp_elems() {
  typedef DS<R, NX, NY> S;
  return 4 * S::MN + 2 * DSS<R, NX, NY>::MB + S::MW + S::MN + S::VB;
}

template <typename R, int NX, int NY>
SS_DEV void load_sb_b(SB<R> e, R* Gv, const R* rec, int64_t stride, int B) {
  typedef DS<R, NX, NY> S;
  g2s<R, NX, NX, S::LDN>(e.E, rec);
  g2s<R, NX, NX, S::LDN>(e.D, rec + NX * NX);
  load_rows<R, NX, NY>(Gv, rec, stride, 2 * NX * NX, B);
}
template <typename R, int NX, int NY>
SS_DEV void store_sb_b(R* rec, int64_t stride, SB<R> e, const R* Gv, int B) {
  typedef DS<R, NX, NY> S;
  s2g<R, NX, NX, S::LDN>(rec, e.E);
  s2g<R, NX, NX, S::LDN>(rec + NX * NX, e.D);
  store_rows<R, NX, NY>(rec, stride, 2 * NX * NX, Gv, B);
}

// Level-1 smoothing summaries of chunk j (all sequences), or level lv -> lv+1 groups.
template <typename R, int NX, int NY>
__global__ void __launch_bounds__(32 * SFOLD_WARPS)
    sfold_b_kernel(DenseArgs<R> a, int lv, int B, int64_t n_lo, int64_t n_hi, int64_t T) {
  typedef DS<R, NX, NY> S;
  typedef DSS<R, NX, NY> SS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5;
  R* p = reinterpret_cast<R*>(smem_raw) + warp * sfold_b_warp_elems<R, NX, NY>();
  const ScanArgs<R>& sa = a.s;
  const int64_t q = (int64_t)blockIdx.x * SFOLD_WARPS + warp;
  if (q >= n_hi) return;
  zero(p, sfold_b_warp_elems<R, NX, NY>());
  SB<R> acc, e;
  acc.E = p; p += S::MN; acc.D = p; p += S::MN;
  e.E = p; p += S::MN; e.D = p; p += S::MN;
  R* Ga = p; p += SS::MB;
  R* Ge = p; p += SS::MB;
  R* Wm = p; p += S::MW;
  R* Tm = p; p += S::MN;
  R* vb = p;
  // level 1 folds the chunk's per-step elements (stride T per sequence), higher levels the
  // level-lv summaries (stride n_lo)
  const R* src = lv == 0 ? sa.selem : sa.ssum[lv];
  const int64_t width = lv == 0 ? (int64_t)sa.g.C : (int64_t)sa.g.G;
  const int64_t m0 = q * width, m1 = min(m0 + width, n_lo);
  load_sb_b<R, NX, NY>(acc, Ga, src + m0 * S::SE, n_lo * S::SE, B);
  for (int64_t m = m0 + 1; m < m1; ++m) {
    load_sb_b<R, NX, NY>(e, Ge, src + m * S::SE, n_lo * S::SE, B);
    sfold_b<R, NX, NY>(acc, Ga, e, Ge, Wm, Tm, vb);
  }
  store_sb_b<R, NX, NY>(sa.ssum[lv == 0 ? 1 : lv + 1] + q * S::SE, n_hi * S::SE, acc, Ga, B);
}

template <typename R, int NX, int NY>
__host__ __device__ constexpr int sapply_b_warp_elems() {
  typedef DS<R, NX, NY> S;
  return S::MN + 2 * S::MN + 3 * DSS<R, NX, NY>::MB + S::MW + S::VB;
}

// Smoothed states entering items [m1-1 .. m0] at level lv, from (L, Mv) at the end.
template <typename R, int NX, int NY>
SS_DEV void swalk_items_b(const ScanArgs<R>& sa, int lv, int B, int64_t n, int64_t m0, int64_t m1, R* L, R* Mv,
                          SB<R> e, R* Ge, R* Wm, R* Tm, R* vb) {
  typedef DS<R, NX, NY> S;
  for (int64_t m = m1 - 1; m >= m0; --m) {
    R* st = sa.sst[lv] + m * S::ST;
    s2g<R, NX, NX, S::LDN>(st, L);
    store_rows<R, NX, NY>(st, n * S::ST, NX * NX, Mv, B);
    if (m > m0) {
      load_sb_b<R, NX, NY>(e, Ge, sa.ssum[lv] + m * S::SE, n * S::SE, B);
      sapply_b<R, NX, NY>(L, Mv, e, Ge, Wm, Tm, vb);
    }
  }
}

template <typename R, int NX, int NY>
__global__ void __launch_bounds__(32) stop_b_kernel(DenseArgs<R> a, int B, int64_t n, int64_t T) {
  typedef DS<R, NX, NY> S;
  typedef DSS<R, NX, NY> SS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* p = reinterpret_cast<R*>(smem_raw);
  const ScanArgs<R>& sa = a.s;
  zero(p, sapply_b_warp_elems<R, NX, NY>());
  R* L = p; p += S::MN;
  SB<R> e;
  e.E = p; p += S::MN; e.D = p; p += S::MN;
  R* Mv = p; p += SS::MB;
  R* Ge = p; p += SS::MB;
  R* Tm = p; p += SS::MB;
  R* Wm = p; p += S::MW;
  R* vb = p;
  g2s<R, NX, NX, S::LDN>(L, sa.fT);
  load_rows<R, NX, NY>(Mv, sa.fT, S::ST, NX * NX, B);
  out_rows<R, NX, NY>(sa, B, T + 1, T, L, Mv);
  swalk_items_b<R, NX, NY>(sa, sa.g.L, B, n, 0, n, L, Mv, e, Ge, Wm, Tm, vb);
}

template <typename R, int NX, int NY>
__global__ void __launch_bounds__(32) sdown_b_kernel(DenseArgs<R> a, int lv, int B, int64_t n_lo, int64_t n_hi) {
  typedef DS<R, NX, NY> S;
  typedef DSS<R, NX, NY> SS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* p = reinterpret_cast<R*>(smem_raw);
  const ScanArgs<R>& sa = a.s;
  const int64_t q = blockIdx.x;
  if (q >= n_hi) return;
  zero(p, sapply_b_warp_elems<R, NX, NY>());
  R* L = p; p += S::MN;
  SB<R> e;
  e.E = p; p += S::MN; e.D = p; p += S::MN;
  R* Mv = p; p += SS::MB;
  R* Ge = p; p += SS::MB;
  R* Tm = p; p += SS::MB;
  R* Wm = p; p += S::MW;
  R* vb = p;
  const R* st = sa.sst[lv + 1] + q * S::ST;
  g2s<R, NX, NX, S::LDN>(L, st);
  load_rows<R, NX, NY>(Mv, st, n_hi * S::ST, NX * NX, B);
  const int64_t m0 = q * sa.g.G, m1 = min(m0 + (int64_t)sa.g.G, n_lo);
  swalk_items_b<R, NX, NY>(sa, lv, B, n_lo, m0, m1, L, Mv, e, Ge, Wm, Tm, vb);
}

template <typename R, int NX, int NY>
__host__ __device__ constexpr int swalk_b_warps() {
  constexpr int w = 200 * 1024 / (int)sizeof(R) / sapply_b_warp_elems<R, NX, NY>();
  return w < 1 ? 1 : (w > 4 ? 4 : w);
}

// RTS steps of chunk j of every sequence from the smoothed state at its end.
template <typename R, int NX, int NY>
__global__ void __launch_bounds__(32 * swalk_b_warps<R, NX, NY>())
    swalk_b_kernel(DenseArgs<R> a, int B, int64_t n_chunks, int64_t T) {
  typedef DS<R, NX, NY> S;
  typedef DSS<R, NX, NY> SS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5;
  R* p = reinterpret_cast<R*>(smem_raw) + warp * sapply_b_warp_elems<R, NX, NY>();
  const ScanArgs<R>& sa = a.s;
  const int64_t j = (int64_t)blockIdx.x * swalk_b_warps<R, NX, NY>() + warp;
  if (j >= n_chunks) return;
  zero(p, sapply_b_warp_elems<R, NX, NY>());
  R* L = p; p += S::MN;
  SB<R> e;
  e.E = p; p += S::MN; e.D = p; p += S::MN;
  R* Mv = p; p += SS::MB;
  R* Ge = p; p += SS::MB;
  R* Tm = p; p += SS::MB;
  R* Wm = p; p += S::MW;
  R* vb = p;
  const int64_t t0 = j * sa.g.C, t1 = min(t0 + (int64_t)sa.g.C, T);
  const R* st = sa.sst[1] + j * S::ST;
  g2s<R, NX, NX, S::LDN>(L, st);
  load_rows<R, NX, NY>(Mv, st, n_chunks * S::ST, NX * NX, B);
  for (int64_t t = t1 - 1; t >= t0; --t) {
    load_sb_b<R, NX, NY>(e, Ge, sa.selem + t * S::SE, T * S::SE, B);
    sapply_b<R, NX, NY>(L, Mv, e, Ge, Wm, Tm, vb);
    out_rows<R, NX, NY>(sa, B, T + 1, t, L, Mv);
  }
}

}  // namespace dense
}  // namespace ss
