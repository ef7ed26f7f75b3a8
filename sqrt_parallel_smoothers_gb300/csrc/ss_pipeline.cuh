// Kernels and host orchestration of the ragged, multi-level square-root
// parallel filter and smoother.
//
// Work decomposition (one thread = one chunk of C consecutive steps of one
// sequence at level 1, or one group of G consecutive summaries at higher
// levels):
//   lin_kernel        thread per step: linearise transition at nominal[t] and
//                     observation at nominal[t+1] -> per-step Lin record
//   filter_leaf       level-1 item: the chunk's filtering summary (its first
//                     step's element, extended one conditional Kalman step at
//                     a time: filter_extend)
//   filter_up         level l -> l+1 summaries (fold of G summaries)
//   filter_top        one thread per sequence: walk the top level from the
//                     prior, writing the state that enters each item
//   filter_down       level l+1 -> l entry states
//   filter_walk       level-1 item: Kalman steps from the entry state; emits
//                     the smoothing elements, folds them into the chunk's
//                     smoothing summary, optional filtered output and
//                     log-likelihood partial sums
//   smoother_up/top/down/walk: the same scan run backwards from the last
//                     filtered state; the walk writes the smoothed trajectory.
#pragma once
#include <cub/block/block_scan.cuh>

#include "ss_lin.cuh"
#include "ss_ops.cuh"

namespace ss {

constexpr int MAX_LEVELS = 8;

// Record sizes (elements; _P: padded to whole 16-byte units).  Lower-triangular
// factors are stored as their lower entries only (pack_tri).
template <typename R, int NX, int NY>
struct Rec {
  static constexpr int TX = NX * (NX + 1) / 2, TY = NY * (NY + 1) / 2;
  static constexpr int LIN = NX * NX + TX + NX + NY * NX + TY + NY;   // F, cQ, bq, H, cR, c
  static constexpr int LIN_P = Padded<R, LIN>::n;
  static constexpr int FE = 2 * NX * NX + TX + 2 * NX;                 // A, b, U, eta, Z
  static constexpr int FE_P = Padded<R, FE>::n;
  static constexpr int SE = NX + NX * NX + TX;                         // g, E, D
  static constexpr int SE_P = Padded<R, SE>::n;
  static constexpr int ST = NX + TX;                                   // m, L
  static constexpr int ST_P = Padded<R, ST>::n;
};

// ----------------------------------------------------------------------------- records

template <typename R, int NX, int NY>
SS_DEV void pack_lin(R (&r)[Rec<R, NX, NY>::LIN_P], const Lin<R, NX, NY>& l) {
  typedef Rec<R, NX, NY> Q;
  int o = 0;
  pack<R, NX, NX>(r, o, l.F); o += NX * NX;
  pack_tri<R, NX>(r, o, l.cQ); o += Q::TX;
  pack_vec<R, NX>(r, o, l.bq); o += NX;
  pack<R, NY, NX>(r, o, l.H); o += NY * NX;
  pack_tri<R, NY>(r, o, l.cR); o += Q::TY;
  pack_vec<R, NY>(r, o, l.c); o += NY;
  SS_UNROLL
  for (int k = Q::LIN; k < Q::LIN_P; ++k) r[k] = R(0);
}

template <typename R, int NX, int NY>
SS_DEV void unpack_lin(const R (&r)[Rec<R, NX, NY>::LIN_P], Lin<R, NX, NY>& l) {
  typedef Rec<R, NX, NY> Q;
  int o = 0;
  unpack<R, NX, NX>(r, o, l.F); o += NX * NX;
  unpack_tri<R, NX>(r, o, l.cQ); o += Q::TX;
  unpack_vec<R, NX>(r, o, l.bq); o += NX;
  unpack<R, NY, NX>(r, o, l.H); o += NY * NX;
  unpack_tri<R, NY>(r, o, l.cR); o += Q::TY;
  unpack_vec<R, NY>(r, o, l.c);
}

// The two halves of pack_lin written straight into a record row (shared
// memory), in the same layout.
template <typename R, int NX, int NY>
SS_DEV void write_lin_transition(R* row, const R (&F)[NX][NX], const R (&cQ)[NX][NX], const R (&bq)[NX]) {
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) row[i * NX + j] = F[i][j];
  }
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j <= i; ++j) row[NX * NX + i * (i + 1) / 2 + j] = cQ[i][j];
  }
  SS_UNROLL
  for (int i = 0; i < NX; ++i) row[NX * NX + Rec<R, NX, NY>::TX + i] = bq[i];
}
template <typename R, int NX, int NY>
SS_DEV void write_lin_observation(R* row, const R (&H)[NY][NX], const R (&cR)[NY][NY], const R (&c)[NY]) {
  typedef Rec<R, NX, NY> Q;
  constexpr int o = NX * NX + Q::TX + NX;
  SS_UNROLL
  for (int i = 0; i < NY; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) row[o + i * NX + j] = H[i][j];
  }
  SS_UNROLL
  for (int i = 0; i < NY; ++i) {
    SS_UNROLL
    for (int j = 0; j <= i; ++j) row[o + NY * NX + i * (i + 1) / 2 + j] = cR[i][j];
  }
  SS_UNROLL
  for (int i = 0; i < NY; ++i) row[o + NY * NX + Q::TY + i] = c[i];
  SS_UNROLL
  for (int q = Q::LIN; q < Q::LIN_P; ++q) row[q] = R(0);
}

template <typename R, int NX, int NY>
SS_DEV void load_lin(const R* p, Lin<R, NX, NY>& l) {
  typedef Rec<R, NX, NY> Q;
  R r[Q::LIN_P];
  load_rec<R, Q::LIN>(p, r);
  unpack_lin<R, NX, NY>(r, l);
}

template <typename R, int NX, int NY>
SS_DEV void store_lin(R* p, const Lin<R, NX, NY>& l) {
  typedef Rec<R, NX, NY> Q;
  R r[Q::LIN_P];
  pack_lin<R, NX, NY>(r, l);
  store_rec<R, Q::LIN>(p, r);
}

template <typename R, int NX>
SS_DEV void pack_fe(R (&r)[Rec<R, NX, 1>::FE_P], const FElem<R, NX>& e) {
  typedef Rec<R, NX, 1> Q;
  int o = 0;
  pack<R, NX, NX>(r, o, e.A); o += NX * NX;
  pack_vec<R, NX>(r, o, e.b); o += NX;
  pack_tri<R, NX>(r, o, e.U); o += Q::TX;
  pack_vec<R, NX>(r, o, e.eta); o += NX;
  pack<R, NX, NX>(r, o, e.Z); o += NX * NX;
  SS_UNROLL
  for (int k = Q::FE; k < Q::FE_P; ++k) r[k] = R(0);
}

template <typename R, int NX>
SS_DEV void unpack_fe(const R (&r)[Rec<R, NX, 1>::FE_P], FElem<R, NX>& e) {
  typedef Rec<R, NX, 1> Q;
  int o = 0;
  unpack<R, NX, NX>(r, o, e.A); o += NX * NX;
  unpack_vec<R, NX>(r, o, e.b); o += NX;
  unpack_tri<R, NX>(r, o, e.U); o += Q::TX;
  unpack_vec<R, NX>(r, o, e.eta); o += NX;
  unpack<R, NX, NX>(r, o, e.Z);
}

template <typename R, int NX>
SS_DEV void load_fe(const R* p, FElem<R, NX>& e) {
  typedef Rec<R, NX, 1> Q;
  R r[Q::FE_P];
  load_rec<R, Q::FE>(p, r);
  unpack_fe<R, NX>(r, e);
}

template <typename R, int NX>
SS_DEV void store_fe(R* p, const FElem<R, NX>& e) {
  typedef Rec<R, NX, 1> Q;
  R r[Q::FE_P];
  pack_fe<R, NX>(r, e);
  store_rec<R, Q::FE>(p, r);
}

template <typename R, int NX>
SS_DEV void pack_se(R (&r)[Rec<R, NX, 1>::SE_P], const SElem<R, NX>& e) {
  typedef Rec<R, NX, 1> Q;
  int o = 0;
  pack_vec<R, NX>(r, o, e.g); o += NX;
  pack<R, NX, NX>(r, o, e.E); o += NX * NX;
  pack_tri<R, NX>(r, o, e.D); o += Q::TX;
  SS_UNROLL
  for (int k = Q::SE; k < Q::SE_P; ++k) r[k] = R(0);
}

template <typename R, int NX>
SS_DEV void unpack_se(const R (&r)[Rec<R, NX, 1>::SE_P], SElem<R, NX>& e) {
  int o = 0;
  unpack_vec<R, NX>(r, o, e.g); o += NX;
  unpack<R, NX, NX>(r, o, e.E); o += NX * NX;
  unpack_tri<R, NX>(r, o, e.D);
}

template <typename R, int NX>
SS_DEV void load_se(const R* p, SElem<R, NX>& e) {
  typedef Rec<R, NX, 1> Q;
  R r[Q::SE_P];
  load_rec<R, Q::SE>(p, r);
  unpack_se<R, NX>(r, e);
}

template <typename R, int NX>
SS_DEV void store_se(R* p, const SElem<R, NX>& e) {
  typedef Rec<R, NX, 1> Q;
  R r[Q::SE_P];
  pack_se<R, NX>(r, e);
  store_rec<R, Q::SE>(p, r);
}

template <typename R, int NX>
SS_DEV void load_st(const R* p, State<R, NX>& s) {
  typedef Rec<R, NX, 1> Q;
  R r[Q::ST_P];
  load_rec<R, Q::ST>(p, r);
  unpack_vec<R, NX>(r, 0, s.m);
  unpack_tri<R, NX>(r, NX, s.L);
}

template <typename R, int NX>
SS_DEV void store_st(R* p, const State<R, NX>& s) {
  typedef Rec<R, NX, 1> Q;
  R r[Q::ST_P];
  pack_vec<R, NX>(r, 0, s.m);
  pack_tri<R, NX>(r, NX, s.L);
  SS_UNROLL
  for (int k = Q::ST; k < Q::ST_P; ++k) r[k] = R(0);
  store_rec<R, Q::ST>(p, r);
}

// Trajectory in the user layout: means (N, NX), factors (N, NX, NX).
template <typename R, int NX>
SS_DEV void load_traj(const R* __restrict__ m, const R* __restrict__ L, int64_t s, State<R, NX>& st) {
  SS_UNROLL
  for (int i = 0; i < NX; ++i) st.m[i] = m[s * NX + i];
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) st.L[i][j] = (j <= i) ? L[(s * NX + i) * NX + j] : R(0);
  }
}

template <typename R, int NX>
SS_DEV void store_traj(R* __restrict__ m, R* __restrict__ L, int64_t s, const State<R, NX>& st) {
  SS_UNROLL
  for (int i = 0; i < NX; ++i) m[s * NX + i] = st.m[i];
  SS_UNROLL
  for (int i = 0; i < NX; ++i) {
    SS_UNROLL
    for (int j = 0; j < NX; ++j) L[(s * NX + i) * NX + j] = (j <= i) ? st.L[i][j] : R(0);
  }
}

// ----------------------------------------------------------------------------- geometry

// Largest i in [0, n) with off[i] <= k (off non-decreasing, off[0] <= k < off[n]).
SS_DEV int64_t find_seq(const int64_t* __restrict__ off, int64_t n, int64_t k) {
  int64_t lo = 0, hi = n;
  while (hi - lo > 1) {
    const int64_t mid = (lo + hi) >> 1;
    if (__ldg(off + mid) <= k) lo = mid; else hi = mid;
  }
  return lo;
}

struct Geo {
  const int64_t* off;              // B+1 step offsets
  int64_t B;
  int C, G, L;                     // chunk, group, number of levels
  const int64_t* lvl[MAX_LEVELS + 1];  // lvl[l], l = 1..L: B+1 item offsets at level l
};

// Per-level item offsets: level 1 items are chunks of C steps, level l+1
// items are groups of G level-l items.  One block; B processed in tiles.
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) plan_kernel(Geo g, int64_t* lvl0, int64_t stride) {
  typedef cub::BlockScan<int64_t, BLOCK> Scan;
  __shared__ typename Scan::TempStorage tmp;
  __shared__ int64_t carry[MAX_LEVELS + 1];
  if (threadIdx.x <= MAX_LEVELS) carry[threadIdx.x] = 0;
  __syncthreads();
  for (int64_t base = 0; base < g.B; base += BLOCK) {
    const int64_t i = base + threadIdx.x;
    int64_t n = (i < g.B) ? (g.off[i + 1] - g.off[i]) : 0;
    for (int l = 1; l <= g.L; ++l) {
      const int64_t d = (l == 1) ? g.C : g.G;
      n = (n + d - 1) / d;
      int64_t excl, total;
      Scan(tmp).ExclusiveSum(n, excl, total);
      int64_t* out = lvl0 + (l - 1) * stride;
      if (i < g.B) out[i] = carry[l] + excl;
      __syncthreads();
      if (threadIdx.x == 0) carry[l] += total;
      __syncthreads();
    }
  }
  if (threadIdx.x == 0) {
    for (int l = 1; l <= g.L; ++l) lvl0[(l - 1) * stride + g.B] = carry[l];
  }
}

// ----------------------------------------------------------------------------- linearisation

template <typename R>
struct LinArgs {
  const int64_t* off;
  int64_t B, total;
  const R* nom_m;        // nominal trajectory or null (zero means, identity factors)
  const R* nom_L;
  const R* nom_rec;      // or the nominal as packed state records (m, lower L)
  const int32_t* active; // null or B flags
  ModelArgs<R> tm, om;
  const R* tq_m;         // transition noise mean / chol
  const R* tq_L;
  const R* oq_m;         // observation noise mean / chol
  const R* oq_L;
  RuleArgs rule;
  int slr_form;
  int trans_only;
  R* out;                // per-step Lin records
};


template <typename R, int N>
SS_DEV void load_nominal(const R* nm, const R* nL, int64_t s, R (&m)[N], R (&C)[N][N]) {
  if (nm == nullptr) {
    SS_UNROLL
    for (int i = 0; i < N; ++i) {
      m[i] = R(0);
      SS_UNROLL
      for (int j = 0; j < N; ++j) C[i][j] = (i == j) ? R(1) : R(0);
    }
  } else {
    SS_UNROLL
    for (int i = 0; i < N; ++i) {
      m[i] = nm[s * N + i];
      SS_UNROLL
      for (int j = 0; j < N; ++j) C[i][j] = (j <= i) ? nL[(s * N + i) * N + j] : R(0);
    }
  }
}

// The nominal state at s from LinArgs: packed records, the caller's layout, or
// the default (zero mean, identity factor).
template <typename R, int NX>
SS_DEV void load_nominal_any(const LinArgs<R>& a, int64_t s, R (&m)[NX], R (&C)[NX][NX]) {
  if (a.nom_rec != nullptr) {
    State<R, NX> st;
    load_st<R, NX>(a.nom_rec + s * Rec<R, NX, 1>::ST_P, st);
    SS_UNROLL
    for (int r = 0; r < NX; ++r) {
      m[r] = st.m[r];
      SS_UNROLL
      for (int c = 0; c < NX; ++c) C[r][c] = st.L[r][c];
    }
  } else {
    load_nominal<R, NX>(a.nom_m, a.nom_L, s, m, C);
  }
}


template <typename R, int D>
SS_DEV void load_noise(const R* qm, const R* qL, R (&m)[D], R (&L)[D][D]) {
  SS_UNROLL
  for (int i = 0; i < D; ++i) {
    m[i] = ldg(qm + i);
    SS_UNROLL
    for (int j = 0; j < D; ++j) L[i][j] = (j <= i) ? ldg(qL + i * D + j) : R(0);   // lower factor
  }
}

template <typename R, int NX, int NY, class TF, class OF, int METHOD>
__global__ void __launch_bounds__(128) lin_kernel(LinArgs<R> a) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.total) return;
  const int64_t i = find_seq(a.off, a.B, k);
  if (a.active != nullptr && a.active[i] == 0) return;
  const int64_t t = k - a.off[i];
  const int64_t s = a.off[i] + i + t;  // state index of nominal[t]
  Lin<R, NX, NY> l;
  {
    TF f;
    f.init(a.tm);
    R m[NX], C[NX][NX], qm[NX], qL[NX][NX];
    load_nominal<R, NX>(a.nom_m, a.nom_L, s, m, C);
    load_noise<R, NX>(a.tq_m, a.tq_L, qm, qL);
    linearize<R, NX, NX, TF, METHOD>(f, m, C, qm, qL, a.rule, a.slr_form, l.F, l.cQ, l.bq);
  }
  if (a.trans_only) {
    SS_UNROLL
    for (int r = 0; r < NY; ++r) {
      l.c[r] = R(0);
      SS_UNROLL
      for (int j = 0; j < NX; ++j) l.H[r][j] = R(0);
      SS_UNROLL
      for (int j = 0; j < NY; ++j) l.cR[r][j] = R(0);
    }
  } else {
    OF h;
    h.init(a.om);
    R m[NX], C[NX][NX], qm[NY], qL[NY][NY];
    load_nominal<R, NX>(a.nom_m, a.nom_L, s + 1, m, C);
    load_noise<R, NY>(a.oq_m, a.oq_L, qm, qL);
    linearize<R, NX, NY, OF, METHOD>(h, m, C, qm, qL, a.rule, a.slr_form, l.H, l.cR, l.c);
  }
  store_lin<R, NX, NY>(a.out + k * Rec<R, NX, NY>::LIN_P, l);
}

// Linearise one model at n independent points (the ss_linearize entry point).
template <typename R>
struct PointArgs {
  int64_t n;
  const R* m;
  const R* L;
  ModelArgs<R> model;
  const R* q_m;
  const R* q_L;
  RuleArgs rule;
  int slr_form;
  R* F;
  R* chol;
  R* b;
};

template <typename R, int DIN, int DOUT, class Fn, int METHOD>
__global__ void __launch_bounds__(128) lin_points_kernel(PointArgs<R> a) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.n) return;
  Fn f;
  f.init(a.model);
  R m[DIN], C[DIN][DIN], qm[DOUT], qL[DOUT][DOUT], F[DOUT][DIN], L[DOUT][DOUT], b[DOUT];
  load_nominal<R, DIN>(a.m, a.L, k, m, C);
  load_noise<R, DOUT>(a.q_m, a.q_L, qm, qL);
  linearize<R, DIN, DOUT, Fn, METHOD>(f, m, C, qm, qL, a.rule, a.slr_form, F, L, b);
  SS_UNROLL
  for (int i = 0; i < DOUT; ++i) {
    a.b[k * DOUT + i] = b[i];
    SS_UNROLL
    for (int j = 0; j < DIN; ++j) a.F[(k * DOUT + i) * DIN + j] = F[i][j];
    SS_UNROLL
    for (int j = 0; j < DOUT; ++j) a.chol[(k * DOUT + i) * DOUT + j] = (j <= i) ? L[i][j] : R(0);
  }
}

// ----------------------------------------------------------------------------- scan kernels

template <typename R>
struct ScanArgs {
  Geo g;
  const int32_t* active;
  const R* ys;             // (sum T, NY)
  const R* lin;            // per-step Lin records
  R* selem;                // per-step smoothing elements
  R* fsum[MAX_LEVELS + 1]; // filtering summaries per level
  R* fst[MAX_LEVELS + 1];  // filtering entry states per level
  R* ssum[MAX_LEVELS + 1]; // smoothing summaries per level
  R* sst[MAX_LEVELS + 1];  // smoothing end states per level
  R* fT;                   // (B) last filtered state
  const R* m0;             // prior means (B or 1, NX)
  const R* L0;             // prior factors
  int64_t prior_stride;    // 0 (shared prior) or 1
  // outputs / options
  R* filt_m;               // filtered trajectory or null
  R* filt_L;
  double* ll_chunk;        // per level-1 item partial log-likelihood or null
  int emit_smoother;       // filter_walk writes smoothing elements and summaries
  const R* in_m;           // filtered trajectory given to the smoother (standalone smoothing) or null
  const R* in_L;
  R* out_m;                // smoothed trajectory
  R* out_L;
  R* out_rec;              // or the smoothed trajectory as packed state records
  const R* prev_m;         // nominal means of this pass (convergence test) or null
  const R* prev_L;
  const R* prev_rec;       // or the nominal as packed state records
  double* mse;             // (B) accumulated squared mean change or null
  uint32_t* flags;         // (B) status bits or null
};

SS_DEV bool seq_inactive(const int32_t* active, int64_t i) { return active != nullptr && active[i] == 0; }

// Level-1 item j -> (sequence, first step, end step).
SS_DEV void chunk_of(const Geo& g, int64_t j, int64_t& i, int64_t& t0, int64_t& t1) {
  i = find_seq(g.lvl[1], g.B, j);
  const int64_t c = j - g.lvl[1][i];
  const int64_t T = g.off[i + 1] - g.off[i];
  t0 = c * g.C;
  t1 = min(t0 + (int64_t)g.C, T);
}

// Level-(l+1) item j -> (sequence, first, end) member indices at level l (global).
SS_DEV void group_of(const Geo& g, int l, int64_t j, int64_t& i, int64_t& m0, int64_t& m1) {
  i = find_seq(g.lvl[l + 1], g.B, j);
  const int64_t q = j - g.lvl[l + 1][i];
  const int64_t base = g.lvl[l][i];
  const int64_t n = g.lvl[l][i + 1] - base;
  m0 = base + q * g.G;
  m1 = base + min(q * g.G + (int64_t)g.G, n);
}

template <typename R, int NX, int NY>
__global__ void __launch_bounds__(128) filter_leaf_kernel(ScanArgs<R> a) {
  typedef Rec<R, NX, NY> Q;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.g.lvl[1][a.g.B]) return;
  int64_t i, t0, t1;
  chunk_of(a.g, j, i, t0, t1);
  if (seq_inactive(a.active, i)) return;
  const int64_t base = a.g.off[i];
  FElem<R, NX> acc;
  for (int64_t t = t0; t < t1; ++t) {
    Lin<R, NX, NY> l;
    load_lin<R, NX, NY>(a.lin + (base + t) * Q::LIN_P, l);
    R y[NY];
    SS_UNROLL
    for (int k = 0; k < NY; ++k) y[k] = a.ys[(base + t) * NY + k];
    if (t == t0) {
      filter_element<R, NX, NY>(l, y, acc);
    } else {
      filter_extend<R, NX, NY, ElemZ<NX, NY>::ZK>(acc, l, y);
    }
  }
  store_fe<R, NX>(a.fsum[1] + j * Q::FE_P, acc);
}

template <typename R, int NX>
__global__ void __launch_bounds__(128) filter_up_kernel(ScanArgs<R> a, int l) {
  pdl_enter();
  typedef Rec<R, NX, 1> Q;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.g.lvl[l + 1][a.g.B]) return;
  int64_t i, m0, m1;
  group_of(a.g, l, j, i, m0, m1);
  if (seq_inactive(a.active, i)) return;
  FElem<R, NX> acc;
  load_fe<R, NX>(a.fsum[l] + m0 * Q::FE_P, acc);
  for (int64_t m = m0 + 1; m < m1; ++m) {
    FElem<R, NX> e;
    load_fe<R, NX>(a.fsum[l] + m * Q::FE_P, e);
    filter_combine<R, NX>(acc, e);
  }
  store_fe<R, NX>(a.fsum[l + 1] + j * Q::FE_P, acc);
}

template <typename R, int NX>
SS_DEV void load_prior(const ScanArgs<R>& a, int64_t i, State<R, NX>& s) {
  const int64_t p = i * a.prior_stride;
  SS_UNROLL
  for (int r = 0; r < NX; ++r) {
    s.m[r] = a.m0[p * NX + r];
    SS_UNROLL
    for (int c = 0; c < NX; ++c) s.L[r][c] = (c <= r) ? a.L0[(p * NX + r) * NX + c] : R(0);
  }
}

template <typename R, int NX>
__global__ void __launch_bounds__(128) filter_top_kernel(ScanArgs<R> a) {
  pdl_enter();
  typedef Rec<R, NX, 1> Q;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.g.B) return;
  if (seq_inactive(a.active, i)) return;
  State<R, NX> s;
  load_prior<R, NX>(a, i, s);
  if (a.filt_m != nullptr) store_traj<R, NX>(a.filt_m, a.filt_L, a.g.off[i] + i, s);
  const int L = a.g.L;
  const int64_t b = a.g.lvl[L][i], e = a.g.lvl[L][i + 1];
  if (b == e) {  // empty sequence: the last filtered state is the prior
    store_st<R, NX>(a.fT + i * Q::ST_P, s);
    return;
  }
  for (int64_t m = b; m < e; ++m) {
    store_st<R, NX>(a.fst[L] + m * Q::ST_P, s);
    if (m + 1 < e) {
      FElem<R, NX> el;
      load_fe<R, NX>(a.fsum[L] + m * Q::FE_P, el);
      filter_apply<R, NX>(s, el);
    }
  }
}

template <typename R, int NX>
__global__ void __launch_bounds__(128) filter_down_kernel(ScanArgs<R> a, int l) {
  pdl_enter();
  typedef Rec<R, NX, 1> Q;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.g.lvl[l + 1][a.g.B]) return;
  int64_t i, m0, m1;
  group_of(a.g, l, j, i, m0, m1);
  if (seq_inactive(a.active, i)) return;
  State<R, NX> s;
  load_st<R, NX>(a.fst[l + 1] + j * Q::ST_P, s);
  for (int64_t m = m0; m < m1; ++m) {
    store_st<R, NX>(a.fst[l] + m * Q::ST_P, s);
    if (m + 1 < m1) {
      FElem<R, NX> el;
      load_fe<R, NX>(a.fsum[l] + m * Q::FE_P, el);
      filter_apply<R, NX>(s, el);
    }
  }
}

// Kalman steps of one chunk from its entry state (see ss_ops.cuh).
template <typename R, int NX, int NY>
__global__ void __launch_bounds__(128) filter_walk_kernel(ScanArgs<R> a) {
  typedef Rec<R, NX, NY> Q;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.g.lvl[1][a.g.B]) return;
  int64_t i, t0, t1;
  chunk_of(a.g, j, i, t0, t1);
  if (seq_inactive(a.active, i)) return;
  const int64_t base = a.g.off[i];
  State<R, NX> s;
  load_st<R, NX>(a.fst[1] + j * Q::ST_P, s);
  SElem<R, NX> acc;
  constexpr int NC = 1 + Tangents<R>::n;   // log-likelihood value (+ tangents), FP64
  double ll[NC];
  SS_UNROLL
  for (int k = 0; k < NC; ++k) ll[k] = 0.0;
  for (int64_t t = t0; t < t1; ++t) {
    Lin<R, NX, NY> l;
    load_lin<R, NX, NY>(a.lin + (base + t) * Q::LIN_P, l);
    R y[NY];
    SS_UNROLL
    for (int k = 0; k < NY; ++k) y[k] = a.ys[(base + t) * NY + k];
    R X[2 * NX][2 * NX], mp[NX];
    SElem<R, NX> se;
    smoother_element<R, NX>(l.F, l.cQ, l.bq, s, se, X, mp);
    if (a.emit_smoother) {
      store_se<R, NX>(a.selem + (base + t) * Q::SE_P, se);
      if (t == t0) acc = se; else smoother_fold<R, NX>(acc, se);
    }
    double c[NC];
    to_components(filter_update<R, NX, NY>(s, l, y, X, mp), c);
    SS_UNROLL
    for (int k = 0; k < NC; ++k) ll[k] += c[k];
    if (a.filt_m != nullptr) store_traj<R, NX>(a.filt_m, a.filt_L, base + i + t + 1, s);
  }
  if (a.emit_smoother) store_se<R, NX>(a.ssum[1] + j * Q::SE_P, acc);
  if (a.ll_chunk != nullptr) {
    SS_UNROLL
    for (int k = 0; k < NC; ++k) a.ll_chunk[j * NC + k] = ll[k];
  }
  if (t1 == a.g.off[i + 1] - base) store_st<R, NX>(a.fT + i * Q::ST_P, s);
}

// Smoothing elements of a given filtered trajectory (standalone smoothing).
template <typename R, int NX, int NY>
__global__ void __launch_bounds__(128) smoother_leaf_kernel(ScanArgs<R> a) {
  typedef Rec<R, NX, NY> Q;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.g.lvl[1][a.g.B]) return;
  int64_t i, t0, t1;
  chunk_of(a.g, j, i, t0, t1);
  const int64_t base = a.g.off[i];
  SElem<R, NX> acc;
  for (int64_t t = t0; t < t1; ++t) {
    Lin<R, NX, NY> l;
    load_lin<R, NX, NY>(a.lin + (base + t) * Q::LIN_P, l);
    State<R, NX> s;
    load_traj<R, NX>(a.in_m, a.in_L, base + i + t, s);
    R X[2 * NX][2 * NX], mp[NX];
    SElem<R, NX> se;
    smoother_element<R, NX>(l.F, l.cQ, l.bq, s, se, X, mp);
    store_se<R, NX>(a.selem + (base + t) * Q::SE_P, se);
    if (t == t0) acc = se; else smoother_fold<R, NX>(acc, se);
  }
  store_se<R, NX>(a.ssum[1] + j * Q::SE_P, acc);
  if (t1 == a.g.off[i + 1] - base) {
    State<R, NX> s;
    load_traj<R, NX>(a.in_m, a.in_L, base + i + t1, s);
    store_st<R, NX>(a.fT + i * Q::ST_P, s);
  }
}

template <typename R, int NX>
__global__ void __launch_bounds__(128) smoother_up_kernel(ScanArgs<R> a, int l) {
  pdl_enter();
  typedef Rec<R, NX, 1> Q;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.g.lvl[l + 1][a.g.B]) return;
  int64_t i, m0, m1;
  group_of(a.g, l, j, i, m0, m1);
  if (seq_inactive(a.active, i)) return;
  SElem<R, NX> acc;
  load_se<R, NX>(a.ssum[l] + m0 * Q::SE_P, acc);
  for (int64_t m = m0 + 1; m < m1; ++m) {
    SElem<R, NX> e;
    load_se<R, NX>(a.ssum[l] + m * Q::SE_P, e);
    smoother_fold<R, NX>(acc, e);
  }
  store_se<R, NX>(a.ssum[l + 1] + j * Q::SE_P, acc);
}

template <typename R, int NX>
SS_DEV void accumulate_change(const ScanArgs<R>& a, int64_t i, int64_t s, const State<R, NX>& st) {
  if (a.mse != nullptr) {
    double d2 = 0.0;
    SS_UNROLL
    for (int r = 0; r < NX; ++r) {
      const R pm = a.prev_rec != nullptr ? a.prev_rec[s * Rec<R, NX, 1>::ST_P + r] : a.prev_m[s * NX + r];
      const double d = (double)st.m[r] - (double)pm;
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

// The smoothed state at s into the output trajectory (caller's layout or packed records).
template <typename R, int NX>
SS_DEV void store_out(const ScanArgs<R>& a, int64_t s, const State<R, NX>& st) {
  if (a.out_rec != nullptr) store_st<R, NX>(a.out_rec + s * Rec<R, NX, 1>::ST_P, st);
  else store_traj<R, NX>(a.out_m, a.out_L, s, st);
}

template <typename R, int NX>
SS_DEV void copy_state(const ScanArgs<R>& a, int64_t s) {
  State<R, NX> st;
  if (a.prev_rec != nullptr) load_st<R, NX>(a.prev_rec + s * Rec<R, NX, 1>::ST_P, st);
  else load_traj<R, NX>(a.prev_m, a.prev_L, s, st);
  store_out<R, NX>(a, s, st);
}

template <typename R, int NX>
__global__ void __launch_bounds__(128) smoother_top_kernel(ScanArgs<R> a) {
  pdl_enter();
  typedef Rec<R, NX, 1> Q;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.g.B) return;
  const int64_t T = a.g.off[i + 1] - a.g.off[i];
  const int64_t sT = a.g.off[i] + i + T;
  if (seq_inactive(a.active, i)) {
    copy_state<R, NX>(a, sT);
    return;
  }
  State<R, NX> s;
  load_st<R, NX>(a.fT + i * Q::ST_P, s);
  store_out<R, NX>(a, sT, s);
  accumulate_change<R, NX>(a, i, sT, s);
  const int L = a.g.L;
  const int64_t b = a.g.lvl[L][i], e = a.g.lvl[L][i + 1];
  for (int64_t m = e - 1; m >= b; --m) {
    store_st<R, NX>(a.sst[L] + m * Q::ST_P, s);
    if (m > b) {
      SElem<R, NX> el;
      load_se<R, NX>(a.ssum[L] + m * Q::SE_P, el);
      smoother_apply<R, NX>(s, el);
    }
  }
}

template <typename R, int NX>
__global__ void __launch_bounds__(128) smoother_down_kernel(ScanArgs<R> a, int l) {
  pdl_enter();
  typedef Rec<R, NX, 1> Q;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.g.lvl[l + 1][a.g.B]) return;
  int64_t i, m0, m1;
  group_of(a.g, l, j, i, m0, m1);
  if (seq_inactive(a.active, i)) return;
  State<R, NX> s;
  load_st<R, NX>(a.sst[l + 1] + j * Q::ST_P, s);
  for (int64_t m = m1 - 1; m >= m0; --m) {
    store_st<R, NX>(a.sst[l] + m * Q::ST_P, s);
    if (m > m0) {
      SElem<R, NX> el;
      load_se<R, NX>(a.ssum[l] + m * Q::SE_P, el);
      smoother_apply<R, NX>(s, el);
    }
  }
}

// RTS steps of one chunk from the smoothed state at its end.
template <typename R, int NX>
__global__ void __launch_bounds__(128) smoother_walk_kernel(ScanArgs<R> a) {
  typedef Rec<R, NX, 1> Q;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.g.lvl[1][a.g.B]) return;
  int64_t i, t0, t1;
  chunk_of(a.g, j, i, t0, t1);
  const int64_t base = a.g.off[i];
  if (seq_inactive(a.active, i)) {
    for (int64_t t = t0; t < t1; ++t) copy_state<R, NX>(a, base + i + t);
    return;
  }
  State<R, NX> s;
  load_st<R, NX>(a.sst[1] + j * Q::ST_P, s);
  for (int64_t t = t1 - 1; t >= t0; --t) {
    SElem<R, NX> e;
    load_se<R, NX>(a.selem + (base + t) * Q::SE_P, e);
    smoother_apply<R, NX>(s, e);
    store_out<R, NX>(a, base + i + t, s);
    accumulate_change<R, NX>(a, i, base + i + t, s);
  }
}

// The last state of each sequence of a given (filtered) trajectory into fT: the
// start of a standalone smoothing pass, also for sequences without steps.
template <typename R, int NX>
__global__ void __launch_bounds__(128) last_state_kernel(ScanArgs<R> a) {
  typedef Rec<R, NX, 1> Q;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.g.B) return;
  State<R, NX> s;
  load_traj<R, NX>(a.in_m, a.in_L, a.g.off[i + 1] + i, s);
  store_st<R, NX>(a.fT + i * Q::ST_P, s);
}

// ----------------------------------------------------------------------------- pathwise sampler

// Posterior trajectories of parsmooth/_pathwise_sampler.py:13-127: from the
// last filtered state x_T = m_T + L_T e_T, then x_t = E_t x_{t+1} + g_t + D_t e_t
// with (g_t, E_t, D_t) the per-step smoothing elements (the sampler's gain,
// increment mean and increment factor, :107-127).  One thread per (sequence,
// sample); e and x in the trajectory layout (state, sample, nx).
template <typename R, int NX>
__global__ void __launch_bounds__(128) sample_kernel(ScanArgs<R> a, int S, const R* __restrict__ eps,
                                                     R* __restrict__ out) {
  typedef Rec<R, NX, 1> Q;
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.g.B * (int64_t)S) return;
  const int64_t i = k / S;
  const int64_t smp = k - i * S;
  const int64_t base = a.g.off[i];
  const int64_t T = a.g.off[i + 1] - base;
  const int64_t s0 = base + i;   // state index of t = 0
  State<R, NX> f;
  load_st<R, NX>(a.fT + i * Q::ST_P, f);
  R x[NX];
  {
    const R* e = eps + ((s0 + T) * S + smp) * NX;
    R* o = out + ((s0 + T) * S + smp) * NX;
    SS_UNROLL
    for (int r = 0; r < NX; ++r) {
      R v = f.m[r];
      SS_UNROLL
      for (int c = 0; c <= r; ++c) v += f.L[r][c] * e[c];
      x[r] = v;
      o[r] = v;
    }
  }
  for (int64_t t = T - 1; t >= 0; --t) {
    SElem<R, NX> se;
    load_se<R, NX>(a.selem + (base + t) * Q::SE_P, se);
    const R* e = eps + ((s0 + t) * S + smp) * NX;
    R* o = out + ((s0 + t) * S + smp) * NX;
    R xn[NX];
    SS_UNROLL
    for (int r = 0; r < NX; ++r) {
      R v = se.g[r];
      SS_UNROLL
      for (int c = 0; c < NX; ++c) v += se.E[r][c] * x[c];
      SS_UNROLL
      for (int c = 0; c <= r; ++c) v += se.D[r][c] * e[c];
      xn[r] = v;
    }
    SS_UNROLL
    for (int r = 0; r < NX; ++r) {
      x[r] = xn[r];
      o[r] = xn[r];
    }
  }
}

// Parallel in time, for few draws of long sequences.  The backward recursion is
// a composition of affine maps x_t = E_t x_{t+1} + (g_t + D_t e_t), associative
// as in the reference's _par_sampling scan (parsmooth/_pathwise_sampler.py:13-38).
// The sequence is cut into chunks (geometry g, one level): sample_leaf_kernel
// composes each chunk's maps into x_{t0} = A x_{t1} + c per (chunk, draw),
// sample_top_kernel walks the chunk maps of each (sequence, draw) backwards from
// x_T and stores every chunk's end state, and sample_walk_kernel replays each
// chunk from its end state.  One thread per (chunk, draw) or (sequence, draw);
// maps hold NX * NX + NX values and ends NX values per (chunk, draw).
template <typename R, int NX>
__global__ void __launch_bounds__(128) sample_leaf_kernel(Geo g, const R* __restrict__ selem, int S,
                                                          const R* __restrict__ eps, R* __restrict__ maps) {
  typedef Rec<R, NX, 1> Q;
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= g.lvl[1][g.B] * (int64_t)S) return;
  const int64_t j = k / S, smp = k - j * S;
  int64_t i, t0, t1;
  chunk_of(g, j, i, t0, t1);
  const int64_t base = g.off[i], s0 = base + i;
  R A[NX][NX], c[NX];
  SS_UNROLL
  for (int r = 0; r < NX; ++r) {
    c[r] = R(0);
    SS_UNROLL
    for (int q = 0; q < NX; ++q) A[r][q] = (r == q) ? R(1) : R(0);
  }
  for (int64_t t = t1 - 1; t >= t0; --t) {
    SElem<R, NX> se;
    load_se<R, NX>(selem + (base + t) * Q::SE_P, se);
    const R* e = eps + ((s0 + t) * S + smp) * NX;
    R nA[NX][NX], nc[NX];
    SS_UNROLL
    for (int r = 0; r < NX; ++r) {
      R v = se.g[r];
      SS_UNROLL
      for (int q = 0; q < NX; ++q) v += se.E[r][q] * c[q];
      SS_UNROLL
      for (int q = 0; q <= r; ++q) v += se.D[r][q] * e[q];
      nc[r] = v;
      SS_UNROLL
      for (int q = 0; q < NX; ++q) {
        R a = R(0);
        SS_UNROLL
        for (int p = 0; p < NX; ++p) a += se.E[r][p] * A[p][q];
        nA[r][q] = a;
      }
    }
    SS_UNROLL
    for (int r = 0; r < NX; ++r) {
      c[r] = nc[r];
      SS_UNROLL
      for (int q = 0; q < NX; ++q) A[r][q] = nA[r][q];
    }
  }
  R* o = maps + k * (NX * NX + NX);
  SS_UNROLL
  for (int r = 0; r < NX; ++r) {
    o[NX * NX + r] = c[r];
    SS_UNROLL
    for (int q = 0; q < NX; ++q) o[r * NX + q] = A[r][q];
  }
}

template <typename R, int NX>
__global__ void __launch_bounds__(128) sample_top_kernel(Geo g, const R* __restrict__ fT, int S,
                                                         const R* __restrict__ eps, const R* __restrict__ maps,
                                                         R* __restrict__ ends, R* __restrict__ out) {
  typedef Rec<R, NX, 1> Q;
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= g.B * (int64_t)S) return;
  const int64_t i = k / S, smp = k - i * S;
  const int64_t T = g.off[i + 1] - g.off[i];
  const int64_t s0 = g.off[i] + i;
  State<R, NX> f;
  load_st<R, NX>(fT + i * Q::ST_P, f);
  R x[NX];
  {
    const R* e = eps + ((s0 + T) * S + smp) * NX;
    R* o = out + ((s0 + T) * S + smp) * NX;
    SS_UNROLL
    for (int r = 0; r < NX; ++r) {
      R v = f.m[r];
      SS_UNROLL
      for (int c = 0; c <= r; ++c) v += f.L[r][c] * e[c];
      x[r] = v;
      o[r] = v;
    }
  }
  for (int64_t j = g.lvl[1][i + 1] - 1; j >= g.lvl[1][i]; --j) {
    const int64_t kk = j * S + smp;
    SS_UNROLL
    for (int r = 0; r < NX; ++r) ends[kk * NX + r] = x[r];
    const R* mp = maps + kk * (NX * NX + NX);
    R xn[NX];
    SS_UNROLL
    for (int r = 0; r < NX; ++r) {
      R v = mp[NX * NX + r];
      SS_UNROLL
      for (int q = 0; q < NX; ++q) v += mp[r * NX + q] * x[q];
      xn[r] = v;
    }
    SS_UNROLL
    for (int r = 0; r < NX; ++r) x[r] = xn[r];
  }
}

template <typename R, int NX>
__global__ void __launch_bounds__(128) sample_walk_kernel(Geo g, const R* __restrict__ selem, int S,
                                                          const R* __restrict__ eps, const R* __restrict__ ends,
                                                          R* __restrict__ out) {
  typedef Rec<R, NX, 1> Q;
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= g.lvl[1][g.B] * (int64_t)S) return;
  const int64_t j = k / S, smp = k - j * S;
  int64_t i, t0, t1;
  chunk_of(g, j, i, t0, t1);
  const int64_t base = g.off[i], s0 = base + i;
  R x[NX];
  SS_UNROLL
  for (int r = 0; r < NX; ++r) x[r] = ends[k * NX + r];
  for (int64_t t = t1 - 1; t >= t0; --t) {
    SElem<R, NX> se;
    load_se<R, NX>(selem + (base + t) * Q::SE_P, se);
    const R* e = eps + ((s0 + t) * S + smp) * NX;
    R* o = out + ((s0 + t) * S + smp) * NX;
    R xn[NX];
    SS_UNROLL
    for (int r = 0; r < NX; ++r) {
      R v = se.g[r];
      SS_UNROLL
      for (int c = 0; c < NX; ++c) v += se.E[r][c] * x[c];
      SS_UNROLL
      for (int c = 0; c <= r; ++c) v += se.D[r][c] * e[c];
      xn[r] = v;
    }
    SS_UNROLL
    for (int r = 0; r < NX; ++r) {
      x[r] = xn[r];
      o[r] = xn[r];
    }
  }
}

// ----------------------------------------------------------------------------- finishing kernels

// Per-sequence log-likelihood: sum of chunk partials plus the constant
// -T ny/2 log(2 pi), all in FP64.  With NC > 1 the chunk partials carry
// tangent components too; component c goes to grad[i * grad_ld + grad_col + c - 1].
static __global__ void ll_reduce_kernel(Geo g, int ny, int NC, const double* __restrict__ ll_chunk,
                                        double* __restrict__ out, double* __restrict__ grad, int grad_ld,
                                        int grad_col, uint32_t* flags) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.B) return;
  const int64_t T = g.off[i + 1] - g.off[i];
  for (int c = 0; c < NC; ++c) {
    double s = (c == 0) ? -0.5 * (double)T * (double)ny * 1.8378770664093453 : 0.0;  // log(2 pi)
    for (int64_t j = g.lvl[1][i]; j < g.lvl[1][i + 1]; ++j) s += ll_chunk[j * NC + c];
    if (c == 0) {
      out[i] = s;
      if (flags != nullptr && !isfinite(s)) atomicOr(flags + i, 2u);
    } else if (grad != nullptr) {
      grad[i * grad_ld + grad_col + (c - 1)] = s;
    }
  }
}

// After one filter-smoother call in tolerance mode: count the call, stop
// sequences whose mean squared change is <= tol, reset the accumulator.
static __global__ void converge_kernel(Geo g, int nx, double tol, double* mse, int32_t* active,
                                int32_t* iters) {
  pdl_enter();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.B) return;
  if (active[i]) {
    iters[i] += 1;
    const int64_t T = g.off[i + 1] - g.off[i];
    if (mse[i] / ((double)(T + 1) * nx) <= tol) active[i] = 0;
  }
  mse[i] = 0.0;
}

static __global__ void init_iter_kernel(int64_t B, int32_t* active, int32_t* iters, double* mse,
                                 uint32_t* flags, int32_t count_first) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B) return;
  active[i] = 1;
  iters[i] = count_first;
  mse[i] = 0.0;
  if (flags != nullptr) flags[i] = 0u;
}

static __global__ void finish_iter_kernel(int64_t B, const int32_t* active, const int32_t* iters,
                                   int32_t* out_iters, uint32_t* flags, int32_t tol_mode) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B) return;
  if (out_iters != nullptr) out_iters[i] = iters[i];
  if (flags != nullptr && tol_mode && active[i]) atomicOr(flags + i, 4u);
}

}  // namespace ss
