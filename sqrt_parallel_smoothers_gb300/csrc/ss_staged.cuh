// The four per-step kernels of the filter-smoother pass with their global
// traffic staged through shared memory (see ss_stage.cuh): the per-step
// linearisation, the chunk's filtering summary, the chunk Kalman walk
// and the chunk RTS walk.  Used for float and double; the per-lane variants
// in ss_pipeline.cuh remain for dual numbers.
#pragma once
#include "ss_pipeline.cuh"
#include "ss_stage.cuh"

namespace ss {

// Records are packed and unpacked by the functions of ss_pipeline.cuh.

constexpr int STAGED_BLOCK = 128;
// Minimum resident blocks per SM requested from the register allocator for the
// per-step kernels, each chosen by measurement: the FP32 linearisation runs four
// blocks (128 registers, a few words of spill, 12 % faster than three; FP64
// two, where three would spill 0.8 kB), the
// smoother walk three, the filter leaf and walk one (they hold a 2nx x 2nx tria
// and lose more to spills than they gain in occupancy).
#ifndef SS_LIN_MINB
#define SS_LIN_MINB 4
#endif
#ifndef SS_LIN_MINB_F64
#define SS_LIN_MINB_F64 2
#endif
// FP64 registers come in pairs: its linearisation keeps fewer blocks
template <typename R>
struct LinMinBlocks { static constexpr int value = sizeof(R) == 4 ? SS_LIN_MINB : SS_LIN_MINB_F64; };
#ifndef SS_SWALK_MINB
#define SS_SWALK_MINB 3
#endif
#ifndef SS_SCAN_MINB
#define SS_SCAN_MINB 1
#endif
#ifndef SS_LEAF_MINB
#define SS_LEAF_MINB SS_SCAN_MINB
#endif
#ifndef SS_WALK_ACC_SMEM
#define SS_WALK_ACC_SMEM 1
#endif
#ifndef SS_WALK_Y_PREFETCH
#define SS_WALK_Y_PREFETCH 1
#endif
constexpr int STAGED_WARPS = STAGED_BLOCK / 32;

// A smoothing summary held in shared memory, one column per thread (element q
// of thread t at col[q * STAGED_BLOCK + t]): conflict-free and off the
// register file between the per-step folds.
template <typename R, int NX>
SS_DEV void col_load_se(const R* col, SElem<R, NX>& e) {
  typedef Rec<R, NX, 1> Q;
  R r[Q::SE_P];
  SS_UNROLL
  for (int q = 0; q < Q::SE_P; ++q) r[q] = q < Q::SE ? col[q * STAGED_BLOCK] : R(0);
  unpack_se<R, NX>(r, e);
}
template <typename R, int NX>
SS_DEV void col_store_se(R* col, const SElem<R, NX>& e) {
  typedef Rec<R, NX, 1> Q;
  R r[Q::SE_P];
  pack_se<R, NX>(r, e);
  SS_UNROLL
  for (int q = 0; q < Q::SE; ++q) col[q * STAGED_BLOCK] = r[q];
}

// Dynamic shared memory (bytes) of each staged kernel.
template <typename R, int NX, int NY>
struct StagedSmem {
  typedef Rec<R, NX, NY> Q;
  static constexpr size_t lin = sizeof(R) * STAGED_WARPS * StageTile<R, Q::LIN>::WARP_ELEMS;
  static constexpr size_t leaf = 2 * lin;
  // the filter walk keeps each thread's chunk smoothing summary in shared
  // memory, one column per thread, when that fits a block's 227 KB
  static constexpr size_t fwalk_tiles = 2 * lin + sizeof(R) * STAGED_WARPS * StageTile<R, Q::SE>::WARP_ELEMS;
  static constexpr size_t walk_acc_bytes = sizeof(R) * STAGED_BLOCK * Q::SE;
  static constexpr bool walk_acc_smem = SS_WALK_ACC_SMEM && fwalk_tiles + walk_acc_bytes <= 232448;
  static constexpr size_t walk_acc = walk_acc_smem ? walk_acc_bytes : 0;
  static constexpr size_t fwalk = fwalk_tiles + walk_acc;
  // the smoother walk's output tile: a row holds nx x nx words (the caller's
  // layout) or one packed state record
  static constexpr int out_stride = ((NX * NX) | 1) > StageTile<R, Q::ST>::STRIDE ? ((NX * NX) | 1)
                                                                                  : StageTile<R, Q::ST>::STRIDE;
  static constexpr size_t swalk = sizeof(R) * STAGED_WARPS *
                                  (2 * StageTile<R, Q::SE>::WARP_ELEMS + 32 * out_stride);
  // every staged kernel's tiles fit one block's 227 KB (not FP64 at nx >= 6, whose records
  // run through the unstaged kernels)
  static constexpr bool fits = lin <= 232448 && leaf <= 232448 && fwalk <= 232448 && swalk <= 232448;
};

template <typename R>
SS_DEV R* warp_smem(unsigned char* raw, size_t warp_elems) {
  return reinterpret_cast<R*>(raw) + (threadIdx.x >> 5) * warp_elems;
}

// ---------------------------------------------------------------------------
template <typename R, int NX, int NY, class TF, class OF, int METHOD>
__global__ void __launch_bounds__(STAGED_BLOCK, LinMinBlocks<R>::value) lin_staged_kernel(LinArgs<R> a) {
  pdl_enter();
  typedef Rec<R, NX, NY> Q;
  extern __shared__ __align__(16) unsigned char ss_smem[];
  R* tile = warp_smem<R>(ss_smem, StageTile<R, Q::LIN>::WARP_ELEMS);
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool work = k < a.total;
  int64_t i = 0;
  if (work) {
    i = find_seq(a.off, a.B, k);
    if (a.active != nullptr && a.active[i] == 0) work = false;
  }
  // The record is written into this lane's shared row in two parts, the
  // transition's before the observation is linearised, so the transition's
  // results do not stay live in registers.
  R* row = stage_row<R, Q::LIN>(tile);
  if (work) {
    const int64_t t = k - a.off[i];
    const int64_t s = a.off[i] + i + t;
    {
      TF f;
      f.init(a.tm);
      R m[NX], C[NX][NX], qm[NX], qL[NX][NX], F[NX][NX], cQ[NX][NX], bq[NX];
      load_nominal_any<R, NX>(a, s, m, C);
      load_noise<R, NX>(a.tq_m, a.tq_L, qm, qL);
      linearize<R, NX, NX, TF, METHOD>(f, m, C, qm, qL, a.rule, a.slr_form, F, cQ, bq);
      write_lin_transition<R, NX, NY>(row, F, cQ, bq);
    }
    R H[NY][NX], cR[NY][NY], c[NY];
    if (a.trans_only) {
      SS_UNROLL
      for (int r = 0; r < NY; ++r) {
        c[r] = R(0);
        SS_UNROLL
        for (int jj = 0; jj < NX; ++jj) H[r][jj] = R(0);
        SS_UNROLL
        for (int jj = 0; jj < NY; ++jj) cR[r][jj] = R(0);
      }
    } else {
      OF h;
      h.init(a.om);
      R m[NX], C[NX][NX], qm[NY], qL[NY][NY];
      load_nominal_any<R, NX>(a, s + 1, m, C);
      load_noise<R, NY>(a.oq_m, a.oq_L, qm, qL);
      linearize<R, NX, NY, OF, METHOD>(h, m, C, qm, qL, a.rule, a.slr_form, H, cR, c);
    }
    write_lin_observation<R, NX, NY>(row, H, cR, c);
  }
  stage_flush<R, Q::LIN>(tile, work ? a.out + k * Q::LIN_P : nullptr);
}

// ---------------------------------------------------------------------------
template <typename R, int NX, int NY>
__global__ void __launch_bounds__(STAGED_BLOCK, SS_LEAF_MINB) filter_leaf_staged_kernel(ScanArgs<R> a) {
  pdl_enter();
  typedef Rec<R, NX, NY> Q;
  typedef StageTile<R, Q::LIN> TL;
  extern __shared__ __align__(16) unsigned char ss_smem[];
  R* tiles = warp_smem<R>(ss_smem, 2 * TL::WARP_ELEMS);
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool work = j < a.g.lvl[1][a.g.B];
  int64_t i = 0, t0 = 0, t1 = 0;
  if (work) {
    chunk_of(a.g, j, i, t0, t1);
    if (seq_inactive(a.active, i)) work = false;
  }
  const int n = work ? (int)(t1 - t0) : 0;
  const int64_t first = work ? a.g.off[i] + t0 : 0;
  stage_load_async<R, Q::LIN>(n > 0 ? a.lin + first * Q::LIN_P : nullptr, tiles);
  cp_async_commit();
  FElem<R, NX> acc;
  for (int s = 0; s < a.g.C; ++s) {
    if (!__any_sync(FULL_MASK, s < n)) break;
    stage_load_async<R, Q::LIN>(s + 1 < n ? a.lin + (first + s + 1) * Q::LIN_P : nullptr,
                                tiles + ((s + 1) & 1) * TL::WARP_ELEMS);
    cp_async_commit();
    cp_async_wait<1>();
    __syncwarp();
    if (s < n) {
      R rec[Q::LIN_P];
      stage_read<R, Q::LIN>(tiles + (s & 1) * TL::WARP_ELEMS, rec);
      Lin<R, NX, NY> l;
      unpack_lin<R, NX, NY>(rec, l);
      R y[NY];
      SS_UNROLL
      for (int k = 0; k < NY; ++k) y[k] = a.ys[(first + s) * NY + k];
      if (s == 0) {
        filter_element<R, NX, NY>(l, y, acc);
      } else {
        filter_extend<R, NX, NY, ElemZ<NX, NY>::ZK>(acc, l, y);
      }
    }
    __syncwarp();
  }
  cp_async_wait<0>();
  if (work) store_fe<R, NX>(a.fsum[1] + j * Q::FE_P, acc);
}

// ---------------------------------------------------------------------------
template <typename R, int NX, int NY>
__global__ void __launch_bounds__(STAGED_BLOCK, SS_SCAN_MINB) filter_walk_staged_kernel(ScanArgs<R> a) {
  pdl_enter();
  typedef Rec<R, NX, NY> Q;
  typedef StageTile<R, Q::LIN> TL;
  typedef StageTile<R, Q::SE> TS;
  extern __shared__ __align__(16) unsigned char ss_smem[];
  R* tiles = warp_smem<R>(ss_smem, 2 * TL::WARP_ELEMS);
  R* stile = reinterpret_cast<R*>(ss_smem) + STAGED_WARPS * 2 * TL::WARP_ELEMS + (threadIdx.x >> 5) * TS::WARP_ELEMS;
  constexpr bool ACC_SMEM = StagedSmem<R, NX, NY>::walk_acc_smem;
  R* acol = reinterpret_cast<R*>(ss_smem) + STAGED_WARPS * (2 * TL::WARP_ELEMS + TS::WARP_ELEMS) + threadIdx.x;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool work = j < a.g.lvl[1][a.g.B];
  int64_t i = 0, t0 = 0, t1 = 0;
  if (work) {
    chunk_of(a.g, j, i, t0, t1);
    if (seq_inactive(a.active, i)) work = false;
  }
  const int n = work ? (int)(t1 - t0) : 0;
  const int64_t base = work ? a.g.off[i] : 0;
  const int64_t first = base + t0;
  State<R, NX> s;
  if (work) load_st<R, NX>(a.fst[1] + j * Q::ST_P, s);
  stage_load_async<R, Q::LIN>(n > 0 ? a.lin + first * Q::LIN_P : nullptr, tiles);
  cp_async_commit();
  SElem<R, NX> acc;
  double ll = 0.0;
  R yn[NY];   // observation of the step (read one step ahead)
  SS_UNROLL
  for (int q = 0; q < NY; ++q) yn[q] = (SS_WALK_Y_PREFETCH && n > 0) ? a.ys[first * NY + q] : R(0);
  for (int k = 0; k < a.g.C; ++k) {
    if (!__any_sync(FULL_MASK, k < n)) break;
    stage_load_async<R, Q::LIN>(k + 1 < n ? a.lin + (first + k + 1) * Q::LIN_P : nullptr,
                                tiles + ((k + 1) & 1) * TL::WARP_ELEMS);
    cp_async_commit();
    R y[NY];
    SS_UNROLL
    for (int q = 0; q < NY; ++q) {
      y[q] = yn[q];
      if (SS_WALK_Y_PREFETCH && k + 1 < n) yn[q] = a.ys[(first + k + 1) * NY + q];
    }
    cp_async_wait<1>();
    __syncwarp();
    // Order within a step, chosen by measurement: the smoothing element is
    // staged out and folded while the predicted factor waits, then the record's
    // observation part is read again from shared memory for the Kalman update.
    const R* tile = tiles + (k & 1) * TL::WARP_ELEMS;
    R X[2 * NX][2 * NX], mp[NX];
    SElem<R, NX> se;
    {
      R srec[Q::SE_P];
      SS_UNROLL
      for (int q = 0; q < Q::SE_P; ++q) srec[q] = R(0);
      if (k < n) {
        R rec[Q::LIN_P];
        stage_read<R, Q::LIN>(tile, rec);
        Lin<R, NX, NY> l;
        unpack_lin<R, NX, NY>(rec, l);
        smoother_element<R, NX>(l.F, l.cQ, l.bq, s, se, X, mp);
        if (a.emit_smoother) pack_se<R, NX>(srec, se);
      }
      if (a.emit_smoother)
        stage_store<R, Q::SE>(stile, srec, k < n ? a.selem + (first + k) * Q::SE_P : nullptr);
    }
    if (k < n && a.emit_smoother) {
      if constexpr (ACC_SMEM) {
        if (k == 0) {
          col_store_se<R, NX>(acol, se);
        } else {
          SElem<R, NX> ac;
          col_load_se<R, NX>(acol, ac);
          smoother_fold<R, NX>(ac, se);
          col_store_se<R, NX>(acol, ac);
        }
      } else {
        if (k == 0) acc = se; else smoother_fold<R, NX>(acc, se);
      }
    }
    if (k < n) {
      R rec[Q::LIN_P];
      stage_read<R, Q::LIN>(tile, rec);
      Lin<R, NX, NY> l;
      unpack_lin<R, NX, NY>(rec, l);
      if (!SS_WALK_Y_PREFETCH) {
        SS_UNROLL
        for (int q = 0; q < NY; ++q) y[q] = a.ys[(first + k) * NY + q];
      }
      ll += (double)filter_update<R, NX, NY>(s, l, y, X, mp);
      if (a.filt_m != nullptr) store_traj<R, NX>(a.filt_m, a.filt_L, first + i + k + 1, s);
    }
    __syncwarp();
  }
  cp_async_wait<0>();
  if (work) {
    if (a.emit_smoother) {
      if constexpr (ACC_SMEM) col_load_se<R, NX>(acol, acc);
      store_se<R, NX>(a.ssum[1] + j * Q::SE_P, acc);
    }
    if (a.ll_chunk != nullptr) a.ll_chunk[j] = ll;
    if (t1 == a.g.off[i + 1] - base) store_st<R, NX>(a.fT + i * Q::ST_P, s);
  }
}

// ---------------------------------------------------------------------------
template <typename R, int NX>
__global__ void __launch_bounds__(STAGED_BLOCK, SS_SWALK_MINB) smoother_walk_staged_kernel(ScanArgs<R> a) {
  pdl_enter();
  typedef Rec<R, NX, 1> Q;
  typedef StageTile<R, Q::SE> TS;
  constexpr int LW = StagedSmem<R, NX, 1>::out_stride;
  extern __shared__ __align__(16) unsigned char ss_smem[];
  R* tiles = warp_smem<R>(ss_smem, 2 * TS::WARP_ELEMS);
  R* otile = reinterpret_cast<R*>(ss_smem) + STAGED_WARPS * 2 * TS::WARP_ELEMS + (threadIdx.x >> 5) * 32 * LW;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool work = j < a.g.lvl[1][a.g.B];
  int64_t i = 0, t0 = 0, t1 = 0;
  if (work) chunk_of(a.g, j, i, t0, t1);
  const int64_t base = work ? a.g.off[i] : 0;
  if (work && seq_inactive(a.active, i)) {
    for (int64_t t = t0; t < t1; ++t) copy_state<R, NX>(a, base + i + t);
    work = false;
  }
  const int n = work ? (int)(t1 - t0) : 0;
  State<R, NX> s;
  if (work) load_st<R, NX>(a.sst[1] + j * Q::ST_P, s);
  // step k handles t = t1 - 1 - k
  stage_load_async<R, Q::SE>(n > 0 ? a.selem + (base + t1 - 1) * Q::SE_P : nullptr, tiles);
  cp_async_commit();
  for (int k = 0; k < a.g.C; ++k) {
    if (!__any_sync(FULL_MASK, k < n)) break;
    stage_load_async<R, Q::SE>(k + 1 < n ? a.selem + (base + t1 - 2 - k) * Q::SE_P : nullptr,
                               tiles + ((k + 1) & 1) * TS::WARP_ELEMS);
    cp_async_commit();
    cp_async_wait<1>();
    __syncwarp();
    R mrow[NX], Lrow[NX * NX];
    SS_UNROLL
    for (int q = 0; q < NX; ++q) mrow[q] = R(0);
    SS_UNROLL
    for (int q = 0; q < NX * NX; ++q) Lrow[q] = R(0);
    const int64_t st = base + i + t1 - 1 - k;
    if (k < n) {
      R rec[Q::SE_P];
      stage_read<R, Q::SE>(tiles + (k & 1) * TS::WARP_ELEMS, rec);
      SElem<R, NX> e;
      unpack_se<R, NX>(rec, e);
      smoother_apply<R, NX>(s, e);
      accumulate_change<R, NX>(a, i, st, s);
      SS_UNROLL
      for (int r = 0; r < NX; ++r) {
        mrow[r] = s.m[r];
        SS_UNROLL
        for (int c = 0; c < NX; ++c) Lrow[r * NX + c] = (c <= r) ? s.L[r][c] : R(0);
      }
    }
    if (a.out_rec != nullptr) {
      // packed state records (the next nominal): whole 16-byte pieces
      R srec[Q::ST_P];
      SS_UNROLL
      for (int q = 0; q < Q::ST_P; ++q) srec[q] = R(0);
      SS_UNROLL
      for (int r = 0; r < NX; ++r) {
        srec[r] = mrow[r];
        SS_UNROLL
        for (int c = 0; c <= r; ++c) srec[NX + r * (r + 1) / 2 + c] = Lrow[r * NX + c];
      }
      stage_store<R, Q::ST>(otile, srec, k < n ? a.out_rec + st * Q::ST_P : nullptr);
    } else {
      stage_store_words<R, NX>(otile, mrow, k < n ? a.out_m + st * NX : nullptr);
      stage_store_words<R, NX * NX>(otile, Lrow, k < n ? a.out_L + st * NX * NX : nullptr);
    }
  }
  cp_async_wait<0>();
}

}  // namespace ss
