// Warp-cooperative staging of per-lane records through shared memory.
//
// The chunk kernels give each lane its own sequence segment, so in any one
// step the 32 lanes of a warp touch 32 records that lie far apart; loading
// them lane by lane costs 32 sectors per request and saturates the load/store
// unit.  Here the warp moves the 32 records together: the lanes trade record
// pointers by shuffle and copy consecutive 16-byte pieces, so every request
// covers one or two contiguous records (a few full sectors).  Loads are
// asynchronous (cp.async, 16 bytes), so the next step's records stream in
// while the current step computes.  Each lane then reads its own row of the
// staging tile; rows are padded to an odd number of 16-byte units so that
// 16-byte shared loads are bank-conflict free.
#pragma once
#include "ss_la.cuh"

namespace ss {

constexpr unsigned FULL_MASK = 0xffffffffu;

template <typename R, int N>
struct StageTile {
  static constexpr int VW = Vec16<R>::n;                 // elements per 16 bytes
  static constexpr int NV = Padded<R, N>::n / VW;        // 16-byte pieces per record
  static constexpr int STRIDE_V = NV | 1;                 // odd row stride (16-byte units)
  static constexpr int STRIDE = STRIDE_V * VW;            // row stride (elements)
  static constexpr int WARP_ELEMS = 32 * STRIDE;          // one warp's tile
};

SS_DEV void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
SS_DEV void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
SS_DEV void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Issue the asynchronous copy of every lane's record (src == nullptr: none)
// into the warp's tile; the caller commits and waits.
template <typename R, int N>
SS_DEV void stage_load_async(const R* src, R* tile) {
  typedef StageTile<R, N> S;
  const int lane = threadIdx.x & 31;
  const unsigned long long mine = reinterpret_cast<unsigned long long>(src);
  SS_UNROLL
  for (int it = 0; it < S::NV; ++it) {
    const int q = it * 32 + lane;
    const int r = q / S::NV;
    const int p = q - r * S::NV;
    const R* g = reinterpret_cast<const R*>(__shfl_sync(FULL_MASK, mine, r));
    if (g != nullptr) cp_async16(tile + r * S::STRIDE + p * S::VW, g + p * S::VW);
  }
}

// This lane's row of the tile -> registers (16-byte shared loads).
template <typename R, int N>
SS_DEV void stage_read(const R* tile, R (&dst)[Padded<R, N>::n]) {
  typedef StageTile<R, N> S;
  typedef typename Vec16<R>::type V;
  const int lane = threadIdx.x & 31;
  const V* row = reinterpret_cast<const V*>(tile + lane * S::STRIDE);
  SS_UNROLL
  for (int k = 0; k < S::NV; ++k) vec_to(row[k], dst + k * S::VW);
}

// Registers -> this lane's row, then the warp stores every lane's record to
// its destination (dst == nullptr: none) in 16-byte pieces.
template <typename R, int N>
SS_DEV void stage_store(R* tile, const R (&src)[Padded<R, N>::n], R* dst) {
  typedef StageTile<R, N> S;
  typedef typename Vec16<R>::type V;
  const int lane = threadIdx.x & 31;
  V* row = reinterpret_cast<V*>(tile + lane * S::STRIDE);
  SS_UNROLL
  for (int k = 0; k < S::NV; ++k) row[k] = vec_from(src + k * S::VW);
  __syncwarp();
  const unsigned long long mine = reinterpret_cast<unsigned long long>(dst);
  SS_UNROLL
  for (int it = 0; it < S::NV; ++it) {
    const int q = it * 32 + lane;
    const int r = q / S::NV;
    const int p = q - r * S::NV;
    R* g = reinterpret_cast<R*>(__shfl_sync(FULL_MASK, mine, r));
    if (g != nullptr) reinterpret_cast<V*>(g)[p] = reinterpret_cast<const V*>(tile + r * S::STRIDE)[p];
  }
  __syncwarp();
}

// Two-phase form of stage_store for records built in parts: each lane writes
// its row (stage_row) element by element, then the warp copies every lane's
// row to its destination (stage_flush).
template <typename R, int N>
SS_DEV R* stage_row(R* tile) {
  return tile + (threadIdx.x & 31) * StageTile<R, N>::STRIDE;
}
template <typename R, int N>
SS_DEV void stage_flush(const R* tile, R* dst) {
  typedef StageTile<R, N> S;
  typedef typename Vec16<R>::type V;
  const int lane = threadIdx.x & 31;
  __syncwarp();
  const unsigned long long mine = reinterpret_cast<unsigned long long>(dst);
  SS_UNROLL
  for (int it = 0; it < S::NV; ++it) {
    const int q = it * 32 + lane;
    const int r = q / S::NV;
    const int p = q - r * S::NV;
    R* g = reinterpret_cast<R*>(__shfl_sync(FULL_MASK, mine, r));
    if (g != nullptr) reinterpret_cast<V*>(g)[p] = reinterpret_cast<const V*>(tile + r * S::STRIDE)[p];
  }
  __syncwarp();
}

// Element-granular variant for destinations without 16-byte alignment (the
// caller's trajectory rows): W elements per lane, row stride W | 1.
template <typename R, int W>
SS_DEV void stage_store_words(R* tile, const R (&src)[W], R* dst) {
  constexpr int STRIDE = W | 1;
  const int lane = threadIdx.x & 31;
  SS_UNROLL
  for (int k = 0; k < W; ++k) tile[lane * STRIDE + k] = src[k];
  __syncwarp();
  const unsigned long long mine = reinterpret_cast<unsigned long long>(dst);
  SS_UNROLL
  for (int it = 0; it < W; ++it) {
    const int q = it * 32 + lane;
    const int r = q / W;
    const int p = q - r * W;
    R* g = reinterpret_cast<R*>(__shfl_sync(FULL_MASK, mine, r));
    if (g != nullptr) g[p] = tile[r * STRIDE + p];
  }
  __syncwarp();
}

}  // namespace ss
