// Warp-cooperative dense linear algebra for the large-state path.
//
// A matrix lives in the warp's slice of shared memory, row-major, with a row
// stride of an odd number of 16-byte units: eight lanes that each touch their
// own row with a 16-byte access then hit eight distinct bank groups, and a
// warp that reads one row (a broadcast) or one column (consecutive
// addresses) is conflict-free as well.  Every operation hands row r of its
// result to lane r % 32 (rows 32..63 are a lane's second slot), computes that
// row in registers and writes it back, then synchronises the warp.
//
// Shapes are compile-time; column counts of blocks that are written inside a
// larger matrix are multiples of the 16-byte vector width, so no write spills
// into a neighbouring block.  No operation may write a matrix it reads.
#pragma once
#include <utility>

#include "ss_la.cuh"

namespace ss {
namespace dense {

template <typename R>
struct Vec;
template <>
struct Vec<float> {
  static constexpr int n = 4;
  float v[4];
};
template <>
struct Vec<double> {
  static constexpr int n = 2;
  double v[2];
};

SS_DEV Vec<float> ld16(const float* p) {
  const float4 t = *reinterpret_cast<const float4*>(p);
  Vec<float> r;
  r.v[0] = t.x;
  r.v[1] = t.y;
  r.v[2] = t.z;
  r.v[3] = t.w;
  return r;
}
SS_DEV Vec<double> ld16(const double* p) {
  const double2 t = *reinterpret_cast<const double2*>(p);
  Vec<double> r;
  r.v[0] = t.x;
  r.v[1] = t.y;
  return r;
}
SS_DEV void st16(float* p, const Vec<float>& v) {
  *reinterpret_cast<float4*>(p) = make_float4(v.v[0], v.v[1], v.v[2], v.v[3]);
}
SS_DEV void st16(double* p, const Vec<double>& v) {
  *reinterpret_cast<double2*>(p) = make_double2(v.v[0], v.v[1]);
}

// Row geometry of an N-column matrix: n = padded row length (whole 16-byte
// units), ld = row stride (an odd number of 16-byte units).
template <typename R, int N>
struct Pad {
  static constexpr int W = Vec<R>::n;
  static constexpr int n = (N + W - 1) / W * W;
  static constexpr int q = n / W;
  static constexpr int ld = ((q & 1) ? q : q + 1) * W;
};

SS_DEV int lane_id() { return threadIdx.x & 31; }

// Zero n elements (n a multiple of the vector width, p 16-byte aligned).
template <typename R>
SS_DEV void zero(R* p, int n) {
  Vec<R> z;
  SS_UNROLL
  for (int u = 0; u < Vec<R>::n; ++u) z.v[u] = R(0);
  for (int q = lane_id() * Vec<R>::n; q < n; q += 32 * Vec<R>::n) st16(p + q, z);
  __syncwarp();
}

template <typename R, int COLS, int LD>
SS_DEV void load_row(const R* M, int r, R (&x)[Pad<R, COLS>::n]) {
  constexpr int W = Vec<R>::n;
  SS_UNROLL
  for (int j = 0; j < Pad<R, COLS>::n; j += W) {
    const Vec<R> v = ld16(M + r * LD + j);
    SS_UNROLL
    for (int u = 0; u < W; ++u) x[j + u] = (j + u < COLS) ? v.v[u] : R(0);
  }
}

template <typename R, int COLS, int LD>
SS_DEV void store_row(R* M, int r, const R (&x)[Pad<R, COLS>::n]) {
  constexpr int W = Vec<R>::n;
  SS_UNROLL
  for (int j = 0; j < Pad<R, COLS>::n; j += W) {
    Vec<R> v;
    SS_UNROLL
    for (int u = 0; u < W; ++u) v.v[u] = (j + u < COLS) ? x[j + u] : R(0);
    st16(M + r * LD + j, v);
  }
}

// Columns [OFF, OFF + N) of a register row into row r of a shared matrix.
template <typename R, int N, int LD, int OFF, int CPX>
SS_DEV void store_part(R* M, int r, const R (&x)[CPX]) {
  constexpr int W = Vec<R>::n;
  static_assert(OFF + Pad<R, N>::n <= CPX, "part outside the row");
  SS_UNROLL
  for (int j = 0; j < Pad<R, N>::n; j += W) {
    Vec<R> v;
    SS_UNROLL
    for (int u = 0; u < W; ++u) v.v[u] = (j + u < N) ? x[OFF + j + u] : R(0);
    st16(M + r * LD + j, v);
  }
}

// ----------------------------------------------------------------------------- tria

// Parlett's reflector for x = (x0, rest), sig = |rest|^2: v0 = x0 - |x| computed
// without cancellation, tau = 2 / (v0^2 + sig) (0 for a zero vector).  FP32 uses
// the hardware reciprocal square root and reciprocal (within 2 ulp).
template <typename R>
SS_DEV void parlett(R x0, R sig, R& v0, R& tau) {
  const R nrm = ss_sqrt(x0 * x0 + sig);
  v0 = (x0 <= R(0)) ? x0 - nrm : -sig / (x0 + nrm);
  const R vv = v0 * v0 + sig;
  tau = (vv > R(0)) ? R(2) / vv : R(0);
}
SS_DEV void parlett(float x0, float sig, float& v0, float& tau) {
  if (!SS_FAST_FP32) {
    const float nrm = sqrtf(x0 * x0 + sig);
    v0 = (x0 <= 0.0f) ? x0 - nrm : -sig / (x0 + nrm);
    const float vv = v0 * v0 + sig;
    tau = (vv > 0.0f) ? 2.0f / vv : 0.0f;
    return;
  }
  const float s = x0 * x0 + sig;
  const float nrm = (s > 0.0f) ? s * rsqrtf(s) : 0.0f;
  v0 = (x0 <= 0.0f) ? x0 - nrm : __fdividef(-sig, x0 + nrm);
  const float vv = v0 * v0 + sig;
  tau = (vv > 0.0f) ? __fdividef(2.0f, vv) : 0.0f;
}

// M <- [L 0] = M Q, Q orthogonal, L lower triangular with a non-negative
// diagonal: Householder reflections from the right (Golub & Van Loan,
// Algorithm 5.1.1, with Parlett's formula for the sign-free reflector, so the
// diagonal comes out non-negative without a second pass).
//
// Per pivot p the pivot lane publishes its row x (16-byte stores, no masking)
// and the squared norm of its part right of p (four partial sums) in one of
// two alternating buffers, so one warp barrier per pivot suffices.  The
// reflector v equals x right of p, v_p = x_p - ||x||-like (Parlett), zero left
// of p; every lane forms row . v and row -= tau (row . v) v over the published
// x and corrects the eight columns of the pivot block, the pivot row included
// (it becomes (.., ||x||, ~0, ..) up to rounding).  The strict upper triangle
// is cleared once at the end.  Pivots are processed in blocks of eight so that
// every register index is compile-time.  vb holds two buffers of
// Pad<COLS>::n + W elements (16-byte aligned): tria_scratch().
// ROLL: the pivot loop of a block needs no compile-time pivot index; kept
// rolled, the code of the large triangularisations shrinks (measured: the
// per-sequence walk and the scan levels 10 % faster, fewer instruction-cache
// stalls), while the shared-covariance walk measured 7 % faster unrolled.
template <typename R, int ROWS, int COLS, int LD, bool ROLL = true>
struct Tria {
  static constexpr int W = Vec<R>::n;
  static constexpr int CP = Pad<R, COLS>::n;
  static constexpr int NS = (ROWS + 31) / 32;
  static constexpr int VS = CP + W;   // one reflector buffer
  static_assert(ROWS <= COLS, "tria needs rows <= cols");
  static_assert(LD >= CP, "row stride too small");

  template <int J0>
  static SS_DEV void block(R (&row)[NS][CP], R* vb, int lane) {
    // rows r < J0 are final: from pivot 32 on, a lane's first slot (rows 0..31)
    // takes no more reflector work (a warp-wide saving, not a per-lane mask)
    constexpr int S0 = (J0 >= 32) ? 1 : 0;
    const int pend = (J0 + 8 < ROWS) ? J0 + 8 : ROWS;
    if constexpr (ROLL) {
#pragma unroll 1
      for (int p = J0; p < pend; ++p) pivot<J0, S0>(p, row, vb, lane);
    } else {
      for (int p = J0; p < pend; ++p) pivot<J0, S0>(p, row, vb, lane);
    }
  }

  template <int J0, int S0>
  static SS_DEV void pivot(int p, R (&row)[NS][CP], R* vb, int lane) {
    constexpr int JB = (J0 + 8 < CP) ? J0 + 8 : CP;   // end of the pivot block's columns
    {
      R* v = vb + (p & 1) * VS;
      if (lane == (p & 31)) {
        const int ps = p >> 5;
        R sq[4] = {R(0), R(0), R(0), R(0)};
        SS_UNROLL
        for (int j = J0; j < CP; j += W) {
          Vec<R> o;
          SS_UNROLL
          for (int u = 0; u < W; ++u) {
            const int jj = j + u;
            R xj = row[0][jj];
            if constexpr (NS > 1) {
              if (ps == 1) xj = row[1][jj];
            }
            o.v[u] = xj;
            if (jj >= JB) sq[jj & 3] += xj * xj;
            else if (jj > p) sq[jj & 3] += xj * xj;
          }
          st16(v + j, o);
        }
        v[CP] = (sq[0] + sq[1]) + (sq[2] + sq[3]);
      }
      __syncwarp();
      const R sig = v[CP];
      const R x0 = v[p];
      R v0, tau;
      parlett(x0, sig, v0, tau);
      // v - x on the pivot block: -x_j left of p, v_p - x_p at p, 0 right of p
      R cb[JB - J0];
      SS_UNROLL
      for (int j = J0; j < JB; j += W) {
        const Vec<R> x = ld16(v + j);
        SS_UNROLL
        for (int u = 0; u < W; ++u) {
          const int jj = j + u;
          cb[jj - J0] = (jj < p) ? -x.v[u] : ((jj == p) ? v0 - x0 : R(0));
        }
      }
      R d[NS][4];
      SS_UNROLL
      for (int s = S0; s < NS; ++s) {
        SS_UNROLL
        for (int k = 0; k < 4; ++k) d[s][k] = R(0);
      }
      SS_UNROLL
      for (int j = J0; j < CP; j += W) {
        const Vec<R> x = ld16(v + j);
        SS_UNROLL
        for (int u = 0; u < W; ++u) {
          SS_UNROLL
          for (int s = S0; s < NS; ++s) {
            R vj = x.v[u];
            if (j + u < JB) vj += cb[j + u - J0];
            d[s][(j + u) & 3] += row[s][j + u] * vj;
          }
        }
      }
      R f[NS];
      SS_UNROLL
      for (int s = S0; s < NS; ++s) {
        const int r = lane + 32 * s;
        const R dd = (d[s][0] + d[s][1]) + (d[s][2] + d[s][3]);
        f[s] = (r >= p && r < ROWS) ? tau * dd : R(0);
      }
      SS_UNROLL
      for (int j = J0; j < CP; j += W) {
        const Vec<R> x = ld16(v + j);
        SS_UNROLL
        for (int u = 0; u < W; ++u) {
          R vj = x.v[u];
          if (j + u < JB) vj += cb[j + u - J0];
          SS_UNROLL
          for (int s = S0; s < NS; ++s) row[s][j + u] -= f[s] * vj;
        }
      }
    }
  }

  template <int... B>
  static SS_DEV void blocks(R (&row)[NS][CP], R* vb, int lane, std::integer_sequence<int, B...>) {
    (block<8 * B>(row, vb, lane), ...);
  }

  // The rows already in registers (row r = lane r % 32, slot r / 32; rows >= ROWS and
  // columns >= COLS zero).
  static SS_DEV void clear_upper(R (&row)[NS][CP], int lane) {
    SS_UNROLL
    for (int s = 0; s < NS; ++s) {
      const int r = lane + 32 * s;
      SS_UNROLL
      for (int j = 0; j < CP; ++j)
        if (j > r) row[s][j] = R(0);
    }
  }

  static SS_DEV void run_regs(R (&row)[NS][CP], R* vb) {
    const int lane = lane_id();
    blocks(row, vb, lane, std::make_integer_sequence<int, (ROWS + 7) / 8>{});
    clear_upper(row, lane);
    __syncwarp();
  }

  static SS_DEV void run(R* M, R* vb) {
    const int lane = lane_id();
    R row[NS][CP];
    SS_UNROLL
    for (int s = 0; s < NS; ++s) {
      const int r = lane + 32 * s;
      if (r < ROWS) {
        load_row<R, COLS, LD>(M, r, row[s]);
      } else {
        SS_UNROLL
        for (int j = 0; j < CP; ++j) row[s][j] = R(0);
      }
    }
    blocks(row, vb, lane, std::make_integer_sequence<int, (ROWS + 7) / 8>{});
    clear_upper(row, lane);
    SS_UNROLL
    for (int s = 0; s < NS; ++s) {
      const int r = lane + 32 * s;
      if (r < ROWS) store_row<R, COLS, LD>(M, r, row[s]);
    }
    __syncwarp();
  }
};

// Scratch elements tria<., COLS> needs for its reflector buffers.
template <typename R, int COLS>
__host__ __device__ constexpr int tria_scratch() { return 2 * (Pad<R, COLS>::n + Vec<R>::n); }

template <typename R, int ROWS, int COLS, int LD>
SS_DEV void tria(R* M, R* vb) {
  Tria<R, ROWS, COLS, LD>::run(M, vb);
}

// ----------------------------------------------------------------------------- products

// FP32 products on the tensor cores: warp-level mma.sync m16n8k8 with TF32
// operands and FP32 accumulation, each operand split into a TF32 high part and
// a TF32 remainder (x = hi + lo) and the product accumulated as
// lo*hi + hi*lo + hi*hi ("3xTF32"): the dropped lo*lo term is below FP32
// rounding, so the result has FP32 accuracy while the multiply-adds run on the
// tensor pipe.  Fragment layout of m16n8k8 (g = lane / 4, t = lane % 4):
// A (16 x 8) a0 (g, t), a1 (g + 8, t), a2 (g, t + 4), a3 (g + 8, t + 4);
// B (8 x 8) b0 (k = t, n = g), b1 (k = t + 4, n = g);
// C (16 x 8) c0, c1 (g, 2t, 2t + 1), c2, c3 (g + 8, 2t, 2t + 1).
SS_DEV uint32_t tf32_hi(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}
SS_DEV void tf32_split(float x, uint32_t& hi, uint32_t& lo) {
  hi = tf32_hi(x);
  lo = tf32_hi(x - __uint_as_float(hi));
}
SS_DEV void mma_tf32(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, "
               "{%8, %9}, {%0, %1, %2, %3};"
               : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
               : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

template <int M, int K, int N, bool TA, bool TB, int LDA, int LDB, int LDC, bool LB>
SS_DEV void mm_tc(float* C, const float* A, const float* B, float alpha, bool acc) {
  static_assert(M % 16 == 0 && K % 8 == 0 && N % 8 == 0, "tensor-core tiles");
  constexpr int KT = K / 8;
  const int lane = lane_id();
  const int g = lane >> 2, t = lane & 3;
  auto a_at = [&](int m, int k) -> float { return TA ? A[k * LDA + m] : A[m * LDA + k]; };
  auto b_at = [&](int k, int n) -> float {
    if (LB && n > k) return 0.0f;
    return TB ? B[n * LDB + k] : B[k * LDB + n];
  };
#pragma unroll 1
  for (int m0 = 0; m0 < M; m0 += 16) {
    uint32_t ah[KT][4], al[KT][4];
    SS_UNROLL
    for (int kt = 0; kt < KT; ++kt) {
      const int k0 = kt * 8;
      tf32_split(a_at(m0 + g, k0 + t), ah[kt][0], al[kt][0]);
      tf32_split(a_at(m0 + g + 8, k0 + t), ah[kt][1], al[kt][1]);
      tf32_split(a_at(m0 + g, k0 + t + 4), ah[kt][2], al[kt][2]);
      tf32_split(a_at(m0 + g + 8, k0 + t + 4), ah[kt][3], al[kt][3]);
    }
#pragma unroll 1
    for (int n0 = 0; n0 < N; n0 += 8) {
      float d[4] = {0.0f, 0.0f, 0.0f, 0.0f};
      SS_UNROLL
      for (int kt = 0; kt < KT; ++kt) {
        const int k0 = kt * 8;
        uint32_t bh[2], bl[2];
        tf32_split(b_at(k0 + t, n0 + g), bh[0], bl[0]);
        tf32_split(b_at(k0 + t + 4, n0 + g), bh[1], bl[1]);
        mma_tf32(d, al[kt], bh);
        mma_tf32(d, ah[kt], bl);
        mma_tf32(d, ah[kt], bh);
      }
      const int r0 = m0 + g, c0 = n0 + 2 * t;
      float* p0 = C + r0 * LDC + c0;
      float* p1 = C + (r0 + 8) * LDC + c0;
      const float o0 = acc ? p0[0] : 0.0f, o1 = acc ? p0[1] : 0.0f;
      const float o2 = acc ? p1[0] : 0.0f, o3 = acc ? p1[1] : 0.0f;
      p0[0] = o0 + alpha * d[0];
      p0[1] = o1 + alpha * d[1];
      p1[0] = o2 + alpha * d[2];
      p1[1] = o3 + alpha * d[3];
    }
  }
  __syncwarp();
}

// C = alpha op(A) op(B) (+ C when acc), C: M x N, op(A): M x K, op(B): K x N,
// op(X) = X^T when the flag is set.
// LB: B is lower triangular (its strict upper part is skipped).
// FP32 shapes that tile into 16 x 8 x 8 run on the tensor cores (mm_tc).
template <typename R, int M, int K, int N, bool TA, bool TB, int LDA, int LDB, int LDC, bool LB = false>
SS_DEV void mm(R* C, const R* A, const R* B, R alpha = R(1), bool acc = false) {
  if constexpr (std::is_same<R, float>::value && M % 16 == 0 && K % 8 == 0 && N % 8 == 0) {
    mm_tc<M, K, N, TA, TB, LDA, LDB, LDC, LB>(C, A, B, alpha, acc);
    return;
  }
  constexpr int W = Vec<R>::n;
  constexpr int KP = Pad<R, K>::n, NP = Pad<R, N>::n;
  const int lane = lane_id();
#pragma unroll 1
  for (int s = 0; s < (M + 31) / 32; ++s) {
    const int i = lane + 32 * s;
    const int ii = i < M ? i : M - 1;
    R a[KP];
    if constexpr (TA) {
      SS_UNROLL
      for (int k = 0; k < KP; ++k) a[k] = (k < K) ? A[k * LDA + ii] : R(0);
    } else {
      load_row<R, K, LDA>(A, ii, a);
    }
    R c[NP];
    if constexpr (!TB) {
      SS_UNROLL
      for (int j = 0; j < NP; ++j) c[j] = R(0);
      SS_UNROLL
      for (int k = 0; k < K; ++k) {
        SS_UNROLL
        for (int j = 0; j < NP; j += W) {
          if (LB && j > k) continue;
          const Vec<R> b = ld16(B + k * LDB + j);
          SS_UNROLL
          for (int u = 0; u < W; ++u) c[j + u] += a[k] * b.v[u];
        }
      }
    } else {
      SS_UNROLL
      for (int j = 0; j < NP; ++j) {
        R t = R(0);
        if (j < N) {
          SS_UNROLL
          for (int k = 0; k < KP; k += W) {
            const Vec<R> b = ld16(B + j * LDB + k);
            SS_UNROLL
            for (int u = 0; u < W; ++u)
              if (k + u < K) t += a[k + u] * b.v[u];
          }
        }
        c[j] = t;
      }
    }
    if (i < M) {
      SS_UNROLL
      for (int j = 0; j < NP; j += W) {
        Vec<R> o;
        if (acc) {
          o = ld16(C + i * LDC + j);
        } else {
          SS_UNROLL
          for (int u = 0; u < W; ++u) o.v[u] = R(0);
        }
        SS_UNROLL
        for (int u = 0; u < W; ++u) o.v[u] += (j + u < N) ? alpha * c[j + u] : R(0);
        st16(C + i * LDC + j, o);
      }
    }
  }
  __syncwarp();
}

// X <- X L^{-1}, L lower triangular (N x N); the ROWS rows of X are independent.
template <typename R, int ROWS, int N, int LDX, int LDL>
SS_DEV void trsm_rl(R* X, const R* L) {
  constexpr int W = Vec<R>::n, NP = Pad<R, N>::n;
  const int lane = lane_id();
#pragma unroll 1
  for (int s = 0; s < (ROWS + 31) / 32; ++s) {
    const int i = lane + 32 * s;
    const int ii = i < ROWS ? i : ROWS - 1;
    R x[NP];
    load_row<R, N, LDX>(X, ii, x);
    SS_UNROLL
    for (int k = N - 1; k >= 0; --k) {
      x[k] = x[k] * ss_rcp(L[k * LDL + k]);
      SS_UNROLL
      for (int j = 0; j < k; j += W) {
        const Vec<R> l = ld16(L + k * LDL + j);
        SS_UNROLL
        for (int u = 0; u < W; ++u)
          if (j + u < k) x[j + u] -= x[k] * l.v[u];
      }
    }
    __syncwarp();
    if (i < ROWS) store_row<R, N, LDX>(X, i, x);
  }
  __syncwarp();
}

// X <- X L^{-T}, L lower triangular (N x N).
template <typename R, int ROWS, int N, int LDX, int LDL>
SS_DEV void trsm_rlt(R* X, const R* L) {
  constexpr int W = Vec<R>::n, NP = Pad<R, N>::n;
  const int lane = lane_id();
#pragma unroll 1
  for (int s = 0; s < (ROWS + 31) / 32; ++s) {
    const int i = lane + 32 * s;
    const int ii = i < ROWS ? i : ROWS - 1;
    R x[NP];
    load_row<R, N, LDX>(X, ii, x);
    SS_UNROLL
    for (int k = 0; k < N; ++k) {
      R t = x[k];
      SS_UNROLL
      for (int j = 0; j < k; j += W) {
        const Vec<R> l = ld16(L + k * LDL + j);
        SS_UNROLL
        for (int u = 0; u < W; ++u)
          if (j + u < k) t -= x[j + u] * l.v[u];
      }
      x[k] = t * ss_rcp(L[k * LDL + k]);
    }
    __syncwarp();
    if (i < ROWS) store_row<R, N, LDX>(X, i, x);
  }
  __syncwarp();
}

// D (ROWS x COLS block) <- S, or <- S^T when T (S is then COLS x ROWS).
template <typename R, int ROWS, int COLS, bool T, int LDD, int LDS>
SS_DEV void copy(R* D, const R* S) {
  const int lane = lane_id();
  constexpr int CP = Pad<R, COLS>::n;
#pragma unroll 1
  for (int s = 0; s < (ROWS + 31) / 32; ++s) {
    const int i = lane + 32 * s;
    if (i < ROWS) {
      R x[CP];
      if constexpr (T) {
        SS_UNROLL
        for (int j = 0; j < CP; ++j) x[j] = (j < COLS) ? S[j * LDS + i] : R(0);
      } else {
        load_row<R, COLS, LDS>(S, i, x);
      }
      store_row<R, COLS, LDD>(D, i, x);
    }
  }
  __syncwarp();
}

// D (ROWS x COLS block) <- diag * I (rows >= COLS or columns >= ROWS zero).
template <typename R, int ROWS, int COLS, int LDD>
SS_DEV void fill_diag(R* D, R diag) {
  const int lane = lane_id();
  constexpr int CP = Pad<R, COLS>::n;
#pragma unroll 1
  for (int s = 0; s < (ROWS + 31) / 32; ++s) {
    const int i = lane + 32 * s;
    if (i < ROWS) {
      R x[CP];
      SS_UNROLL
      for (int j = 0; j < CP; ++j) x[j] = (j == i) ? diag : R(0);
      store_row<R, COLS, LDD>(D, i, x);
    }
  }
  __syncwarp();
}

// Lane i < M: sum_k op(A)[i][k] x[k] (x a padded shared vector).
template <typename R, int M, int K, bool TA, int LDA>
SS_DEV R rowdot(const R* A, const R* x, int i) {
  constexpr int W = Vec<R>::n, KP = Pad<R, K>::n;
  const int ii = i < M ? i : M - 1;
  R t = R(0);
  if constexpr (TA) {
    SS_UNROLL
    for (int k = 0; k < K; ++k) t += A[k * LDA + ii] * x[k];
  } else {
    SS_UNROLL
    for (int k = 0; k < KP; k += W) {
      const Vec<R> a = ld16(A + ii * LDA + k);
      const Vec<R> b = ld16(x + k);
      SS_UNROLL
      for (int u = 0; u < W; ++u)
        if (k + u < K) t += a.v[u] * b.v[u];
    }
  }
  return t;
}

// Cooperative copies between a contiguous global (ROWS x COLS, row-major)
// array and a shared matrix; COLS a multiple of the vector width, both
// addresses 16-byte aligned.
template <typename R, int ROWS, int COLS, int LD>
SS_DEV void g2s(R* S, const R* G) {
  constexpr int W = Vec<R>::n, U = COLS / W;
  static_assert(COLS % W == 0, "columns must fill whole 16-byte units");
  for (int q = lane_id(); q < ROWS * U; q += 32) {
    const int r = q / U, c = (q - r * U) * W;
    st16(S + r * LD + c, ld16(G + (size_t)r * COLS + c));
  }
  __syncwarp();
}

template <typename R, int ROWS, int COLS, int LD>
SS_DEV void s2g(R* G, const R* S) {
  constexpr int W = Vec<R>::n, U = COLS / W;
  static_assert(COLS % W == 0, "columns must fill whole 16-byte units");
  for (int q = lane_id(); q < ROWS * U; q += 32) {
    const int r = q / U, c = (q - r * U) * W;
    st16(G + (size_t)r * COLS + c, ld16(S + r * LD + c));
  }
  __syncwarp();
}

// Element-wise version for arrays of unknown alignment (model matrices).
template <typename R, int ROWS, int COLS, int LD>
SS_DEV void g2s_any(R* S, const R* G) {
  for (int q = lane_id(); q < ROWS * COLS; q += 32) {
    const int r = q / COLS, c = q - r * COLS;
    S[r * LD + c] = G[q];
  }
  __syncwarp();
}

// Global -> global copy of n elements (16-byte aligned, n a multiple of W).
template <typename R>
SS_DEV void g2g(R* D, const R* S, int n) {
  constexpr int W = Vec<R>::n;
  for (int q = lane_id() * W; q < n; q += 32 * W) st16(D + q, ld16(S + q));
  __syncwarp();
}

SS_DEV float warp_sum(float v) {
  SS_UNROLL
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
SS_DEV double warp_sum(double v) {
  SS_UNROLL
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

}  // namespace dense
}  // namespace ss
