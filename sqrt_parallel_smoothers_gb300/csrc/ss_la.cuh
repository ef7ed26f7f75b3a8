// Small dense linear algebra for one thread: fixed-size row-major arrays that
// the compiler keeps in registers (every loop bound is a template constant and
// every loop is unrolled).  These are the building blocks of the per-timestep
// element construction and of the associative-scan combines.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <type_traits>

#define SS_DEV __device__ __forceinline__
#define SS_UNROLL _Pragma("unroll")

namespace ss {

SS_DEV float ss_sqrt(float x) { return sqrtf(x); }
SS_DEV double ss_sqrt(double x) { return sqrt(x); }
SS_DEV float ss_abs(float x) { return fabsf(x); }
SS_DEV double ss_abs(double x) { return fabs(x); }
SS_DEV float ss_log(float x) { return logf(x); }
SS_DEV double ss_log(double x) { return log(x); }
SS_DEV bool ss_isfinite(float x) { return isfinite(x); }
SS_DEV bool ss_isfinite(double x) { return isfinite(x); }

// FP32 factorisations use the hardware reciprocal and reciprocal square root
// (__fdividef, rsqrtf: within 2 ulp) in the Householder reflectors and the
// triangular solves' pivots; FP64 stays correctly rounded.  Other scalar types
// (dual numbers) use their division.
#ifndef SS_FAST_FP32
#define SS_FAST_FP32 1
#endif
SS_DEV float ss_rcp(float x) { return SS_FAST_FP32 ? __fdividef(1.0f, x) : __frcp_rn(x); }
SS_DEV double ss_rcp(double x) { return __drcp_rn(x); }
template <typename R>
SS_DEV R ss_rcp(const R& x) { return R(1) / x; }

// One Householder reflector's scalars from x0 = M[i][i] and sigma = the sum of
// squares of the rest of row i (> 0): beta = -sign(x0) sqrt(x0^2 + sigma),
// v0 = x0 - beta and k = 1 / (beta v0) = -1 / (|beta| (|beta| + |x0|)).
template <typename R>
SS_DEV void reflector(R x0, R sigma, R& beta, R& v0, R& k) {
  const R nrm = ss_sqrt(x0 * x0 + sigma);
  beta = (x0 <= R(0)) ? nrm : -nrm;   // opposite sign of x0: no cancellation in v0
  v0 = x0 - beta;
  k = R(1) / (beta * v0);
}
SS_DEV void reflector(float x0, float sigma, float& beta, float& v0, float& k) {
  if (SS_FAST_FP32) {
    const float s = x0 * x0 + sigma;
    const float ri = rsqrtf(s);
    const float nrm = s * ri;
    beta = (x0 <= 0.0f) ? nrm : -nrm;
    v0 = x0 - beta;
    k = __fdividef(-ri, nrm + fabsf(x0));
  } else {
    const float nrm = sqrtf(x0 * x0 + sigma);
    beta = (x0 <= 0.0f) ? nrm : -nrm;
    v0 = x0 - beta;
    k = 1.0f / (beta * v0);
  }
}

// Range guard of the FP32 reflectors.  A reflector takes the unscaled sum of
// squares of its row, which overflows once an entry passes about 1.8e19 (and
// the products of its update a little earlier), and underflows below about
// 1e-19.  When x0^2 + sigma leaves [2^-64, 2^64] (or is not finite) the row is
// scaled by a power of two first, as LAPACK's scaled norm does: every step of
// the reflector is then exact in range, and the reflector itself is unchanged
// (H = I + k u u^T is invariant under u -> a u, k -> k / a^2), so only beta is
// scaled back.  Typical rows never take this path; FP64 (range 1e308) and dual
// numbers never do.  The guard is not free even when no row takes it (with it
// on every tria the batched smoother measured 16 % slower, the filter walk
// 28 %), so tria and tria_sp take it as a template flag, set where FP32 entries
// can grow without bound: the information-factor update of the chunk leaf,
// whose rows carry the chunk's product of linearised transitions
// (filter_extend, csrc/ss_ops.cuh; 1.5 % of the batched smoother's time).
template <typename R>
SS_DEV bool reflector_out_of_range(const R&, const R&) { return false; }
SS_DEV bool reflector_out_of_range(float x0, float sigma) {
  const float s = x0 * x0 + sigma;
  return !(s <= 0x1p64f && s >= 0x1p-64f);
}
// 2^-e for the exponent e of amax (amax > 0), so that amax * 2^-e lies in
// [1, 2); e is clamped so that both 2^-e and 2^e are normal floats.
SS_DEV float pow2_inverse_scale(float amax) {
  int e = ((__float_as_int(amax) >> 23) & 0xff) - 127;
  e = e < -125 ? -125 : (e > 125 ? 125 : e);
  return __int_as_float((127 - e) << 23);
}
template <typename R>
SS_DEV R pow2_inverse_scale(const R&) { return R(1); }

// Whether row i still needs a reflector.  In FP32 a row whose whole sum of
// squares x0^2 + sigma is below the smallest normal float is taken as already
// reduced: the hardware reciprocal square root flushes such a denormal to zero
// and would turn the reflector into inf * 0 = NaN, while the entries it would
// rotate are below 1.1e-19, far under the rounding of any normal-range factor.
// (The range-guarded triangularisations rescale such rows instead.)
#ifndef SS_TINY_ROWS_REDUCED
#define SS_TINY_ROWS_REDUCED 1
#endif
template <typename R>
SS_DEV bool reflector_live(const R& x0, const R& sigma) { return sigma != R(0); }
SS_DEV bool reflector_live(float x0, float sigma) {
  return sigma != 0.0f && (!SS_TINY_ROWS_REDUCED || x0 * x0 + sigma >= 0x1p-126f);
}

// Programmatic dependent launch (sm_90 and later).  The per-pass kernels are
// launched with programmatic stream serialisation, so a kernel's launch is
// prepared while its predecessor on the stream drains.  Each such kernel calls
// pdl_enter() first: griddepcontrol.wait blocks until the predecessor has
// completed and its writes are visible (a no-op without a programmatic
// predecessor).  Every kernel of the chain waits before it completes, so a
// kernel also sees the writes of all earlier kernels on its stream.  An early
// launch_dependents (SS_PDL_TRIGGER=1) lets the successor's blocks take SM
// slots while they wait; measured, that is 8 % slower than the trigger at
// block exit, which is the default.
#ifndef SS_PDL_TRIGGER
#define SS_PDL_TRIGGER 0
#endif
SS_DEV void pdl_enter() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  if (SS_PDL_TRIGGER) asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// ---------------------------------------------------------------------------
// tria: on return M[:, :ROWS] holds the lower-triangular L (diag >= 0) with
// L L^T = M M^T (input M), and M[:, ROWS:] is zero.  Householder reflections
// applied from the right, one per row (the transpose of QR of M^T).  This is
// the single primitive every square-root step uses
// (parsmooth/_utils.py:22-24 computes the same factor through jnp.linalg.qr).
template <typename R, int ROWS, int COLS, bool GUARD = false>
SS_DEV void tria(R (&M)[ROWS][COLS]) {
  static_assert(COLS >= ROWS, "tria expects at least as many columns as rows");
  SS_UNROLL
  for (int i = 0; i < ROWS; ++i) {
    // two partial sums: halves the dependent chain of the norm
    R sig0 = R(0), sig1 = R(0);
    SS_UNROLL
    for (int j = i + 1; j < COLS; ++j) {
      if ((j - i) & 1) sig0 += M[i][j] * M[i][j];
      else sig1 += M[i][j] * M[i][j];
    }
    R sigma = sig0 + sig1;
    R x0 = M[i][i];
    R beta = x0;
    if (sigma != R(0)) {
      R unscale = R(1);
      if (GUARD && reflector_out_of_range(x0, sigma)) {
        R amax = ss_abs(x0);
        SS_UNROLL
        for (int j = i + 1; j < COLS; ++j) amax = ss_abs(M[i][j]) > amax ? ss_abs(M[i][j]) : amax;
        const R sc = pow2_inverse_scale(amax);
        unscale = R(1) / sc;
        x0 *= sc;
        sigma = R(0);
        SS_UNROLL
        for (int j = i + 1; j < COLS; ++j) {
          M[i][j] *= sc;
          sigma += M[i][j] * M[i][j];
        }
      }
      const R nrm = ss_sqrt(x0 * x0 + sigma);
      beta = (x0 <= R(0)) ? nrm : -nrm;   // opposite sign of x0: no cancellation in v0
      const R v0 = x0 - beta;
      const R tau = -v0 / beta;
      const R inv = R(1) / v0;
      R v[COLS];
      SS_UNROLL
      for (int j = i + 1; j < COLS; ++j) v[j] = M[i][j] * inv;
      SS_UNROLL
      for (int r = i + 1; r < ROWS; ++r) {
        R w0 = M[r][i], w1 = R(0);
        SS_UNROLL
        for (int j = i + 1; j < COLS; ++j) {
          if ((j - i) & 1) w1 += M[r][j] * v[j];
          else w0 += M[r][j] * v[j];
        }
        const R w = (w0 + w1) * tau;
        M[r][i] -= w;
        SS_UNROLL
        for (int j = i + 1; j < COLS; ++j) M[r][j] -= w * v[j];
      }
      SS_UNROLL
      for (int j = i + 1; j < COLS; ++j) M[i][j] = R(0);
      beta *= unscale;
    }
    // canonical sign: non-negative diagonal (flip column i)
    if (beta < R(0)) {
      M[i][i] = -beta;
      SS_UNROLL
      for (int r = i + 1; r < ROWS; ++r) M[r][i] = -M[r][i];
    } else {
      M[i][i] = beta;
    }
  }
}

// ---------------------------------------------------------------------------
// tria_sp: the same factor as tria, for inputs with a known zero pattern.
//
// Every square-root step factors a block matrix whose blocks are full,
// lower-triangular or zero ([[F L, cQ], [L, 0]] and the like).  A Householder
// reflection from the right only spreads non-zeros within the columns it
// touches, so the pattern of every intermediate matrix follows from the input
// pattern alone.  TriaPlan runs that propagation at compile time: for each
// reflector i, the columns > i it carries (sup) and the rows > i it changes
// (touch).  The device loop then skips products with structural zeros (exact
// zeros in tria's arithmetic).  Each reflector is applied in the unscaled form
// H = I + u u^T / (beta v0), one reciprocal per reflector, so the result equals
// tria's up to rounding.
//
// PAT::nz(r, c) is true where the input may be non-zero; entries it calls zero
// are taken as zero.
template <int ROWS, int COLS>
struct TriaPlan {
  unsigned long long sup[ROWS];
  unsigned long long touch[ROWS];
};

template <int ROWS, int COLS, class PAT>
__host__ __device__ constexpr TriaPlan<ROWS, COLS> make_tria_plan() {
  static_assert(COLS <= 64 && ROWS <= 64, "patterns are 64-bit masks");
  TriaPlan<ROWS, COLS> p{};
  unsigned long long nz[ROWS] = {};
  for (int r = 0; r < ROWS; ++r)
    for (int c = 0; c < COLS; ++c)
      if (PAT::nz(r, c)) nz[r] |= 1ull << c;
  for (int i = 0; i < ROWS; ++i) {
    const unsigned long long below = (i + 1 < 64) ? ~((2ull << i) - 1) : 0ull;
    const unsigned long long s = nz[i] & below;
    const unsigned long long cols = s | (1ull << i);
    p.sup[i] = s;
    p.touch[i] = 0;
    if (s != 0) {
      for (int r = i + 1; r < ROWS; ++r) {
        if (nz[r] & cols) {
          p.touch[i] |= 1ull << r;
          nz[r] |= cols;
        }
      }
    }
    nz[i] = 1ull << i;
  }
  return p;
}

// Block patterns.  Rows [0, RT) over columns [0, CL) are full; rows [0, RT)
// over columns [CL, COLS) are lower triangular with KB leading full columns
// (entry (r, CL + c) non-zero iff c <= r or c < KB); rows [RT, ROWS) are lower
// triangular (full when BL_FULL) over columns [0, CL) and zero beyond.
template <int RT, int CL, int KB = 0, bool BL_FULL = false>
struct PatBlocks {
  __host__ __device__ static constexpr bool nz(int r, int c) {
    if (r < RT) return c < CL || (c - CL) <= r || (c - CL) < KB;
    return c < CL && (BL_FULL || c <= r - RT);
  }
};

struct PatFull {
  __host__ __device__ static constexpr bool nz(int, int) { return true; }
};

// Reflector I of tria_sp applied to the rows it touches: M[r] += c u with
// u = (v0, M[I][I+1:]) and c = k (M[r] . u).
template <typename R, int ROWS, int COLS, int I, unsigned long long SUP, unsigned long long TOUCH>
SS_DEV void tria_sp_apply(R (&M)[ROWS][COLS], const R& v0, const R& k) {
  constexpr int i = I;
  SS_UNROLL
  for (int r = i + 1; r < ROWS; ++r) {
    if ((TOUCH >> r) & 1) {
      R d0 = M[r][i] * v0, d1 = R(0);
      SS_UNROLL
      for (int j = i + 1; j < COLS; ++j) {
        if ((SUP >> j) & 1) {
          if ((j - i) & 1) d1 += M[r][j] * M[i][j];
          else d0 += M[r][j] * M[i][j];
        }
      }
      const R c = (d0 + d1) * k;
      M[r][i] += c * v0;
      SS_UNROLL
      for (int j = i + 1; j < COLS; ++j)
        if ((SUP >> j) & 1) M[r][j] += c * M[i][j];
    }
  }
}

// A row whose part right of the diagonal is already zero (sigma == 0) needs no
// reflector.  With SS_TRIA_SELECT that case is taken by selects (v0 = k = 0
// makes the update a no-op, beta = x0) instead of a branch around the
// reflector, so the code of a triangularisation is one basic block and the
// scheduler can overlap each reflector's row updates with the next one's norm
// (the range guard's rare rescaling keeps its branch).
#ifndef SS_TRIA_SELECT
#define SS_TRIA_SELECT 1
#endif

template <typename R, int ROWS, int COLS, class PAT, int I, bool GUARD>
SS_DEV void tria_sp_step(R (&M)[ROWS][COLS]) {
  if constexpr (I < ROWS) {
    constexpr TriaPlan<ROWS, COLS> P = make_tria_plan<ROWS, COLS, PAT>();
    constexpr unsigned long long SUP = P.sup[I];
    constexpr unsigned long long TOUCH = P.touch[I];
    constexpr int i = I;
    R beta = M[i][i];
    if constexpr (SUP != 0) {
      R sig0 = R(0), sig1 = R(0);
      SS_UNROLL
      for (int j = i + 1; j < COLS; ++j) {
        if ((SUP >> j) & 1) {
          if ((j - i) & 1) sig0 += M[i][j] * M[i][j];
          else sig1 += M[i][j] * M[i][j];
        }
      }
      R sigma = sig0 + sig1;
      R x0 = M[i][i];
      const bool live = GUARD ? sigma != R(0) : reflector_live(x0, sigma);
      if (SS_TRIA_SELECT || live) {
        // H = I + u u^T / (beta v0), u = (v0, M[i][i+1:]), v0 = x0 - beta:
        // one reciprocal per reflector, no scaled copy of the row (except in
        // the FP32 range guard, which scales the row in place).
        R v0, k, b, unscale = R(1);
        if (GUARD && live && reflector_out_of_range(x0, sigma)) {
          R amax = ss_abs(x0);
          SS_UNROLL
          for (int j = i + 1; j < COLS; ++j)
            if ((SUP >> j) & 1) amax = ss_abs(M[i][j]) > amax ? ss_abs(M[i][j]) : amax;
          const R sc = pow2_inverse_scale(amax);
          unscale = R(1) / sc;
          x0 *= sc;
          sigma = R(0);
          SS_UNROLL
          for (int j = i + 1; j < COLS; ++j) {
            if ((SUP >> j) & 1) {
              M[i][j] *= sc;
              sigma += M[i][j] * M[i][j];
            }
          }
        }
        reflector(x0, sigma, b, v0, k);
        beta = live ? b * unscale : beta;
        v0 = live ? v0 : R(0);
        k = live ? k : R(0);
        tria_sp_apply<R, ROWS, COLS, I, SUP, TOUCH>(M, v0, k);
      }
    }
    SS_UNROLL
    for (int j = i + 1; j < COLS; ++j) M[i][j] = R(0);
    if (beta < R(0)) {
      M[i][i] = -beta;
      SS_UNROLL
      for (int r = i + 1; r < ROWS; ++r) M[r][i] = -M[r][i];
    } else {
      M[i][i] = beta;
    }
    tria_sp_step<R, ROWS, COLS, PAT, I + 1, GUARD>(M);
  }
}

template <typename R, int ROWS, int COLS, class PAT, bool GUARD = false>
SS_DEV void tria_sp(R (&M)[ROWS][COLS]) {
  static_assert(COLS >= ROWS, "tria expects at least as many columns as rows");
  if constexpr (COLS > 64) {
    // wider than a 64-bit pattern mask (sigma-point regressions of conditional models at
    // nx >= 8): the unpatterned triangularisation
    tria<R, ROWS, COLS, GUARD>(M);
    return;
  }
  // entries outside the pattern are zero: say so, so that they cost no registers
  SS_UNROLL
  for (int r = 0; r < ROWS; ++r) {
    SS_UNROLL
    for (int c = 0; c < COLS; ++c)
      if (!PAT::nz(r, c)) M[r][c] = R(0);
  }
  tria_sp_step<R, ROWS, COLS, PAT, 0, GUARD>(M);
}

// ---------------------------------------------------------------------------
// Triangular solves against the lower-triangular N x N block of M that starts
// at (R0, C0) (only its lower part is read).

// B <- L^{-1} B   (B: N x K)
template <typename R, int N, int K, int R0 = 0, int C0 = 0, int MR, int MC>
SS_DEV void solve_lower(const R (&M)[MR][MC], R (&B)[N][K]) {
  SS_UNROLL
  for (int i = 0; i < N; ++i) {
    const R inv = ss_rcp(M[R0 + i][C0 + i]);
    SS_UNROLL
    for (int k = 0; k < K; ++k) {
      R s = B[i][k];
      SS_UNROLL
      for (int j = 0; j < i; ++j) s -= M[R0 + i][C0 + j] * B[j][k];
      B[i][k] = s * inv;
    }
  }
}

// b <- L^{-1} b
template <typename R, int N, int R0 = 0, int C0 = 0, int MR, int MC>
SS_DEV void solve_lower_vec(const R (&M)[MR][MC], R (&b)[N]) {
  SS_UNROLL
  for (int i = 0; i < N; ++i) {
    R s = b[i];
    SS_UNROLL
    for (int j = 0; j < i; ++j) s -= M[R0 + i][C0 + j] * b[j];
    b[i] = s * ss_rcp(M[R0 + i][C0 + i]);
  }
}

// B <- L^{-T} B   (B: N x K)
template <typename R, int N, int K, int R0 = 0, int C0 = 0, int MR, int MC>
SS_DEV void solve_lower_T(const R (&M)[MR][MC], R (&B)[N][K]) {
  SS_UNROLL
  for (int i = N - 1; i >= 0; --i) {
    const R inv = ss_rcp(M[R0 + i][C0 + i]);
    SS_UNROLL
    for (int k = 0; k < K; ++k) {
      R s = B[i][k];
      SS_UNROLL
      for (int j = i + 1; j < N; ++j) s -= M[R0 + j][C0 + i] * B[j][k];
      B[i][k] = s * inv;
    }
  }
}

// ---------------------------------------------------------------------------
// Givens: L <- tria([L, v]) for lower-triangular L (D x D) with diag >= 0.
// Handles L == 0 (first column of a streamed factor) and zero pivots.
template <typename R, int D>
SS_DEV void chol_add_column(R (&L)[D][D], R (&v)[D]) {
  SS_UNROLL
  for (int j = 0; j < D; ++j) {
    const R a = L[j][j];
    const R b = v[j];
    const R r = ss_sqrt(a * a + b * b);
    if (r != R(0)) {
      const R c = a / r, s = b / r;
      L[j][j] = r;
      SS_UNROLL
      for (int i = j + 1; i < D; ++i) {
        const R lij = L[i][j];
        const R vi = v[i];
        L[i][j] = c * lij + s * vi;
        v[i] = c * vi - s * lij;
      }
    }
  }
}

// Rank-1 update (mult = +1) or downdate (mult = -1) of a lower Cholesky
// factor, column sweep of Algorithm 3.1 of Krause & Igel as written in
// parsmooth/_utils.py:39-81; non-finite entries of the result become 0.
template <typename R, int D>
SS_DEV void chol_update(R (&L)[D][D], const R (&v)[D], R mult) {
  R omega[D];
  SS_UNROLL
  for (int i = 0; i < D; ++i) omega[i] = v[i];
  R b = R(1);
  R out[D][D];
  SS_UNROLL
  for (int j = 0; j < D; ++j) {
    const R d = L[j][j];
    const R w = omega[j];
    const R nd = ss_sqrt(d * d + mult / b * w * w);
    const R gamma = d * d * b + mult * w * w;
    const R wd = w / d;
    SS_UNROLL
    for (int i = j; i < D; ++i) omega[i] -= wd * L[i][j];
    const R coef = mult * w / gamma;
    SS_UNROLL
    for (int i = j + 1; i < D; ++i) out[i][j] = nd * (L[i][j] / d + coef * omega[i]);
    out[j][j] = nd;
    b += mult * wd * wd;
  }
  SS_UNROLL
  for (int i = 0; i < D; ++i) {
    SS_UNROLL
    for (int j = 0; j <= i; ++j) L[i][j] = ss_isfinite(out[i][j]) ? out[i][j] : R(0);
  }
}

// ---------------------------------------------------------------------------
// Products.

// C = A B   (A: M x K, B: K x N)
template <typename R, int M, int K, int N>
SS_DEV void matmul(const R (&A)[M][K], const R (&B)[K][N], R (&C)[M][N]) {
  SS_UNROLL
  for (int i = 0; i < M; ++i) {
    SS_UNROLL
    for (int j = 0; j < N; ++j) {
      R s = R(0);
      SS_UNROLL
      for (int k = 0; k < K; ++k) s += A[i][k] * B[k][j];
      C[i][j] = s;
    }
  }
}

// C = A^T B   (A: K x M, B: K x N)
template <typename R, int K, int M, int N>
SS_DEV void matmul_tn(const R (&A)[K][M], const R (&B)[K][N], R (&C)[M][N]) {
  SS_UNROLL
  for (int i = 0; i < M; ++i) {
    SS_UNROLL
    for (int j = 0; j < N; ++j) {
      R s = R(0);
      SS_UNROLL
      for (int k = 0; k < K; ++k) s += A[k][i] * B[k][j];
      C[i][j] = s;
    }
  }
}

// y = A x
template <typename R, int M, int N>
SS_DEV void matvec(const R (&A)[M][N], const R (&x)[N], R (&y)[M]) {
  SS_UNROLL
  for (int i = 0; i < M; ++i) {
    R s = R(0);
    SS_UNROLL
    for (int j = 0; j < N; ++j) s += A[i][j] * x[j];
    y[i] = s;
  }
}

// y = A^T x
template <typename R, int M, int N>
SS_DEV void matvec_t(const R (&A)[M][N], const R (&x)[M], R (&y)[N]) {
  SS_UNROLL
  for (int j = 0; j < N; ++j) {
    R s = R(0);
    SS_UNROLL
    for (int i = 0; i < M; ++i) s += A[i][j] * x[i];
    y[j] = s;
  }
}

// ---------------------------------------------------------------------------
// Global-memory records.  Every per-step / per-summary record is a flat array
// of R; records are padded to a multiple of 16 bytes so that each thread moves
// them with 16-byte vector accesses.

template <typename R>
struct Vec16 {  // scalar types without a 16-byte vector form are moved element by element
  static constexpr int n = 1;
  static constexpr bool vec = false;
};
template <>
struct Vec16<float> {
  typedef float4 type;
  static constexpr int n = 4;
  static constexpr bool vec = true;
};
template <>
struct Vec16<double> {
  typedef double2 type;
  static constexpr int n = 2;
  static constexpr bool vec = true;
};

template <typename R, int N>
struct Padded {
  static constexpr int n = ((N + Vec16<R>::n - 1) / Vec16<R>::n) * Vec16<R>::n;
};

// Read-only cached load for built-in scalars, plain load otherwise.
SS_DEV float ldg(const float* p) { return __ldg(p); }
SS_DEV double ldg(const double* p) { return __ldg(p); }
template <typename R>
SS_DEV R ldg(const R* p) { return *p; }

// Global side must be 16-byte aligned (records sit at 16-byte multiples in a
// 256-byte aligned workspace); the register side is copied element by element.
SS_DEV void vec_to(const float4& v, float* d) { d[0] = v.x; d[1] = v.y; d[2] = v.z; d[3] = v.w; }
SS_DEV void vec_to(const double2& v, double* d) { d[0] = v.x; d[1] = v.y; }
SS_DEV float4 vec_from(const float* s) { return make_float4(s[0], s[1], s[2], s[3]); }
SS_DEV double2 vec_from(const double* s) { return make_double2(s[0], s[1]); }

template <typename R, int N>
SS_DEV void load_rec(const R* __restrict__ src, R (&dst)[Padded<R, N>::n]) {
  if constexpr (Vec16<R>::vec) {
    typedef typename Vec16<R>::type V;
    constexpr int W = Vec16<R>::n;
    const V* s = reinterpret_cast<const V*>(src);
    SS_UNROLL
    for (int k = 0; k < Padded<R, N>::n / W; ++k) vec_to(__ldg(s + k), dst + k * W);
  } else {
    SS_UNROLL
    for (int k = 0; k < N; ++k) dst[k] = src[k];
  }
}

template <typename R, int N>
SS_DEV void store_rec(R* __restrict__ dst, const R (&src)[Padded<R, N>::n]) {
  if constexpr (Vec16<R>::vec) {
    typedef typename Vec16<R>::type V;
    constexpr int W = Vec16<R>::n;
    V* d = reinterpret_cast<V*>(dst);
    SS_UNROLL
    for (int k = 0; k < Padded<R, N>::n / W; ++k) d[k] = vec_from(src + k * W);
  } else {
    SS_UNROLL
    for (int k = 0; k < N; ++k) dst[k] = src[k];
  }
}

// Copy helpers between flat records and matrices.
template <typename R, int M, int N, int P>
SS_DEV void unpack(const R (&rec)[P], int off, R (&A)[M][N]) {
  SS_UNROLL
  for (int i = 0; i < M; ++i) {
    SS_UNROLL
    for (int j = 0; j < N; ++j) A[i][j] = rec[off + i * N + j];
  }
}
// Lower-triangular factor stored as its N (N + 1) / 2 lower entries, row by
// row; unpacking sets the upper entries to zero, so the compiler treats them
// as constants.
template <typename R, int N, int P>
SS_DEV void pack_tri(R (&rec)[P], int off, const R (&A)[N][N]) {
  SS_UNROLL
  for (int i = 0; i < N; ++i) {
    SS_UNROLL
    for (int j = 0; j <= i; ++j) rec[off + i * (i + 1) / 2 + j] = A[i][j];
  }
}
template <typename R, int N, int P>
SS_DEV void unpack_tri(const R (&rec)[P], int off, R (&A)[N][N]) {
  SS_UNROLL
  for (int i = 0; i < N; ++i) {
    SS_UNROLL
    for (int j = 0; j < N; ++j) A[i][j] = (j <= i) ? rec[off + i * (i + 1) / 2 + j] : R(0);
  }
}
template <typename R, int N, int P>
SS_DEV void unpack_vec(const R (&rec)[P], int off, R (&a)[N]) {
  SS_UNROLL
  for (int i = 0; i < N; ++i) a[i] = rec[off + i];
}
template <typename R, int M, int N, int P>
SS_DEV void pack(R (&rec)[P], int off, const R (&A)[M][N]) {
  SS_UNROLL
  for (int i = 0; i < M; ++i) {
    SS_UNROLL
    for (int j = 0; j < N; ++j) rec[off + i * N + j] = A[i][j];
  }
}
template <typename R, int N, int P>
SS_DEV void pack_vec(R (&rec)[P], int off, const R (&a)[N]) {
  SS_UNROLL
  for (int i = 0; i < N; ++i) rec[off + i] = a[i];
}

}  // namespace ss
