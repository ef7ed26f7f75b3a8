// Host orchestration of one API call for a compile-time (R, NX, NY).
#pragma once
#include <algorithm>
#include <cmath>
#include <cstring>

#include "ss_dims.h"
#include "ss_staged.cuh"

namespace ss {

enum { OP_WORKSPACE = 0, OP_LINEARIZE = 1, OP_FILTER = 2, OP_SMOOTH = 3, OP_ITERATED = 4, OP_SUPPORTED = 5,
       OP_SAMPLE = 6, OP_ADJOINT = 7 };

// One entry-point call, dtype-erased.
struct Call {
  int op;
  const ss_problem* p;
  size_t* ws_bytes_out;
  // linearize
  int32_t which;
  int64_t n_points;
  const void* pt_m;
  const void* pt_L;
  void* pt_F;
  void* pt_chol;
  void* pt_b;
  // filter / smoother / iterated
  const void* ys;
  const void* m0;
  const void* L0;
  int32_t prior_per_sequence;
  const void* nom_m;
  const void* nom_L;
  const void* in_m;
  const void* in_L;
  void* out_m;
  void* out_L;
  double* out_ell;
  double* out_grad;   // (B, grad_ld) gradient output; this run writes column grad_col
  int32_t grad_ld;
  int32_t grad_col;
  int32_t n_iter;
  double tol;
  int32_t* out_iters;
  uint32_t* out_flags;
  void* ws;
  size_t ws_bytes;
  cudaStream_t stream;
  const ss_tangents* tangents;  // forward-mode directions of the model scalars (gradient runs)
  int32_t n_samples;            // sampler: draws per sequence
  const void* eps;              // sampler: standard normals (states, n_samples, nx)
  const ss_adjoints* adjoints;  // reverse-mode gradient outputs (ss_filter_adjoint)
};

typedef int (*RunFn)(const Call&);

inline size_t align_up(size_t x, size_t a = 256) { return (x + a - 1) / a * a; }

struct Layout {
  int C, G, L;
  int64_t items[MAX_LEVELS + 1];
  size_t lvl, lvl_stride;  // int64 [L][B+1]
  size_t lin, selem, fT, ll, mse, active, iters, nomA_m, nomA_L, nomB_m, nomB_L;
  size_t fsum[MAX_LEVELS + 1], fst[MAX_LEVELS + 1], ssum[MAX_LEVELS + 1], sst[MAX_LEVELS + 1];
  size_t bytes;
};

template <typename R, int NX, int NY>
inline int make_layout(const ss_problem& p, Layout& y) {
  typedef Rec<R, NX, NY> Q;
  const int64_t B = p.batch, N = p.total_steps;
  y.C = p.chunk > 0 ? p.chunk : 16;
  y.G = p.group > 1 ? p.group : 8;
  if (p.chunk <= 0 && p.group <= 1) {
    // Automatic geometry.  A problem whose level-1 chunks fit in one wave of
    // resident threads (152 SMs x 256 threads at the chunk kernels' register
    // use) is latency-bound: the time is the chain one thread walks (C steps at
    // the leaf, G summaries per level, up to 4G at the top), so the smallest
    // chunk that still fits one wave, with G = 4, is the shortest chain.
    // FP64 arithmetic is slow per thread on this GPU, so FP64 prefers groups of
    // two (more levels, half the sequential combines per level; measured 24 %
    // faster for one sequence of 4096 steps) when the levels fit.
    constexpr int64_t ONE_WAVE = 152 * 256;
    for (int c : {4, 8}) {
      if (N / c + B <= ONE_WAVE) {
        for (int g : {sizeof(typename Tangents<R>::scalar) == 8 ? 2 : 4, 4}) {
          int64_t n = (p.max_len + c - 1) / c;
          int levels = 1;
          while (n > 4 * g) { n = (n + g - 1) / g; ++levels; }
          if (levels <= MAX_LEVELS) { y.C = c; y.G = g; break; }
        }
        break;
      }
    }
  }
  const int64_t top = 4 * (int64_t)y.G;
  int64_t n = (p.max_len + y.C - 1) / y.C;
  y.L = 1;
  while (n > top) {
    n = (n + y.G - 1) / y.G;
    ++y.L;
    if (y.L > MAX_LEVELS) return SS_ERR_INVALID;
  }
  y.items[0] = N;
  y.items[1] = (N + y.C - 1) / y.C + B;
  for (int l = 2; l <= y.L; ++l) y.items[l] = (y.items[l - 1] + y.G - 1) / y.G + B;
  size_t o = 0;
  auto take = [&](size_t bytes) { size_t r = o; o = align_up(o + bytes); return r; };
  y.lvl_stride = (size_t)(B + 1);
  y.lvl = take(sizeof(int64_t) * y.lvl_stride * y.L);
  y.lin = take(sizeof(R) * Q::LIN_P * (size_t)N);
  y.selem = take(sizeof(R) * Q::SE_P * (size_t)N);
  for (int l = 1; l <= y.L; ++l) {
    y.fsum[l] = take(sizeof(R) * Q::FE_P * (size_t)y.items[l]);
    y.fst[l] = take(sizeof(R) * Q::ST_P * (size_t)y.items[l]);
    y.ssum[l] = take(sizeof(R) * Q::SE_P * (size_t)y.items[l]);
    y.sst[l] = take(sizeof(R) * Q::ST_P * (size_t)y.items[l]);
  }
  y.fT = take(sizeof(R) * Q::ST_P * (size_t)B);
  y.ll = take(sizeof(double) * (size_t)y.items[1] * (1 + Tangents<R>::n));
  y.mse = take(sizeof(double) * (size_t)B);
  y.active = take(sizeof(int32_t) * (size_t)B);
  y.iters = take(sizeof(int32_t) * (size_t)B);
  const size_t S = (size_t)(N + B);
  // The factor buffers also hold the loop's intermediate nominals as packed
  // state records (run_iterated), which for nx <= 3 are longer than nx * nx.
  constexpr size_t NOM_L = (size_t)(NX * NX > Q::ST_P ? NX * NX : Q::ST_P);
  y.nomA_m = take(sizeof(R) * S * NX);
  y.nomA_L = take(sizeof(R) * S * NOM_L);
  y.nomB_m = take(sizeof(R) * S * NX);
  y.nomB_L = take(sizeof(R) * S * NOM_L);
  y.bytes = o;
  return SS_OK;
}

// Host-side rule constants (unscented weights, Gauss-Hermite roots/weights).
int fill_rule(const ss_problem& p, RuleArgs& r);

template <typename R>
inline ModelArgs<R> model_args(const ss_model& m) {
  ModelArgs<R> a;
  a.mat = static_cast<const R*>(m.matrix);
  for (int k = 0; k < 4; ++k) a.p[k] = R(m.params[k]);
  return a;
}

inline int slr_form_of(const ss_problem& p, bool fp32) {
  if (p.slr_form == SS_SLR_DOWNDATE || p.slr_form == SS_SLR_RESIDUAL) return p.slr_form;
  // the residual form needs a rule with identity second moment: not GH of order 1
  if (p.lin_method == SS_LIN_GAUSS_HERMITE && p.gh_order < 2) return SS_SLR_DOWNDATE;
  return fp32 ? SS_SLR_RESIDUAL : SS_SLR_DOWNDATE;
}

// Instrumentation (ss_capi.cu): a launch counter and optional per-kernel
// CUDA-event timing.  Events are recorded on the launching stream around each
// kernel, so they also time kernels replayed from a captured CUDA graph.
void count_launch();
bool profiling_on();
void profile_push(const char* name, cudaEvent_t start, cudaEvent_t stop);

// During stream capture an event record only becomes a graph node (re-recorded
// by every replay) with cudaEventRecordExternal.
inline void record_event(cudaEvent_t e, cudaStream_t st) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(st, &cs);
  cudaEventRecordWithFlags(e, st, cs == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : cudaEventRecordDefault);
}

#define SS_LAUNCH(NAME, ST, ...)                                           \
  do {                                                                     \
    cudaEvent_t ss_e0_ = nullptr;                                          \
    const bool ss_prof_ = ss::profiling_on();                              \
    if (ss_prof_) {                                                        \
      cudaEventCreate(&ss_e0_);                                            \
      ss::record_event(ss_e0_, ST);                                        \
    }                                                                      \
    __VA_ARGS__;                                                           \
    if (cudaGetLastError() != cudaSuccess) return SS_ERR_CUDA;             \
    ss::count_launch();                                                    \
    if (ss_prof_) {                                                        \
      cudaEvent_t ss_e1_ = nullptr;                                        \
      cudaEventCreate(&ss_e1_);                                            \
      ss::record_event(ss_e1_, ST);                                        \
      ss::profile_push(NAME, ss_e0_, ss_e1_);                              \
    }                                                                      \
  } while (0)

// Launch with programmatic stream serialisation (the kernel must begin with
// pdl_enter()), or plainly when that is switched off (SQRTSMOOTH_PDL=0).
bool pdl_on();
template <typename... KArgs, typename... Args>
inline void launch_pdl(void (*kernel)(KArgs...), unsigned grid, int block, size_t smem, cudaStream_t st,
                       Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl_on() ? 1 : 0;
  cudaLaunchKernelEx(&cfg, kernel, args...);
}

// The scan-level kernels (up, top, down) have few, long-running items; one warp
// per block spreads them over every SM.
constexpr int LEVEL_BLOCK = 32;

inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block > 0 ? (n + block - 1) / block : 1); }

// The shared-memory staged kernels (ss_staged.cuh) serve types with a 16-byte
// vector form whose staging tiles fit a block; the others take the plain kernels.
template <typename R, int NX, int NY>
constexpr bool use_staged() {
  if constexpr (Vec16<R>::vec) return StagedSmem<R, NX, NY>::fits;
  else return false;
}

// Lin-kernel dispatch over the model pair and method.
template <typename R, int NX, int NY, class TF, class OF, int METHOD>
inline int launch_lin_one(const LinArgs<R>& a, cudaStream_t st) {
  const unsigned grid = grid_for(a.total, STAGED_BLOCK);
  if constexpr (use_staged<R, NX, NY>()) {
    constexpr int sm = (int)StagedSmem<R, NX, NY>::lin;
    cudaFuncSetAttribute(lin_staged_kernel<R, NX, NY, TF, OF, METHOD>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    SS_LAUNCH("lin", st, launch_pdl(lin_staged_kernel<R, NX, NY, TF, OF, METHOD>, grid, STAGED_BLOCK, sm, st, a));
  } else {
    SS_LAUNCH("lin", st, lin_kernel<R, NX, NY, TF, OF, METHOD><<<grid, 128, 0, st>>>(a));
  }
  return SS_OK;
}

template <typename R, int NX, int NY, class TF, class OF>
inline int launch_lin_method(const LinArgs<R>& a, int method, cudaStream_t st) {
  switch (method) {
    case SS_LIN_EXTENDED: return launch_lin_one<R, NX, NY, TF, OF, SS_LIN_EXTENDED>(a, st);
    case SS_LIN_CUBATURE: return launch_lin_one<R, NX, NY, TF, OF, SS_LIN_CUBATURE>(a, st);
    case SS_LIN_UNSCENTED: return launch_lin_one<R, NX, NY, TF, OF, SS_LIN_UNSCENTED>(a, st);
    case SS_LIN_GAUSS_HERMITE:
      if constexpr (Tangents<R>::n == 0) return launch_lin_one<R, NX, NY, TF, OF, SS_LIN_GAUSS_HERMITE>(a, st);
      else return SS_ERR_UNSUPPORTED;
    default: return SS_ERR_UNSUPPORTED;
  }
}

template <int NX>
constexpr bool ct_ok() { return NX == 5; }
template <int NX, int NY>
constexpr bool bearings_ok() { return NY == 2 && NX >= 2; }

template <int NX, int NY>
constexpr bool poisson_ok() { return NY <= NX; }

template <typename R, int NX, int NY>
inline bool models_supported(int tk, int ok) {
  const bool t = tk == SS_MODEL_LINEAR || (tk == SS_MODEL_COORDINATED_TURN && ct_ok<NX>()) ||
                 tk == SS_MODEL_RICKER;
  const bool o = ok == SS_MODEL_LINEAR || (ok == SS_MODEL_BEARINGS && bearings_ok<NX, NY>()) ||
                 (ok == SS_MODEL_POISSON_EXP && poisson_ok<NX, NY>());
  return t && o;
}

template <typename R, int NX, int NY, class TF>
inline int launch_lin_obs(const LinArgs<R>& a, int ok, int method, cudaStream_t st) {
  if (ok == SS_MODEL_LINEAR) return launch_lin_method<R, NX, NY, TF, LinearFn<R, NX, NY>>(a, method, st);
  if constexpr (bearings_ok<NX, NY>()) {
    if (ok == SS_MODEL_BEARINGS) return launch_lin_method<R, NX, NY, TF, BearingsFn<R, NX, NY>>(a, method, st);
  }
  if constexpr (poisson_ok<NX, NY>()) {
    if (ok == SS_MODEL_POISSON_EXP) return launch_lin_method<R, NX, NY, TF, PoissonExpFn<R, NX, NY>>(a, method, st);
  }
  return SS_ERR_UNSUPPORTED;
}

template <typename R, int NX, int NY>
inline int launch_lin(const LinArgs<R>& a, int tk, int ok, int method, cudaStream_t st) {
  if (a.total == 0) return SS_OK;
  if constexpr (Tangents<R>::n > 0) {
    // gradient runs: the bearings pair at (5, 2) and linear pairs only
    if constexpr (ct_ok<NX>() && bearings_ok<NX, NY>()) {
      if (tk == SS_MODEL_COORDINATED_TURN && ok == SS_MODEL_BEARINGS)
        return launch_lin_method<R, NX, NY, CoordinatedTurnFn<R, NX, NX>, BearingsFn<R, NX, NY>>(a, method, st);
    }
    if (tk == SS_MODEL_LINEAR && ok == SS_MODEL_LINEAR)
      return launch_lin_method<R, NX, NY, LinearFn<R, NX, NX>, LinearFn<R, NX, NY>>(a, method, st);
    return SS_ERR_UNSUPPORTED;
  } else {
    if (tk == SS_MODEL_LINEAR) return launch_lin_obs<R, NX, NY, LinearFn<R, NX, NX>>(a, ok, method, st);
    if constexpr (ct_ok<NX>()) {
      if (tk == SS_MODEL_COORDINATED_TURN)
        return launch_lin_obs<R, NX, NY, CoordinatedTurnFn<R, NX, NX>>(a, ok, method, st);
    }
    if (tk == SS_MODEL_RICKER) return launch_lin_obs<R, NX, NY, RickerFn<R, NX, NX>>(a, ok, method, st);
    return SS_ERR_UNSUPPORTED;
  }
}

template <typename R, int DIN, int DOUT, class Fn>
inline int launch_points_method(const PointArgs<R>& a, int method, cudaStream_t st) {
  const unsigned grid = grid_for(a.n, 128);
  switch (method) {
    case SS_LIN_EXTENDED: SS_LAUNCH("lin_points", st, lin_points_kernel<R, DIN, DOUT, Fn, SS_LIN_EXTENDED><<<grid, 128, 0, st>>>(a)); break;
    case SS_LIN_CUBATURE: SS_LAUNCH("lin_points", st, lin_points_kernel<R, DIN, DOUT, Fn, SS_LIN_CUBATURE><<<grid, 128, 0, st>>>(a)); break;
    case SS_LIN_UNSCENTED: SS_LAUNCH("lin_points", st, lin_points_kernel<R, DIN, DOUT, Fn, SS_LIN_UNSCENTED><<<grid, 128, 0, st>>>(a)); break;
    case SS_LIN_GAUSS_HERMITE: SS_LAUNCH("lin_points", st, lin_points_kernel<R, DIN, DOUT, Fn, SS_LIN_GAUSS_HERMITE><<<grid, 128, 0, st>>>(a)); break;
    default: return SS_ERR_UNSUPPORTED;
  }
  return SS_OK;
}

// ----------------------------------------------------------------------------- runner

template <typename R, int NX, int NY>
struct Runner {
  typedef Rec<R, NX, NY> Q;
  const Call& c;
  const ss_problem& p;
  Layout y;
  char* ws;
  cudaStream_t st;
  Geo geo;
  ScanArgs<R> sa;
  LinArgs<R> la;

  explicit Runner(const Call& call) : c(call), p(*call.p), ws(static_cast<char*>(call.ws)), st(call.stream) {}

  template <typename T>
  T* at(size_t off) const { return reinterpret_cast<T*>(ws + off); }

  int prepare() {
    int rc = make_layout<R, NX, NY>(p, y);
    if (rc) return rc;
    if (c.ws_bytes < y.bytes || ws == nullptr) return SS_ERR_WORKSPACE;
    geo.off = p.offsets;
    geo.B = p.batch;
    geo.C = y.C;
    geo.G = y.G;
    geo.L = y.L;
    for (int l = 0; l <= MAX_LEVELS; ++l) geo.lvl[l] = nullptr;
    for (int l = 1; l <= y.L; ++l) geo.lvl[l] = at<int64_t>(y.lvl) + (size_t)(l - 1) * y.lvl_stride;
    SS_LAUNCH("plan", st, plan_kernel<512><<<1, 512, 0, st>>>(geo, at<int64_t>(y.lvl), (int64_t)y.lvl_stride));
    std::memset(&sa, 0, sizeof(sa));
    sa.g = geo;
    sa.ys = static_cast<const R*>(c.ys);
    sa.lin = at<R>(y.lin);
    sa.selem = at<R>(y.selem);
    for (int l = 1; l <= y.L; ++l) {
      sa.fsum[l] = at<R>(y.fsum[l]);
      sa.fst[l] = at<R>(y.fst[l]);
      sa.ssum[l] = at<R>(y.ssum[l]);
      sa.sst[l] = at<R>(y.sst[l]);
    }
    sa.fT = at<R>(y.fT);
    sa.m0 = static_cast<const R*>(c.m0);
    sa.L0 = static_cast<const R*>(c.L0);
    sa.prior_stride = c.prior_per_sequence ? 1 : 0;
    std::memset(&la, 0, sizeof(la));
    la.off = p.offsets;
    la.B = p.batch;
    la.total = p.total_steps;
    la.tm = model_args<R>(p.transition);
    la.om = model_args<R>(p.observation);
    if constexpr (Tangents<R>::n > 0) {
      if (c.tangents != nullptr) {
        for (int dir = 0; dir < c.tangents->n_dir && dir < Tangents<R>::n; ++dir) {
          for (int k = 0; k < 4; ++k) {
            la.tm.p[k].d[dir] = c.tangents->trans_params[dir][k];
            la.om.p[k].d[dir] = c.tangents->obs_params[dir][k];
          }
        }
      }
    }
    la.tq_m = static_cast<const R*>(p.transition.noise_mean);
    la.tq_L = static_cast<const R*>(p.transition.noise_chol);
    la.oq_m = static_cast<const R*>(p.observation.noise_mean);
    la.oq_L = static_cast<const R*>(p.observation.noise_chol);
    rc = fill_rule(p, la.rule);
    if (rc) return rc;
    la.slr_form = slr_form_of(p, sizeof(typename Tangents<R>::scalar) == 4);
    la.out = at<R>(y.lin);
    return SS_OK;
  }

  int lin(const R* nm, const R* nL, const int32_t* active, bool trans_only, const R* nrec = nullptr) {
    la.nom_m = nm;
    la.nom_L = nL;
    la.nom_rec = nrec;
    la.active = active;
    la.trans_only = trans_only ? 1 : 0;
    return launch_lin<R, NX, NY>(la, p.transition.kind, trans_only ? SS_MODEL_LINEAR : p.observation.kind,
                                 p.lin_method, st);
  }

  // Filter scan: level-1 summaries must already be in fsum[1] (filter_leaf).
  int filter_scan() {
    for (int l = 1; l < y.L; ++l) {
      SS_LAUNCH("filter_up", st, launch_pdl(filter_up_kernel<R, NX>, grid_for(y.items[l + 1], LEVEL_BLOCK), LEVEL_BLOCK, 0, st, sa, l));
    }
    SS_LAUNCH("filter_top", st, launch_pdl(filter_top_kernel<R, NX>, grid_for(p.batch, LEVEL_BLOCK), LEVEL_BLOCK, 0, st, sa));
    for (int l = y.L - 1; l >= 1; --l) {
      SS_LAUNCH("filter_down", st, launch_pdl(filter_down_kernel<R, NX>, grid_for(y.items[l + 1], LEVEL_BLOCK), LEVEL_BLOCK, 0, st, sa, l));
    }
    return SS_OK;
  }

  int filter_pass(bool emit_smoother) {
    const unsigned g1 = grid_for(y.items[1], STAGED_BLOCK);
    if constexpr (use_staged<R, NX, NY>()) {
      constexpr int sm = (int)StagedSmem<R, NX, NY>::leaf;
      cudaFuncSetAttribute(filter_leaf_staged_kernel<R, NX, NY>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
      SS_LAUNCH("filter_leaf", st, launch_pdl(filter_leaf_staged_kernel<R, NX, NY>, g1, STAGED_BLOCK, sm, st, sa));
    } else {
      SS_LAUNCH("filter_leaf", st, filter_leaf_kernel<R, NX, NY><<<grid_for(y.items[1], 128), 128, 0, st>>>(sa));
    }
    int rc = filter_scan();
    if (rc) return rc;
    sa.emit_smoother = emit_smoother ? 1 : 0;
    if constexpr (use_staged<R, NX, NY>()) {
      constexpr int sm = (int)StagedSmem<R, NX, NY>::fwalk;
      cudaFuncSetAttribute(filter_walk_staged_kernel<R, NX, NY>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
      SS_LAUNCH("filter_walk", st, launch_pdl(filter_walk_staged_kernel<R, NX, NY>, g1, STAGED_BLOCK, sm, st, sa));
    } else {
      SS_LAUNCH("filter_walk", st, filter_walk_kernel<R, NX, NY><<<grid_for(y.items[1], 128), 128, 0, st>>>(sa));
    }
    return SS_OK;
  }

  int smoother_scan_and_walk() {
    for (int l = 1; l < y.L; ++l) {
      SS_LAUNCH("smoother_up", st, launch_pdl(smoother_up_kernel<R, NX>, grid_for(y.items[l + 1], LEVEL_BLOCK), LEVEL_BLOCK, 0, st, sa, l));
    }
    SS_LAUNCH("smoother_top", st, launch_pdl(smoother_top_kernel<R, NX>, grid_for(p.batch, LEVEL_BLOCK), LEVEL_BLOCK, 0, st, sa));
    for (int l = y.L - 1; l >= 1; --l) {
      SS_LAUNCH("smoother_down", st, launch_pdl(smoother_down_kernel<R, NX>, grid_for(y.items[l + 1], LEVEL_BLOCK), LEVEL_BLOCK, 0, st, sa, l));
    }
    if constexpr (use_staged<R, NX, NY>()) {
      constexpr int sm = (int)StagedSmem<R, NX, NY>::swalk;
      cudaFuncSetAttribute(smoother_walk_staged_kernel<R, NX>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
      SS_LAUNCH("smoother_walk", st,
                launch_pdl(smoother_walk_staged_kernel<R, NX>, grid_for(y.items[1], STAGED_BLOCK), STAGED_BLOCK, sm, st, sa));
    } else {
      SS_LAUNCH("smoother_walk", st, smoother_walk_kernel<R, NX><<<grid_for(y.items[1], 128), 128, 0, st>>>(sa));
    }
    return SS_OK;
  }

  int run_filter() {
    int rc = prepare();
    if (rc) return rc;
    rc = lin(static_cast<const R*>(c.nom_m), static_cast<const R*>(c.nom_L), nullptr, false);
    if (rc) return rc;
    sa.filt_m = static_cast<R*>(c.out_m);
    sa.filt_L = static_cast<R*>(c.out_L);
    sa.ll_chunk = c.out_ell ? at<double>(y.ll) : nullptr;
    rc = filter_pass(false);
    if (rc) return rc;
    if (c.out_ell) {
      SS_LAUNCH("ll_reduce", st, ll_reduce_kernel<<<grid_for(p.batch, 128), 128, 0, st>>>(geo, NY, 1 + Tangents<R>::n, at<double>(y.ll), c.out_ell, c.out_grad, c.grad_ld, c.grad_col, nullptr));
    }
    return SS_OK;
  }

  int run_smooth() {
    int rc = prepare();
    if (rc) return rc;
    rc = lin(static_cast<const R*>(c.nom_m), static_cast<const R*>(c.nom_L), nullptr, true);
    if (rc) return rc;
    sa.in_m = static_cast<const R*>(c.in_m);
    sa.in_L = static_cast<const R*>(c.in_L);
    sa.out_m = static_cast<R*>(c.out_m);
    sa.out_L = static_cast<R*>(c.out_L);
    SS_LAUNCH("smoother_leaf", st, smoother_leaf_kernel<R, NX, NY><<<grid_for(y.items[1], 128), 128, 0, st>>>(sa));
    SS_LAUNCH("last_state", st, last_state_kernel<R, NX><<<grid_for(p.batch, 128), 128, 0, st>>>(sa));
    return smoother_scan_and_walk();
  }

  // Pathwise sampler: the smoothing elements of the given filtered trajectory
  // (smoother_leaf_kernel), then one backward recursion per (sequence, sample).
  int run_sample() {
    int rc = prepare();
    if (rc) return rc;
    rc = lin(static_cast<const R*>(c.nom_m), static_cast<const R*>(c.nom_L), nullptr, true);
    if (rc) return rc;
    sa.in_m = static_cast<const R*>(c.in_m);
    sa.in_L = static_cast<const R*>(c.in_L);
    SS_LAUNCH("smoother_leaf", st, smoother_leaf_kernel<R, NX, NY><<<grid_for(y.items[1], 128), 128, 0, st>>>(sa));
    SS_LAUNCH("last_state", st, last_state_kernel<R, NX><<<grid_for(p.batch, 128), 128, 0, st>>>(sa));
    const int S = c.n_samples;
    const int64_t n = p.batch * (int64_t)S;
    const R* eps = static_cast<const R*>(c.eps);
    R* out = static_cast<R*>(c.out_m);
    // Few independent walkers on long sequences: the parallel-in-time sampler, with chunks of
    // about sqrt(T) steps (three chains of that length instead of one of T).  Its chunk maps
    // and end states go to the level-1 summary regions of the workspace, which sampling does
    // not otherwise use, and its one-level geometry to the level offsets, which the smoother
    // leaf has finished with (stream order); when they do not fit, the per-walker kernel runs.
    constexpr int64_t SAMPLE_SERIAL_MIN = 16384;
    if (n < SAMPLE_SERIAL_MIN && p.max_len >= 64) {
      const int cs = std::max(16, (int)std::ceil(std::sqrt((double)p.max_len)));
      const int64_t items = (p.total_steps + cs - 1) / cs + p.batch;
      const bool fits = (size_t)(items * S) * (NX * NX + NX) <= (size_t)y.items[1] * Q::FE_P &&
                        (size_t)(items * S) * NX <= (size_t)y.items[1] * Q::ST_P;
      if (fits) {
        Geo gs = geo;
        gs.C = cs;
        gs.L = 1;
        for (int l = 2; l <= MAX_LEVELS; ++l) gs.lvl[l] = nullptr;
        SS_LAUNCH("plan", st, plan_kernel<512><<<1, 512, 0, st>>>(gs, at<int64_t>(y.lvl), (int64_t)y.lvl_stride));
        R* maps = at<R>(y.fsum[1]);
        R* ends = at<R>(y.fst[1]);
        SS_LAUNCH("sample_leaf", st, sample_leaf_kernel<R, NX><<<grid_for(items * S, 128), 128, 0, st>>>(gs, sa.selem, S, eps, maps));
        SS_LAUNCH("sample_top", st, sample_top_kernel<R, NX><<<grid_for(n, 128), 128, 0, st>>>(gs, sa.fT, S, eps, maps, ends, out));
        SS_LAUNCH("sample_walk", st, sample_walk_kernel<R, NX><<<grid_for(items * S, 128), 128, 0, st>>>(gs, sa.selem, S, eps, ends, out));
        return SS_OK;
      }
    }
    SS_LAUNCH("sample", st, sample_kernel<R, NX><<<grid_for(n, 128), 128, 0, st>>>(sa, S, eps, out));
    return SS_OK;
  }

  int run_iterated() {
    int rc = prepare();
    if (rc) return rc;
    const bool tol_mode = c.tol > 0.0;
    int32_t* active = at<int32_t>(y.active);
    int32_t* iters = at<int32_t>(y.iters);
    double* mse = at<double>(y.mse);
    const bool has_init = c.nom_m != nullptr;
    SS_LAUNCH("init_iter", st, init_iter_kernel<<<grid_for(p.batch, 128), 128, 0, st>>>(p.batch, active, iters, mse, c.out_flags, 0));
    const int calls = c.n_iter > 1 ? c.n_iter : 1;
    R* bufm[2] = {at<R>(y.nomA_m), at<R>(y.nomB_m)};
    R* bufL[2] = {at<R>(y.nomA_L), at<R>(y.nomB_L)};
    // Intermediate nominals are packed state records (m, lower L: whole 16-byte
    // pieces, 80 bytes for nx = 5) in the factor buffers; only the caller's
    // initial nominal and the final output use the caller's layout.  The
    // dual-number kernels keep the caller's layout throughout.
    constexpr bool packed = use_staged<R, NX, NY>();
    const R* cur_m = static_cast<const R*>(c.nom_m);
    const R* cur_L = static_cast<const R*>(c.nom_L);
    const R* cur_rec = nullptr;
    int next = 0;
    // pass 0 (init_nominal None): filter-smoother at the default nominal
    const int first = has_init ? 1 : 0;
    for (int k = first; k <= calls; ++k) {
      const bool last = (k == calls);
      const bool counted = (k >= 1);
      R* om = last ? static_cast<R*>(c.out_m) : (packed ? nullptr : bufm[next]);
      R* oL = last ? static_cast<R*>(c.out_L) : (packed ? nullptr : bufL[next]);
      R* orec = (!last && packed) ? bufL[next] : nullptr;
      const int32_t* act = (tol_mode && counted) ? active : nullptr;
      rc = lin(cur_m, cur_L, act, false, cur_rec);
      if (rc) return rc;
      sa.active = act;
      sa.filt_m = nullptr;
      sa.filt_L = nullptr;
      sa.ll_chunk = nullptr;
      rc = filter_pass(true);
      if (rc) return rc;
      sa.out_m = om;
      sa.out_L = oL;
      sa.out_rec = orec;
      sa.prev_m = cur_m;
      sa.prev_L = cur_L;
      sa.prev_rec = cur_rec;
      sa.mse = (tol_mode && counted) ? mse : nullptr;
      sa.flags = last ? c.out_flags : nullptr;
      rc = smoother_scan_and_walk();
      if (rc) return rc;
      if (tol_mode && counted) {
        SS_LAUNCH("converge", st, launch_pdl(converge_kernel, grid_for(p.batch, 128), 128, 0, st, geo, NX, c.tol, mse, active, iters));
      }
      cur_m = om;
      cur_L = oL;
      cur_rec = orec;
      next ^= 1;
    }
    sa.out_rec = nullptr;
    sa.prev_rec = nullptr;
    sa.active = nullptr;
    sa.mse = nullptr;
    sa.flags = nullptr;
    if (c.out_ell) {
      rc = lin(cur_m, cur_L, nullptr, false);
      if (rc) return rc;
      sa.ll_chunk = at<double>(y.ll);
      rc = filter_pass(false);
      if (rc) return rc;
      SS_LAUNCH("ll_reduce", st, ll_reduce_kernel<<<grid_for(p.batch, 128), 128, 0, st>>>(geo, NY, 1 + Tangents<R>::n, at<double>(y.ll), c.out_ell, c.out_grad, c.grad_ld, c.grad_col, c.out_flags));
    }
    if (c.out_iters || (c.out_flags && tol_mode)) {
      if (!tol_mode) {
        SS_LAUNCH("init_iter", st, init_iter_kernel<<<grid_for(p.batch, 128), 128, 0, st>>>(p.batch, active, iters, mse, nullptr, calls));
      }
      SS_LAUNCH("finish_iter", st, finish_iter_kernel<<<grid_for(p.batch, 128), 128, 0, st>>>(p.batch, active, iters, c.out_iters, c.out_flags,
                                                                 tol_mode ? 1 : 0));
    }
    return SS_OK;
  }

  int run_linearize() {
    PointArgs<R> a;
    std::memset(&a, 0, sizeof(a));
    const ss_model& mdl = c.which == 0 ? p.transition : p.observation;
    a.n = c.n_points;
    a.m = static_cast<const R*>(c.pt_m);
    a.L = static_cast<const R*>(c.pt_L);
    a.model = model_args<R>(mdl);
    a.q_m = static_cast<const R*>(mdl.noise_mean);
    a.q_L = static_cast<const R*>(mdl.noise_chol);
    int rc = fill_rule(p, a.rule);
    if (rc) return rc;
    a.slr_form = slr_form_of(p, sizeof(typename Tangents<R>::scalar) == 4);
    a.F = static_cast<R*>(c.pt_F);
    a.chol = static_cast<R*>(c.pt_chol);
    a.b = static_cast<R*>(c.pt_b);
    if (a.n == 0) return SS_OK;
    if (c.which == 0) {
      if (mdl.kind == SS_MODEL_LINEAR) return launch_points_method<R, NX, NX, LinearFn<R, NX, NX>>(a, p.lin_method, st);
      if constexpr (ct_ok<NX>()) {
        if (mdl.kind == SS_MODEL_COORDINATED_TURN)
          return launch_points_method<R, NX, NX, CoordinatedTurnFn<R, NX, NX>>(a, p.lin_method, st);
      }
      if (mdl.kind == SS_MODEL_RICKER) return launch_points_method<R, NX, NX, RickerFn<R, NX, NX>>(a, p.lin_method, st);
    } else {
      if (mdl.kind == SS_MODEL_LINEAR) return launch_points_method<R, NX, NY, LinearFn<R, NX, NY>>(a, p.lin_method, st);
      if constexpr (bearings_ok<NX, NY>()) {
        if (mdl.kind == SS_MODEL_BEARINGS)
          return launch_points_method<R, NX, NY, BearingsFn<R, NX, NY>>(a, p.lin_method, st);
      }
      if constexpr (poisson_ok<NX, NY>()) {
        if (mdl.kind == SS_MODEL_POISSON_EXP)
          return launch_points_method<R, NX, NY, PoissonExpFn<R, NX, NY>>(a, p.lin_method, st);
      }
    }
    return SS_ERR_UNSUPPORTED;
  }
};

// Covariance-form calls (ss_problem.options & SS_OPT_COVARIANCE_FORM): defined in
// ss_std_run.cuh and instantiated in their own translation units (inst_std_*.cu),
// which keeps the parallel build's longest unit short.
template <typename R, int NX, int NY>
int run_std(const Call& c);

template <typename R, int NX, int NY>
int run(const Call& c) {
  if (c.op == OP_SUPPORTED)
    return models_supported<R, NX, NY>(c.p->transition.kind, c.p->observation.kind) ? SS_OK : SS_ERR_UNSUPPORTED;
  if (!models_supported<R, NX, NY>(c.p->transition.kind, c.p->observation.kind)) return SS_ERR_UNSUPPORTED;
  if (c.p->options & SS_OPT_COVARIANCE_FORM) {
    if constexpr (Tangents<R>::n == 0 && NX <= SS_MAX_NX && NY <= SS_MAX_NY) return run_std<R, NX, NY>(c);
    else return SS_ERR_UNSUPPORTED;
  }
  if (c.op == OP_WORKSPACE) {
    Layout y;
    const int rc = make_layout<R, NX, NY>(*c.p, y);
    if (rc) return rc;
    *c.ws_bytes_out = y.bytes;
    return SS_OK;
  }
  Runner<R, NX, NY> r(c);
  switch (c.op) {
    case OP_LINEARIZE: return r.run_linearize();
    case OP_FILTER: return r.run_filter();
    case OP_SMOOTH: return r.run_smooth();
    case OP_ITERATED: return r.run_iterated();
    case OP_SAMPLE:
      if constexpr (Tangents<R>::n == 0) return r.run_sample();
      else return SS_ERR_UNSUPPORTED;
    default: return SS_ERR_INVALID;
  }
}

}  // namespace ss

#define SS_INST(R, TAG, NX, NY) \
  namespace ss {                \
  int run_##TAG##_##NX##_##NY(const Call& c) { return run<R, NX, NY>(c); } \
  }
