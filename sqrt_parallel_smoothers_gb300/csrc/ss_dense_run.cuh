// Host orchestration of the large-state path (per-sequence and shared-covariance modes).
#pragma once
#include "ss_dense_shared.cuh"

namespace ss {
namespace dense {

// ----------------------------------------------------------------------------- host

struct DLayout {
  int C, G, L;
  int64_t items[MAX_LEVELS + 1];
  size_t lvl, lvl_stride, tab, selem, fT, ll, mse, active, iters, nomA_m, nomA_L, nomB_m, nomB_L;
  size_t fsum[MAX_LEVELS + 1], fst[MAX_LEVELS + 1], ssum[MAX_LEVELS + 1], sst[MAX_LEVELS + 1];
  size_t bytes;
};

template <typename R, int NX, int NY>
inline int make_dlayout(const ss_problem& p, DLayout& y) {
  typedef DS<R, NX, NY> S;
  const int64_t B = p.batch, N = p.total_steps;
  y.C = p.chunk > 0 ? p.chunk : 32;
  y.G = p.group > 1 ? p.group : 8;
  if (y.C > 4096) return SS_ERR_INVALID;
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
  y.tab = take(sizeof(R) * S::table_elems(y.C));
  y.selem = take(sizeof(R) * S::SE * (size_t)N);
  for (int l = 1; l <= y.L; ++l) {
    y.fsum[l] = take(sizeof(R) * S::FE * (size_t)y.items[l]);
    y.fst[l] = take(sizeof(R) * S::ST * (size_t)y.items[l]);
    y.ssum[l] = take(sizeof(R) * S::SE * (size_t)y.items[l]);
    y.sst[l] = take(sizeof(R) * S::ST * (size_t)y.items[l]);
  }
  y.fT = take(sizeof(R) * S::ST * (size_t)B);
  y.ll = take(sizeof(double) * (size_t)y.items[1]);
  y.mse = take(sizeof(double) * (size_t)B);
  y.active = take(sizeof(int32_t) * (size_t)B);
  y.iters = take(sizeof(int32_t) * (size_t)B);
  const size_t St = (size_t)(N + B);
  y.nomA_m = take(sizeof(R) * St * NX);
  y.nomA_L = take(sizeof(R) * St * NX * NX);
  y.nomB_m = take(sizeof(R) * St * NX);
  y.nomB_L = take(sizeof(R) * St * NX * NX);
  y.bytes = o;
  return SS_OK;
}

inline bool aligned16(const void* p) { return p == nullptr || (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

template <typename Kern>
inline void set_smem(Kern k, size_t bytes) {
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <typename R, int NX, int NY>
struct DRunner {
  typedef DS<R, NX, NY> S;
  const Call& c;
  const ss_problem& p;
  DLayout y;
  char* ws;
  cudaStream_t st;
  Geo geo;
  DenseArgs<R> a;
  bool shared = false;          // shared-covariance mode (ss_dense_shared.cuh)
  int64_t T = 0;                // sequence length in shared mode
  int64_t nl[MAX_LEVELS + 2];   // items per sequence at each level in shared mode

  explicit DRunner(const Call& call) : c(call), p(*call.p), ws(static_cast<char*>(call.ws)), st(call.stream) {}

  template <typename T>
  T* at(size_t off) const { return reinterpret_cast<T*>(ws + off); }

  int prepare() {
    int rc = make_dlayout<R, NX, NY>(p, y);
    if (rc) return rc;
    if (c.ws_bytes < y.bytes || ws == nullptr) return SS_ERR_WORKSPACE;
    if (!aligned16(c.out_m) || !aligned16(c.out_L) || !aligned16(c.in_m) || !aligned16(c.in_L) ||
        !aligned16(c.nom_m) || !aligned16(c.nom_L) || !aligned16(ws))
      return SS_ERR_INVALID;
    geo.off = p.offsets;
    geo.B = p.batch;
    geo.C = y.C;
    geo.G = y.G;
    geo.L = y.L;
    for (int l = 0; l <= MAX_LEVELS; ++l) geo.lvl[l] = nullptr;
    for (int l = 1; l <= y.L; ++l) geo.lvl[l] = at<int64_t>(y.lvl) + (size_t)(l - 1) * y.lvl_stride;
    SS_LAUNCH("plan", st, plan_kernel<512><<<1, 512, 0, st>>>(geo, at<int64_t>(y.lvl), (int64_t)y.lvl_stride));
    std::memset(&a, 0, sizeof(a));
    ScanArgs<R>& sa = a.s;
    sa.g = geo;
    sa.ys = static_cast<const R*>(c.ys);
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
    a.F = static_cast<const R*>(p.transition.matrix);
    a.qm = static_cast<const R*>(p.transition.noise_mean);
    a.qc = static_cast<const R*>(p.transition.noise_chol);
    a.H = static_cast<const R*>(p.observation.matrix);
    a.rm = static_cast<const R*>(p.observation.noise_mean);
    a.rc = static_cast<const R*>(p.observation.noise_chol);
    a.tab = at<R>(y.tab);
    a.C = y.C;
    // equal lengths <=> sum T_i = B max T_i; a shared prior; at most 32 sequences (one per lane)
    shared = !(p.options & SS_OPT_PER_SEQUENCE_COVARIANCE) && !c.prior_per_sequence && p.batch >= 2 &&
             p.batch <= SB_ROWS && p.max_len >= 1 && p.total_steps == p.batch * p.max_len;
    if (shared) {
      T = p.max_len;
      nl[1] = (T + y.C - 1) / y.C;
      for (int l = 2; l <= y.L; ++l) nl[l] = (nl[l - 1] + y.G - 1) / y.G;
    }
    return SS_OK;
  }

  int setup() {
    const size_t sm = sizeof(R) * setup_elems<R, NX, NY>();
    set_smem(setup_kernel<R, NX, NY>, sm);
    SS_LAUNCH("dense_setup", st, setup_kernel<R, NX, NY><<<1, 32, sm, st>>>(a));
    return SS_OK;
  }

  int filter_pass_shared(bool emit_smoother) {
    const int B = (int)p.batch;
    const int32_t* act = a.s.active;
    a.s.active = nullptr;  // a linear model's passes do not depend on the nominal: compute every sequence
    {
      const size_t sm = sizeof(R) * leaf_elems<R, NX, NY>();
      set_smem(leaf_kernel<R, NX, NY>, sm);
      SS_LAUNCH("filter_leaf", st, leaf_kernel<R, NX, NY><<<grid_for(y.items[1], LEAF_WARPS), 32 * LEAF_WARPS, sm, st>>>(a));
    }
    const size_t sm_up = sizeof(R) * up_b_elems<R, NX, NY>();
    const size_t sm_ap = sizeof(R) * apply_b_elems<R, NX, NY>();
    set_smem(up_b_kernel<R, NX, NY>, sm_up);
    set_smem(top_b_kernel<R, NX, NY>, sm_ap);
    set_smem(down_b_kernel<R, NX, NY>, sm_ap);
    for (int l = 1; l < y.L; ++l) {
      SS_LAUNCH("filter_up", st, up_b_kernel<R, NX, NY><<<(unsigned)nl[l + 1], 32, sm_up, st>>>(a, l, B, nl[l], nl[l + 1]));
    }
    SS_LAUNCH("filter_top", st, top_b_kernel<R, NX, NY><<<1, 32, sm_ap, st>>>(a, B, nl[y.L], T));
    for (int l = y.L - 1; l >= 1; --l) {
      SS_LAUNCH("filter_down", st, down_b_kernel<R, NX, NY><<<(unsigned)nl[l + 1], 32, sm_ap, st>>>(a, l, B, nl[l], nl[l + 1]));
    }
    a.s.emit_smoother = emit_smoother ? 1 : 0;
    constexpr int WW = walk_b_warps<R, NX, NY>();
    const size_t sm_w = sizeof(R) * walk_b_elems<R, NX, NY>();
    set_smem(walk_b_kernel<R, NX, NY>, sm_w);
    SS_LAUNCH("filter_walk", st, walk_b_kernel<R, NX, NY><<<grid_for(nl[1], WW), 32 * WW, sm_w, st>>>(a, B, nl[1], T));
    a.s.active = act;
    return SS_OK;
  }

  int smoother_pass_shared() {
    const int B = (int)p.batch;
    const size_t sm_f = sizeof(R) * SFOLD_WARPS * sfold_b_warp_elems<R, NX, NY>();
    set_smem(sfold_b_kernel<R, NX, NY>, sm_f);
    SS_LAUNCH("smoother_leaf", st, sfold_b_kernel<R, NX, NY><<<grid_for(nl[1], SFOLD_WARPS), 32 * SFOLD_WARPS, sm_f, st>>>(a, 0, B, T, nl[1], T));
    for (int l = 1; l < y.L; ++l) {
      SS_LAUNCH("smoother_up", st, sfold_b_kernel<R, NX, NY><<<grid_for(nl[l + 1], SFOLD_WARPS), 32 * SFOLD_WARPS, sm_f, st>>>(a, l, B, nl[l], nl[l + 1], T));
    }
    const size_t sm_a = sizeof(R) * sapply_b_warp_elems<R, NX, NY>();
    set_smem(stop_b_kernel<R, NX, NY>, sm_a);
    set_smem(sdown_b_kernel<R, NX, NY>, sm_a);
    SS_LAUNCH("smoother_top", st, stop_b_kernel<R, NX, NY><<<1, 32, sm_a, st>>>(a, B, nl[y.L], T));
    for (int l = y.L - 1; l >= 1; --l) {
      SS_LAUNCH("smoother_down", st, sdown_b_kernel<R, NX, NY><<<(unsigned)nl[l + 1], 32, sm_a, st>>>(a, l, B, nl[l], nl[l + 1]));
    }
    constexpr int SW = swalk_b_warps<R, NX, NY>();
    const size_t sm_w = sizeof(R) * SW * sapply_b_warp_elems<R, NX, NY>();
    set_smem(swalk_b_kernel<R, NX, NY>, sm_w);
    SS_LAUNCH("smoother_walk", st, swalk_b_kernel<R, NX, NY><<<grid_for(nl[1], SW), 32 * SW, sm_w, st>>>(a, B, nl[1], T));
    return SS_OK;
  }

  int filter_pass(bool emit_smoother) {
    if (shared) return filter_pass_shared(emit_smoother);
    {
      const size_t sm = sizeof(R) * leaf_elems<R, NX, NY>();
      set_smem(leaf_kernel<R, NX, NY>, sm);
      SS_LAUNCH("filter_leaf", st, leaf_kernel<R, NX, NY><<<grid_for(y.items[1], LEAF_WARPS), 32 * LEAF_WARPS, sm, st>>>(a));
    }
    const size_t sm_up = sizeof(R) * up_elems<R, NX, NY>();
    const size_t sm_ap = sizeof(R) * apply_elems<R, NX, NY>();
    set_smem(up_kernel<R, NX, NY>, sm_up);
    set_smem(top_kernel<R, NX, NY>, sm_ap);
    set_smem(down_kernel<R, NX, NY>, sm_ap);
    for (int l = 1; l < y.L; ++l) {
      SS_LAUNCH("filter_up", st, up_kernel<R, NX, NY><<<(unsigned)y.items[l + 1], 32, sm_up, st>>>(a, l));
    }
    SS_LAUNCH("filter_top", st, top_kernel<R, NX, NY><<<(unsigned)p.batch, 32, sm_ap, st>>>(a));
    for (int l = y.L - 1; l >= 1; --l) {
      SS_LAUNCH("filter_down", st, down_kernel<R, NX, NY><<<(unsigned)y.items[l + 1], 32, sm_ap, st>>>(a, l));
    }
    a.s.emit_smoother = emit_smoother ? 1 : 0;
    if constexpr (std::is_same<R, float>::value) {
      const size_t sm_r = sizeof(R) * walk_r_elems<R, NX, NY>();
      set_smem(walk_r_kernel<R, NX, NY>, sm_r);
      SS_LAUNCH("filter_walk", st,
                walk_r_kernel<R, NX, NY><<<grid_for(y.items[1], WALK_R_WARPS), 32 * WALK_R_WARPS, sm_r, st>>>(a));
    } else {
      constexpr int WW = walk_warps<R, NX, NY>();
      const size_t sm_w = sizeof(R) * walk_elems<R, NX, NY>();
      set_smem(walk_kernel<R, NX, NY>, sm_w);
      SS_LAUNCH("filter_walk", st, walk_kernel<R, NX, NY><<<grid_for(y.items[1], WW), 32 * WW, sm_w, st>>>(a));
    }
    return SS_OK;
  }

  int smoother_pass() {
    if (shared) return smoother_pass_shared();
    const size_t sm_f = sizeof(R) * SFOLD_WARPS * sfold_warp_elems<R, NX, NY>();
    set_smem(sleaf_kernel<R, NX, NY>, sm_f);
    set_smem(sup_kernel<R, NX, NY>, sm_f);
    SS_LAUNCH("smoother_leaf", st, sleaf_kernel<R, NX, NY><<<grid_for(y.items[1], SFOLD_WARPS), 32 * SFOLD_WARPS, sm_f, st>>>(a));
    for (int l = 1; l < y.L; ++l) {
      SS_LAUNCH("smoother_up", st, sup_kernel<R, NX, NY><<<grid_for(y.items[l + 1], SFOLD_WARPS), 32 * SFOLD_WARPS, sm_f, st>>>(a, l));
    }
    const size_t sm_a = sizeof(R) * sapply_warp_elems<R, NX, NY>();
    set_smem(stop_kernel<R, NX, NY>, sm_a);
    set_smem(sdown_kernel<R, NX, NY>, sm_a);
    SS_LAUNCH("smoother_top", st, stop_kernel<R, NX, NY><<<(unsigned)p.batch, 32, sm_a, st>>>(a));
    for (int l = y.L - 1; l >= 1; --l) {
      SS_LAUNCH("smoother_down", st, sdown_kernel<R, NX, NY><<<(unsigned)y.items[l + 1], 32, sm_a, st>>>(a, l));
    }
    const size_t sm_w = sizeof(R) * SWALK_WARPS * sapply_warp_elems<R, NX, NY>();
    set_smem(swalk_kernel<R, NX, NY>, sm_w);
    SS_LAUNCH("smoother_walk", st, swalk_kernel<R, NX, NY><<<grid_for(y.items[1], SWALK_WARPS), 32 * SWALK_WARPS, sm_w, st>>>(a));
    return SS_OK;
  }

  int run_filter() {
    int rc = prepare();
    if (rc) return rc;
    rc = setup();
    if (rc) return rc;
    a.s.filt_m = static_cast<R*>(c.out_m);
    a.s.filt_L = static_cast<R*>(c.out_L);
    a.s.ll_chunk = c.out_ell ? at<double>(y.ll) : nullptr;
    rc = filter_pass(false);
    if (rc) return rc;
    if (c.out_ell) {
      SS_LAUNCH("ll_reduce", st, ll_reduce_kernel<<<grid_for(p.batch, 128), 128, 0, st>>>(geo, NY, 1, at<double>(y.ll), c.out_ell, nullptr, 0, 0, nullptr));
    }
    return SS_OK;
  }

  int run_smooth() {
    int rc = prepare();
    if (rc) return rc;
    shared = false;
    a.s.in_m = static_cast<const R*>(c.in_m);
    a.s.in_L = static_cast<const R*>(c.in_L);
    a.s.out_m = static_cast<R*>(c.out_m);
    a.s.out_L = static_cast<R*>(c.out_L);
    const size_t sm = sizeof(R) * (mc_elems<R, NX, NY>() + SELEM_WARPS * selem_warp_elems<R, NX, NY>());
    set_smem(selem_kernel<R, NX, NY>, sm);
    SS_LAUNCH("smoother_elements", st, selem_kernel<R, NX, NY><<<grid_for(y.items[1], SELEM_WARPS), 32 * SELEM_WARPS, sm, st>>>(a));
    SS_LAUNCH("last_state", st, last_state_kernel<R, NX, NY><<<(unsigned)p.batch, 32, 0, st>>>(a));
    return smoother_pass();
  }

  int run_iterated() {
    int rc = prepare();
    if (rc) return rc;
    rc = setup();
    if (rc) return rc;
    ScanArgs<R>& sa = a.s;
    const bool tol_mode = c.tol > 0.0;
    int32_t* active = at<int32_t>(y.active);
    int32_t* iters = at<int32_t>(y.iters);
    double* mse = at<double>(y.mse);
    const bool has_init = c.nom_m != nullptr;
    SS_LAUNCH("init_iter", st, init_iter_kernel<<<grid_for(p.batch, 128), 128, 0, st>>>(p.batch, active, iters, mse, c.out_flags, 0));
    const int calls = c.n_iter > 1 ? c.n_iter : 1;
    R* bufm[2] = {at<R>(y.nomA_m), at<R>(y.nomB_m)};
    R* bufL[2] = {at<R>(y.nomA_L), at<R>(y.nomB_L)};
    const R* cur_m = static_cast<const R*>(c.nom_m);
    const R* cur_L = static_cast<const R*>(c.nom_L);
    int next = 0;
    const int first = has_init ? 1 : 0;
    for (int k = first; k <= calls; ++k) {
      const bool last = (k == calls);
      const bool counted = (k >= 1);
      R* om = last ? static_cast<R*>(c.out_m) : bufm[next];
      R* oL = last ? static_cast<R*>(c.out_L) : bufL[next];
      const int32_t* act = (tol_mode && counted) ? active : nullptr;
      sa.active = act;
      sa.filt_m = nullptr;
      sa.filt_L = nullptr;
      sa.ll_chunk = nullptr;
      rc = filter_pass(true);
      if (rc) return rc;
      sa.out_m = om;
      sa.out_L = oL;
      sa.prev_m = cur_m;
      sa.prev_L = cur_L;
      // the first pass of a run without an initial trajectory has no previous iterate
      sa.mse = (tol_mode && counted && cur_m != nullptr) ? mse : nullptr;
      sa.flags = last ? c.out_flags : nullptr;
      rc = smoother_pass();
      if (rc) return rc;
      if (tol_mode && counted) {
        SS_LAUNCH("converge", st, converge_kernel<<<grid_for(p.batch, 128), 128, 0, st>>>(geo, NX, c.tol, mse, active, iters));
      }
      cur_m = om;
      cur_L = oL;
      next ^= 1;
    }
    sa.active = nullptr;
    sa.mse = nullptr;
    sa.flags = nullptr;
    if (c.out_ell) {
      sa.ll_chunk = at<double>(y.ll);
      rc = filter_pass(false);
      if (rc) return rc;
      SS_LAUNCH("ll_reduce", st, ll_reduce_kernel<<<grid_for(p.batch, 128), 128, 0, st>>>(geo, NY, 1, at<double>(y.ll), c.out_ell, nullptr, 0, 0, c.out_flags));
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
    const ss_model& mdl = c.which == 0 ? p.transition : p.observation;
    if (c.n_points == 0) return SS_OK;
    const int tria_chol = p.lin_method == SS_LIN_EXTENDED ? 0 : 1;
    const R* A = static_cast<const R*>(mdl.matrix);
    const R* qm = static_cast<const R*>(mdl.noise_mean);
    const R* qc = static_cast<const R*>(mdl.noise_chol);
    R* F = static_cast<R*>(c.pt_F);
    R* ch = static_cast<R*>(c.pt_chol);
    R* b = static_cast<R*>(c.pt_b);
    if (c.which == 0) {
      const size_t sm = sizeof(R) * (NX * Pad<R, NX>::ld + tria_scratch<R, NX>());
      set_smem(lin_points_kernel<R, NX, NX>, sm);
      SS_LAUNCH("lin_points", st, lin_points_kernel<R, NX, NX><<<(unsigned)c.n_points, 32, sm, st>>>(c.n_points, A, qm, qc, tria_chol, F, ch, b));
    } else {
      const size_t sm = sizeof(R) * (NY * Pad<R, NY>::ld + tria_scratch<R, NY>());
      set_smem(lin_points_kernel<R, NX, NY>, sm);
      SS_LAUNCH("lin_points", st, lin_points_kernel<R, NX, NY><<<(unsigned)c.n_points, 32, sm, st>>>(c.n_points, A, qm, qc, tria_chol, F, ch, b));
    }
    return SS_OK;
  }
};

template <typename R, int NX, int NY>
int run(const Call& c) {
  const bool ok = c.p->transition.kind == SS_MODEL_LINEAR && c.p->observation.kind == SS_MODEL_LINEAR;
  if (c.op == OP_SUPPORTED) return ok ? SS_OK : SS_ERR_UNSUPPORTED;
  if (!ok) return SS_ERR_UNSUPPORTED;
  if (c.op == OP_WORKSPACE) {
    DLayout y;
    const int rc = make_dlayout<R, NX, NY>(*c.p, y);
    if (rc) return rc;
    *c.ws_bytes_out = y.bytes;
    return SS_OK;
  }
  DRunner<R, NX, NY> r(c);
  switch (c.op) {
    case OP_LINEARIZE: return r.run_linearize();
    case OP_FILTER: return r.run_filter();
    case OP_SMOOTH: return r.run_smooth();
    case OP_ITERATED: return r.run_iterated();
    case OP_SAMPLE: return SS_ERR_UNSUPPORTED;
    default: return SS_ERR_INVALID;
  }
}

}  // namespace dense
}  // namespace ss

#define SS_INST_DENSE(R, TAG, NX, NY) \
  namespace ss {                      \
  int dense_##TAG##_##NX##_##NY(const Call& c) { return dense::run<R, NX, NY>(c); } \
  }
