// Host orchestration of the covariance-form filter, smoother and iterated
// smoother (kernels in ss_std.cuh) for a compile-time (R, NX, NY).  It shares
// the square-root Runner's geometry, launch helpers and finishing kernels
// (ss_run.cuh) and is compiled in its own units (inst_std_*.cu).  Every factor
// argument of the call (prior, nominal, model noises, trajectories) is a
// covariance here.
#pragma once
#include "ss_run.cuh"
#include "ss_std.cuh"

namespace ss {

// The square-root layout's geometry with covariance-form record sizes.
template <typename R, int NX, int NY>
inline int make_std_layout(const ss_problem& p, Layout& y) {
  typedef SRec<R, NX, NY> Q;
  int rc = make_layout<R, NX, NY>(p, y);   // geometry (chunk, group, levels, items)
  if (rc) return rc;
  const int64_t B = p.batch, N = p.total_steps;
  size_t o = 0;
  auto take = [&](size_t bytes) { size_t r = o; o = align_up(o + bytes); return r; };
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
  y.ll = take(sizeof(double) * (size_t)y.items[1]);
  y.mse = take(sizeof(double) * (size_t)B);
  y.active = take(sizeof(int32_t) * (size_t)B);
  y.iters = take(sizeof(int32_t) * (size_t)B);
  const size_t S = (size_t)(N + B);
  y.nomA_m = take(sizeof(R) * S * NX);
  y.nomA_L = take(sizeof(R) * S * NX * NX);
  y.nomB_m = take(sizeof(R) * S * NX);
  y.nomB_L = take(sizeof(R) * S * NX * NX);
  y.bytes = o;
  return SS_OK;
}

template <typename R, int NX, int NY, class TF, class OF>
inline int launch_std_lin_pair(const LinArgs<R>& a, cudaStream_t st) {
  SS_LAUNCH("std_lin", st, std_lin_kernel<R, NX, NY, TF, OF><<<grid_for(a.total, 128), 128, 0, st>>>(a));
  return SS_OK;
}

template <typename R, int NX, int NY, class TF>
inline int launch_std_lin_obs(const LinArgs<R>& a, int ok, cudaStream_t st) {
  if (ok == SS_MODEL_LINEAR) return launch_std_lin_pair<R, NX, NY, TF, LinearFn<R, NX, NY>>(a, st);
  if constexpr (bearings_ok<NX, NY>()) {
    if (ok == SS_MODEL_BEARINGS) return launch_std_lin_pair<R, NX, NY, TF, BearingsFn<R, NX, NY>>(a, st);
  }
  if constexpr (poisson_ok<NX, NY>()) {
    if (ok == SS_MODEL_POISSON_EXP) return launch_std_lin_pair<R, NX, NY, TF, PoissonExpFn<R, NX, NY>>(a, st);
  }
  return SS_ERR_UNSUPPORTED;
}

template <typename R, int NX, int NY>
inline int launch_std_lin(const LinArgs<R>& a, int tk, int ok, cudaStream_t st) {
  if (a.total == 0) return SS_OK;
  if (tk == SS_MODEL_LINEAR) return launch_std_lin_obs<R, NX, NY, LinearFn<R, NX, NX>>(a, ok, st);
  if constexpr (ct_ok<NX>()) {
    if (tk == SS_MODEL_COORDINATED_TURN) return launch_std_lin_obs<R, NX, NY, CoordinatedTurnFn<R, NX, NX>>(a, ok, st);
  }
  if (tk == SS_MODEL_RICKER) return launch_std_lin_obs<R, NX, NY, RickerFn<R, NX, NX>>(a, ok, st);
  return SS_ERR_UNSUPPORTED;
}

template <typename R, int NX, int NY>
struct StdRunner {
  const Call& c;
  const ss_problem& p;
  Layout y;
  char* ws;
  cudaStream_t st;
  Geo geo;
  ScanArgs<R> sa;
  LinArgs<R> la;

  explicit StdRunner(const Call& call) : c(call), p(*call.p), ws(static_cast<char*>(call.ws)), st(call.stream) {}

  template <typename T>
  T* at(size_t off) const { return reinterpret_cast<T*>(ws + off); }

  int prepare() {
    int rc = make_std_layout<R, NX, NY>(p, y);
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
    la.tq_m = static_cast<const R*>(p.transition.noise_mean);
    la.tq_L = static_cast<const R*>(p.transition.noise_chol);
    la.oq_m = static_cast<const R*>(p.observation.noise_mean);
    la.oq_L = static_cast<const R*>(p.observation.noise_chol);
    rc = fill_rule(p, la.rule);
    if (rc) return rc;
    la.out = at<R>(y.lin);
    return SS_OK;
  }

  int lin(const R* nm, const R* nP, const int32_t* active, bool trans_only) {
    la.nom_m = nm;
    la.nom_L = nP;
    la.nom_rec = nullptr;
    la.active = active;
    la.trans_only = trans_only ? 1 : 0;
    return launch_std_lin<R, NX, NY>(la, p.transition.kind, trans_only ? SS_MODEL_LINEAR : p.observation.kind, st);
  }

  int filter_pass(bool emit_smoother) {
    const unsigned g1 = grid_for(y.items[1], 128);
    SS_LAUNCH("std_filter_leaf", st, std_filter_leaf_kernel<R, NX, NY><<<g1, 128, 0, st>>>(sa));
    for (int l = 1; l < y.L; ++l) {
      SS_LAUNCH("std_filter_up", st, std_filter_up_kernel<R, NX><<<grid_for(y.items[l + 1], LEVEL_BLOCK), LEVEL_BLOCK, 0, st>>>(sa, l));
    }
    SS_LAUNCH("std_filter_top", st, std_filter_top_kernel<R, NX><<<grid_for(p.batch, LEVEL_BLOCK), LEVEL_BLOCK, 0, st>>>(sa));
    for (int l = y.L - 1; l >= 1; --l) {
      SS_LAUNCH("std_filter_down", st, std_filter_down_kernel<R, NX><<<grid_for(y.items[l + 1], LEVEL_BLOCK), LEVEL_BLOCK, 0, st>>>(sa, l));
    }
    sa.emit_smoother = emit_smoother ? 1 : 0;
    SS_LAUNCH("std_filter_walk", st, std_filter_walk_kernel<R, NX, NY><<<g1, 128, 0, st>>>(sa));
    return SS_OK;
  }

  int smoother_scan_and_walk() {
    for (int l = 1; l < y.L; ++l) {
      SS_LAUNCH("std_smoother_up", st, std_smoother_up_kernel<R, NX><<<grid_for(y.items[l + 1], LEVEL_BLOCK), LEVEL_BLOCK, 0, st>>>(sa, l));
    }
    SS_LAUNCH("std_smoother_top", st, std_smoother_top_kernel<R, NX><<<grid_for(p.batch, LEVEL_BLOCK), LEVEL_BLOCK, 0, st>>>(sa));
    for (int l = y.L - 1; l >= 1; --l) {
      SS_LAUNCH("std_smoother_down", st, std_smoother_down_kernel<R, NX><<<grid_for(y.items[l + 1], LEVEL_BLOCK), LEVEL_BLOCK, 0, st>>>(sa, l));
    }
    SS_LAUNCH("std_smoother_walk", st, std_smoother_walk_kernel<R, NX><<<grid_for(y.items[1], 128), 128, 0, st>>>(sa));
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
      SS_LAUNCH("ll_reduce", st, ll_reduce_kernel<<<grid_for(p.batch, 128), 128, 0, st>>>(geo, NY, 1, at<double>(y.ll), c.out_ell, nullptr, 0, 0, nullptr));
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
    SS_LAUNCH("std_smoother_leaf", st, std_smoother_leaf_kernel<R, NX, NY><<<grid_for(y.items[1], 128), 128, 0, st>>>(sa));
    SS_LAUNCH("std_last_state", st, std_last_state_kernel<R, NX><<<grid_for(p.batch, 128), 128, 0, st>>>(sa));
    return smoother_scan_and_walk();
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
    R* bufP[2] = {at<R>(y.nomA_L), at<R>(y.nomB_L)};
    const R* cur_m = static_cast<const R*>(c.nom_m);
    const R* cur_P = static_cast<const R*>(c.nom_L);
    int next = 0;
    const int first = has_init ? 1 : 0;
    for (int k = first; k <= calls; ++k) {
      const bool last = (k == calls);
      const bool counted = (k >= 1);
      R* om = last ? static_cast<R*>(c.out_m) : bufm[next];
      R* oP = last ? static_cast<R*>(c.out_L) : bufP[next];
      const int32_t* act = (tol_mode && counted) ? active : nullptr;
      rc = lin(cur_m, cur_P, act, false);
      if (rc) return rc;
      sa.active = act;
      sa.filt_m = nullptr;
      sa.filt_L = nullptr;
      sa.ll_chunk = nullptr;
      rc = filter_pass(true);
      if (rc) return rc;
      sa.out_m = om;
      sa.out_L = oP;
      sa.out_rec = nullptr;
      // a sequence stopped by the tolerance test keeps its previous trajectory (every
      // sequence is active in the uncounted first pass at the default nominal)
      sa.prev_m = cur_m;
      sa.prev_L = cur_P;
      sa.prev_rec = nullptr;
      sa.mse = (tol_mode && counted) ? mse : nullptr;
      sa.flags = last ? c.out_flags : nullptr;
      rc = smoother_scan_and_walk();
      if (rc) return rc;
      if (tol_mode && counted) {
        SS_LAUNCH("converge", st, converge_kernel<<<grid_for(p.batch, 128), 128, 0, st>>>(geo, NX, c.tol, mse, active, iters));
      }
      cur_m = om;
      cur_P = oP;
      next ^= 1;
    }
    sa.active = nullptr;
    sa.mse = nullptr;
    sa.flags = nullptr;
    if (c.out_ell) {
      rc = lin(cur_m, cur_P, nullptr, false);
      if (rc) return rc;
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
    a.F = static_cast<R*>(c.pt_F);
    a.chol = static_cast<R*>(c.pt_chol);
    a.b = static_cast<R*>(c.pt_b);
    if (a.n == 0) return SS_OK;
    const unsigned grid = grid_for(a.n, 128);
    if (c.which == 0) {
      if (mdl.kind == SS_MODEL_LINEAR) {
        SS_LAUNCH("std_lin_points", st, std_lin_points_kernel<R, NX, NX, LinearFn<R, NX, NX>><<<grid, 128, 0, st>>>(a));
        return SS_OK;
      }
      if constexpr (ct_ok<NX>()) {
        if (mdl.kind == SS_MODEL_COORDINATED_TURN) {
          SS_LAUNCH("std_lin_points", st, std_lin_points_kernel<R, NX, NX, CoordinatedTurnFn<R, NX, NX>><<<grid, 128, 0, st>>>(a));
          return SS_OK;
        }
      }
      if (mdl.kind == SS_MODEL_RICKER) {
        SS_LAUNCH("std_lin_points", st, std_lin_points_kernel<R, NX, NX, RickerFn<R, NX, NX>><<<grid, 128, 0, st>>>(a));
        return SS_OK;
      }
    } else {
      if (mdl.kind == SS_MODEL_LINEAR) {
        SS_LAUNCH("std_lin_points", st, std_lin_points_kernel<R, NX, NY, LinearFn<R, NX, NY>><<<grid, 128, 0, st>>>(a));
        return SS_OK;
      }
      if constexpr (bearings_ok<NX, NY>()) {
        if (mdl.kind == SS_MODEL_BEARINGS) {
          SS_LAUNCH("std_lin_points", st, std_lin_points_kernel<R, NX, NY, BearingsFn<R, NX, NY>><<<grid, 128, 0, st>>>(a));
          return SS_OK;
        }
      }
      if constexpr (poisson_ok<NX, NY>()) {
        if (mdl.kind == SS_MODEL_POISSON_EXP) {
          SS_LAUNCH("std_lin_points", st, std_lin_points_kernel<R, NX, NY, PoissonExpFn<R, NX, NY>><<<grid, 128, 0, st>>>(a));
          return SS_OK;
        }
      }
    }
    return SS_ERR_UNSUPPORTED;
  }
};

// Covariance-form calls (ss_problem.options & SS_OPT_COVARIANCE_FORM).
template <typename R, int NX, int NY>
int run_std(const Call& c) {
  if (c.op == OP_WORKSPACE) {
    Layout y;
    const int rc = make_std_layout<R, NX, NY>(*c.p, y);
    if (rc) return rc;
    *c.ws_bytes_out = y.bytes;
    return SS_OK;
  }
  StdRunner<R, NX, NY> r(c);
  switch (c.op) {
    case OP_LINEARIZE: return r.run_linearize();
    case OP_FILTER: return r.run_filter();
    case OP_SMOOTH: return r.run_smooth();
    case OP_ITERATED: return r.run_iterated();
    default: return SS_ERR_UNSUPPORTED;
  }
}

}  // namespace ss

// Explicit instantiation of the covariance-form entry for one (dtype, nx, ny).
#define SS_INST_STD(R, NX, NY) template int ss::run_std<R, NX, NY>(const ss::Call& c);
