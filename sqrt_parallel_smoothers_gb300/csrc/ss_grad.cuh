// Gradient of the filter's log-likelihood by forward-mode (tangent-linear)
// propagation: the whole filter pipeline instantiated on Dual<T, 1>, one
// pass per parameter direction (a wider dual type multiplies the register
// footprint of the square-root combines past what a thread can hold).
//
// The iterated form (OP_ITERATED) runs the whole fixed-point loop of
// parsmooth/methods.py:54-76 in dual numbers, so the tangent of each nominal
// trajectory is carried into the next call's linearisation, and returns the
// derivative of the log-likelihood at the final nominal: the exact derivative
// of the n_iter-call iteration, which tends to the implicit-function
// derivative of the fixed point (parsmooth/_utils.py:113-133) as the
// iteration converges.
#pragma once
#include "ss_run.cuh"

namespace ss {

constexpr int GRAD_NT = 1;

// out[k] = (x[k], dx[0][k], ..., dx[n_dir-1][k]); missing tangents are zero.
template <typename T>
static __global__ void lift_kernel(const T* __restrict__ x, const T* __restrict__ dx, int n_dir, int64_t n,
                                   Dual<T, GRAD_NT>* __restrict__ out) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  Dual<T, GRAD_NT> d;
  d.v = x[k];
  for (int r = 0; r < GRAD_NT; ++r) d.d[r] = (dx != nullptr && r < n_dir) ? dx[(int64_t)r * n + k] : T(0);
  out[k] = d;
}

struct GradLayout {
  Layout inner;
  size_t ys, m0, L0, nm, nL, tmat, omat, tqm, tqL, oqm, oqL, om, oL, inner_base, bytes;
};

template <typename T, int NX, int NY>
inline int make_grad_layout(const ss_problem& p, int64_t n_prior, bool iterated, GradLayout& g) {
  typedef Dual<T, GRAD_NT> D;
  int rc = make_layout<D, NX, NY>(p, g.inner);
  if (rc) return rc;
  size_t o = 0;
  auto take = [&](size_t n) { size_t r = o; o = align_up(o + n * sizeof(D)); return r; };
  const size_t S = (size_t)(p.total_steps + p.batch);
  g.ys = take((size_t)p.total_steps * NY);
  g.m0 = take((size_t)n_prior * NX);
  g.L0 = take((size_t)n_prior * NX * NX);
  g.nm = take(S * NX);
  g.nL = take(S * NX * NX);
  g.tmat = take(NX * NX);
  g.omat = take(NY * NX);
  g.tqm = take(NX);
  g.tqL = take(NX * NX);
  g.oqm = take(NY);
  g.oqL = take(NY * NY);
  g.om = take(iterated ? S * NX : 0);        // the iterated run's final trajectory (unused)
  g.oL = take(iterated ? S * NX * NX : 0);
  g.inner_base = o;
  g.bytes = o + g.inner.bytes;
  return SS_OK;
}

template <typename T>
inline int lift(const void* x, const void* dx, int n_dir, int64_t n, char* dst, cudaStream_t st) {
  if (n == 0) return SS_OK;
  SS_LAUNCH("lift", st, lift_kernel<T><<<grid_for(n, 256), 256, 0, st>>>(static_cast<const T*>(x),
                                                                            static_cast<const T*>(dx), n_dir, n,
                                                                            reinterpret_cast<Dual<T, GRAD_NT>*>(dst)));
  return SS_OK;
}

template <typename T, int NX, int NY>
int run_grad(const Call& c) {
  typedef Dual<T, GRAD_NT> D;
  const ss_problem& p = *c.p;
  if (p.lin_method == SS_LIN_GAUSS_HERMITE) return SS_ERR_UNSUPPORTED;
  if (!models_supported<T, NX, NY>(p.transition.kind, p.observation.kind)) return SS_ERR_UNSUPPORTED;
  const int64_t n_prior = c.prior_per_sequence ? p.batch : 1;
  const bool iterated = c.n_iter > 0;
  GradLayout g;
  int rc = make_grad_layout<T, NX, NY>(p, n_prior, iterated, g);
  if (rc) return rc;
  if (c.op == OP_WORKSPACE) {
    *c.ws_bytes_out = g.bytes;
    return SS_OK;
  }
  if (c.ws == nullptr || c.ws_bytes < g.bytes) return SS_ERR_WORKSPACE;
  const ss_tangents* tg = c.tangents;
  if (tg == nullptr || tg->n_dir < 1 || tg->n_dir > SS_MAX_TANGENTS) return SS_ERR_INVALID;
  char* w = static_cast<char*>(c.ws);
  cudaStream_t st = c.stream;
  const int nd = tg->n_dir;
  const size_t S = (size_t)(p.total_steps + p.batch);
  // inputs that carry no tangent: lifted once
  if ((rc = lift<T>(c.ys, nullptr, 0, p.total_steps * NY, w + g.ys, st))) return rc;
  if ((rc = lift<T>(c.m0, nullptr, 0, n_prior * NX, w + g.m0, st))) return rc;
  if ((rc = lift<T>(c.L0, nullptr, 0, n_prior * NX * NX, w + g.L0, st))) return rc;
  if (c.nom_m != nullptr) {
    if ((rc = lift<T>(c.nom_m, nullptr, 0, (int64_t)S * NX, w + g.nm, st))) return rc;
    if ((rc = lift<T>(c.nom_L, nullptr, 0, (int64_t)S * NX * NX, w + g.nL, st))) return rc;
  }
  auto dir_ptr = [](const void* base, int dir, int64_t n) -> const void* {
    return base == nullptr ? nullptr : static_cast<const T*>(base) + (int64_t)dir * n;
  };
  for (int dir = 0; dir < nd; ++dir) {
    ss_problem p2 = p;
    if (p.transition.kind == SS_MODEL_LINEAR) {
      if ((rc = lift<T>(p.transition.matrix, dir_ptr(tg->trans_matrix, dir, NX * NX), 1, NX * NX, w + g.tmat, st)))
        return rc;
      p2.transition.matrix = w + g.tmat;
    }
    if (p.observation.kind == SS_MODEL_LINEAR) {
      if ((rc = lift<T>(p.observation.matrix, dir_ptr(tg->obs_matrix, dir, NY * NX), 1, NY * NX, w + g.omat, st)))
        return rc;
      p2.observation.matrix = w + g.omat;
    }
    if ((rc = lift<T>(p.transition.noise_mean, dir_ptr(tg->trans_noise_mean, dir, NX), 1, NX, w + g.tqm, st)))
      return rc;
    if ((rc = lift<T>(p.transition.noise_chol, dir_ptr(tg->trans_noise_chol, dir, NX * NX), 1, NX * NX,
                      w + g.tqL, st)))
      return rc;
    if ((rc = lift<T>(p.observation.noise_mean, dir_ptr(tg->obs_noise_mean, dir, NY), 1, NY, w + g.oqm, st)))
      return rc;
    if ((rc = lift<T>(p.observation.noise_chol, dir_ptr(tg->obs_noise_chol, dir, NY * NY), 1, NY * NY,
                      w + g.oqL, st)))
      return rc;
    p2.transition.noise_mean = w + g.tqm;
    p2.transition.noise_chol = w + g.tqL;
    p2.observation.noise_mean = w + g.oqm;
    p2.observation.noise_chol = w + g.oqL;
    ss_tangents one;
    std::memset(&one, 0, sizeof(one));
    one.n_dir = 1;
    for (int k = 0; k < 4; ++k) {
      one.trans_params[0][k] = tg->trans_params[dir][k];
      one.obs_params[0][k] = tg->obs_params[dir][k];
    }
    Call c2 = c;
    c2.op = iterated ? OP_ITERATED : OP_FILTER;
    c2.p = &p2;
    c2.tangents = &one;
    c2.ys = w + g.ys;
    c2.m0 = w + g.m0;
    c2.L0 = w + g.L0;
    c2.nom_m = c.nom_m ? w + g.nm : nullptr;
    c2.nom_L = c.nom_m ? w + g.nL : nullptr;
    c2.out_m = iterated ? w + g.om : nullptr;
    c2.out_L = iterated ? w + g.oL : nullptr;
    c2.tol = 0.0;
    c2.out_iters = nullptr;
    c2.out_flags = nullptr;
    c2.grad_ld = nd;
    c2.grad_col = dir;
    c2.ws = w + g.inner_base;
    c2.ws_bytes = g.inner.bytes;
    Runner<D, NX, NY> r(c2);
    if ((rc = iterated ? r.run_iterated() : r.run_filter())) return rc;
  }
  return SS_OK;
}

}  // namespace ss

#define SS_INST_GRAD(R, TAG, NX, NY) \
  namespace ss {                     \
  int grad_##TAG##_##NX##_##NY(const Call& c) { return run_grad<R, NX, NY>(c); } \
  }
