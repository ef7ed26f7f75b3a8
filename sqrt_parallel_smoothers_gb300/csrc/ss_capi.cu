// C ABI of the library: argument validation and dispatch to the compiled
// (dtype, nx, ny) instantiations.
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <cstdlib>
#include <mutex>
#include <string>
#include <vector>

#include "ss_dims.h"
#include "ss_run.cuh"

namespace ss {

#define SS_DECL(NX, NY)                      \
  int run_f32_##NX##_##NY(const Call& c);    \
  int run_f64_##NX##_##NY(const Call& c);
SS_FOR_DIMS(SS_DECL)
#undef SS_DECL
#define SS_DECL(NX, NY)                      \
  int grad_f32_##NX##_##NY(const Call& c);   \
  int grad_f64_##NX##_##NY(const Call& c);
SS_FOR_GRAD_DIMS(SS_DECL)
#undef SS_DECL
#define SS_DECL(NX, NY)                      \
  int adj_f32_##NX##_##NY(const Call& c);    \
  int adj_f64_##NX##_##NY(const Call& c);
SS_FOR_ADJ_DIMS(SS_DECL)
#undef SS_DECL
#define SS_DECL(NX, NY)                      \
  int dense_f32_##NX##_##NY(const Call& c);  \
  int dense_f64_##NX##_##NY(const Call& c);
SS_FOR_DENSE_DIMS(SS_DECL)
#undef SS_DECL

static RunFn find_grad(int dtype, int nx, int ny) {
#define SS_CASE(NX, NY) \
  if (nx == NX && ny == NY) return dtype == SS_F32 ? grad_f32_##NX##_##NY : grad_f64_##NX##_##NY;
  SS_FOR_GRAD_DIMS(SS_CASE)
#undef SS_CASE
  return nullptr;
}

static RunFn find_adj(int dtype, int nx, int ny) {
#define SS_CASE(NX, NY) \
  if (nx == NX && ny == NY) return dtype == SS_F32 ? adj_f32_##NX##_##NY : adj_f64_##NX##_##NY;
  SS_FOR_ADJ_DIMS(SS_CASE)
#undef SS_CASE
  return nullptr;
}

static RunFn find_run(int dtype, int nx, int ny) {
#define SS_CASE(NX, NY) \
  if (nx == NX && ny == NY) return dtype == SS_F32 ? run_f32_##NX##_##NY : run_f64_##NX##_##NY;
  SS_FOR_DIMS(SS_CASE)
#undef SS_CASE
#define SS_CASE(NX, NY) \
  if (nx == NX && ny == NY) return dtype == SS_F32 ? dense_f32_##NX##_##NY : dense_f64_##NX##_##NY;
  SS_FOR_DENSE_DIMS(SS_CASE)
#undef SS_CASE
  return nullptr;
}

// Physicists' Hermite polynomial H_n(x) by the three-term recurrence
// H_k = 2x H_{k-1} - 2(k-1) H_{k-2} (parsmooth/linearization/_gh.py:129-151
// builds the same coefficients).
static double hermite(int n, double x) {
  if (n == 0) return 1.0;
  double h0 = 1.0, h1 = 2.0 * x;
  for (int k = 2; k <= n; ++k) {
    const double h2 = 2.0 * x * h1 - 2.0 * (k - 1) * h0;
    h0 = h1;
    h1 = h2;
  }
  return h1;
}

// Roots of H_p: they interlace with the roots of H_{p-1}, so each lies in one
// bracket between consecutive roots of H_{p-1} (or the bound sqrt(2p+1));
// bisection in each bracket.
static void hermite_roots(int p, double* roots) {
  double prev[SS_MAX_GH_ORDER + 1];
  prev[0] = 0.0;
  int np = 0;
  for (int k = 1; k <= p; ++k) {
    const double bound = std::sqrt(2.0 * k + 1.0) + 1.0;
    double cur[SS_MAX_GH_ORDER + 1];
    for (int r = 0; r < k; ++r) {
      double lo = (r == 0) ? -bound : prev[r - 1];
      double hi = (r == k - 1) ? bound : prev[r];
      double flo = hermite(k, lo);
      for (int it = 0; it < 200; ++it) {
        const double mid = 0.5 * (lo + hi);
        const double fm = hermite(k, mid);
        if (fm == 0.0) {
          lo = hi = mid;
          break;
        }
        if ((fm < 0) == (flo < 0)) {
          lo = mid;
          flo = fm;
        } else {
          hi = mid;
        }
      }
      cur[r] = 0.5 * (lo + hi);
    }
    for (int r = 0; r < k; ++r) prev[r] = cur[r];
    np = k;
  }
  for (int r = 0; r < np; ++r) roots[r] = prev[r];
}

int fill_rule(const ss_problem& p, RuleArgs& r) {
  std::memset(&r, 0, sizeof(r));
  r.method = p.lin_method;
  const double n = p.nx;
  if (p.lin_method == SS_LIN_UNSCENTED) {
    // parsmooth/linearization/_unscented.py:64-65 (kappa default 3 + n) and :96-100
    const double kappa = p.ut_kappa_default ? 3.0 + n : p.ut_kappa;
    const double lam = p.ut_alpha * p.ut_alpha * (n + kappa) - n;
    if (!(n + lam > 0)) return SS_ERR_INVALID;
    r.ut_d[0] = std::sqrt(n + lam);
    r.ut_d[1] = lam / (n + lam);
    r.ut_d[2] = lam / (n + lam) + (1.0 - p.ut_alpha * p.ut_alpha + p.ut_beta);
    r.ut_d[3] = 1.0 / (2.0 * (n + lam));
    for (int k = 0; k < 4; ++k) r.ut_f[k] = (float)r.ut_d[k];
  } else if (p.lin_method == SS_LIN_GAUSS_HERMITE) {
    const int order = p.gh_order;
    if (order < 1 || order > SS_MAX_GH_ORDER) return SS_ERR_INVALID;
    r.gh_order = order;
    double roots[SS_MAX_GH_ORDER];
    hermite_roots(order, roots);
    double fact = 1.0;
    for (int k = 2; k <= order; ++k) fact *= k;
    const double sqrt_pi = std::sqrt(M_PI);
    for (int k = 0; k < order; ++k) {
      // parsmooth/linearization/_gh.py:106-109, divided by sqrt(pi) per dimension (:120)
      const double hp = hermite(order - 1, roots[k]);
      const double w = std::pow(2.0, order - 1) * fact * sqrt_pi / (order * order * hp * hp);
      r.gh_root_d[k] = std::sqrt(2.0) * roots[k];
      r.gh_w_d[k] = w / sqrt_pi;
      r.gh_root_f[k] = (float)r.gh_root_d[k];
      r.gh_w_f[k] = (float)r.gh_w_d[k];
    }
  }
  return SS_OK;
}

// ----------------------------------------------------------------------------- instrumentation

static std::atomic<long long> g_launches{0};
static std::atomic<bool> g_profiling{false};
static std::mutex g_prof_mu;
struct ProfRec {
  const char* name;
  cudaEvent_t start, stop;
};
static std::vector<ProfRec> g_prof;

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
bool profiling_on() { return g_profiling.load(std::memory_order_relaxed); }
// Programmatic dependent launch of the per-pass kernels: on unless the
// environment sets SQRTSMOOTH_PDL=0 (read once).
bool pdl_on() {
  static const bool on = [] {
    const char* v = std::getenv("SQRTSMOOTH_PDL");
    return !(v != nullptr && v[0] == '0');
  }();
  return on;
}
void profile_push(const char* name, cudaEvent_t start, cudaEvent_t stop) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  g_prof.push_back({name, start, stop});
}

static int validate(const ss_problem* p) {
  if (p == nullptr) return SS_ERR_INVALID;
  if (p->dtype != SS_F32 && p->dtype != SS_F64) return SS_ERR_INVALID;
  if (p->nx < 1 || p->ny < 1) return SS_ERR_INVALID;
  if (p->lin_method < SS_LIN_EXTENDED || p->lin_method > SS_LIN_GAUSS_HERMITE) return SS_ERR_INVALID;
  if (p->lin_method == SS_LIN_GAUSS_HERMITE && (p->gh_order < 1 || p->gh_order > SS_MAX_GH_ORDER))
    return SS_ERR_INVALID;
  if (p->batch < 1 || p->total_steps < 0 || p->max_len < 0) return SS_ERR_INVALID;
  if (p->chunk < 0 || p->group < 0) return SS_ERR_INVALID;
  if (p->offsets == nullptr) return SS_ERR_INVALID;
  const ss_model* ms[2] = {&p->transition, &p->observation};
  for (const ss_model* m : ms) {
    if (m->noise_mean == nullptr || m->noise_chol == nullptr) return SS_ERR_INVALID;
    if (m->kind == SS_MODEL_LINEAR && m->matrix == nullptr) return SS_ERR_INVALID;
    if (m->kind < SS_MODEL_LINEAR || m->kind > SS_MODEL_POISSON_EXP) return SS_ERR_UNSUPPORTED;
  }
  if (find_run(p->dtype, p->nx, p->ny) == nullptr) return SS_ERR_UNSUPPORTED;
  // the covariance-form kernels exist for the small-state pairs only
  if ((p->options & SS_OPT_COVARIANCE_FORM) && (p->nx > SS_MAX_NX || p->ny > SS_MAX_NY)) return SS_ERR_UNSUPPORTED;
  return SS_OK;
}

static int dispatch(Call& c) {
  int rc = validate(c.p);
  if (rc) return rc;
  return find_run(c.p->dtype, c.p->nx, c.p->ny)(c);
}

}  // namespace ss

using namespace ss;

extern "C" {

int ss_version(void) { return 10000; }

long long ss_launch_count(void) { return g_launches.load(); }

int ss_profile_enable(int on) {
  g_profiling.store(on != 0);
  return SS_OK;
}

int ss_profile_reset(void) {
  std::lock_guard<std::mutex> lk(g_prof_mu);
  for (const ProfRec& r : g_prof) {
    cudaEventDestroy(r.start);
    cudaEventDestroy(r.stop);
  }
  g_prof.clear();
  return SS_OK;
}

int ss_profile_read(char* buf, size_t len) {
  if (buf == nullptr || len == 0) return SS_ERR_INVALID;
  std::map<std::string, std::pair<long long, double>> acc;
  {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    for (const ProfRec& r : g_prof) {
      if (cudaEventSynchronize(r.stop) != cudaSuccess) return SS_ERR_CUDA;
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, r.start, r.stop) != cudaSuccess) return SS_ERR_CUDA;
      auto& a = acc[r.name];
      a.first += 1;
      a.second += ms;
    }
  }
  std::string out = "{";
  bool first = true;
  for (const auto& kv : acc) {
    char item[160];
    std::snprintf(item, sizeof(item), "%s\"%s\": [%lld, %.6f]", first ? "" : ", ", kv.first.c_str(),
                  kv.second.first, kv.second.second);
    out += item;
    first = false;
  }
  out += "}";
  if (out.size() + 1 > len) return SS_ERR_INVALID;
  std::memcpy(buf, out.c_str(), out.size() + 1);
  return SS_OK;
}

const char* ss_status_string(int status) {
  switch (status) {
    case SS_OK: return "ok";
    case SS_ERR_INVALID: return "invalid argument";
    case SS_ERR_UNSUPPORTED: return "unsupported model, method or dimension";
    case SS_ERR_CUDA: return "CUDA error";
    case SS_ERR_WORKSPACE: return "workspace too small";
    default: return "unknown status";
  }
}

int ss_supported(const ss_problem* p) {
  if (validate(p) != SS_OK) return 0;
  Call c;
  std::memset(&c, 0, sizeof(c));
  c.op = OP_SUPPORTED;
  c.p = p;
  return find_run(p->dtype, p->nx, p->ny)(c) == SS_OK ? 1 : 0;
}

int ss_workspace_bytes(const ss_problem* p, size_t* bytes) {
  if (bytes == nullptr) return SS_ERR_INVALID;
  Call c;
  std::memset(&c, 0, sizeof(c));
  c.op = OP_WORKSPACE;
  c.p = p;
  c.ws_bytes_out = bytes;
  return dispatch(c);
}

int ss_linearize(const ss_problem* p, int32_t which, int64_t n, const void* m, const void* chol,
                 void* F, void* chol_out, void* b, ss_stream_t stream) {
  if (which != 0 && which != 1) return SS_ERR_INVALID;
  if (n < 0 || (n > 0 && (m == nullptr || chol == nullptr || F == nullptr || chol_out == nullptr || b == nullptr)))
    return SS_ERR_INVALID;
  Call c;
  std::memset(&c, 0, sizeof(c));
  c.op = OP_LINEARIZE;
  c.p = p;
  c.which = which;
  c.n_points = n;
  c.pt_m = m;
  c.pt_L = chol;
  c.pt_F = F;
  c.pt_chol = chol_out;
  c.pt_b = b;
  c.stream = reinterpret_cast<cudaStream_t>(stream);
  return dispatch(c);
}

int ss_filter(const ss_problem* p, const void* ys, const void* m0, const void* L0,
              int32_t prior_per_sequence, const void* nominal_m, const void* nominal_L, void* out_m,
              void* out_L, double* out_ell, void* workspace, size_t workspace_bytes, ss_stream_t stream) {
  if (p == nullptr || m0 == nullptr || L0 == nullptr || out_m == nullptr || out_L == nullptr) return SS_ERR_INVALID;
  if (p->total_steps > 0 && ys == nullptr) return SS_ERR_INVALID;
  if ((nominal_m == nullptr) != (nominal_L == nullptr)) return SS_ERR_INVALID;
  Call c;
  std::memset(&c, 0, sizeof(c));
  c.op = OP_FILTER;
  c.p = p;
  c.ys = ys;
  c.m0 = m0;
  c.L0 = L0;
  c.prior_per_sequence = prior_per_sequence;
  c.nom_m = nominal_m;
  c.nom_L = nominal_L;
  c.out_m = out_m;
  c.out_L = out_L;
  c.out_ell = out_ell;
  c.ws = workspace;
  c.ws_bytes = workspace_bytes;
  c.stream = reinterpret_cast<cudaStream_t>(stream);
  return dispatch(c);
}

int ss_smooth(const ss_problem* p, const void* filt_m, const void* filt_L, const void* nominal_m,
              const void* nominal_L, void* out_m, void* out_L, void* workspace, size_t workspace_bytes,
              ss_stream_t stream) {
  if (p == nullptr || filt_m == nullptr || filt_L == nullptr || out_m == nullptr || out_L == nullptr)
    return SS_ERR_INVALID;
  if ((nominal_m == nullptr) != (nominal_L == nullptr)) return SS_ERR_INVALID;
  Call c;
  std::memset(&c, 0, sizeof(c));
  c.op = OP_SMOOTH;
  c.p = p;
  c.in_m = filt_m;
  c.in_L = filt_L;
  c.nom_m = nominal_m;
  c.nom_L = nominal_L;
  c.out_m = out_m;
  c.out_L = out_L;
  c.ws = workspace;
  c.ws_bytes = workspace_bytes;
  c.stream = reinterpret_cast<cudaStream_t>(stream);
  return dispatch(c);
}

int ss_filter_grad_workspace_bytes(const ss_problem* p, size_t* bytes) {
  if (bytes == nullptr) return SS_ERR_INVALID;
  int rc = validate(p);
  if (rc) return rc;
  RunFn f = find_grad(p->dtype, p->nx, p->ny);
  if (f == nullptr) return SS_ERR_UNSUPPORTED;
  Call c;
  std::memset(&c, 0, sizeof(c));
  c.op = OP_WORKSPACE;
  c.p = p;
  c.ws_bytes_out = bytes;
  c.prior_per_sequence = 1;  // the larger of the two prior layouts
  return f(c);
}

int ss_filter_grad(const ss_problem* p, const ss_tangents* tangents, const void* ys, const void* m0,
                   const void* L0, int32_t prior_per_sequence, const void* nominal_m, const void* nominal_L,
                   double* out_ell, double* out_grad, void* workspace, size_t workspace_bytes,
                   ss_stream_t stream) {
  if (p == nullptr || tangents == nullptr || m0 == nullptr || L0 == nullptr || out_ell == nullptr ||
      out_grad == nullptr)
    return SS_ERR_INVALID;
  if (p->total_steps > 0 && ys == nullptr) return SS_ERR_INVALID;
  if ((nominal_m == nullptr) != (nominal_L == nullptr)) return SS_ERR_INVALID;
  int rc = validate(p);
  if (rc) return rc;
  RunFn f = find_grad(p->dtype, p->nx, p->ny);
  if (f == nullptr) return SS_ERR_UNSUPPORTED;
  Call c;
  std::memset(&c, 0, sizeof(c));
  c.op = OP_FILTER;
  c.p = p;
  c.tangents = tangents;
  c.ys = ys;
  c.m0 = m0;
  c.L0 = L0;
  c.prior_per_sequence = prior_per_sequence;
  c.nom_m = nominal_m;
  c.nom_L = nominal_L;
  c.out_ell = out_ell;
  c.out_grad = out_grad;
  c.ws = workspace;
  c.ws_bytes = workspace_bytes;
  c.stream = reinterpret_cast<cudaStream_t>(stream);
  return f(c);
}

int ss_sample(const ss_problem* p, const void* filt_m, const void* filt_L, const void* nominal_m,
              const void* nominal_L, int32_t n_samples, const void* eps, void* out, void* workspace,
              size_t workspace_bytes, ss_stream_t stream) {
  if (p == nullptr || filt_m == nullptr || filt_L == nullptr || n_samples < 1 || eps == nullptr || out == nullptr)
    return SS_ERR_INVALID;
  if ((nominal_m == nullptr) != (nominal_L == nullptr)) return SS_ERR_INVALID;
  Call c;
  std::memset(&c, 0, sizeof(c));
  c.op = OP_SAMPLE;
  c.p = p;
  c.in_m = filt_m;
  c.in_L = filt_L;
  c.nom_m = nominal_m;
  c.nom_L = nominal_L;
  c.n_samples = n_samples;
  c.eps = eps;
  c.out_m = out;
  c.ws = workspace;
  c.ws_bytes = workspace_bytes;
  c.stream = reinterpret_cast<cudaStream_t>(stream);
  return dispatch(c);
}

int ss_iterated_grad_workspace_bytes(const ss_problem* p, size_t* bytes) {
  if (bytes == nullptr) return SS_ERR_INVALID;
  int rc = validate(p);
  if (rc) return rc;
  RunFn f = find_grad(p->dtype, p->nx, p->ny);
  if (f == nullptr) return SS_ERR_UNSUPPORTED;
  Call c;
  std::memset(&c, 0, sizeof(c));
  c.op = OP_WORKSPACE;
  c.p = p;
  c.ws_bytes_out = bytes;
  c.prior_per_sequence = 1;
  c.n_iter = 1;  // the iterated layout
  return f(c);
}

int ss_iterated_grad(const ss_problem* p, const ss_tangents* tangents, const void* ys, const void* m0,
                     const void* L0, int32_t prior_per_sequence, const void* init_m, const void* init_L,
                     int32_t n_iter, double* out_ell, double* out_grad, void* workspace,
                     size_t workspace_bytes, ss_stream_t stream) {
  if (p == nullptr || tangents == nullptr || m0 == nullptr || L0 == nullptr || out_ell == nullptr ||
      out_grad == nullptr || n_iter < 1)
    return SS_ERR_INVALID;
  if (p->total_steps > 0 && ys == nullptr) return SS_ERR_INVALID;
  if ((init_m == nullptr) != (init_L == nullptr)) return SS_ERR_INVALID;
  int rc = validate(p);
  if (rc) return rc;
  RunFn f = find_grad(p->dtype, p->nx, p->ny);
  if (f == nullptr) return SS_ERR_UNSUPPORTED;
  Call c;
  std::memset(&c, 0, sizeof(c));
  c.op = OP_ITERATED;
  c.p = p;
  c.tangents = tangents;
  c.ys = ys;
  c.m0 = m0;
  c.L0 = L0;
  c.prior_per_sequence = prior_per_sequence;
  c.nom_m = init_m;
  c.nom_L = init_L;
  c.n_iter = n_iter;
  c.out_ell = out_ell;
  c.out_grad = out_grad;
  c.ws = workspace;
  c.ws_bytes = workspace_bytes;
  c.stream = reinterpret_cast<cudaStream_t>(stream);
  return f(c);
}

int ss_filter_adjoint_workspace_bytes(const ss_problem* p, size_t* bytes) {
  if (bytes == nullptr) return SS_ERR_INVALID;
  int rc = validate(p);
  if (rc) return rc;
  if (p->options & SS_OPT_COVARIANCE_FORM) return SS_ERR_UNSUPPORTED;
  RunFn f = find_adj(p->dtype, p->nx, p->ny);
  if (f == nullptr) return SS_ERR_UNSUPPORTED;
  Call c;
  std::memset(&c, 0, sizeof(c));
  c.op = OP_WORKSPACE;
  c.p = p;
  c.ws_bytes_out = bytes;
  return f(c);
}

int ss_filter_adjoint(const ss_problem* p, const void* ys, const void* m0, const void* L0,
                      int32_t prior_per_sequence, const void* nominal_m, const void* nominal_L,
                      double* out_ell, const ss_adjoints* out, void* workspace, size_t workspace_bytes,
                      ss_stream_t stream) {
  if (p == nullptr || out == nullptr || m0 == nullptr || L0 == nullptr) return SS_ERR_INVALID;
  if (p->total_steps > 0 && ys == nullptr) return SS_ERR_INVALID;
  if ((nominal_m == nullptr) != (nominal_L == nullptr)) return SS_ERR_INVALID;
  int rc = validate(p);
  if (rc) return rc;
  if (p->options & SS_OPT_COVARIANCE_FORM) return SS_ERR_UNSUPPORTED;
  if ((out->trans_params != nullptr || out->obs_params != nullptr) && p->lin_method == SS_LIN_GAUSS_HERMITE)
    return SS_ERR_UNSUPPORTED;
  RunFn f = find_adj(p->dtype, p->nx, p->ny);
  if (f == nullptr) return SS_ERR_UNSUPPORTED;
  Call c;
  std::memset(&c, 0, sizeof(c));
  c.op = OP_ADJOINT;
  c.p = p;
  c.ys = ys;
  c.m0 = m0;
  c.L0 = L0;
  c.prior_per_sequence = prior_per_sequence;
  c.nom_m = nominal_m;
  c.nom_L = nominal_L;
  c.out_ell = out_ell;
  c.adjoints = out;
  c.ws = workspace;
  c.ws_bytes = workspace_bytes;
  c.stream = reinterpret_cast<cudaStream_t>(stream);
  return f(c);
}

int ss_iterated(const ss_problem* p, const void* ys, const void* m0, const void* L0,
                int32_t prior_per_sequence, const void* init_m, const void* init_L, int32_t n_iter,
                double tol, void* out_m, void* out_L, double* out_ell, int32_t* out_iters,
                uint32_t* out_flags, void* workspace, size_t workspace_bytes, ss_stream_t stream) {
  if (p == nullptr || m0 == nullptr || L0 == nullptr || out_m == nullptr || out_L == nullptr) return SS_ERR_INVALID;
  if (p->total_steps > 0 && ys == nullptr) return SS_ERR_INVALID;
  if ((init_m == nullptr) != (init_L == nullptr)) return SS_ERR_INVALID;
  if (n_iter < 0 || !(tol >= 0.0) || (tol > 0.0 && n_iter < 1)) return SS_ERR_INVALID;
  Call c;
  std::memset(&c, 0, sizeof(c));
  c.op = OP_ITERATED;
  c.p = p;
  c.ys = ys;
  c.m0 = m0;
  c.L0 = L0;
  c.prior_per_sequence = prior_per_sequence;
  c.nom_m = init_m;
  c.nom_L = init_L;
  c.n_iter = n_iter;
  c.tol = tol;
  c.out_m = out_m;
  c.out_L = out_L;
  c.out_ell = out_ell;
  c.out_iters = out_iters;
  c.out_flags = out_flags;
  c.ws = workspace;
  c.ws_bytes = workspace_bytes;
  c.stream = reinterpret_cast<cudaStream_t>(stream);
  return dispatch(c);
}

}  // extern "C"
