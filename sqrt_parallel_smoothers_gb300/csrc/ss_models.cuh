// Device-side model registry and linearisation methods.
//
// The reference linearises arbitrary JAX callables; device code cannot call
// Python, so models are C++ functors selected by id.  Each functor evaluates
// f(x) and its Jacobian (the Jacobian is only used by the extended method).
#pragma once
#include "ss_dual.cuh"
#include "../../include/sqrtsmooth.h"

namespace ss {

SS_DEV float ss_sin(float x) { return sinf(x); }
SS_DEV double ss_sin(double x) { return sin(x); }
SS_DEV float ss_cos(float x) { return cosf(x); }
SS_DEV double ss_cos(double x) { return cos(x); }
SS_DEV float ss_atan2(float y, float x) { return atan2f(y, x); }
SS_DEV float ss_exp(float x) { return expf(x); }
SS_DEV double ss_exp(double x) { return exp(x); }
SS_DEV double ss_atan2(double y, double x) { return atan2(y, x); }
template <typename T, int NT>
SS_DEV Dual<T, NT> ss_sin(const Dual<T, NT>& a) { return chain(a, ss_sin(a.v), ss_cos(a.v)); }
template <typename T, int NT>
SS_DEV Dual<T, NT> ss_cos(const Dual<T, NT>& a) { return chain(a, ss_cos(a.v), -ss_sin(a.v)); }
template <typename T, int NT>
SS_DEV Dual<T, NT> ss_exp(const Dual<T, NT>& a) {
  const T e = ss_exp(a.v);
  return chain(a, e, e);
}
// sin and cos of one angle with one range reduction.  In FP32 a small angle
// (|x| <= 1/4, the coordinated turn's omega dt in practice) takes the Taylor
// polynomials to degree 9 / 8, whose truncation error (below 3e-13) is far
// under FP32 rounding; larger angles call sincosf.
SS_DEV void ss_sincos(float x, float& s, float& c) {
  if (fabsf(x) <= 0.25f) {
    const float x2 = x * x;
    s = x * (1.0f - x2 * (1.0f / 6.0f) * (1.0f - x2 * (1.0f / 20.0f) * (1.0f - x2 * (1.0f / 42.0f) *
                                                                          (1.0f - x2 * (1.0f / 72.0f)))));
    c = 1.0f - x2 * 0.5f * (1.0f - x2 * (1.0f / 12.0f) * (1.0f - x2 * (1.0f / 30.0f) * (1.0f - x2 * (1.0f / 56.0f))));
  } else {
    sincosf(x, &s, &c);
  }
}
SS_DEV void ss_sincos(double x, double& s, double& c) { sincos(x, &s, &c); }
template <typename T, int NT>
SS_DEV void ss_sincos(const Dual<T, NT>& a, Dual<T, NT>& s, Dual<T, NT>& c) {
  T sv, cv;
  ss_sincos(a.v, sv, cv);
  s = chain(a, sv, cv);
  c = chain(a, cv, -sv);
}
template <typename T, int NT>
SS_DEV Dual<T, NT> ss_atan2(const Dual<T, NT>& y, const Dual<T, NT>& x) {
  Dual<T, NT> r;
  r.v = ss_atan2(y.v, x.v);
  const T inv = T(1) / (x.v * x.v + y.v * y.v);
  SS_UNROLL
  for (int k = 0; k < NT; ++k) r.d[k] = (x.v * y.d[k] - y.v * x.d[k]) * inv;
  return r;
}

// Parameters of one model as the kernels see them (device pointers / scalars).
template <typename R>
struct ModelArgs {
  const R* mat;   // LINEAR: d_out x d_in row-major matrix
  R p[4];         // COORDINATED_TURN: p[0] = dt; BEARINGS: s1x, s1y, s2x, s2y; RICKER: a; POISSON_EXP: lam
};

// A functor is a conditional-moments model (parsmooth/_base.py:20-22) when it
// defines kConditional = true: eval gives E[y|x] and cond_chol a factor of
// Cov[y|x]; its linearisation then ignores the model's additive noise.
template <class Fn, class = void>
struct IsConditional {
  static constexpr bool value = false;
};
template <class Fn>
struct IsConditional<Fn, decltype(void(Fn::kConditional))> {
  static constexpr bool value = Fn::kConditional;
};

// f(x) = A x  (tests/_lgssm.py:5-35 in the reference)
template <typename R, int DIN, int DOUT>
struct LinearFn {
  R A[DOUT][DIN];
  SS_DEV void init(const ModelArgs<R>& a) {
    SS_UNROLL
    for (int i = 0; i < DOUT; ++i) {
      SS_UNROLL
      for (int j = 0; j < DIN; ++j) A[i][j] = a.mat[i * DIN + j];
    }
  }
  SS_DEV void eval(const R (&x)[DIN], R (&y)[DOUT]) const { matvec<R, DOUT, DIN>(A, x, y); }
  SS_DEV void jac(const R (&)[DIN], R (&J)[DOUT][DIN]) const {
    SS_UNROLL
    for (int i = 0; i < DOUT; ++i) {
      SS_UNROLL
      for (int j = 0; j < DIN; ++j) J[i][j] = A[i][j];
    }
  }
};

// Coordinated turn, state (x, y, vx, vy, w) (tests/bearings/bearings_utils.py:7-44),
// including the |w| < 1e-6 branch.
template <typename R, int DIN, int DOUT>
struct CoordinatedTurnFn {
  static_assert(DIN == 5 && DOUT == 5, "coordinated turn is 5 -> 5");
  R dt;
  SS_DEV void init(const ModelArgs<R>& a) { dt = a.p[0]; }
  SS_DEV void coeffs(R w, R& c, R& s, R& sw, R& cw) const {
    ss_sincos(w * dt, s, c);
    if (ss_abs(w) < R(1e-6)) {
      sw = dt;
      cw = R(0);
    } else {
      const R iw = ss_rcp(w);
      sw = s * iw;
      cw = (c - R(1)) * iw;
    }
  }
  SS_DEV void eval(const R (&x)[DIN], R (&y)[DOUT]) const {
    R c, s, sw, cw;
    coeffs(x[4], c, s, sw, cw);
    y[0] = x[0] + sw * x[2] - cw * x[3];
    y[1] = x[1] + cw * x[2] + sw * x[3];
    y[2] = c * x[2] + s * x[3];
    y[3] = -s * x[2] + c * x[3];
    y[4] = x[4];
  }
  SS_DEV void jac(const R (&x)[DIN], R (&J)[DOUT][DIN]) const {
    const R w = x[4];
    R c, s, sw, cw;
    coeffs(w, c, s, sw, cw);
    R dsw = R(0), dcw = R(0);
    if (!(ss_abs(w) < R(1e-6))) {
      const R iw = ss_rcp(w);
      dsw = (dt * c - sw) * iw;
      dcw = (-dt * s - cw) * iw;
    }
    SS_UNROLL
    for (int i = 0; i < 5; ++i) {
      SS_UNROLL
      for (int j = 0; j < 5; ++j) J[i][j] = R(0);
    }
    J[0][0] = R(1); J[0][2] = sw; J[0][3] = -cw; J[0][4] = dsw * x[2] - dcw * x[3];
    J[1][1] = R(1); J[1][2] = cw; J[1][3] = sw;  J[1][4] = dcw * x[2] + dsw * x[3];
    J[2][2] = c;  J[2][3] = s;  J[2][4] = -dt * s * x[2] + dt * c * x[3];
    J[3][2] = -s; J[3][3] = c;  J[3][4] = -dt * c * x[2] - dt * s * x[3];
    J[4][4] = R(1);
  }
};

// Two bearings atan2(y - s_y, x - s_x) (tests/bearings/bearings_utils.py:47-69).
template <typename R, int DIN, int DOUT>
struct BearingsFn {
  static_assert(DOUT == 2 && DIN >= 2, "bearings maps R^n (n >= 2) to two angles");
  R s[4];
  SS_DEV void init(const ModelArgs<R>& a) {
    SS_UNROLL
    for (int k = 0; k < 4; ++k) s[k] = a.p[k];
  }
  SS_DEV void eval(const R (&x)[DIN], R (&y)[DOUT]) const {
    y[0] = ss_atan2(x[1] - s[1], x[0] - s[0]);
    y[1] = ss_atan2(x[1] - s[3], x[0] - s[2]);
  }
  SS_DEV void jac(const R (&x)[DIN], R (&J)[DOUT][DIN]) const {
    SS_UNROLL
    for (int k = 0; k < 2; ++k) {
      const R dx = x[0] - s[2 * k], dy = x[1] - s[2 * k + 1];
      const R r2 = dx * dx + dy * dy;
      SS_UNROLL
      for (int j = 0; j < DIN; ++j) J[k][j] = R(0);
      const R ir2 = ss_rcp(r2);
      J[k][0] = -dy * ir2;
      J[k][1] = dx * ir2;
    }
  }
};

// Ricker map on the log scale (notebooks/population_model.py:9-21), elementwise:
// f(x)_i = a + x_i - exp(x_i).
template <typename R, int DIN, int DOUT>
struct RickerFn {
  static_assert(DIN == DOUT, "the Ricker map is n -> n");
  R a;
  SS_DEV void init(const ModelArgs<R>& m) { a = m.p[0]; }
  SS_DEV void eval(const R (&x)[DIN], R (&y)[DOUT]) const {
    SS_UNROLL
    for (int i = 0; i < DOUT; ++i) y[i] = a + x[i] - ss_exp(x[i]);
  }
  SS_DEV void jac(const R (&x)[DIN], R (&J)[DOUT][DIN]) const {
    SS_UNROLL
    for (int i = 0; i < DOUT; ++i) {
      SS_UNROLL
      for (int j = 0; j < DIN; ++j) J[i][j] = (i == j) ? R(1) - ss_exp(x[i]) : R(0);
    }
  }
};

// Poisson counts with log-intensity x (notebooks/population_model.py:83-118):
// E[y_k | x] = Var[y_k | x] = lam exp(x_k), k < ny, as conditional moments.
template <typename R, int DIN, int DOUT>
struct PoissonExpFn {
  static_assert(DOUT <= DIN, "one count per leading state component");
  static constexpr bool kConditional = true;
  R lam;
  SS_DEV void init(const ModelArgs<R>& m) { lam = m.p[0]; }
  SS_DEV void eval(const R (&x)[DIN], R (&y)[DOUT]) const {
    SS_UNROLL
    for (int i = 0; i < DOUT; ++i) y[i] = lam * ss_exp(x[i]);
  }
  SS_DEV void jac(const R (&x)[DIN], R (&J)[DOUT][DIN]) const {
    SS_UNROLL
    for (int i = 0; i < DOUT; ++i) {
      SS_UNROLL
      for (int j = 0; j < DIN; ++j) J[i][j] = (i == j) ? lam * ss_exp(x[i]) : R(0);
    }
  }
  SS_DEV void cond_chol(const R (&x)[DIN], R (&C)[DOUT][DOUT]) const {
    SS_UNROLL
    for (int i = 0; i < DOUT; ++i) {
      SS_UNROLL
      for (int j = 0; j < DOUT; ++j) C[i][j] = (i == j) ? ss_sqrt(lam * ss_exp(x[i])) : R(0);
    }
  }
};

// ---------------------------------------------------------------------------
// Sigma-point rules.  Point k is m + chol xi_k.  Host code fills the rule
// (weights of the unscented transform, 1-D Gauss-Hermite roots/weights).
struct RuleArgs {
  int method;          // SS_LIN_*
  int gh_order;        // p (Gauss-Hermite)
  // unscented: {sqrt(n + lambda), wm0, wc0, w}; both precisions so that FP32
  // kernels never touch the FP64 pipe
  double ut_d[4];
  float ut_f[4];
  double gh_root_d[SS_MAX_GH_ORDER];   // sqrt(2) * Hermite roots
  double gh_w_d[SS_MAX_GH_ORDER];      // 1-D weights / sqrt(pi)
  float gh_root_f[SS_MAX_GH_ORDER];
  float gh_w_f[SS_MAX_GH_ORDER];
};

template <typename R>
SS_DEV R rule_ut(const RuleArgs& r, int i) { return R(r.ut_d[i]); }
template <>
SS_DEV float rule_ut<float>(const RuleArgs& r, int i) { return r.ut_f[i]; }
template <>
SS_DEV double rule_ut<double>(const RuleArgs& r, int i) { return r.ut_d[i]; }
template <typename R>
SS_DEV R rule_gh_root(const RuleArgs& r, int i) { return R(r.gh_root_d[i]); }
template <>
SS_DEV float rule_gh_root<float>(const RuleArgs& r, int i) { return r.gh_root_f[i]; }
template <>
SS_DEV double rule_gh_root<double>(const RuleArgs& r, int i) { return r.gh_root_d[i]; }
template <typename R>
SS_DEV R rule_gh_w(const RuleArgs& r, int i) { return R(r.gh_w_d[i]); }
template <>
SS_DEV float rule_gh_w<float>(const RuleArgs& r, int i) { return r.gh_w_f[i]; }
template <>
SS_DEV double rule_gh_w<double>(const RuleArgs& r, int i) { return r.gh_w_d[i]; }

}  // namespace ss
