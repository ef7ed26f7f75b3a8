// Forward-mode dual numbers: a value and NT tangent components.
//
// Every kernel of the filter is written for a generic scalar type R, so
// instantiating it with R = Dual<float, NT> propagates the derivatives of
// every intermediate with respect to NT parameter directions alongside the
// values (tangent-linear mode).  Comparisons look at the value only, which
// reproduces the branch structure of the primal code.
#pragma once
#include "ss_la.cuh"

namespace ss {

template <typename T, int NT>
struct Dual {
  T v;
  T d[NT];
  Dual() = default;
  SS_DEV Dual(double x) : v(T(x)) {
    SS_UNROLL
    for (int k = 0; k < NT; ++k) d[k] = T(0);
  }
  SS_DEV Dual(int x) : Dual(double(x)) {}
  SS_DEV Dual(float x) : Dual(double(x)) {}
  // the value part (convergence tests and bookkeeping look at values only)
  SS_DEV explicit operator double() const { return (double)v; }
  SS_DEV Dual& operator+=(const Dual& o) {
    v += o.v;
    SS_UNROLL
    for (int k = 0; k < NT; ++k) d[k] += o.d[k];
    return *this;
  }
  SS_DEV Dual& operator-=(const Dual& o) {
    v -= o.v;
    SS_UNROLL
    for (int k = 0; k < NT; ++k) d[k] -= o.d[k];
    return *this;
  }
  SS_DEV Dual& operator*=(const Dual& o) {
    SS_UNROLL
    for (int k = 0; k < NT; ++k) d[k] = d[k] * o.v + v * o.d[k];
    v *= o.v;
    return *this;
  }
};

template <typename T, int NT>
SS_DEV Dual<T, NT> operator+(Dual<T, NT> a, const Dual<T, NT>& b) { return a += b; }
template <typename T, int NT>
SS_DEV Dual<T, NT> operator-(Dual<T, NT> a, const Dual<T, NT>& b) { return a -= b; }
template <typename T, int NT>
SS_DEV Dual<T, NT> operator-(const Dual<T, NT>& a) {
  Dual<T, NT> r;
  r.v = -a.v;
  SS_UNROLL
  for (int k = 0; k < NT; ++k) r.d[k] = -a.d[k];
  return r;
}
template <typename T, int NT>
SS_DEV Dual<T, NT> operator*(const Dual<T, NT>& a, const Dual<T, NT>& b) {
  Dual<T, NT> r;
  r.v = a.v * b.v;
  SS_UNROLL
  for (int k = 0; k < NT; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
  return r;
}
template <typename T, int NT>
SS_DEV Dual<T, NT> operator/(const Dual<T, NT>& a, const Dual<T, NT>& b) {
  Dual<T, NT> r;
  const T inv = T(1) / b.v;
  r.v = a.v * inv;
  SS_UNROLL
  for (int k = 0; k < NT; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * inv;
  return r;
}
template <typename T, int NT>
SS_DEV Dual<T, NT>& operator/=(Dual<T, NT>& a, const Dual<T, NT>& b) { return a = a / b; }

#define SS_DUAL_CMP(OP)                                                            \
  template <typename T, int NT>                                                    \
  SS_DEV bool operator OP(const Dual<T, NT>& a, const Dual<T, NT>& b) { return a.v OP b.v; }
SS_DUAL_CMP(<)
SS_DUAL_CMP(<=)
SS_DUAL_CMP(>)
SS_DUAL_CMP(>=)
SS_DUAL_CMP(==)
SS_DUAL_CMP(!=)
#undef SS_DUAL_CMP

// Chain rule helper: r = f(a) with f'(a) = df.
template <typename T, int NT>
SS_DEV Dual<T, NT> chain(const Dual<T, NT>& a, T fv, T df) {
  Dual<T, NT> r;
  r.v = fv;
  SS_UNROLL
  for (int k = 0; k < NT; ++k) r.d[k] = df * a.d[k];
  return r;
}

template <typename T, int NT>
SS_DEV Dual<T, NT> ss_sqrt(const Dual<T, NT>& a) {
  const T s = ss_sqrt(a.v);
  return chain(a, s, s > T(0) ? T(0.5) / s : T(0));
}
template <typename T, int NT>
SS_DEV Dual<T, NT> ss_abs(const Dual<T, NT>& a) { return a.v < T(0) ? -a : a; }
template <typename T, int NT>
SS_DEV Dual<T, NT> ss_log(const Dual<T, NT>& a) { return chain(a, ss_log(a.v), T(1) / a.v); }
template <typename T, int NT>
SS_DEV bool ss_isfinite(const Dual<T, NT>& a) { return ss_isfinite(a.v); }

template <typename T>
struct Tangents {
  static constexpr int n = 0;
  using scalar = T;
};
template <typename T, int NT>
struct Tangents<Dual<T, NT>> {
  static constexpr int n = NT;
  using scalar = T;  // the arithmetic precision of the value and tangents
};

// Value and tangents of a scalar as doubles (for FP64 accumulation).
SS_DEV void to_components(float x, double* c) { c[0] = x; }
SS_DEV void to_components(double x, double* c) { c[0] = x; }
template <typename T, int NT>
SS_DEV void to_components(const Dual<T, NT>& x, double* c) {
  c[0] = x.v;
  SS_UNROLL
  for (int k = 0; k < NT; ++k) c[1 + k] = x.d[k];
}

}  // namespace ss
