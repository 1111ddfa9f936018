// Forward-mode dual numbers: a value and K tangent components, propagated
// through every arithmetic operation (chain rule), for exact derivatives of
// a discrete computation with respect to K scalar parameters.
#pragma once

#include <cuda_runtime.h>

namespace gj {

template <int K>
struct Dual {
  double v;
  double t[K];

  __host__ __device__ Dual() : v(0.0) {
    for (int i = 0; i < K; ++i) t[i] = 0.0;
  }
  __host__ __device__ Dual(double x) : v(x) {  // NOLINT: constants promote implicitly
    for (int i = 0; i < K; ++i) t[i] = 0.0;
  }
  __host__ __device__ static Dual seed(double x, int which) {
    Dual d(x);
    d.t[which] = 1.0;
    return d;
  }
};

#define GJ_DUAL_BIN(OP, VAL, TAN)                                                       \
  template <int K>                                                                      \
  __host__ __device__ inline Dual<K> operator OP(const Dual<K>& a, const Dual<K>& b) {  \
    Dual<K> r;                                                                          \
    r.v = VAL;                                                                          \
    for (int i = 0; i < K; ++i) r.t[i] = TAN;                                           \
    return r;                                                                           \
  }
GJ_DUAL_BIN(+, a.v + b.v, a.t[i] + b.t[i])
GJ_DUAL_BIN(-, a.v - b.v, a.t[i] - b.t[i])
GJ_DUAL_BIN(*, a.v * b.v, a.t[i] * b.v + a.v * b.t[i])
#undef GJ_DUAL_BIN

template <int K>
__host__ __device__ inline Dual<K> operator/(const Dual<K>& a, const Dual<K>& b) {
  Dual<K> r;
  const double ib = 1.0 / b.v;
  r.v = a.v * ib;
  for (int i = 0; i < K; ++i) r.t[i] = (a.t[i] - r.v * b.t[i]) * ib;
  return r;
}
template <int K>
__host__ __device__ inline Dual<K> operator-(const Dual<K>& a) {
  Dual<K> r;
  r.v = -a.v;
  for (int i = 0; i < K; ++i) r.t[i] = -a.t[i];
  return r;
}
template <int K>
__host__ __device__ inline Dual<K> operator+(const Dual<K>& a, double b) { return a + Dual<K>(b); }
template <int K>
__host__ __device__ inline Dual<K> operator+(double a, const Dual<K>& b) { return Dual<K>(a) + b; }
template <int K>
__host__ __device__ inline Dual<K> operator-(const Dual<K>& a, double b) { return a - Dual<K>(b); }
template <int K>
__host__ __device__ inline Dual<K> operator-(double a, const Dual<K>& b) { return Dual<K>(a) - b; }
template <int K>
__host__ __device__ inline Dual<K> operator*(const Dual<K>& a, double b) {
  Dual<K> r;
  r.v = a.v * b;
  for (int i = 0; i < K; ++i) r.t[i] = a.t[i] * b;
  return r;
}
template <int K>
__host__ __device__ inline Dual<K> operator*(double a, const Dual<K>& b) { return b * a; }
template <int K>
__host__ __device__ inline Dual<K> operator/(const Dual<K>& a, double b) { return a * (1.0 / b); }
template <int K>
__host__ __device__ inline Dual<K> operator/(double a, const Dual<K>& b) { return Dual<K>(a) / b; }
template <int K>
__host__ __device__ inline Dual<K>& operator+=(Dual<K>& a, const Dual<K>& b) { return a = a + b; }
template <int K>
__host__ __device__ inline Dual<K>& operator-=(Dual<K>& a, const Dual<K>& b) { return a = a - b; }
template <int K>
__host__ __device__ inline Dual<K>& operator*=(Dual<K>& a, const Dual<K>& b) { return a = a * b; }

// elementary functions: f(v) and f'(v) times the tangents
template <int K>
__host__ __device__ inline Dual<K> chain(const Dual<K>& a, double f, double df) {
  Dual<K> r;
  r.v = f;
  for (int i = 0; i < K; ++i) r.t[i] = df * a.t[i];
  return r;
}
template <int K>
__device__ inline Dual<K> sqrt(const Dual<K>& a) {
  const double s = ::sqrt(a.v);
  return chain(a, s, 0.5 / s);
}
template <int K>
__device__ inline Dual<K> exp(const Dual<K>& a) {
  const double e = ::exp(a.v);
  return chain(a, e, e);
}
template <int K>
__device__ inline Dual<K> log(const Dual<K>& a) {
  return chain(a, ::log(a.v), 1.0 / a.v);
}
template <int K>
__device__ inline Dual<K> log1p(const Dual<K>& a) {
  return chain(a, ::log1p(a.v), 1.0 / (1.0 + a.v));
}

// plain-double versions so templated code resolves for S = double inside gj
__device__ inline double sqrt(double a) { return ::sqrt(a); }
__device__ inline double exp(double a) { return ::exp(a); }
__device__ inline double log(double a) { return ::log(a); }
__device__ inline double log1p(double a) { return ::log1p(a); }

template <int K>
__host__ __device__ inline double value(const Dual<K>& a) { return a.v; }
__host__ __device__ inline double value(double a) { return a; }

}  // namespace gj
