// Registered target families: per-chain device operators (one thread owns one
// chain; vectors of length d live in the caller's local arrays).
//
// The reference takes user callables logdensity_fn / metric_fn and obtains
// gradients, HVPs (util.py:120-121, jvp of grad) and metric derivatives
// (lmcmc/metrics.py:165, jacfwd) by JAX autodiff.  Here each family states
// them in closed form:
//   funnel  : examples/funnel/main.py:28-54 (v = theta[D-1], sigma = p0)
//   logreg  : sum_n [y_n a_n - log(1+e^a_n)] + log N(beta; 0, p0*I), a = X beta;
//             Fisher G = X^T Lambda X + I/p0
//   hier    : theta = [theta_1..theta_J, mu, v]; y_j ~ N(theta_j, s_j^2),
//             theta_j ~ N(mu, e^v), mu ~ N(0, p0^2), v ~ N(0, p1^2);
//             arrowhead Fisher metric
// Scalars that sum many terms (log densities) are accumulated in float64.
#pragma once

#include "common.cuh"

namespace gj {

__host__ __device__ inline bool metric_is_diag(int metric) {
  return metric == GJ_METRIC_DIAG_FISHER;
}

// ---------------------------------------------------------------------------
// log density and gradient
// ---------------------------------------------------------------------------
template <typename T>
__device__ __noinline__ double logdensity_grad(const TargetDev& t, const T* q, T* g) {
  const int d = t.d;
  if (t.family == GJ_FUNNEL) {
    const T v = q[d - 1];
    const T ev = dexp<T>(-v);
    const double s = t.p0;
    T sx = 0;
    for (int i = 0; i < d - 1; ++i) {
      sx += q[i] * q[i];
      g[i] = -q[i] * ev;
    }
    g[d - 1] = T(-double(v) / (s * s) - 0.5 * (d - 1)) + T(0.5) * ev * sx;
    // norm.logpdf(v;0,s) + sum norm.logpdf(x_i;0,e^{v/2})
    double ld = -0.5 * double(v) * double(v) / (s * s) - log(s) - 0.5 * kLog2Pi;
    ld += -0.5 * double(ev) * double(sx) - (d - 1) * (0.5 * double(v) + 0.5 * kLog2Pi);
    return ld;
  } else if (t.family == GJ_LOGREG) {
    const T* X = static_cast<const T*>(t.X);
    const T* y = static_cast<const T*>(t.y);
    const double pv = t.p0;
    for (int k = 0; k < d; ++k) g[k] = T(0);
    double ld = 0.0;
    for (int n = 0; n < t.n; ++n) {
      const T* x = X + (size_t)n * d;
      T a = 0;
      for (int k = 0; k < d; ++k) a += x[k] * q[k];
      const T sg = dsigmoid<T>(a);
      const T r = y[n] - sg;
      ld += double(y[n]) * double(a) - double(dlog1pexp<T>(a));
      for (int k = 0; k < d; ++k) g[k] += r * x[k];
    }
    double qq = 0.0;
    for (int k = 0; k < d; ++k) {
      qq += double(q[k]) * double(q[k]);
      g[k] -= q[k] * T(1.0 / pv);
    }
    ld += -0.5 * qq / pv - 0.5 * d * (kLog2Pi + log(pv));
    return ld;
  } else {  // GJ_HIERGAUSS
    const int J = t.n;
    const T* y = static_cast<const T*>(t.y);
    const T* sg = static_cast<const T*>(t.s);
    const T mu = q[J], v = q[J + 1];
    const T ev = dexp<T>(-v);
    const double sm = t.p0, sv = t.p1;
    T sr = 0, srr = 0;
    double ld = 0.0;
    for (int j = 0; j < J; ++j) {
      const T r = q[j] - mu;
      const T e = y[j] - q[j];
      const T is2 = T(1) / (sg[j] * sg[j]);
      g[j] = e * is2 - r * ev;
      sr += r;
      srr += r * r;
      ld += -0.5 * double(e) * double(e) * double(is2) - log(double(sg[j])) - 0.5 * kLog2Pi;
    }
    ld += -0.5 * double(ev) * double(srr) - J * (0.5 * double(v) + 0.5 * kLog2Pi);
    ld += -0.5 * double(mu) * double(mu) / (sm * sm) - log(sm) - 0.5 * kLog2Pi;
    ld += -0.5 * double(v) * double(v) / (sv * sv) - log(sv) - 0.5 * kLog2Pi;
    g[J] = sr * ev - mu * T(1.0 / (sm * sm));
    g[J + 1] = T(0.5) * ev * srr - T(0.5 * J) - v * T(1.0 / (sv * sv));
    return ld;
  }
}

// ---------------------------------------------------------------------------
// Hessian-vector product of the log density (util.py:120-121)
// ---------------------------------------------------------------------------
template <typename T>
__device__ __noinline__ void hvp(const TargetDev& t, const T* q, const T* u, T* out) {
  const int d = t.d;
  if (t.family == GJ_FUNNEL) {
    const T v = q[d - 1];
    const T ev = dexp<T>(-v);
    const T uv = u[d - 1];
    T sx = 0, xu = 0;
    for (int i = 0; i < d - 1; ++i) {
      sx += q[i] * q[i];
      xu += q[i] * u[i];
      out[i] = ev * (-u[i] + q[i] * uv);
    }
    out[d - 1] = ev * xu + (T(-1.0 / (t.p0 * t.p0)) - T(0.5) * ev * sx) * uv;
  } else if (t.family == GJ_LOGREG) {
    const T* X = static_cast<const T*>(t.X);
    for (int k = 0; k < d; ++k) out[k] = -u[k] * T(1.0 / t.p0);
    for (int n = 0; n < t.n; ++n) {
      const T* x = X + (size_t)n * d;
      T a = 0, xu = 0;
      for (int k = 0; k < d; ++k) {
        a += x[k] * q[k];
        xu += x[k] * u[k];
      }
      const T sg = dsigmoid<T>(a);
      const T c = -sg * (T(1) - sg) * xu;
      for (int k = 0; k < d; ++k) out[k] += c * x[k];
    }
  } else {
    const int J = t.n;
    const T* sg = static_cast<const T*>(t.s);
    const T mu = q[J], v = q[J + 1];
    const T ev = dexp<T>(-v);
    const T um = u[J], uv = u[J + 1];
    T sr = 0, srr = 0, sut = 0, sru = 0;
    for (int j = 0; j < J; ++j) {
      const T r = q[j] - mu;
      sr += r;
      srr += r * r;
      sut += u[j];
      sru += r * u[j];
      out[j] = -(T(1) / (sg[j] * sg[j]) + ev) * u[j] + ev * um + r * ev * uv;
    }
    out[J] = ev * sut + (T(-J) * ev - T(1.0 / (t.p0 * t.p0))) * um - ev * sr * uv;
    out[J + 1] = ev * sru - ev * sr * um + (T(-0.5) * ev * srr - T(1.0 / (t.p1 * t.p1))) * uv;
  }
}

// ---------------------------------------------------------------------------
// Metric G(q): diagonal metrics fill G[0..d); dense metrics fill G[d*d]
// (row-major).  Stored in float64; computed in T.
// ---------------------------------------------------------------------------
template <typename T, int DMAX>
__device__ void logreg_metric_onepass(const TargetDev& t, const T* q, double* G);

template <typename T, int DMAX>
__device__ __noinline__ void metric(const TargetDev& t, const T* q, double* G) {
  const int d = t.d;
  if (t.metric == GJ_METRIC_IDENTITY) {
    for (int i = 0; i < d * d; ++i) G[i] = 0.0;
    for (int i = 0; i < d; ++i) G[i * d + i] = 1.0;
    return;
  }
  if (t.family == GJ_FUNNEL) {
    const T v = q[d - 1];
    const T ev = dexp<T>(-v);
    if (t.metric == GJ_METRIC_DIAG_FISHER) {
      for (int i = 0; i < d - 1; ++i) G[i] = double(ev);
      G[d - 1] = 1.0 / (t.p0 * t.p0) + 0.5 * (d - 1);
      return;
    }
    // pull-back J^{-T} J^{-1}
    for (int i = 0; i < d * d; ++i) G[i] = 0.0;
    T sx = 0;
    for (int i = 0; i < d - 1; ++i) {
      G[i * d + i] = double(ev);
      const T c = T(-0.5) * ev * q[i];
      G[i * d + d - 1] = double(c);
      G[(d - 1) * d + i] = double(c);
      sx += q[i] * q[i];
    }
    G[d * d - 1] = double(T(0.25) * ev * sx) + 1.0 / (t.p0 * t.p0);
  } else if (t.family == GJ_LOGREG) {
    logreg_metric_onepass<T, DMAX>(t, q, G);
  } else {
    const int J = t.n;
    const T* sg = static_cast<const T*>(t.s);
    const T ev = dexp<T>(-q[J + 1]);
    for (int i = 0; i < d * d; ++i) G[i] = 0.0;
    for (int j = 0; j < J; ++j) {
      G[j * d + j] = double(T(1) / (sg[j] * sg[j]) + ev);
      G[j * d + J] = -double(ev);
      G[J * d + j] = -double(ev);
    }
    G[J * d + J] = double(T(J) * ev) + 1.0 / (t.p0 * t.p0);
    G[(J + 1) * d + J + 1] = 0.5 * J + 1.0 / (t.p1 * t.p1);
  }
}

// Logistic-regression Gram in one pass over the data (used by the per-chain
// kernels instead of the entry-wise loop above when d is known to be small).
template <typename T, int DMAX>
__device__ __noinline__ void logreg_metric_onepass(const TargetDev& t, const T* q, double* G) {
  const int d = t.d;
  const T* X = static_cast<const T*>(t.X);
  T acc[DMAX * (DMAX + 1) / 2];
  const int P = d * (d + 1) / 2;
  for (int i = 0; i < P; ++i) acc[i] = T(0);
  for (int n = 0; n < t.n; ++n) {
    const T* x = X + (size_t)n * d;
    T a = 0;
    for (int m = 0; m < d; ++m) a += x[m] * q[m];
    const T sg = dsigmoid<T>(a);
    const T lam = sg * (T(1) - sg);
    int idx = 0;
    for (int j = 0; j < d; ++j) {
      const T lx = lam * x[j];
      for (int k = j; k < d; ++k) acc[idx++] += lx * x[k];
    }
  }
  int idx = 0;
  for (int j = 0; j < d; ++j)
    for (int k = j; k < d; ++k) {
      G[j * d + k] = double(acc[idx]);
      G[k * d + j] = double(acc[idx]);
      ++idx;
    }
  for (int j = 0; j < d; ++j) G[j * d + j] += 1.0 / t.p0;
}

// ∂G/∂q_k: diagonal metrics fill dG[0..d), dense fill dG[d*d].
template <typename T>
__device__ __noinline__ void metric_deriv(const TargetDev& t, const T* q, int k, double* dG) {
  const int d = t.d;
  if (t.metric == GJ_METRIC_IDENTITY) {
    for (int i = 0; i < d * d; ++i) dG[i] = 0.0;
    return;
  }
  if (t.family == GJ_FUNNEL) {
    const T ev = dexp<T>(-q[d - 1]);
    if (t.metric == GJ_METRIC_DIAG_FISHER) {
      for (int i = 0; i < d; ++i) dG[i] = 0.0;
      if (k == d - 1)
        for (int i = 0; i < d - 1; ++i) dG[i] = -double(ev);
      return;
    }
    for (int i = 0; i < d * d; ++i) dG[i] = 0.0;
    if (k < d - 1) {
      dG[k * d + d - 1] = -0.5 * double(ev);
      dG[(d - 1) * d + k] = -0.5 * double(ev);
      dG[d * d - 1] = 0.5 * double(ev * q[k]);
    } else {
      T sx = 0;
      for (int i = 0; i < d - 1; ++i) {
        dG[i * d + i] = -double(ev);
        dG[i * d + d - 1] = 0.5 * double(ev * q[i]);
        dG[(d - 1) * d + i] = 0.5 * double(ev * q[i]);
        sx += q[i] * q[i];
      }
      dG[d * d - 1] = -0.25 * double(ev * sx);
    }
  } else if (t.family == GJ_LOGREG) {
    const T* X = static_cast<const T*>(t.X);
    for (int i = 0; i < d * d; ++i) dG[i] = 0.0;
    for (int n = 0; n < t.n; ++n) {
      const T* x = X + (size_t)n * d;
      T a = 0;
      for (int m = 0; m < d; ++m) a += x[m] * q[m];
      const T sg = dsigmoid<T>(a);
      const double c = double(sg * (T(1) - sg) * (T(1) - T(2) * sg) * x[k]);
      for (int i = 0; i < d; ++i)
        for (int j = 0; j < d; ++j) dG[i * d + j] += c * double(x[i]) * double(x[j]);
    }
  } else {
    const int J = t.n;
    for (int i = 0; i < d * d; ++i) dG[i] = 0.0;
    if (k != J + 1) return;
    const double ev = double(dexp<T>(-q[J + 1]));
    for (int j = 0; j < J; ++j) {
      dG[j * d + j] = -ev;
      dG[j * d + J] = ev;
      dG[J * d + j] = ev;
    }
    dG[J * d + J] = -J * ev;
  }
}

// ∂K/∂q_k = ½ tr(G⁻¹ ∂_k G) − ½ uᵀ ∂_k G u with u = G⁻¹ p — what
// jax.grad of the Gaussian kinetic energy gives (rmhmc/integrators.py:112-114,
// rmhmc/metrics.py:60-74).  Ginv: for diagonal metrics the d reciprocals,
// for dense metrics the d*d inverse.  Closed forms per family.
template <typename T>
__device__ __noinline__ void kinetic_dq(const TargetDev& t, const T* q, const double* Ginv, const double* u,
                           double* dK) {
  const int d = t.d;
  for (int k = 0; k < d; ++k) dK[k] = 0.0;
  if (t.metric == GJ_METRIC_IDENTITY) return;
  if (t.family == GJ_FUNNEL) {
    const double ev = double(dexp<T>(-q[d - 1]));
    if (t.metric == GJ_METRIC_DIAG_FISHER) {
      // only ∂_v G_x = -e^{-v}: Σ_i (½/G_i − ½u_i²)(−e^{-v})
      double acc = 0.0;
      for (int i = 0; i < d - 1; ++i) acc += (0.5 * Ginv[i] - 0.5 * u[i] * u[i]) * (-ev);
      dK[d - 1] = acc;
      return;
    }
    const int vi = d - 1;
    double trv = 0.0, quv = 0.0, sx = 0.0, xu = 0.0, xg = 0.0, su2 = 0.0;
    for (int i = 0; i < d - 1; ++i) {
      const double x = double(q[i]);
      const double tr_k = ev * (-Ginv[i * d + vi] + 0.5 * x * Ginv[vi * d + vi]);
      const double qu_k = ev * (-u[i] * u[vi] + 0.5 * x * u[vi] * u[vi]);
      dK[i] = 0.5 * tr_k - 0.5 * qu_k;
      trv += Ginv[i * d + i];
      xg += x * Ginv[i * d + vi];
      sx += x * x;
      xu += x * u[i];
      su2 += u[i] * u[i];
    }
    const double tr_v = ev * (-trv + xg - 0.25 * sx * Ginv[vi * d + vi]);
    const double qu_v = ev * (-su2 + u[vi] * xu - 0.25 * sx * u[vi] * u[vi]);
    dK[vi] = 0.5 * tr_v - 0.5 * qu_v;
  } else if (t.family == GJ_LOGREG) {
    // ∂K/∂β_k = ½ Σ_n Λ'_n x_nk [x_nᵀG⁻¹x_n − (x_nᵀu)²]
    const T* X = static_cast<const T*>(t.X);
    for (int n = 0; n < t.n; ++n) {
      const T* x = X + (size_t)n * d;
      T a = 0;
      for (int m = 0; m < d; ++m) a += x[m] * q[m];
      const T sg = dsigmoid<T>(a);
      const double lp = double(sg * (T(1) - sg) * (T(1) - T(2) * sg));
      double w = 0.0, s = 0.0;
      for (int i = 0; i < d; ++i) {
        double gx = 0.0;
        for (int j = 0; j < d; ++j) gx += Ginv[i * d + j] * double(x[j]);
        w += double(x[i]) * gx;
        s += double(x[i]) * u[i];
      }
      const double c = 0.5 * lp * (w - s * s);
      for (int k = 0; k < d; ++k) dK[k] += c * double(x[k]);
    }
  } else {
    const int J = t.n;
    const double ev = double(dexp<T>(-q[J + 1]));
    double tr = 0.0, qu = 0.0, su = 0.0;
    for (int j = 0; j < J; ++j) {
      tr += -Ginv[j * d + j] + 2.0 * Ginv[j * d + J];
      qu += -u[j] * u[j];
      su += u[j];
    }
    tr += -J * Ginv[J * d + J];
    qu += 2.0 * u[J] * su - J * u[J] * u[J];
    dK[J + 1] = 0.5 * ev * tr - 0.5 * ev * qu;
  }
}

}  // namespace gj
