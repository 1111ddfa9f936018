// Per-chain kernels: one thread owns one chain for a whole transition.
//
// This is the "plain per-chain" form of every sampler and target family
// (precision float64 or mixed), and the path for small-d targets:
//   rmhmc_chain_kernel    rmhmc/rmhmc.py:131-174 + rmhmc_proposal :376-440,
//                          integrators rmhmc/integrators.py:53-156 (implicit
//                          midpoint) or the generalized leapfrog
//                          (Girolami & Calderhead 2011, eqs. 16-18)
//   lmc_chain_kernel      lmcmc/lmc.py:135-180, lmcmc/integrators.py:51-144,
//                          lmcmc/metrics.py:75-219
//   monge_chain_kernel    lmcmonge/lmc.py:151-236, lmcmonge/integrators.py:52-194,
//                          lmcmonge/metrics.py:44-284
//   operator kernels      value_and_grad, hvp, metric
// Chain state lives in per-thread arrays of compile-time capacity DMAX
// (registers / local memory); the metric linear algebra is float64.
#include "chain_kernels.cuh"
#include "linalg.cuh"
#include "targets.cuh"

namespace gj {

// ---------------------------------------------------------------------------
// factored metric at one position
// ---------------------------------------------------------------------------
template <int DMAX>
struct MetricEval {
  double L[DMAX * DMAX];     // diag: G_i in L[0..d); dense: Cholesky factor
  double Ginv[DMAX * DMAX];  // diag: 1/G_i; dense: inverse (when requested)
  double logdet;
  bool diag;
};

template <typename T, int DMAX>
__device__ __noinline__ void eval_metric(const TargetDev& t, const T* q, MetricEval<DMAX>& M, bool want_inv,
                            bool* bad) {
  const int d = t.d;
  M.diag = metric_is_diag(t.metric);
  metric<T, DMAX>(t, q, M.L);
  if (M.diag) {
    double ld = 0.0;
    for (int i = 0; i < d; ++i) {
      if (!(M.L[i] > 0.0)) *bad = true;
      M.Ginv[i] = 1.0 / M.L[i];
      ld += log(M.L[i]);
    }
    M.logdet = ld;
    return;
  }
  M.logdet = chol_inplace(M.L, d, bad);
  if (want_inv) {
    double e[DMAX], y[DMAX];
    chol_inverse(M.L, d, M.Ginv, e, y);
  }
}

// u = G^{-1} p
template <typename T, int DMAX>
__device__ __noinline__ void metric_solve(const MetricEval<DMAX>& M, int d, const T* p, double* u) {
  if (M.diag) {
    for (int i = 0; i < d; ++i) u[i] = M.Ginv[i] * double(p[i]);
    return;
  }
  double b[DMAX], y[DMAX];
  for (int i = 0; i < d; ++i) b[i] = double(p[i]);
  chol_fwd(M.L, d, b, y);
  chol_bwd(M.L, d, y, u);
}

// K = ½ pᵀG⁻¹p + ½ log det G + d/2 log 2π  (rmhmc/metrics.py:60-74)
template <typename T, int DMAX>
__device__ __noinline__ double kinetic_rm(const MetricEval<DMAX>& M, int d, const T* p) {
  double quad = 0.0;
  if (M.diag) {
    for (int i = 0; i < d; ++i) quad += double(p[i]) * double(p[i]) * M.Ginv[i];
  } else {
    double b[DMAX], y[DMAX];
    for (int i = 0; i < d; ++i) b[i] = double(p[i]);
    chol_fwd(M.L, d, b, y);
    for (int i = 0; i < d; ++i) quad += y[i] * y[i];
  }
  return 0.5 * quad + 0.5 * M.logdet + 0.5 * d * kLog2Pi;
}

__device__ __forceinline__ bool fp_continue(int n, int max_iters, double norm, double tol) {
  return (n < max_iters) && isfinite(norm) && (norm < 1e10) && (norm > tol);
}

// ---------------------------------------------------------------------------
// RMHMC integrators
// ---------------------------------------------------------------------------
// One evaluation of the implicit-midpoint map (rmhmc/integrators.py:119-142):
// (qo, po) = (qs + h/2 G(qi)⁻¹pi, ps − h/2 [∂_qK(qi, pi) − ∇ℓ(qi)]).
template <typename T, int DMAX>
__device__ __noinline__ void im_map(const TargetDev& t, double hh, const T* qi, const T* pi, const T* qs,
                       const T* ps, T* qo, T* po, MetricEval<DMAX>& M, bool* bad) {
  const int d = t.d;
  T gi[DMAX];
  logdensity_grad<T>(t, qi, gi);
  eval_metric<T, DMAX>(t, qi, M, true, bad);
  double u[DMAX], dK[DMAX];
  metric_solve<T, DMAX>(M, d, pi, u);
  kinetic_dq<T>(t, qi, M.Ginv, u, dK);
  for (int i = 0; i < d; ++i) {
    qo[i] = T(double(qs[i]) + hh * u[i]);
    po[i] = T(double(ps[i]) - hh * (dK[i] - double(gi[i])));
  }
}

template <typename T>
__device__ __forceinline__ double inf_norm2(const T* a, const T* b, const T* c, const T* e, int d) {
  double m = 0.0;
  for (int i = 0; i < d; ++i) {
    m = fmax(m, fabs(double(a[i]) - double(b[i])));
    m = fmax(m, fabs(double(c[i]) - double(e[i])));
  }
  // NaN must survive the max (jnp.max propagates NaN)
  for (int i = 0; i < d; ++i)
    if (isnan(double(a[i]) - double(b[i])) || isnan(double(c[i]) - double(e[i]))) return NAN;
  return m;
}

template <typename T>
__device__ __forceinline__ double inf_norm1(const T* a, const T* b, int d) {
  double m = 0.0;
  bool nan = false;
  for (int i = 0; i < d; ++i) {
    const double x = double(a[i]) - double(b[i]);
    nan |= isnan(x);
    m = fmax(m, fabs(x));
  }
  return nan ? NAN : m;
}

// implicit_midpoint.one_step (rmhmc/integrators.py:116-154): q, p in/out,
// g, ld out.  Returns the fixed-point iteration count; *conv = success.
template <typename T, int DMAX>
__device__ __noinline__ int im_step(const TargetDev& t, const StepDev& sp, T* q, T* p, T* g, double* ld,
                       MetricEval<DMAX>& M, bool* conv, bool* bad) {
  const int d = t.d;
  const double hh = 0.5 * sp.h;
  T q0[DMAX], p0[DMAX], qc[DMAX], pc[DMAX], qn[DMAX], pn[DMAX];
  for (int i = 0; i < d; ++i) {
    q0[i] = q[i];
    p0[i] = p[i];
  }
  im_map<T, DMAX>(t, hh, q0, p0, q0, p0, qn, pn, M, bad);  // eager first eval (:84)
  double nrm = inf_norm2(qn, q0, pn, p0, d);
  int it = 0;
  while (fp_continue(it, sp.max_iters, nrm, sp.tol)) {
    for (int i = 0; i < d; ++i) {
      qc[i] = qn[i];
      pc[i] = pn[i];
    }
    im_map<T, DMAX>(t, hh, qc, pc, q0, p0, qn, pn, M, bad);
    nrm = inf_norm2(qn, qc, pn, pc, d);
    ++it;
  }
  *conv = isfinite(nrm) && nrm <= sp.tol;
  im_map<T, DMAX>(t, hh, qn, pn, qn, pn, q, p, M, bad);  // explicit half step (:147-148)
  *ld = logdensity_grad<T>(t, q, g);
  return it;
}

// Generalized leapfrog: q, p, g (gradient at q on entry) in/out, ld out.
template <typename T, int DMAX>
__device__ __noinline__ int gl_step(const TargetDev& t, const StepDev& sp, T* q, T* p, T* g, double* ld,
                       MetricEval<DMAX>& M, bool* conv, bool* bad) {
  const int d = t.d;
  const double hh = 0.5 * sp.h;
  T p0[DMAX], q0[DMAX], xc[DMAX], xn[DMAX];
  double u[DMAX], dK[DMAX], u0[DMAX];
  for (int i = 0; i < d; ++i) {
    p0[i] = p[i];
    q0[i] = q[i];
  }
  // (1) p½ = p − h/2 ∂_qH(q, p½): the metric at q is fixed during this solve
  eval_metric<T, DMAX>(t, q0, M, true, bad);
  auto pmap = [&](const T* pi, T* po) {
    metric_solve<T, DMAX>(M, d, pi, u);
    kinetic_dq<T>(t, q0, M.Ginv, u, dK);
    for (int i = 0; i < d; ++i) po[i] = T(double(p0[i]) - hh * (dK[i] - double(g[i])));
  };
  pmap(p0, xn);
  double nrm = inf_norm1(xn, p0, d);
  int it = 0, it_total = 0;
  while (fp_continue(it, sp.max_iters, nrm, sp.tol)) {
    for (int i = 0; i < d; ++i) xc[i] = xn[i];
    pmap(xc, xn);
    nrm = inf_norm1(xn, xc, d);
    ++it;
  }
  bool ok = isfinite(nrm) && nrm <= sp.tol;
  it_total += it;
  for (int i = 0; i < d; ++i) p[i] = xn[i];  // p½
  metric_solve<T, DMAX>(M, d, p, u0);
  // (2) q' = q + h/2 [G⁻¹(q) + G⁻¹(q')] p½
  auto qmap = [&](const T* qi, T* qo) {
    eval_metric<T, DMAX>(t, qi, M, false, bad);
    metric_solve<T, DMAX>(M, d, p, u);
    for (int i = 0; i < d; ++i) qo[i] = T(double(q0[i]) + hh * (u0[i] + u[i]));
  };
  qmap(q0, xn);
  nrm = inf_norm1(xn, q0, d);
  it = 0;
  while (fp_continue(it, sp.max_iters, nrm, sp.tol)) {
    for (int i = 0; i < d; ++i) xc[i] = xn[i];
    qmap(xc, xn);
    nrm = inf_norm1(xn, xc, d);
    ++it;
  }
  ok = ok && isfinite(nrm) && nrm <= sp.tol;
  it_total += it;
  for (int i = 0; i < d; ++i) q[i] = xn[i];
  // (3) p' = p½ − h/2 ∂_qH(q', p½)
  *ld = logdensity_grad<T>(t, q, g);
  eval_metric<T, DMAX>(t, q, M, true, bad);
  metric_solve<T, DMAX>(M, d, p, u);
  kinetic_dq<T>(t, q, M.Ginv, u, dK);
  for (int i = 0; i < d; ++i) p[i] = T(double(p[i]) - hh * (dK[i] - double(g[i])));
  *conv = ok;
  return it_total;
}

template <typename T, int DMAX>
__global__ void __launch_bounds__(128) rmhmc_chain_kernel(TargetDev t, StepDev sp, T* pos, T* grad,
                                                          double* logdens, const T* z,
                                                          const double* uacc, InfoDev<T> info,
                                                          int C) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  const int d = t.d;
  T q[DMAX], p[DMAX], g[DMAX];
  for (int i = 0; i < d; ++i) {
    q[i] = pos[(size_t)c * d + i];
    g[i] = grad[(size_t)c * d + i];
  }
  const double ld0 = logdens[c];
  bool bad = false;
  MetricEval<DMAX> M;
  // momentum p = chol(G)·z or sqrt(G)⊙z (rmhmc/metrics.py:45-58, util.py:83)
  eval_metric<T, DMAX>(t, q, M, false, &bad);
  for (int i = 0; i < d; ++i) {
    if (M.diag) {
      p[i] = T(sqrt(M.L[i]) * double(z[(size_t)c * d + i]));
    } else {
      double s = 0.0;
      for (int k = 0; k <= i; ++k) s += M.L[i * d + k] * double(z[(size_t)c * d + k]);
      p[i] = T(s);
    }
    if (info.momentum) info.momentum[(size_t)c * d + i] = p[i];
  }
  const double H0 = -ld0 + kinetic_rm<T, DMAX>(M, d, p);  // hmc_energy (mcmc/metrics.py:160-166)
  double ld = ld0;
  int iters = 0;
  bool all_conv = true;
  for (int s = 0; s < sp.L; ++s) {  // static_integration (mcmc/trajectory.py:121-139)
    bool conv = true;
    if (sp.integrator == GJ_GENERALIZED_LEAPFROG)
      iters += gl_step<T, DMAX>(t, sp, q, p, g, &ld, M, &conv, &bad);
    else
      iters += im_step<T, DMAX>(t, sp, q, p, g, &ld, M, &conv, &bad);
    all_conv &= conv;
  }
  // flip_momentum (rmhmc.py:443-462) does not change K; H1 at the proposal
  eval_metric<T, DMAX>(t, q, M, false, &bad);
  const double H1 = -ld + kinetic_rm<T, DMAX>(M, d, p);
  if (info.prop_q || info.prop_v) {  // RMHMCInfo.proposal.state: q_L and −G⁻¹(q_L)p_L
    double vel[DMAX];
    metric_solve<T, DMAX>(M, d, p, vel);
    for (int i = 0; i < d; ++i) {
      if (info.prop_q) info.prop_q[(size_t)c * d + i] = q[i];
      if (info.prop_v) info.prop_v[(size_t)c * d + i] = T(-vel[i]);
    }
  }
  const AcceptOut a = metropolis(H0, H1, uacc[c], sp.div_threshold);
  if (a.accept) {
    for (int i = 0; i < d; ++i) {
      pos[(size_t)c * d + i] = q[i];
      grad[(size_t)c * d + i] = g[i];
    }
    logdens[c] = ld;
  }
  if (info.acc_rate) info.acc_rate[c] = a.p_acc;
  if (info.accepted) info.accepted[c] = a.accept;
  if (info.divergent) info.divergent[c] = a.divergent;
  if (info.energy) info.energy[c] = H1;
  if (info.fp_iters) info.fp_iters[c] = iters;
  if (info.status)
    info.status[c] = (all_conv ? 0u : GJ_CHAIN_FP_NOT_CONVERGED) |
                     (isfinite(H1) ? 0u : GJ_CHAIN_NONFINITE) | (bad ? GJ_CHAIN_NOT_SPD : 0u);
}


// ---------------------------------------------------------------------------
// iterative NUTS with the Riemannian metric (rmhmc/nuts.py), thread per chain
// ---------------------------------------------------------------------------
// One chain's trajectory: the extreme states are integrated in place (the
// subtrajectory of expansion k starts at the extreme on its side and that
// extreme becomes its last state, which is where the merged trajectory of
// mcmc/trajectory.py:635-640 ends), the momentum / velocity sums, the
// sampled proposal and the numpyro-style U-turn checkpoints
// (mcmc/termination.py:30-119).  Uniforms: u[k] the direction of expansion k,
// u[M + k] its biased merge, u[2M + 2^k − 1 + j] step j of expansion k.
constexpr int kNutsMaxDoublings = 16;

__device__ __forceinline__ double logaddexp(double a, double b) {
  if (a == -INFINITY) return b;
  if (b == -INFINITY) return a;
  const double m = fmax(a, b);
  return m + log1p(exp(-fabs(a - b)));
}
__device__ __forceinline__ double expit(double x) {
  if (x >= 0.0) return 1.0 / (1.0 + exp(-x));
  const double e = exp(x);
  return e / (1.0 + e);  // NaN stays NaN
}

// the generalized U-turn of rmhmc/metrics.py:76-118 (criterion 0 "euc",
// 1 "bet", 2 "riem")
template <int DMAX>
__device__ bool nuts_turning(int d, int crit, const double* m_l, const double* m_r,
                             const double* m_sum, const double* v_l, const double* v_r,
                             const double* v_sum) {
  const double* rho = crit == 1 ? m_sum : v_sum;
  const double* a = crit == 2 ? m_l : v_l;
  const double* b = crit == 2 ? m_r : v_r;
  double sa = 0.0, sb = 0.0;
  for (int i = 0; i < d; ++i) {
    sa += a[i] * rho[i];
    sb += b[i] * rho[i];
  }
  return sa <= 0.0 || sb <= 0.0;
}

// ---------------------------------------------------------------------------
// dense-metric LMC (lmcmc/*)
// ---------------------------------------------------------------------------
// Ω̃(q, v, h) = G + h/2·½(P1 + P2 − P3) (lmcmc/metrics.py:158-179) written
// into Om; also returns ∇ log det G (lmcmc/metrics.py:181-189) when gld != 0.
template <typename T, int DMAX>
__device__ __noinline__ void omega_tilde(const TargetDev& t, const T* q, const double* v, double h,
                            const double* G, const double* Ginv, bool diag, double* Om,
                            double* gld) {
  const int d = t.d;
  const double c = 0.25 * h;
  double dG[DMAX * DMAX];
  for (int i = 0; i < d * d; ++i) Om[i] = 0.0;
  if (diag) {
    for (int a = 0; a < d; ++a) Om[a * d + a] = G[a];
    for (int k = 0; k < d; ++k) {
      metric_deriv<T>(t, q, k, dG);  // dG[a] = ∂G_a/∂q_k
      double tr = 0.0;
      for (int a = 0; a < d; ++a) {
        Om[a * d + a] += c * dG[a] * v[k];  // P1 = diag(Σ_k ∂_kG_a v_k)
        Om[a * d + k] += c * dG[a] * v[a];  // P2[a][k] = ∂_kG_a v_a
        Om[k * d + a] -= c * dG[a] * v[a];  // −P2ᵀ
        tr += Ginv[a] * dG[a];
      }
      if (gld) gld[k] = tr;
    }
    return;
  }
  for (int i = 0; i < d * d; ++i) Om[i] = G[i];
  for (int k = 0; k < d; ++k) {
    metric_deriv<T>(t, q, k, dG);  // dG[a*d+b] = ∂G_ab/∂q_k
    double tr = 0.0;
    for (int a = 0; a < d; ++a)
      for (int b = 0; b < d; ++b) tr += Ginv[a * d + b] * dG[b * d + a];
    if (gld) gld[k] = tr;
    for (int l = 0; l < d; ++l) {
      double s2 = 0.0;
      for (int i = 0; i < d; ++i) s2 += v[i] * dG[i * d + l];
      Om[l * d + k] += c * s2;  // P2[l][k] = Σ_i v_i ∂_kG_il
      for (int j = 0; j < d; ++j) Om[l * d + j] += c * v[k] * dG[j * d + l];  // P1
    }
    for (int j = 0; j < d; ++j) {
      double s3 = 0.0;
      for (int i = 0; i < d; ++i) s3 += v[i] * dG[i * d + j];
      Om[k * d + j] -= c * s3;  // P3[k][j] = Σ_i v_i ∂_kG_ij
    }
  }
}

template <int DMAX>
struct LmcWork {
  double G[DMAX * DMAX];
  double Ginv[DMAX * DMAX];
  double Om[DMAX * DMAX];
};

// G (symmetrised), its inverse and log det at q
template <typename T, int DMAX>
__device__ __noinline__ double lmc_metric(const TargetDev& t, const T* q, LmcWork<DMAX>& W, bool diag,
                             bool* bad) {
  const int d = t.d;
  metric<T, DMAX>(t, q, W.G);
  if (diag) {
    double ld = 0.0;
    for (int i = 0; i < d; ++i) {
      if (!(W.G[i] > 0.0)) *bad = true;
      W.Ginv[i] = 1.0 / W.G[i];
      ld += log(W.G[i]);
    }
    return ld;
  }
  for (int i = 0; i < d; ++i)
    for (int j = 0; j < i; ++j) {
      const double s = 0.5 * (W.G[i * d + j] + W.G[j * d + i]);
      W.G[i * d + j] = s;
      W.G[j * d + i] = s;
    }
  for (int i = 0; i < d * d; ++i) W.Om[i] = W.G[i];
  const double ld = chol_inplace(W.Om, d, bad);
  double e[DMAX], y[DMAX];
  chol_inverse(W.Om, d, W.Ginv, e, y);
  return ld;
}

// half_step_fn (lmcmc/integrators.py:61-91); v in/out (double), J in/out.
template <typename T, int DMAX>
__device__ __noinline__ void lmc_half_step(const TargetDev& t, const T* q, double* v, double* J, const T* g,
                              double h, LmcWork<DMAX>& W, bool diag, bool* bad) {
  const int d = t.d;
  int piv[DMAX];
  double gld[DMAX], vt[DMAX];
  lmc_metric<T, DMAX>(t, q, W, diag, bad);
  omega_tilde<T, DMAX>(t, q, v, h, W.G, W.Ginv, diag, W.Om, gld);
  *J -= lu_inplace(W.Om, piv, d);
  for (int i = 0; i < d; ++i) {
    double gv = 0.0;
    if (diag) {
      gv = W.G[i] * v[i];
    } else {
      for (int j = 0; j < d; ++j) gv += W.G[i * d + j] * v[j];
    }
    const double dphi = -double(g[i]) + 0.5 * gld[i];
    vt[i] = gv - 0.5 * h * dphi;
  }
  lu_solve(W.Om, piv, d, vt);
  for (int i = 0; i < d; ++i) v[i] = vt[i];
  omega_tilde<T, DMAX>(t, q, v, -h, W.G, W.Ginv, diag, W.Om, nullptr);
  *J += lu_inplace(W.Om, piv, d);
}

// K = −½ log det G + ½ vᵀGv (lmcmc/metrics.py:93-112)
template <int DMAX>
__device__ double lmc_kinetic(const LmcWork<DMAX>& W, int d, double logdet, const double* v,
                              bool diag) {
  double quad = 0.0;
  for (int i = 0; i < d; ++i) {
    if (diag) {
      quad += W.G[i] * v[i] * v[i];
    } else {
      double s = 0.0;
      for (int j = 0; j < d; ++j) s += W.G[i * d + j] * v[j];
      quad += v[i] * s;
    }
  }
  return -0.5 * logdet + 0.5 * quad;
}

template <typename T, int DMAX>
__global__ void __launch_bounds__(128) lmc_chain_kernel(TargetDev t, StepDev sp, T* pos, T* grad,
                                                        double* logdens, double* vol,
                                                        const T* z, const double* uacc,
                                                        InfoDev<T> info, int C) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  const int d = t.d;
  const bool diag = metric_is_diag(t.metric);
  T q[DMAX], g[DMAX];
  double v[DMAX];
  for (int i = 0; i < d; ++i) {
    q[i] = pos[(size_t)c * d + i];
    g[i] = grad[(size_t)c * d + i];
  }
  const double ld0 = logdens[c];
  const double J0 = vol[c];
  bool bad = false;
  LmcWork<DMAX> W;
  // velocity v = L^{-T} z (lmcmc/metrics.py:75-91)
  double logdet = lmc_metric<T, DMAX>(t, q, W, diag, &bad);
  if (diag) {
    for (int i = 0; i < d; ++i) v[i] = double(z[(size_t)c * d + i]) / sqrt(W.G[i]);
  } else {
    double zz[DMAX];
    for (int i = 0; i < d; ++i) zz[i] = double(z[(size_t)c * d + i]);
    chol_bwd(W.Om, d, zz, v);  // W.Om holds the Cholesky factor after lmc_metric
  }
  for (int i = 0; i < d; ++i)
    if (info.momentum) info.momentum[(size_t)c * d + i] = T(v[i]);
  const double H0 = -ld0 + lmc_kinetic<DMAX>(W, d, logdet, v, diag) - J0;  // lmc_energy
  double ld = ld0, J = J0;
  for (int s = 0; s < sp.L; ++s) {  // lan_integrator.one_step (lmcmc/integrators.py:93-144)
    lmc_half_step<T, DMAX>(t, q, v, &J, g, sp.h, W, diag, &bad);
    for (int i = 0; i < d; ++i) q[i] = T(double(q[i]) + sp.h * v[i]);
    ld = logdensity_grad<T>(t, q, g);
    lmc_half_step<T, DMAX>(t, q, v, &J, g, sp.h, W, diag, &bad);
  }
  logdet = lmc_metric<T, DMAX>(t, q, W, diag, &bad);
  const double H1 = -ld + lmc_kinetic<DMAX>(W, d, logdet, v, diag) - J;
  for (int i = 0; i < d; ++i) {  // LMCInfo.proposal.state: q_L and −v_L (flip_velocity)
    if (info.prop_q) info.prop_q[(size_t)c * d + i] = q[i];
    if (info.prop_v) info.prop_v[(size_t)c * d + i] = T(-v[i]);
  }
  const AcceptOut a = metropolis(H0, H1, uacc[c], sp.div_threshold);
  if (a.accept) {
    for (int i = 0; i < d; ++i) {
      pos[(size_t)c * d + i] = q[i];
      grad[(size_t)c * d + i] = g[i];
    }
    logdens[c] = ld;
    vol[c] = J;
  }
  if (info.acc_rate) info.acc_rate[c] = a.p_acc;
  if (info.accepted) info.accepted[c] = a.accept;
  if (info.divergent) info.divergent[c] = a.divergent;
  if (info.energy) info.energy[c] = H1;
  if (info.fp_iters) info.fp_iters[c] = 0;
  if (info.status)
    info.status[c] = (isfinite(H1) ? 0u : GJ_CHAIN_NONFINITE) | (bad ? GJ_CHAIN_NOT_SPD : 0u);
}

// ---------------------------------------------------------------------------
// LMC on a Monge patch, one thread per chain (lmcmonge/*)
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ double dotd(const T* a, const T* b, int d) {
  double s = 0.0;
  for (int i = 0; i < d; ++i) s += double(a[i]) * double(b[i]);
  return s;
}

// half_step_omega (lmcmonge/integrators.py:158-194)
template <typename T, int DMAX>
__device__ __noinline__ void monge_half(double a2, T* v, double* J, const T* dl, const T* Hv, double L,
                           const T* dl_ig, const T* Hdl_ig, const T* ig_Hdl_ig, double eps,
                           int fix, int d) {
  const double det1 = 1.0 + 0.5 * eps * a2 * dotd(Hv, dl_ig, d);
  *J -= log(fabs(det1));
  const double sL = sqrt(L);
  double dphi_dl = 0.0;
  for (int i = 0; i < d; ++i) dphi_dl += (-double(dl[i]) + a2 * double(Hdl_ig[i]) / sL) * double(dl_ig[i]);
  T vt[DMAX];
  for (int i = 0; i < d; ++i) {
    const double dphi_ig = -double(dl_ig[i]) + a2 * double(ig_Hdl_ig[i]) / sL;
    vt[i] = T(double(v[i]) - 0.5 * eps * sL * (dphi_ig - a2 * dphi_dl * double(dl_ig[i])));
  }
  double corr = 0.5 * eps * dotd(vt, Hv, d) / det1;
  if (fix) corr *= a2;
  for (int i = 0; i < d; ++i) v[i] = T(double(vt[i]) - corr * double(dl_ig[i]));
  *J += log(fabs(1.0 - 0.5 * eps * a2 * dotd(Hdl_ig, v, d)));
}

template <typename T, int DMAX>
__global__ void __launch_bounds__(128) monge_chain_kernel(TargetDev t, StepDev sp, T* pos, T* grad,
                                                          double* logdens, double* vol,
                                                          const T* z, const double* uacc,
                                                          InfoDev<T> info, int C) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  const int d = t.d;
  const double a2 = sp.alpha2;
  const T* imv = static_cast<const T*>(sp.inv_mass);
  T q[DMAX], g[DMAX], v[DMAX], gn[DMAX], dl_ig[DMAX], Hdl[DMAX], igH[DMAX], hv[DMAX], im[DMAX];
  double slm = 0.0;  // Σ log M
  for (int i = 0; i < d; ++i) {
    q[i] = pos[(size_t)c * d + i];
    g[i] = grad[(size_t)c * d + i];
    im[i] = imv ? imv[i] : T(1);
    slm += -log(double(im[i]));
  }
  const double ld0 = logdens[c];
  const double J0 = vol[c];
  // setup (lmcmonge/lmc.py:177-208)
  double L = 0.0;
  for (int i = 0; i < d; ++i) L += double(im[i]) * double(g[i]) * double(g[i]);
  L = 1.0 + a2 * L;
  double sL = sqrt(L);
  for (int i = 0; i < d; ++i) {
    gn[i] = T(double(g[i]) / sL);
    dl_ig[i] = im[i] * gn[i];
  }
  hvp<T>(t, q, dl_ig, Hdl);
  for (int i = 0; i < d; ++i) {
    Hdl[i] = T(double(Hdl[i]) / sL);
    igH[i] = im[i] * Hdl[i];
  }
  // velocity: closed-form factor of diag(M⁻¹) − α² w wᵀ (lmcmonge/metrics.py:155-166)
  {
    double suf = 0.0;
    double tau_next[DMAX];
    for (int i = d - 1; i >= 0; --i) {
      const double ui = double(dl_ig[i]) / sqrt(double(im[i]));
      suf += ui * ui;
      tau_next[i] = 1.0 / L + a2 * suf - a2 * ui * ui;  // τ_{i+1}
    }
    double pre = 0.0;
    for (int i = 0; i < d; ++i) {
      const double ui = double(dl_ig[i]) / sqrt(double(im[i]));
      const double tn = tau_next[i];
      const double ta = tn + a2 * ui * ui;  // τ_i
      const double zi = double(z[(size_t)c * d + i]);
      const double y = sqrt(tn / ta) * zi - a2 * ui * pre;
      pre += ui * zi / sqrt(ta * tn);
      v[i] = T(sqrt(double(im[i])) * y);
      if (info.momentum) info.momentum[(size_t)c * d + i] = v[i];
    }
  }
  hvp<T>(t, q, v, hv);
  for (int i = 0; i < d; ++i) hv[i] = T(double(hv[i]) / sL);
  // K (lmcmonge/metrics.py:168-186) and H0 = −ℓ + K − J
  auto kinetic = [&](double Lc) {
    double vmv = 0.0;
    for (int i = 0; i < d; ++i) vmv += double(v[i]) * double(v[i]) / double(im[i]);
    const double vg = dotd(v, gn, d);
    return -0.5 * (log(Lc) + slm) + 0.5 * vmv + 0.5 * Lc * a2 * vg * vg;
  };
  const double H0 = -ld0 + kinetic(L) - J0;
  double ld = ld0, J = J0;
  for (int s = 0; s < sp.L; ++s) {  // lan_integrator.one_step (integrators.py:63-155)
    monge_half<T, DMAX>(a2, v, &J, gn, hv, L, dl_ig, Hdl, igH, sp.h, sp.alpha2_fix, d);
    for (int i = 0; i < d; ++i) q[i] = T(double(q[i]) + sp.h * double(v[i]));
    ld = logdensity_grad<T>(t, q, g);
    L = 0.0;
    for (int i = 0; i < d; ++i) L += double(im[i]) * double(g[i]) * double(g[i]);
    L = 1.0 + a2 * L;
    sL = sqrt(L);
    for (int i = 0; i < d; ++i) gn[i] = T(double(g[i]) / sL);
    hvp<T>(t, q, v, hv);
    for (int i = 0; i < d; ++i) {
      hv[i] = T(double(hv[i]) / sL);
      dl_ig[i] = im[i] * gn[i];
    }
    hvp<T>(t, q, dl_ig, Hdl);
    for (int i = 0; i < d; ++i) {
      Hdl[i] = T(double(Hdl[i]) / sL);
      igH[i] = im[i] * Hdl[i];
    }
    monge_half<T, DMAX>(a2, v, &J, gn, hv, L, dl_ig, Hdl, igH, sp.h, sp.alpha2_fix, d);
    hvp<T>(t, q, v, hv);
    for (int i = 0; i < d; ++i) hv[i] = T(double(hv[i]) / sL);
  }
  const double H1 = -ld + kinetic(L) - J;  // flip_velocity leaves K unchanged
  for (int i = 0; i < d; ++i) {  // LMCInfo.proposal.state: q_L and −v_L
    if (info.prop_q) info.prop_q[(size_t)c * d + i] = q[i];
    if (info.prop_v) info.prop_v[(size_t)c * d + i] = T(-double(v[i]));
  }
  const AcceptOut a = metropolis(H0, H1, uacc[c], sp.div_threshold);
  if (a.accept) {
    for (int i = 0; i < d; ++i) {
      pos[(size_t)c * d + i] = q[i];
      grad[(size_t)c * d + i] = T(double(gn[i]) * sL);  // lmc.py:231
    }
    logdens[c] = ld;
    vol[c] = J;
  }
  if (info.acc_rate) info.acc_rate[c] = a.p_acc;
  if (info.accepted) info.accepted[c] = a.accept;
  if (info.divergent) info.divergent[c] = a.divergent;
  if (info.energy) info.energy[c] = H1;
  if (info.fp_iters) info.fp_iters[c] = 0;
  if (info.status) info.status[c] = isfinite(H1) ? 0u : GJ_CHAIN_NONFINITE;
}

// ---------------------------------------------------------------------------
// NUTS dynamics: one integrator step of a chain's extreme state, in place.
// Each policy holds its per-chain work space and exposes, per state, the
// momentum m and velocity u in float64 for the U-turn criterion.
// ---------------------------------------------------------------------------
// RMHMC (rmhmc/nuts.py): IntegratorState (q, p, v = G⁻¹p, ℓ, ∇ℓ), energy
// −ℓ + K (mcmc/metrics.py:160-166)
template <typename T, int DMAX>
struct RmDyn {
  struct State {
    T q[DMAX], p[DMAX], g[DMAX];
    double m[DMAX], u[DMAX];
    double ld;
  };
  TargetDev t;
  StepDev sp;
  MetricEval<DMAX> Mv;
  bool bad = false, conv_all = true;
  int iters = 0;

  __device__ double start(State& s, const T* q, const T* g, double ld, double, const T* z,
                          T* draw_out) {
    const int d = t.d;
    for (int i = 0; i < d; ++i) {
      s.q[i] = q[i];
      s.g[i] = g[i];
    }
    s.ld = ld;
    // p = chol(G)·z, v = G⁻¹p (rmhmc/nuts.py:144-146)
    eval_metric<T, DMAX>(t, s.q, Mv, false, &bad);
    for (int i = 0; i < d; ++i) {
      if (Mv.diag) {
        s.p[i] = T(sqrt(Mv.L[i]) * double(z[i]));
      } else {
        double acc = 0.0;
        for (int k = 0; k <= i; ++k) acc += Mv.L[i * d + k] * double(z[k]);
        s.p[i] = T(acc);
      }
      s.m[i] = double(s.p[i]);
      if (draw_out) draw_out[i] = s.p[i];
    }
    metric_solve<T, DMAX>(Mv, d, s.p, s.u);
    return -s.ld + kinetic_rm<T, DMAX>(Mv, d, s.p);
  }
  __device__ double step(State& s, double h) {
    const int d = t.d;
    StepDev sd = sp;
    sd.h = h;
    bool conv = true;
    if (sp.integrator == GJ_GENERALIZED_LEAPFROG)
      iters += gl_step<T, DMAX>(t, sd, s.q, s.p, s.g, &s.ld, Mv, &conv, &bad);
    else
      iters += im_step<T, DMAX>(t, sd, s.q, s.p, s.g, &s.ld, Mv, &conv, &bad);
    conv_all &= conv;
    eval_metric<T, DMAX>(t, s.q, Mv, false, &bad);
    metric_solve<T, DMAX>(Mv, d, s.p, s.u);
    for (int i = 0; i < d; ++i) s.m[i] = double(s.p[i]);
    return -s.ld + kinetic_rm<T, DMAX>(Mv, d, s.p);
  }
  __device__ void store(const State& s, T* q, T* g, double* ld, double*) const {
    for (int i = 0; i < t.d; ++i) {
      q[i] = s.q[i];
      g[i] = s.g[i];
    }
    *ld = s.ld;
  }
  __device__ uint8_t status() const {
    return (conv_all ? 0u : GJ_CHAIN_FP_NOT_CONVERGED) | (bad ? GJ_CHAIN_NOT_SPD : 0u);
  }
};

// dense LMC (lmcmc/nuts.py): IntegratorState (q, Gv, v, ℓ, ∇ℓ, J), energy
// −ℓ + K − J (lmcmc/metrics.py:209-219), the lan integrator
// (lmcmc/integrators.py:93-144)
template <typename T, int DMAX>
struct LmcDyn {
  struct State {
    T q[DMAX], g[DMAX];
    double m[DMAX], u[DMAX];
    double ld, J;
  };
  TargetDev t;
  StepDev sp;
  LmcWork<DMAX> W;
  bool bad = false, conv_all = true;
  int iters = 0;

  __device__ double finish(State& s) {  // Gv and the energy at s.q (W holds G after lmc_metric)
    const int d = t.d;
    const bool diag = metric_is_diag(t.metric);
    const double logdet = lmc_metric<T, DMAX>(t, s.q, W, diag, &bad);
    for (int i = 0; i < d; ++i) {
      if (diag) {
        s.m[i] = W.G[i] * s.u[i];
      } else {
        double acc = 0.0;
        for (int k = 0; k < d; ++k) acc += W.G[i * d + k] * s.u[k];
        s.m[i] = acc;
      }
    }
    return -s.ld + lmc_kinetic<DMAX>(W, d, logdet, s.u, diag) - s.J;
  }
  __device__ double start(State& s, const T* q, const T* g, double ld, double J, const T* z,
                          T* draw_out) {
    const int d = t.d;
    const bool diag = metric_is_diag(t.metric);
    for (int i = 0; i < d; ++i) {
      s.q[i] = q[i];
      s.g[i] = g[i];
    }
    s.ld = ld;
    s.J = J;
    // v = L⁻ᵀz (lmcmc/metrics.py:75-91)
    lmc_metric<T, DMAX>(t, s.q, W, diag, &bad);
    if (diag) {
      for (int i = 0; i < d; ++i) s.u[i] = double(z[i]) / sqrt(W.G[i]);
    } else {
      double zz[DMAX];
      for (int i = 0; i < d; ++i) zz[i] = double(z[i]);
      chol_bwd(W.Om, d, zz, s.u);
    }
    for (int i = 0; i < d; ++i)
      if (draw_out) draw_out[i] = T(s.u[i]);
    return finish(s);
  }
  __device__ double step(State& s, double h) {
    const int d = t.d;
    const bool diag = metric_is_diag(t.metric);
    lmc_half_step<T, DMAX>(t, s.q, s.u, &s.J, s.g, h, W, diag, &bad);
    for (int i = 0; i < d; ++i) s.q[i] = T(double(s.q[i]) + h * s.u[i]);
    s.ld = logdensity_grad<T>(t, s.q, s.g);
    lmc_half_step<T, DMAX>(t, s.q, s.u, &s.J, s.g, h, W, diag, &bad);
    return finish(s);
  }
  __device__ void store(const State& s, T* q, T* g, double* ld, double* vol) const {
    for (int i = 0; i < t.d; ++i) {
      q[i] = s.q[i];
      g[i] = s.g[i];
    }
    *ld = s.ld;
    *vol = s.J;
  }
  __device__ uint8_t status() const { return bad ? GJ_CHAIN_NOT_SPD : 0u; }
};

// LMC-Monge (lmcmonge/nuts.py): RiemannianIntegratorState (lmcmonge/
// integrators.py:26-40), energy −ℓ + K − J (lmcmonge/metrics.py:267-284),
// momentum = the metric-vector product with the raw gradient
// (lmcmonge/metrics.py:243-255, as lmc.py:202-204 calls it)
template <typename T, int DMAX>
struct MongeDyn {
  struct State {
    T q[DMAX], v[DMAX], gn[DMAX], dl_ig[DMAX], Hdl[DMAX], igH[DMAX], hv[DMAX];
    double m[DMAX], u[DMAX];
    double ld, L, J;
  };
  TargetDev t;
  StepDev sp;
  T im[DMAX];
  double slm = 0.0;  // Σ log M
  bool bad = false, conv_all = true;
  int iters = 0;

  __device__ void init_mass() {
    const T* imv = static_cast<const T*>(sp.inv_mass);
    for (int i = 0; i < t.d; ++i) {
      im[i] = imv ? imv[i] : T(1);
      slm += -log(double(im[i]));
    }
  }
  __device__ double finish(State& s) {  // momentum, u = v and the energy
    const int d = t.d;
    const double a2 = sp.alpha2, sL = sqrt(s.L);
    double vg = 0.0, vgn = 0.0, vmv = 0.0;
    for (int i = 0; i < d; ++i) {
      vg += double(s.v[i]) * double(s.gn[i]) * sL;
      vgn += double(s.v[i]) * double(s.gn[i]);
      vmv += double(s.v[i]) * double(s.v[i]) / double(im[i]);
    }
    for (int i = 0; i < d; ++i) {
      s.u[i] = double(s.v[i]);
      s.m[i] = double(s.v[i]) / double(im[i]) + a2 * s.L * vg * double(s.gn[i]) * sL;
    }
    const double K = -0.5 * (log(s.L) + slm) + 0.5 * vmv + 0.5 * s.L * a2 * vgn * vgn;
    return -s.ld + K - s.J;
  }
  __device__ void at_q(State& s, const T* g) {  // L, normalised and weighted gradients, HVP
    const int d = t.d;
    const double a2 = sp.alpha2;
    double L = 0.0;
    for (int i = 0; i < d; ++i) L += double(im[i]) * double(g[i]) * double(g[i]);
    s.L = 1.0 + a2 * L;
    const double sL = sqrt(s.L);
    for (int i = 0; i < d; ++i) {
      s.gn[i] = T(double(g[i]) / sL);
      s.dl_ig[i] = im[i] * s.gn[i];
    }
    hvp<T>(t, s.q, s.dl_ig, s.Hdl);
    for (int i = 0; i < d; ++i) {
      s.Hdl[i] = T(double(s.Hdl[i]) / sL);
      s.igH[i] = im[i] * s.Hdl[i];
    }
  }
  __device__ void hv_at(State& s) {
    const double sL = sqrt(s.L);
    hvp<T>(t, s.q, s.v, s.hv);
    for (int i = 0; i < t.d; ++i) s.hv[i] = T(double(s.hv[i]) / sL);
  }
  __device__ double start(State& s, const T* q, const T* g, double ld, double J, const T* z,
                          T* draw_out) {
    const int d = t.d;
    const double a2 = sp.alpha2;
    init_mass();
    for (int i = 0; i < d; ++i) s.q[i] = q[i];
    s.ld = ld;
    s.J = J;
    at_q(s, g);
    // velocity: the closed-form factor of diag(M⁻¹) − α²·w·wᵀ
    // (lmcmonge/metrics.py:155-166)
    double suf = 0.0, tau_next[DMAX];
    for (int i = d - 1; i >= 0; --i) {
      const double ui = double(s.dl_ig[i]) / sqrt(double(im[i]));
      suf += ui * ui;
      tau_next[i] = 1.0 / s.L + a2 * suf - a2 * ui * ui;
    }
    double pre = 0.0;
    for (int i = 0; i < d; ++i) {
      const double ui = double(s.dl_ig[i]) / sqrt(double(im[i]));
      const double tn = tau_next[i], ta = tn + a2 * ui * ui;
      const double zi = double(z[i]);
      const double y = sqrt(tn / ta) * zi - a2 * ui * pre;
      pre += ui * zi / sqrt(ta * tn);
      s.v[i] = T(sqrt(double(im[i])) * y);
      if (draw_out) draw_out[i] = s.v[i];
    }
    hv_at(s);
    return finish(s);
  }
  __device__ double step(State& s, double h) {  // lan_integrator.one_step
    const int d = t.d;
    const double a2 = sp.alpha2;
    monge_half<T, DMAX>(a2, s.v, &s.J, s.gn, s.hv, s.L, s.dl_ig, s.Hdl, s.igH, h, sp.alpha2_fix, d);
    for (int i = 0; i < d; ++i) s.q[i] = T(double(s.q[i]) + h * double(s.v[i]));
    T g[DMAX];
    s.ld = logdensity_grad<T>(t, s.q, g);
    at_q(s, g);
    hv_at(s);
    monge_half<T, DMAX>(a2, s.v, &s.J, s.gn, s.hv, s.L, s.dl_ig, s.Hdl, s.igH, h, sp.alpha2_fix, d);
    hv_at(s);
    return finish(s);
  }
  __device__ void store(const State& s, T* q, T* g, double* ld, double* vol) const {
    const double sL = sqrt(s.L);
    for (int i = 0; i < t.d; ++i) {
      q[i] = s.q[i];
      g[i] = T(double(s.gn[i]) * sL);  // lmcmonge/nuts.py:197-203
    }
    *ld = s.ld;
    *vol = s.J;
  }
  __device__ uint8_t status() const { return 0u; }
};

// ---------------------------------------------------------------------------
// iterative NUTS (rmhmc/nuts.py, lmcmc/nuts.py, lmcmonge/nuts.py), one
// thread per chain
// ---------------------------------------------------------------------------
// A chain's trajectory: the two extreme states, integrated in place (the
// subtrajectory of expansion k starts at the extreme on its side and that
// extreme becomes its last state, which is where the merged trajectory of
// mcmc/trajectory.py:634-640 ends), the momentum and velocity sums, the
// sampled proposal and the numpyro-style U-turn checkpoints
// (mcmc/termination.py:30-119).  Uniforms: u[k] the direction of expansion
// k, u[M + k] its biased merge, u[2M + 2^k − 1 + j] step j of expansion k.
template <class Dyn, typename T, int DMAX>
__global__ void __launch_bounds__(128) nuts_kernel(TargetDev t, StepDev sp, int M, int crit, T* pos,
                                                   T* grad, double* logdens, double* vol,
                                                   const T* z, const double* uni, int U,
                                                   NutsInfoDev<T> info, int C) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  Dyn dyn;
  dyn.t = t;
  dyn.sp = sp;
  const int d = dyn.t.d;
  const double* u = uni + (size_t)c * U;
  using S = typename Dyn::State;
  S Lf;
  const double H0 = dyn.start(Lf, pos + (size_t)c * d, grad + (size_t)c * d, logdens[c],
                              vol ? vol[c] : 0.0, z + (size_t)c * d,
                              info.momentum ? info.momentum + (size_t)c * d : nullptr);
  S Rt = Lf;
  S prop = Lf;  // the sampled proposal (mcmc/proposal.py:23-38)
  double prop_E = H0, prop_w = 0.0, prop_sl = -INFINITY;
  double psum[DMAX], vsum[DMAX];
  for (int i = 0; i < d; ++i) {
    psum[i] = Lf.m[i];
    vsum[i] = Lf.u[i];
  }
  int n_states = 0;
  double ck_r[kNutsMaxDoublings][DMAX], ck_rs[kNutsMaxDoublings][DMAX];
  double ck_v[kNutsMaxDoublings][DMAX], ck_vs[kNutsMaxDoublings][DMAX];
  for (int k = 0; k < M; ++k)
    for (int i = 0; i < d; ++i) ck_r[k][i] = ck_rs[k][i] = ck_v[k][i] = ck_vs[k][i] = 0.0;
  int step = 0;
  bool div = false, turning = false;
  while (step < M && !div && !turning) {  // dynamic_multiplicative_expansion
    const int dir = u[step] < 0.5 ? 1 : -1;
    S& E = dir > 0 ? Rt : Lf;
    const int base = 2 * M + (1 << step) - 1;
    double spsum[DMAX], svsum[DMAX];
    S sub;
    double s_E = 0.0, s_w = 0.0, s_sl = 0.0;
    int s_n = 0;
    bool sdiv = false, sterm = false;
    for (int j = 0; j < (1 << step) && !sterm && !sdiv; ++j) {  // dynamic_progressive_integration
      const double H1 = dyn.step(E, dir * dyn.sp.h);
      double w = H0 - H1;  // proposal_from_energy_diff (mcmc/proposal.py:87-121)
      if (isnan(w)) w = -INFINITY;
      const double sl = fmin(w, 0.0);
      sdiv = -w > dyn.sp.div_threshold;
      bool take;
      if (j == 0) {
        for (int i = 0; i < d; ++i) {
          spsum[i] = E.m[i];
          svsum[i] = E.u[i];
        }
        s_n = 1;
        take = true;
        s_w = w;
        s_sl = sl;
      } else {  // progressive_uniform_sampling (mcmc/proposal.py:186-212)
        for (int i = 0; i < d; ++i) {
          spsum[i] += E.m[i];
          svsum[i] += E.u[i];
        }
        ++s_n;
        take = u[base + j] < expit(w - s_w);
        s_w = logaddexp(s_w, w);
        s_sl = logaddexp(s_sl, sl);
      }
      if (take) {
        sub = E;
        s_E = H1;
      }
      // iterative U-turn: checkpoint update and check (termination.py:48-119)
      const int hi = __popc((unsigned)j >> 1);
      const int lo = hi - (__ffs(~(unsigned)j) - 1) + 1;
      if (j % 2 == 0)
        for (int i = 0; i < d; ++i) {
          ck_r[hi][i] = E.m[i];
          ck_rs[hi][i] = spsum[i];
          ck_v[hi][i] = E.u[i];
          ck_vs[hi][i] = svsum[i];
        }
      for (int k = hi; k >= lo && !sterm; --k) {
        double srs[DMAX], svs[DMAX];
        for (int i = 0; i < d; ++i) {
          srs[i] = spsum[i] - ck_rs[k][i] + ck_r[k][i];
          svs[i] = svsum[i] - ck_vs[k][i] + ck_v[k][i];
        }
        sterm = nuts_turning<DMAX>(d, crit, ck_r[k], E.m, srs, ck_v[k], E.u, svs);
      }
    }
    // the expansion's proposal (mcmc/trajectory.py:609-632)
    if (sdiv || sterm) {
      prop_sl = logaddexp(prop_sl, s_sl);
    } else {  // progressive_biased_sampling (mcmc/proposal.py:215-245)
      const double pa = fmin(exp(s_w - prop_w), 1.0);
      const bool take = u[M + step] < pa;
      prop_w = logaddexp(prop_w, s_w);
      prop_sl = logaddexp(prop_sl, s_sl);
      if (take) {
        prop = sub;
        prop_E = s_E;
      }
    }
    // merge and the whole trajectory's U-turn (trajectory.py:634-650)
    for (int i = 0; i < d; ++i) {
      psum[i] += spsum[i];
      vsum[i] += svsum[i];
    }
    n_states += s_n;
    const bool whole = nuts_turning<DMAX>(d, crit, Lf.m, Rt.m, psum, Lf.u, Rt.u, vsum);
    div = sdiv;
    turning = sterm || whole;
    ++step;
  }
  double J_out = 0.0;
  dyn.store(prop, pos + (size_t)c * d, grad + (size_t)c * d, &logdens[c], &J_out);
  if (vol) vol[c] = J_out;
  if (info.left_q)
    for (int i = 0; i < d; ++i) info.left_q[(size_t)c * d + i] = Lf.q[i];
  if (info.right_q)
    for (int i = 0; i < d; ++i) info.right_q[(size_t)c * d + i] = Rt.q[i];
  if (info.acc_rate) info.acc_rate[c] = exp(prop_sl) / n_states;
  if (info.divergent) info.divergent[c] = div;
  if (info.turning) info.turning[c] = turning;
  if (info.energy) info.energy[c] = prop_E;
  if (info.doublings) info.doublings[c] = step;
  if (info.steps) info.steps[c] = n_states;
  if (info.fp_iters) info.fp_iters[c] = dyn.iters;
  if (info.status) info.status[c] = dyn.status() | (isfinite(prop_E) ? 0u : GJ_CHAIN_NONFINITE);
}

// ---------------------------------------------------------------------------
// operator kernels
// ---------------------------------------------------------------------------
template <typename T, int DMAX>
__global__ void logdensity_grad_kernel(TargetDev t, const T* q, double* ld, T* g, double* vol,
                                       int C) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  const int d = t.d;
  T qq[DMAX], gg[DMAX];
  for (int i = 0; i < d; ++i) qq[i] = q[(size_t)c * d + i];
  const double l = logdensity_grad<T>(t, qq, gg);
  ld[c] = l;
  for (int i = 0; i < d; ++i) g[(size_t)c * d + i] = gg[i];
  if (vol) vol[c] = 0.0;
}

template <typename T, int DMAX>
__global__ void hvp_kernel(TargetDev t, const T* q, const T* u, T* out, int C) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  const int d = t.d;
  T qq[DMAX], uu[DMAX], oo[DMAX];
  for (int i = 0; i < d; ++i) {
    qq[i] = q[(size_t)c * d + i];
    uu[i] = u[(size_t)c * d + i];
  }
  hvp<T>(t, qq, uu, oo);
  for (int i = 0; i < d; ++i) out[(size_t)c * d + i] = oo[i];
}

template <typename T, int DMAX>
__global__ void metric_kernel(TargetDev t, const T* q, T* out, int C) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  const int d = t.d;
  T qq[DMAX];
  double G[DMAX * DMAX];
  for (int i = 0; i < d; ++i) qq[i] = q[(size_t)c * d + i];
  metric<T, DMAX>(t, qq, G);
  const int n = metric_is_diag(t.metric) ? d : d * d;
  for (int i = 0; i < n; ++i) out[(size_t)c * n + i] = T(G[i]);
}

// Adjoint of the metric operator: out_k = Σ_ab W_ab ∂G_ab/∂q_k (dense W is
// d x d; for diagonal metrics W holds the d cotangents of G_a) — the
// vector-Jacobian product the reference gets from jax.vjp of metric_fn.
template <typename T, int DMAX>
__global__ void metric_vjp_kernel(TargetDev t, const T* q, const T* W, T* out, int C) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  const int d = t.d;
  const bool diag = metric_is_diag(t.metric);
  const int nw = diag ? d : d * d;
  T qq[DMAX];
  double dG[DMAX * DMAX];
  for (int i = 0; i < d; ++i) qq[i] = q[(size_t)c * d + i];
  for (int k = 0; k < d; ++k) {
    metric_deriv<T>(t, qq, k, dG);
    double acc = 0.0;
    for (int i = 0; i < nw; ++i) acc += double(W[(size_t)c * nw + i]) * dG[i];
    out[(size_t)c * d + k] = T(acc);
  }
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
static inline dim3 grid_for(int C, int tpb) { return dim3((C + tpb - 1) / tpb); }

#define GJ_DISPATCH_DMAX(d, MAXD, ...)                  \
  if ((d) <= 8) {                                        \
    constexpr int DM = 8;                                \
    __VA_ARGS__;                                         \
  } else if ((d) <= 32) {                                \
    constexpr int DM = 32;                               \
    __VA_ARGS__;                                         \
  } else if ((MAXD) >= 128 && (d) <= 128) {              \
    constexpr int DM = ((MAXD) >= 128 ? 128 : 32);       \
    __VA_ARGS__;                                         \
  } else {                                               \
    return cudaErrorInvalidValue;                        \
  }

template <typename T>
cudaError_t launch_rmhmc_chain(const TargetDev& t, const StepDev& sp, T* pos, T* grad, double* ld,
                               const T* z, const double* u, const InfoDev<T>& info, int C, int tpb,
                               cudaStream_t st) {
  GJ_DISPATCH_DMAX(t.d, 32, rmhmc_chain_kernel<T, DM><<<grid_for(C, tpb), tpb, 0, st>>>(
                                t, sp, pos, grad, ld, z, u, info, C));
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_nuts(int sampler, const TargetDev& t, const StepDev& sp, int max_doublings,
                        int criterion, T* pos, T* grad, double* ld, double* vol, const T* z,
                        const double* u, int U, const NutsInfoDev<T>& info, int C, int tpb,
                        cudaStream_t st) {
  if (max_doublings < 0 || max_doublings > kNutsMaxDoublings) return cudaErrorInvalidValue;
  if (sampler == GJ_SAMPLER_RMHMC) {
    GJ_DISPATCH_DMAX(t.d, 32, {
      nuts_kernel<RmDyn<T, DM>, T, DM><<<grid_for(C, tpb), tpb, 0, st>>>(
          t, sp, max_doublings, criterion, pos, grad, ld, nullptr, z, u, U, info, C);
    });
  } else if (sampler == GJ_SAMPLER_LMC) {
    GJ_DISPATCH_DMAX(t.d, 32, {
      nuts_kernel<LmcDyn<T, DM>, T, DM><<<grid_for(C, tpb), tpb, 0, st>>>(
          t, sp, max_doublings, criterion, pos, grad, ld, vol, z, u, U, info, C);
    });
  } else {
    GJ_DISPATCH_DMAX(t.d, 32, {
      nuts_kernel<MongeDyn<T, DM>, T, DM><<<grid_for(C, tpb), tpb, 0, st>>>(
          t, sp, max_doublings, criterion, pos, grad, ld, vol, z, u, U, info, C);
    });
  }
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_lmc_chain(const TargetDev& t, const StepDev& sp, T* pos, T* grad, double* ld,
                             double* vol, const T* z, const double* u, const InfoDev<T>& info,
                             int C, int tpb, cudaStream_t st) {
  GJ_DISPATCH_DMAX(t.d, 32, lmc_chain_kernel<T, DM><<<grid_for(C, tpb), tpb, 0, st>>>(
                                t, sp, pos, grad, ld, vol, z, u, info, C));
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_monge_chain(const TargetDev& t, const StepDev& sp, T* pos, T* grad, double* ld,
                               double* vol, const T* z, const double* u, const InfoDev<T>& info,
                               int C, int tpb, cudaStream_t st) {
  GJ_DISPATCH_DMAX(t.d, 128, monge_chain_kernel<T, DM><<<grid_for(C, tpb), tpb, 0, st>>>(
                                 t, sp, pos, grad, ld, vol, z, u, info, C));
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_logdensity_grad(const TargetDev& t, const T* q, double* ld, T* g, double* vol,
                                   int C, cudaStream_t st) {
  GJ_DISPATCH_DMAX(t.d, 128, logdensity_grad_kernel<T, DM><<<grid_for(C, 128), 128, 0, st>>>(
                                 t, q, ld, g, vol, C));
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_hvp(const TargetDev& t, const T* q, const T* u, T* out, int C, cudaStream_t st) {
  GJ_DISPATCH_DMAX(t.d, 128, hvp_kernel<T, DM><<<grid_for(C, 128), 128, 0, st>>>(t, q, u, out, C));
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_metric(const TargetDev& t, const T* q, T* out, int C, cudaStream_t st) {
  GJ_DISPATCH_DMAX(t.d, 32, metric_kernel<T, DM><<<grid_for(C, 128), 128, 0, st>>>(t, q, out, C));
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_metric_vjp(const TargetDev& t, const T* q, const T* W, T* out, int C,
                              cudaStream_t st) {
  GJ_DISPATCH_DMAX(t.d, 32, metric_vjp_kernel<T, DM><<<grid_for(C, 128), 128, 0, st>>>(t, q, W, out, C));
  return cudaGetLastError();
}

#define GJ_INST(T)                                                                               \
  template cudaError_t launch_rmhmc_chain<T>(const TargetDev&, const StepDev&, T*, T*, double*,  \
                                             const T*, const double*, const InfoDev<T>&, int,   \
                                             int, cudaStream_t);                                 \
  template cudaError_t launch_nuts<T>(int, const TargetDev&, const StepDev&, int, int, T*, T*,   \
                                      double*, double*, const T*, const double*, int,           \
                                      const NutsInfoDev<T>&, int, int, cudaStream_t);           \
  template cudaError_t launch_lmc_chain<T>(const TargetDev&, const StepDev&, T*, T*, double*,    \
                                           double*, const T*, const double*, const InfoDev<T>&, \
                                           int, int, cudaStream_t);                              \
  template cudaError_t launch_monge_chain<T>(const TargetDev&, const StepDev&, T*, T*, double*,  \
                                             double*, const T*, const double*,                  \
                                             const InfoDev<T>&, int, int, cudaStream_t);         \
  template cudaError_t launch_logdensity_grad<T>(const TargetDev&, const T*, double*, T*,        \
                                                 double*, int, cudaStream_t);                    \
  template cudaError_t launch_hvp<T>(const TargetDev&, const T*, const T*, T*, int,              \
                                     cudaStream_t);                                              \
  template cudaError_t launch_metric<T>(const TargetDev&, const T*, T*, int, cudaStream_t);    \
  template cudaError_t launch_metric_vjp<T>(const TargetDev&, const T*, const T*, T*, int,      \
                                            cudaStream_t);

// compiled once per precision (GJ_CHAIN_PREC = 1: float, 2: double) so the
// two halves build in parallel
#if !defined(GJ_CHAIN_PREC) || GJ_CHAIN_PREC == 1
GJ_INST(float)
#endif
#if !defined(GJ_CHAIN_PREC) || GJ_CHAIN_PREC == 2
GJ_INST(double)
#endif

}  // namespace gj
