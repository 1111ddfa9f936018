// Differentiated RMHMC trajectory (generalized leapfrog) for Bayesian
// logistic regression: exact derivatives of the acceptance probability and of
// the energy error of one transition with respect to the step size h and the
// metric regulariser λ (G = XᵀΛX + λI), by forward-mode tangent propagation.
//
// With two parameters, two tangent components carried through the discrete
// trajectory (Dual<2>) give the full Jacobian at about three times the cost of
// the primal and O(1) extra memory, so no trajectory has to be stored or
// recomputed.  The fixed-point solves of the generalized leapfrog
// (Girolami & Calderhead 2011, eqs. 16-18) run a fixed number of iterations
// (K_p for the momentum half step, K_q for the position step) so that the
// computed map — and hence its derivative — does not switch iteration
// counts between neighbouring parameter values.
//
// One thread owns one chain; every scalar is float64 (S = double for the
// primal, S = Dual<2> for value + d/dh + d/dλ).  Kinetic energy, momentum
// draw and accept follow rmhmc/metrics.py:45-74 and mcmc/proposal.py:87-185.
#include "common.cuh"
#include "dual.cuh"

namespace gj {

namespace {

struct LrData {
  const double* X;
  const double* y;
  int N, d;
  double prior_var;
};

template <typename S>
__device__ S softplus_s(const S& a) {
  return value(a) > 0.0 ? a + log1p(exp(-a)) : log1p(exp(a));
}

template <typename S, int DMAX>
__device__ S lr_logdensity_grad(const LrData& D, const S* q, S* g) {
  const int d = D.d;
  const double pinv = 1.0 / D.prior_var;
  S ld = 0.0, qq = 0.0;
  for (int k = 0; k < d; ++k) {
    g[k] = q[k] * (-pinv);
    qq += q[k] * q[k];
  }
  for (int n = 0; n < D.N; ++n) {
    const double* x = D.X + (size_t)n * d;
    S a = 0.0;
    for (int k = 0; k < d; ++k) a += q[k] * x[k];
    const S sg = 1.0 / (1.0 + exp(-a));
    ld += a * D.y[n] - softplus_s(a);
    const S r = D.y[n] - sg;
    for (int k = 0; k < d; ++k) g[k] += r * x[k];
  }
  return ld - 0.5 * pinv * qq - 0.5 * d * (kLog2Pi + ::log(D.prior_var));
}

// G = Σ_n Λ_n x_n x_nᵀ + λI factored in place (lower Cholesky); log det G.
template <typename S, int DMAX>
__device__ S lr_metric_chol(const LrData& D, const S* q, const S& lam, S* L) {
  const int d = D.d;
  for (int i = 0; i < d * d; ++i) L[i] = 0.0;
  for (int n = 0; n < D.N; ++n) {
    const double* x = D.X + (size_t)n * d;
    S a = 0.0;
    for (int k = 0; k < d; ++k) a += q[k] * x[k];
    const S sg = 1.0 / (1.0 + exp(-a));
    const S lamn = sg * (1.0 - sg);
    for (int i = 0; i < d; ++i) {
      const S li = lamn * x[i];
      for (int j = 0; j <= i; ++j) L[i * d + j] += li * x[j];
    }
  }
  S logdet = 0.0;
  for (int j = 0; j < d; ++j) {
    S s = L[j * d + j] + lam;
    for (int k = 0; k < j; ++k) s -= L[j * d + k] * L[j * d + k];
    const S ljj = sqrt(s);
    L[j * d + j] = ljj;
    logdet += 2.0 * log(ljj);
    for (int i = j + 1; i < d; ++i) {
      S t = L[i * d + j];
      for (int k = 0; k < j; ++k) t -= L[i * d + k] * L[j * d + k];
      L[i * d + j] = t / ljj;
    }
  }
  return logdet;
}

template <typename S>
__device__ void chol_fwd_s(const S* L, int d, const S* b, S* y) {
  for (int i = 0; i < d; ++i) {
    S s = b[i];
    for (int k = 0; k < i; ++k) s -= L[i * d + k] * y[k];
    y[i] = s / L[i * d + i];
  }
}
template <typename S>
__device__ void chol_bwd_s(const S* L, int d, const S* y, S* x) {
  for (int i = d - 1; i >= 0; --i) {
    S s = y[i];
    for (int k = i + 1; k < d; ++k) s -= L[k * d + i] * x[k];
    x[i] = s / L[i * d + i];
  }
}

// u = G⁻¹ p and G⁻¹ (dense) from the factor
template <typename S, int DMAX>
__device__ void chol_solve_inv(const S* L, int d, const S* p, S* u, S* Ginv) {
  S y[DMAX], e[DMAX];
  chol_fwd_s(L, d, p, y);
  chol_bwd_s(L, d, y, u);
  if (!Ginv) return;
  for (int c = 0; c < d; ++c) {
    for (int i = 0; i < d; ++i) e[i] = (i == c) ? S(1.0) : S(0.0);
    chol_fwd_s(L, d, e, y);
    chol_bwd_s(L, d, y, e);
    for (int i = 0; i < d; ++i) Ginv[i * d + c] = e[i];
  }
}

// ∂K/∂q_k = ½ Σ_n Λ'_n x_nk [x_nᵀG⁻¹x_n − (x_nᵀu)²]
template <typename S, int DMAX>
__device__ void lr_dK(const LrData& D, const S* q, const S* Ginv, const S* u, S* dK) {
  const int d = D.d;
  for (int k = 0; k < d; ++k) dK[k] = 0.0;
  for (int n = 0; n < D.N; ++n) {
    const double* x = D.X + (size_t)n * d;
    S a = 0.0, s = 0.0, w = 0.0;
    for (int k = 0; k < d; ++k) {
      a += q[k] * x[k];
      s += u[k] * x[k];
    }
    for (int i = 0; i < d; ++i) {
      S gx = 0.0;
      for (int j = 0; j < d; ++j) gx += Ginv[i * d + j] * x[j];
      w += gx * x[i];
    }
    const S sg = 1.0 / (1.0 + exp(-a));
    const S lp = sg * (1.0 - sg) * (1.0 - 2.0 * sg);
    const S c = 0.5 * lp * (w - s * s);
    for (int k = 0; k < d; ++k) dK[k] += c * x[k];
  }
}

template <typename S, int DMAX>
__device__ S kinetic(const S* L, int d, const S& logdet, const S* p) {
  S y[DMAX];
  chol_fwd_s(L, d, p, y);
  S quad = 0.0;
  for (int i = 0; i < d; ++i) quad += y[i] * y[i];
  return 0.5 * quad + 0.5 * logdet + 0.5 * d * kLog2Pi;
}

template <typename S, int DMAX>
__global__ void gl_trajectory_kernel(LrData D, int C, const double* q0, const double* z, double h,
                                     double lam, int Lsteps, int Kp, int Kq, double* out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  const int d = D.d;
  S hs, ls;
  if constexpr (sizeof(S) == sizeof(double)) {
    hs = S(h);
    ls = S(lam);
  } else {
    hs = S::seed(h, 0);
    ls = S::seed(lam, 1);
  }
  const S hh = 0.5 * hs;
  S q[DMAX], p[DMAX], g[DMAX], L[DMAX * DMAX], Gi[DMAX * DMAX], u[DMAX], dK[DMAX], q0s[DMAX],
      p0s[DMAX], xn[DMAX], u0[DMAX];
  for (int i = 0; i < d; ++i) q[i] = q0[(size_t)c * d + i];
  S ld = lr_logdensity_grad<S, DMAX>(D, q, g);
  // momentum p = chol(G(q0))·z (rmhmc/metrics.py:45-58)
  S logdet = lr_metric_chol<S, DMAX>(D, q, ls, L);
  for (int i = 0; i < d; ++i) {
    S s = 0.0;
    for (int k = 0; k <= i; ++k) s += L[i * d + k] * z[(size_t)c * d + k];
    p[i] = s;
  }
  const S H0 = -ld + kinetic<S, DMAX>(L, d, logdet, p);
  for (int step = 0; step < Lsteps; ++step) {
    for (int i = 0; i < d; ++i) {
      q0s[i] = q[i];
      p0s[i] = p[i];
    }
    // (1) p½ = p − h/2 (∂_qK(q, p½) − ∇ℓ(q)); metric at q fixed
    lr_metric_chol<S, DMAX>(D, q0s, ls, L);
    for (int it = 0; it < Kp; ++it) {
      chol_solve_inv<S, DMAX>(L, d, p, u, Gi);
      lr_dK<S, DMAX>(D, q0s, Gi, u, dK);
      for (int i = 0; i < d; ++i) xn[i] = p0s[i] - hh * (dK[i] - g[i]);
      for (int i = 0; i < d; ++i) p[i] = xn[i];
    }
    chol_solve_inv<S, DMAX>(L, d, p, u0, nullptr);
    // (2) q' = q + h/2 [G⁻¹(q) + G⁻¹(q')] p½
    for (int it = 0; it < Kq; ++it) {
      lr_metric_chol<S, DMAX>(D, q, ls, L);
      chol_solve_inv<S, DMAX>(L, d, p, u, nullptr);
      for (int i = 0; i < d; ++i) xn[i] = q0s[i] + hh * (u0[i] + u[i]);
      for (int i = 0; i < d; ++i) q[i] = xn[i];
    }
    // (3) p' = p½ − h/2 (∂_qK(q', p½) − ∇ℓ(q'))
    ld = lr_logdensity_grad<S, DMAX>(D, q, g);
    lr_metric_chol<S, DMAX>(D, q, ls, L);
    chol_solve_inv<S, DMAX>(L, d, p, u, Gi);
    lr_dK<S, DMAX>(D, q, Gi, u, dK);
    for (int i = 0; i < d; ++i) p[i] = p[i] - hh * (dK[i] - g[i]);
  }
  logdet = lr_metric_chol<S, DMAX>(D, q, ls, L);
  const S H1 = -ld + kinetic<S, DMAX>(L, d, logdet, p);
  const S dH = H1 - H0;  // energy error of the proposal
  // p_accept = min(exp(H0 − H1), 1): derivative zero where clipped
  S pa = exp(-dH);
  if (value(pa) >= 1.0) pa = S(1.0);
  double* o = out + (size_t)c * 6;
  if constexpr (sizeof(S) == sizeof(double)) {
    o[0] = value(pa);
    o[3] = value(dH);
    o[1] = o[2] = o[4] = o[5] = 0.0;
  } else {
    o[0] = pa.v;
    o[1] = pa.t[0];
    o[2] = pa.t[1];
    o[3] = dH.v;
    o[4] = dH.t[0];
    o[5] = dH.t[1];
  }
}

}  // namespace

cudaError_t launch_gl_trajectory_jvp(const double* X, const double* y, int N, int d,
                                     double prior_var, int C, const double* q0, const double* z,
                                     double h, double lam, int L, int Kp, int Kq, int tangents,
                                     double* out, cudaStream_t st) {
  LrData D{X, y, N, d, prior_var};
  const int tpb = 32;
  const dim3 grid((C + tpb - 1) / tpb);
  if (d <= 8) {
    if (tangents)
      gl_trajectory_kernel<Dual<2>, 8><<<grid, tpb, 0, st>>>(D, C, q0, z, h, lam, L, Kp, Kq, out);
    else
      gl_trajectory_kernel<double, 8><<<grid, tpb, 0, st>>>(D, C, q0, z, h, lam, L, Kp, Kq, out);
  } else if (d <= 16) {
    if (tangents)
      gl_trajectory_kernel<Dual<2>, 16><<<grid, tpb, 0, st>>>(D, C, q0, z, h, lam, L, Kp, Kq, out);
    else
      gl_trajectory_kernel<double, 16><<<grid, tpb, 0, st>>>(D, C, q0, z, h, lam, L, Kp, Kq, out);
  } else {
    return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace gj
