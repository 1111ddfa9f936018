// Thread-local dense linear algebra in float64 for the per-chain kernels:
// Cholesky (metric momentum draw, kinetic energy log-det and solves,
// rmhmc/metrics.py:45-74,120-127; lmcmc/metrics.py:75-112) and LU with partial
// pivoting (lmcmc/integrators.py:73-89).  Row-major d x d arrays.
#pragma once

#include "common.cuh"

namespace gj {

// In-place lower Cholesky of A (lower triangle read, L written into it,
// upper triangle zeroed).  Returns log det A = 2 Σ log L_ii; sets *bad when a
// pivot is not positive (the factor is then NaN, as LAPACK-in-XLA gives).
static __device__ __noinline__ double chol_inplace(double* A, int d, bool* bad) {
  double logdet = 0.0;
  for (int j = 0; j < d; ++j) {
    double s = A[j * d + j];
    for (int k = 0; k < j; ++k) s -= A[j * d + k] * A[j * d + k];
    if (!(s > 0.0)) {
      *bad = true;
      s = NAN;
    }
    const double ljj = sqrt(s);
    A[j * d + j] = ljj;
    logdet += 2.0 * log(ljj);
    const double inv = 1.0 / ljj;
    for (int i = j + 1; i < d; ++i) {
      double t = A[i * d + j];
      for (int k = 0; k < j; ++k) t -= A[i * d + k] * A[j * d + k];
      A[i * d + j] = t * inv;
    }
    for (int k = j + 1; k < d; ++k) A[j * d + k] = 0.0;
  }
  return logdet;
}

// y = L^{-1} b (forward substitution)
static __device__ __noinline__ void chol_fwd(const double* L, int d, const double* b, double* y) {
  for (int i = 0; i < d; ++i) {
    double s = b[i];
    for (int k = 0; k < i; ++k) s -= L[i * d + k] * y[k];
    y[i] = s / L[i * d + i];
  }
}

// x = L^{-T} y (backward substitution)
static __device__ __noinline__ void chol_bwd(const double* L, int d, const double* y, double* x) {
  for (int i = d - 1; i >= 0; --i) {
    double s = y[i];
    for (int k = i + 1; k < d; ++k) s -= L[k * d + i] * x[k];
    x[i] = s / L[i * d + i];
  }
}

// Ginv = L^{-T} L^{-1}, column by column (uses y as scratch of length d)
static __device__ __noinline__ void chol_inverse(const double* L, int d, double* Ginv, double* e, double* y) {
  for (int c = 0; c < d; ++c) {
    for (int i = 0; i < d; ++i) e[i] = (i == c) ? 1.0 : 0.0;
    chol_fwd(L, d, e, y);
    chol_bwd(L, d, y, e);
    for (int i = 0; i < d; ++i) Ginv[i * d + c] = e[i];
  }
}

// In-place LU with partial pivoting; returns log|det A| = Σ log|U_ii|.
static __device__ __noinline__ double lu_inplace(double* A, int* piv, int d) {
  double logdet = 0.0;
  for (int k = 0; k < d; ++k) {
    int p = k;
    double m = fabs(A[k * d + k]);
    for (int i = k + 1; i < d; ++i) {
      const double a = fabs(A[i * d + k]);
      if (a > m) {
        m = a;
        p = i;
      }
    }
    piv[k] = p;
    if (p != k)
      for (int j = 0; j < d; ++j) {
        const double t = A[k * d + j];
        A[k * d + j] = A[p * d + j];
        A[p * d + j] = t;
      }
    const double ukk = A[k * d + k];
    logdet += log(fabs(ukk));
    const double inv = 1.0 / ukk;
    for (int i = k + 1; i < d; ++i) {
      const double l = A[i * d + k] * inv;
      A[i * d + k] = l;
      for (int j = k + 1; j < d; ++j) A[i * d + j] -= l * A[k * d + j];
    }
  }
  return logdet;
}

// Solve A x = b with the factor of lu_inplace (b overwritten by x).
static __device__ __noinline__ void lu_solve(const double* LU, const int* piv, int d, double* b) {
  for (int k = 0; k < d; ++k) {
    const int p = piv[k];
    if (p != k) {
      const double t = b[k];
      b[k] = b[p];
      b[p] = t;
    }
  }
  for (int i = 0; i < d; ++i) {
    double s = b[i];
    for (int k = 0; k < i; ++k) s -= LU[i * d + k] * b[k];
    b[i] = s;
  }
  for (int i = d - 1; i >= 0; --i) {
    double s = b[i];
    for (int k = i + 1; k < d; ++k) s -= LU[i * d + k] * b[k];
    b[i] = s / LU[i * d + i];
  }
}

}  // namespace gj
