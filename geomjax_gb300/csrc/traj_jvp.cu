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
// One CTA of 256 threads owns one chain; every scalar is float64 (S = double
// for the primal, S = Dual<2> for value + d/dh + d/dλ).  Shared memory holds
// the packed Cholesky factor of G, the chain's vectors, three per-datum
// arrays and a 16-row tile of X; each phase (log density and gradient, Gram,
// factorisation, solves, per-datum w_n = ||L⁻¹x_n||² and Λ'_n, ∂K/∂q) is
// spread over the CTA's threads.  Kinetic energy, momentum draw and accept
// follow rmhmc/metrics.py:45-74 and mcmc/proposal.py:87-185.
#include "common.cuh"
#include "dual.cuh"

namespace gj {

namespace {

constexpr int TT = 256;  // threads per chain
constexpr int XT = 16;   // rows of X per shared-memory tile
constexpr int EPT = 9;   // Gram entries per thread: P <= 9·256 (d <= 67)

struct LrData {
  const double* X;
  const double* y;
  int N, d;
  double prior_var;
};

__device__ __forceinline__ int colstart(int k, int d) { return k * d - (k * (k - 1)) / 2; }

template <typename S>
__device__ S softplus_s(const S& a) {
  return value(a) > 0.0 ? a + log1p(exp(-a)) : log1p(exp(a));
}

__device__ __forceinline__ double shfl_down(double v, int o) {
  return __shfl_down_sync(0xffffffffu, v, o);
}
template <int K>
__device__ __forceinline__ Dual<K> shfl_down(const Dual<K>& v, int o) {
  Dual<K> r;
  r.v = __shfl_down_sync(0xffffffffu, v.v, o);
  for (int i = 0; i < K; ++i) r.t[i] = __shfl_down_sync(0xffffffffu, v.t[i], o);
  return r;
}

// sum over the CTA; every thread gets the result (red: TT/32 slots + 1)
template <typename S>
__device__ S block_sum(S v, S* red) {
  for (int o = 16; o > 0; o >>= 1) v += shfl_down(v, o);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) red[w] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    S s = red[0];
    for (int i = 1; i < TT / 32; ++i) s += red[i];
    red[TT / 32] = s;
  }
  __syncthreads();
  const S r = red[TT / 32];
  __syncthreads();
  return r;
}

// out[k] = base[k] + Σ_n A[n]·x_nk for k < d: (column, part) pairs over the
// threads, partial sums in red[part·d + k], then one thread per column
template <typename S>
__device__ void col_reduce(const LrData& D, const S* A, const S* base, S* out, S* red) {
  const int d = D.d, N = D.N;
  const int parts = TT / d;
  const int chunk = (N + parts - 1) / parts;
  for (int idx = threadIdx.x; idx < d * parts; idx += TT) {
    const int k = idx % d, part = idx / d;
    const int n0 = part * chunk, n1 = min(N, n0 + chunk);
    S s = 0.0;
    for (int n = n0; n < n1; ++n) s += A[n] * D.X[(size_t)n * d + k];
    red[part * d + k] = s;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < d; k += TT) {
    S s = base ? base[k] : S(0.0);
    for (int part = 0; part < parts; ++part) s += red[part * d + k];
    out[k] = s;
  }
  __syncthreads();
}

// shared-memory layout of one chain (offsets in S units, then the X tile)
struct Layout {
  int P, vecs, A, W, LP, red;
  size_t bytes_S, xtile;
};

template <typename S>
__host__ __device__ inline Layout layout(int d, int N) {
  Layout l;
  l.P = d * (d + 1) / 2;
  l.vecs = l.P;                  // 10 vectors of d
  l.A = l.vecs + 10 * d;         // [max(N, XT·d)] scratch per datum
  const int a = N > XT * d ? N : XT * d;
  l.W = l.A + a;                 // [N] w_n
  l.LP = l.W + N;                // [N] Λ'_n
  l.red = l.LP + N;              // [TT] reduction scratch
  l.bytes_S = (size_t)(l.red + TT) * sizeof(S);
  l.xtile = (size_t)XT * (d + 1) * sizeof(double);
  return l;
}

template <typename S>
struct Chain {
  LrData D;
  int d, N, P;
  double pinv;
  S *L, *q, *p, *g, *u, *u0, *dK, *q0s, *p0s, *y, *tmp, *A, *W, *LP, *red;
  double* Xt;  // [XT][d + 1]

  // ℓ(q) and ∇ℓ(q) into g; A holds y_n − σ_n afterwards
  __device__ S logdensity_grad() {
    S part = 0.0;
    for (int n = threadIdx.x; n < N; n += TT) {
      const double* x = D.X + (size_t)n * d;
      S a = 0.0;
      for (int k = 0; k < d; ++k) a += q[k] * x[k];
      const S sg = 1.0 / (1.0 + exp(-a));
      part += a * D.y[n] - softplus_s(a);
      A[n] = D.y[n] - sg;
    }
    S qq = 0.0;
    for (int k = threadIdx.x; k < d; k += TT) {
      qq += q[k] * q[k];
      tmp[k] = q[k] * (-pinv);
    }
    const S ld = block_sum(part, red);
    const S q2 = block_sum(qq, red);
    col_reduce(D, A, tmp, g, red);
    return ld - 0.5 * pinv * q2 - 0.5 * d * (kLog2Pi + ::log(D.prior_var));
  }

  // G(q) = Σ_n Λ_n x_n x_nᵀ + λI into L (packed), factored in place; log det G
  __device__ S metric_chol(const S& lam) {
    for (int n = threadIdx.x; n < N; n += TT) {
      const double* x = D.X + (size_t)n * d;
      S a = 0.0;
      for (int k = 0; k < d; ++k) a += q[k] * x[k];
      const S sg = 1.0 / (1.0 + exp(-a));
      A[n] = sg * (1.0 - sg);
    }
    // the thread's packed entries (row ri, column ci)
    int ri[EPT], ci[EPT];
#pragma unroll
    for (int m = 0; m < EPT; ++m) {
      const int e = threadIdx.x + m * TT;
      int k = 0, rem = e;
      while (k < d && rem >= d - k) {
        rem -= d - k;
        ++k;
      }
      ci[m] = k;
      ri[m] = k + rem;
    }
    S acc[EPT];
#pragma unroll
    for (int m = 0; m < EPT; ++m) acc[m] = 0.0;
    for (int n0 = 0; n0 < N; n0 += XT) {
      const int nr = min(XT, N - n0);
      __syncthreads();  // previous tile consumed (and A written)
      for (int t = threadIdx.x; t < nr * d; t += TT)
        Xt[(t / d) * (d + 1) + t % d] = D.X[(size_t)(n0 + t / d) * d + t % d];
      __syncthreads();
      for (int r = 0; r < nr; ++r) {
        const S lr = A[n0 + r];
        const double* xr = Xt + r * (d + 1);
#pragma unroll
        for (int m = 0; m < EPT; ++m)
          if (threadIdx.x + m * TT < P) acc[m] += lr * (xr[ri[m]] * xr[ci[m]]);
      }
    }
#pragma unroll
    for (int m = 0; m < EPT; ++m) {
      const int e = threadIdx.x + m * TT;
      if (e < P) L[e] = (ri[m] == ci[m]) ? acc[m] + lam : acc[m];
    }
    __syncthreads();
    // right-looking Cholesky of the packed lower triangle
    S logdet = 0.0;  // thread 0's copy is the result
    for (int j = 0, cj = 0; j < d; cj += d - j, ++j) {
      if (threadIdx.x == 0) {
        const S ljj = sqrt(L[cj]);
        L[cj] = ljj;
        tmp[j] = 1.0 / ljj;
        logdet += 2.0 * log(ljj);
      }
      __syncthreads();
      const S inv = tmp[j];
      for (int i = j + 1 + threadIdx.x; i < d; i += TT) L[cj + i - j] *= inv;
      __syncthreads();
      // trailing triangle, columns k > j: T pairs spread over the threads
      const int cols = d - j - 1;
      const int T = cols * (cols + 1) / 2;
      for (int m = threadIdx.x; m < T; m += TT) {
        int k = j + 1, rem = m;
        while (rem >= d - k) {
          rem -= d - k;
          ++k;
        }
        const int i = k + rem;
        L[colstart(k, d) + i - k] -= L[cj + i - j] * L[cj + k - j];
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) red[0] = logdet;
    __syncthreads();
    const S r = red[0];
    __syncthreads();
    return r;
  }

  // x = G⁻¹ b (x may alias b); also returns ||L⁻¹b||² to every thread
  __device__ S solve(const S* b, S* x, bool backward = true) {
    for (int i = threadIdx.x; i < d; i += TT) y[i] = b[i];
    __syncthreads();
    for (int j = 0, cj = 0; j < d; cj += d - j, ++j) {
      if (threadIdx.x == 0) y[j] = y[j] / L[cj];
      __syncthreads();
      const S yj = y[j];
      for (int i = j + 1 + threadIdx.x; i < d; i += TT) y[i] -= L[cj + i - j] * yj;
      __syncthreads();
    }
    S qq = 0.0;
    for (int i = threadIdx.x; i < d; i += TT) qq += y[i] * y[i];
    const S quad = block_sum(qq, red);
    if (!backward) return quad;
    for (int i = threadIdx.x; i < d; i += TT) x[i] = y[i];
    __syncthreads();
    for (int j = d - 1; j >= 0; --j) {
      if (threadIdx.x == 0) x[j] = x[j] / L[colstart(j, d)];
      __syncthreads();
      const S xj = x[j];
      for (int i = threadIdx.x; i < j; i += TT) x[i] -= L[colstart(i, d) + j - i] * xj;
      __syncthreads();
    }
    return quad;
  }

  // W[n] = ||L⁻¹x_n||², LP[n] = Λ'_n at q; A is the [d][XT] scratch of the
  // tile's forward substitutions
  __device__ void per_datum() {
    for (int n = threadIdx.x; n < N; n += TT) {
      const double* x = D.X + (size_t)n * d;
      S a = 0.0;
      for (int k = 0; k < d; ++k) a += q[k] * x[k];
      const S sg = 1.0 / (1.0 + exp(-a));
      LP[n] = sg * (1.0 - sg) * (1.0 - 2.0 * sg);
    }
    for (int n0 = 0; n0 < N; n0 += XT) {
      const int nr = min(XT, N - n0);
      __syncthreads();
      for (int t = threadIdx.x; t < d * XT; t += TT) {
        const int i = t / XT, r = t % XT;
        A[t] = (r < nr) ? S(D.X[(size_t)(n0 + r) * d + i]) : S(0.0);
      }
      __syncthreads();
      for (int k = 0, ck = 0; k < d; ck += d - k, ++k) {
        if (threadIdx.x < XT) A[k * XT + threadIdx.x] = A[k * XT + threadIdx.x] / L[ck];
        __syncthreads();
        for (int t = threadIdx.x; t < (d - k - 1) * XT; t += TT) {
          const int i = k + 1 + t / XT, r = t % XT;
          A[i * XT + r] -= L[ck + i - k] * A[k * XT + r];
        }
        __syncthreads();
      }
      if (threadIdx.x < nr) {
        S s = 0.0;
        for (int i = 0; i < d; ++i) s += A[i * XT + threadIdx.x] * A[i * XT + threadIdx.x];
        W[n0 + threadIdx.x] = s;
      }
    }
    __syncthreads();
  }

  // dK = ∂K/∂q at the per-datum arrays' position for u = G⁻¹p:
  // ½ Σ_n Λ'_n x_nk [w_n − (x_nᵀu)²]
  __device__ void kinetic_dq() {
    for (int n = threadIdx.x; n < N; n += TT) {
      const double* x = D.X + (size_t)n * d;
      S s = 0.0;
      for (int k = 0; k < d; ++k) s += u[k] * x[k];
      A[n] = 0.5 * LP[n] * (W[n] - s * s);
    }
    __syncthreads();
    col_reduce(D, A, static_cast<const S*>(nullptr), dK, red);
  }
};

template <typename S>
__global__ void __launch_bounds__(TT) gl_trajectory_kernel(LrData D, int C, const double* q0,
                                                           const double* z, double h, double lam,
                                                           int Lsteps, int Kp, int Kq,
                                                           double* out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int c = blockIdx.x;
  if (c >= C) return;
  const int d = D.d;
  const Layout ly = layout<S>(d, D.N);
  S* base = reinterpret_cast<S*>(smem_raw);
  Chain<S> ch;
  ch.D = D;
  ch.d = d;
  ch.N = D.N;
  ch.P = ly.P;
  ch.pinv = 1.0 / D.prior_var;
  ch.L = base;
  S* v = base + ly.vecs;
  ch.q = v;
  ch.p = v + d;
  ch.g = v + 2 * d;
  ch.u = v + 3 * d;
  ch.u0 = v + 4 * d;
  ch.dK = v + 5 * d;
  ch.q0s = v + 6 * d;
  ch.p0s = v + 7 * d;
  ch.y = v + 8 * d;
  ch.tmp = v + 9 * d;
  ch.A = base + ly.A;
  ch.W = base + ly.W;
  ch.LP = base + ly.LP;
  ch.red = base + ly.red;
  ch.Xt = reinterpret_cast<double*>(smem_raw + ly.bytes_S);
  S hs, ls;
  if constexpr (sizeof(S) == sizeof(double)) {
    hs = S(h);
    ls = S(lam);
  } else {
    hs = S::seed(h, 0);
    ls = S::seed(lam, 1);
  }
  const S hh = 0.5 * hs;
  for (int i = threadIdx.x; i < d; i += TT) ch.q[i] = q0[(size_t)c * d + i];
  __syncthreads();
  S ld = ch.logdensity_grad();
  // momentum p = chol(G(q0))·z (rmhmc/metrics.py:45-58)
  S logdet = ch.metric_chol(ls);
  for (int i = threadIdx.x; i < d; i += TT) {
    S s = 0.0;
    for (int k = 0; k <= i; ++k) s += ch.L[colstart(k, d) + i - k] * z[(size_t)c * d + k];
    ch.p[i] = s;
  }
  __syncthreads();
  // H0 = −ℓ + ½||L⁻¹p||² + ½ log det G + d/2 log 2π
  const S H0 = -ld + 0.5 * ch.solve(ch.p, ch.u, false) + 0.5 * logdet + 0.5 * d * kLog2Pi;
  // the factor, w and Λ' at each step's start are those of the previous
  // step's final momentum update
  ch.per_datum();
  for (int step = 0; step < Lsteps; ++step) {
    for (int i = threadIdx.x; i < d; i += TT) {
      ch.q0s[i] = ch.q[i];
      ch.p0s[i] = ch.p[i];
    }
    __syncthreads();
    // (1) p½ = p − h/2 (∂_qK(q, p½) − ∇ℓ(q)); metric at q fixed
    for (int it = 0; it < Kp; ++it) {
      ch.solve(ch.p, ch.u);
      ch.kinetic_dq();
      for (int i = threadIdx.x; i < d; i += TT) ch.p[i] = ch.p0s[i] - hh * (ch.dK[i] - ch.g[i]);
      __syncthreads();
    }
    ch.solve(ch.p, ch.u0);
    // (2) q' = q + h/2 [G⁻¹(q) + G⁻¹(q')] p½
    for (int it = 0; it < Kq; ++it) {
      ch.metric_chol(ls);
      ch.solve(ch.p, ch.u);
      for (int i = threadIdx.x; i < d; i += TT)
        ch.q[i] = ch.q0s[i] + hh * (ch.u0[i] + ch.u[i]);
      __syncthreads();
    }
    // (3) p' = p½ − h/2 (∂_qK(q', p½) − ∇ℓ(q'))
    ld = ch.logdensity_grad();
    logdet = ch.metric_chol(ls);
    ch.per_datum();
    ch.solve(ch.p, ch.u);
    ch.kinetic_dq();
    for (int i = threadIdx.x; i < d; i += TT) ch.p[i] = ch.p[i] - hh * (ch.dK[i] - ch.g[i]);
    __syncthreads();
  }
  // L holds the factor of G(q') (with no step, the initial one)
  const S H1 = -ld + 0.5 * ch.solve(ch.p, ch.u, false) + 0.5 * logdet + 0.5 * d * kLog2Pi;
  if (threadIdx.x != 0) return;
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

template <typename S>
size_t smem_bytes(int d, int N) {
  const Layout l = layout<S>(d, N);
  return l.bytes_S + l.xtile;
}

template <typename S>
cudaError_t launch_traj(const LrData& D, int C, const double* q0, const double* z, double h,
                        double lam, int L, int Kp, int Kq, double* out, cudaStream_t st) {
  const size_t smem = smem_bytes<S>(D.d, D.N);
  cudaError_t e = cudaFuncSetAttribute(gl_trajectory_kernel<S>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  gl_trajectory_kernel<S><<<C, TT, smem, st>>>(D, C, q0, z, h, lam, L, Kp, Kq, out);
  return cudaGetLastError();
}

}  // namespace

size_t gl_trajectory_smem(int d, int N, int tangents) {
  return tangents ? smem_bytes<Dual<2>>(d, N) : smem_bytes<double>(d, N);
}

cudaError_t launch_gl_trajectory_jvp(const double* X, const double* y, int N, int d,
                                     double prior_var, int C, const double* q0, const double* z,
                                     double h, double lam, int L, int Kp, int Kq, int tangents,
                                     double* out, cudaStream_t st) {
  if (d > 64 || d * (d + 1) / 2 > EPT * TT) return cudaErrorInvalidValue;
  LrData D{X, y, N, d, prior_var};
  return tangents ? launch_traj<Dual<2>>(D, C, q0, z, h, lam, L, Kp, Kq, out, st)
                  : launch_traj<double>(D, C, q0, z, h, lam, L, Kp, Kq, out, st);
}

}  // namespace gj
