// Dense-Fisher logistic regression, one CTA per chain.
//
// Two samplers over the target ℓ(β) = Σ_n [y_n a_n − log(1 + e^{a_n})] +
// log N(β; 0, s²I), a = Xβ, with the Fisher metric G = XᵀΛX + I/s²
// (Λ = σ(1 − σ), ∂G/∂β_k = Xᵀdiag(Λ'⊙X[:, k])X, Λ' = σ(1 − σ)(1 − 2σ)):
//
//   rmhmc_cta_kernel  rmhmc/rmhmc.py:131-174 (+ rmhmc_proposal :376-440), with
//                     the implicit midpoint (rmhmc/integrators.py:92-156) or the
//                     generalized leapfrog (Girolami & Calderhead 2011, eqs.
//                     16-18); both fixed-point half steps follow
//                     solve_fixed_point_iteration (rmhmc/integrators.py:53-89):
//                     eager first map, ∞-norm, stop at max_iters, non-finite,
//                     ≥ 1e10 or ≤ tol
//   lmc_cta_kernel    lmcmc/lmc.py:135-180 with lan_integrator
//                     (lmcmc/integrators.py:51-144): Ω̃ = G + h/4·Σ_i v_i ∂_iG
//                     (lmcmc/metrics.py:158-179; for this family ∂G is fully
//                     symmetric, so the three einsums coincide), LU with
//                     partial pivoting for log|det Ω̃| and the solve,
//                     ∇log det G = tr(G⁻¹∂_kG) (:181-189), v = L⁻ᵀz (:75-91)
//
// One CTA of 256 threads owns one chain for a whole transition.  Shared memory
// holds the packed factor of G and its inverse, the chain's vectors, the
// per-datum arrays (residual, Λ, Λ', w_n = x_nᵀG⁻¹x_n) and a 16-row tile of X;
// X itself stays in global memory (L2-resident).  Every phase is spread over
// the CTA:
//   * Gram assembly: each thread owns ≤ 9 packed entries and sweeps the X
//     tiles (smem broadcast of the tile row);
//   * right-looking Cholesky: warps over the trailing columns, lanes over rows;
//   * L⁻¹ (packed by rows): warps over columns, lanes over rows; solves are
//     then two triangular mat-vecs (threads over rows), no serial substitution;
//   * w_n = ||L⁻¹x_n||²: a half warp per datum, lanes over rows of L⁻¹;
//   * ∂K/∂q, ∇ℓ, tr(G⁻¹∂G): column reductions over n.
//
// Two instantiations: the plain FP64 form (X, state and every operation in
// float64), and the mixed form (X and state float32; the per-datum arrays,
// the Gram tiles and w_n in float32; the Gram's tile sums, the factor, L⁻¹,
// LU, solves, fixed-point iterates, convergence norms and energies float64).
#include "chain_kernels.cuh"

namespace gj {

namespace {

constexpr int TT = 256;   // threads per chain
constexpr int NW = TT / 32;
constexpr int XT = 16;    // rows of X per shared-memory tile
constexpr int EPT = 9;    // packed entries per thread: P <= 9·256 (d <= 67)
constexpr int NVEC = 16;  // d-vectors per chain
constexpr int RED = TT + 2 * NW + 2;  // reduction scratch (doubles)

__host__ __device__ __forceinline__ int colstart(int k, int d) { return k * d - (k * (k - 1)) / 2; }
__host__ __device__ __forceinline__ int rowstart(int i) { return i * (i + 1) / 2; }

struct CtaLayout {
  int P;
  int L, Li, Gp, Om, vec, red, ndouble;  // offsets in doubles
  size_t LiB, R, LAM, LP, W, A, Xt, piv, bytes;
};

template <typename B>
__host__ __device__ inline CtaLayout cta_layout(int d, int N, bool lmc) {
  CtaLayout l;
  l.P = d * (d + 1) / 2;
  int o = 0;
  l.L = o;
  o += l.P;
  l.Li = o;
  o += l.P;
  l.Gp = o;
  if (lmc) o += l.P;
  l.Om = o;
  if (lmc) o += d * d;
  l.vec = o;
  o += NVEC * d;
  l.red = o;
  o += RED;
  l.ndouble = o;
  size_t b = (size_t)o * sizeof(double);
  l.LiB = b;
  if (sizeof(B) != sizeof(double)) b += (size_t)l.P * sizeof(B);
  const int a = N > XT * d ? N : XT * d;
  l.R = b;
  b += (size_t)N * sizeof(B);
  l.LAM = b;
  b += (size_t)N * sizeof(B);
  l.LP = b;
  b += (size_t)N * sizeof(B);
  l.W = b;
  b += (size_t)N * sizeof(B);
  l.A = b;
  b += (size_t)a * sizeof(B);
  b = (b + 15) & ~(size_t)15;
  l.Xt = b;
  b += (size_t)XT * (d + 1) * sizeof(B);
  b = (b + 15) & ~(size_t)15;
  l.piv = b;
  if (lmc) b += (size_t)d * sizeof(int);
  l.bytes = (b + 15) & ~(size_t)15;
  return l;
}

__device__ __forceinline__ double nanmax(double a, double b) {
  return (a != a || b != b) ? NAN : fmax(a, b);
}

// σ(a), σ(−a) and log(1 + e^a) from e = e^{−|a|}: neither sigmoid is formed
// as 1 − the other (in float32 that costs the small one its relative accuracy)
template <typename B>
__device__ __forceinline__ void sig_pair_b(B a, B* sp, B* sm, B* softplus) {
  const B e = exp(-fabs(a));
  const B big = B(1) / (B(1) + e), small = e * big;
  *sp = a >= B(0) ? big : small;
  *sm = a >= B(0) ? small : big;
  *softplus = (a > B(0) ? a : B(0)) + log1p(e);
}

// One chain's view of its shared memory and the target.  T: dtype of X, y and
// the chain state in global memory; B: the per-datum (bulk) arithmetic.
template <typename T, typename B>
struct Cta {
  const T* X;
  const T* Y;
  int N, d, P;
  double pvar, pinv;
  double *L, *Li, *Gp, *Om, *red, *dinv;
  B *LiB, *R, *LAM, *LP, *W, *A, *Xt;
  int* piv;
  bool bad;  // a non-positive Cholesky pivot (thread 0's copy is the one read)

  __device__ void bind(unsigned char* smem, const T* X_, const T* Y_, int N_, int d_, double pvar_,
                       bool lmc) {
    X = X_;
    Y = Y_;
    N = N_;
    d = d_;
    pvar = pvar_;
    pinv = 1.0 / pvar_;
    const CtaLayout l = cta_layout<B>(d, N, lmc);
    P = l.P;
    double* D = reinterpret_cast<double*>(smem);
    L = D + l.L;
    Li = D + l.Li;
    Gp = D + l.Gp;
    Om = D + l.Om;
    red = D + l.red;
    dinv = D + l.vec;  // vector 0
    if constexpr (sizeof(B) == sizeof(double))
      LiB = reinterpret_cast<B*>(Li);
    else
      LiB = reinterpret_cast<B*>(smem + l.LiB);
    R = reinterpret_cast<B*>(smem + l.R);
    LAM = reinterpret_cast<B*>(smem + l.LAM);
    LP = reinterpret_cast<B*>(smem + l.LP);
    W = reinterpret_cast<B*>(smem + l.W);
    A = reinterpret_cast<B*>(smem + l.A);
    Xt = reinterpret_cast<B*>(smem + l.Xt);
    piv = reinterpret_cast<int*>(smem + l.piv);
    bad = false;
  }
  __device__ double* vec(double* base, int i) const { return base + (size_t)i * d; }

  // sum over the CTA, in a fixed order; every thread gets the result
  __device__ double bsum(double v) {
    v = warp_sum(v);
    __syncthreads();  // earlier readers of the slots are done
    if ((threadIdx.x & 31) == 0) red[TT + (threadIdx.x >> 5)] = v;
    __syncthreads();
    double s = 0.0;
#pragma unroll
    for (int w = 0; w < NW; ++w) s += red[TT + w];
    return s;
  }
  // NaN-propagating max over the CTA (jnp.max propagates NaN)
  __device__ double bmax(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = nanmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[TT + NW + (threadIdx.x >> 5)] = v;
    __syncthreads();
    double m = 0.0;
#pragma unroll
    for (int w = 0; w < NW; ++w) m = nanmax(m, red[TT + NW + w]);
    return m;
  }
  // a value known to thread 0, to every thread
  __device__ double bcast0(double v) {
    __syncthreads();
    if (threadIdx.x == 0) red[TT + 2 * NW] = v;
    __syncthreads();
    return red[TT + 2 * NW];
  }

  // ||a − b||∞ over d entries (NaN-propagating), to every thread
  __device__ double dist_inf(const double* a, const double* b) {
    double m = 0.0;
    for (int i = threadIdx.x; i < d; i += TT) m = nanmax(m, fabs(a[i] - b[i]));
    return bmax(m);
  }

  // the per-datum arrays at q: R = y − σ, LAM = Λ, LP = Λ'; returns the
  // log density (every thread)
  __device__ double point(const double* q) {
    double part = 0.0;
    for (int n = threadIdx.x; n < N; n += TT) {
      const T* x = X + (size_t)n * d;
      B a = B(0);
      for (int k = 0; k < d; ++k) a += B(q[k]) * B(x[k]);
      B sp, sm, spl;
      sig_pair_b(a, &sp, &sm, &spl);
      const B y = B(Y[n]);
      part += double(y * a - spl);
      R[n] = y * sm - (B(1) - y) * sp;  // y − σ(a)
      const B lam = sp * sm;
      LAM[n] = lam;
      LP[n] = lam * (sm - sp);  // Λ(1 − 2σ)
    }
    double qq = 0.0;
    for (int k = threadIdx.x; k < d; k += TT) qq += q[k] * q[k];
    const double lik = bsum(part);
    const double q2 = bsum(qq);
    return lik - 0.5 * pinv * q2 - 0.5 * d * (kLog2Pi + ::log(pvar));
  }

  // out[k] = base_scale·base[k] + Σ_n w[n]·x_nk (float64 sums), then a barrier
  __device__ void col_reduce(const B* w, double* out, const double* base, double base_scale) {
    const int parts = TT / d;
    const int chunk = (N + parts - 1) / parts;
    __syncthreads();  // w complete
    for (int idx = threadIdx.x; idx < d * parts; idx += TT) {
      const int k = idx % d, part = idx / d;
      const int n0 = part * chunk, n1 = min(N, n0 + chunk);
      double s = 0.0;
      for (int n = n0; n < n1; ++n) s += double(w[n]) * double(X[(size_t)n * d + k]);
      red[part * d + k] = s;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < d; k += TT) {
      double s = base ? base_scale * base[k] : 0.0;
      for (int part = 0; part < parts; ++part) s += red[part * d + k];
      out[k] = s;
    }
    __syncthreads();
  }

  // X rows [n0, n0 + nr) into the tile (row stride d + 1)
  __device__ void load_tile(int n0, int nr) {
    __syncthreads();  // the previous tile is consumed
    for (int t = threadIdx.x; t < nr * d; t += TT) {
      const int r = t / d, k = t - r * d;
      Xt[r * (d + 1) + k] = B(X[(size_t)n0 * d + t]);
    }
    __syncthreads();
  }

  // Σ_n w[n] x_n x_nᵀ, packed column-major lower entries e = colstart(c) +
  // r − c.  mode 0: L[e] = sum + λδ_rc (the metric, to be factored);
  // mode 1: dense Om[r][c] = Om[c][r] = Gp[e] + scale·sum.
  __device__ void gram(const B* w, int mode, double lam, double scale) {
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
    // each 16-row tile is summed in B, the tile sums in float64: a float32
    // running sum over N = 1000 positive terms drifts by ~1e-5 relative
    double acc[EPT];
#pragma unroll
    for (int m = 0; m < EPT; ++m) acc[m] = 0.0;
    for (int n0 = 0; n0 < N; n0 += XT) {
      const int nr = min(XT, N - n0);
      load_tile(n0, nr);
      B tile[EPT];
#pragma unroll
      for (int m = 0; m < EPT; ++m) tile[m] = B(0);
      for (int r = 0; r < nr; ++r) {
        const B lr = w[n0 + r];
        const B* xr = Xt + r * (d + 1);
#pragma unroll
        for (int m = 0; m < EPT; ++m)
          if (threadIdx.x + m * TT < P) tile[m] += lr * (xr[ri[m]] * xr[ci[m]]);
      }
#pragma unroll
      for (int m = 0; m < EPT; ++m) acc[m] += double(tile[m]);
    }
#pragma unroll
    for (int m = 0; m < EPT; ++m) {
      const int e = threadIdx.x + m * TT;
      if (e >= P) continue;
      if (mode == 0) {
        L[e] = acc[m] + (ri[m] == ci[m] ? lam : 0.0);
      } else {
        const double v = Gp[e] + scale * acc[m];
        Om[ri[m] * d + ci[m]] = v;
        Om[ci[m] * d + ri[m]] = v;
      }
    }
    __syncthreads();
  }

  // G(q) into L from LAM, a copy into Gp when asked; factored in place,
  // dinv = 1/diag(L), L⁻¹ into Li (and LiB); returns log det G (every thread)
  __device__ double metric_factor(bool keep_g) {
    gram(LAM, 0, pinv, 0.0);
    if (keep_g) {
      for (int e = threadIdx.x; e < P; e += TT) Gp[e] = L[e];
      __syncthreads();
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double logdet = 0.0;  // thread 0's copy
    for (int j = 0; j < d; ++j) {
      const int cj = colstart(j, d);
      if (threadIdx.x == 0) {
        double pv = L[cj];
        if (!(pv > 0.0)) {
          bad = true;
          pv = NAN;
        }
        const double ljj = sqrt(pv);
        L[cj] = ljj;
        dinv[j] = 1.0 / ljj;
        logdet += 2.0 * log(ljj);
      }
      __syncthreads();
      const double inv = dinv[j];
      for (int i = j + 1 + threadIdx.x; i < d; i += TT) L[cj + i - j] *= inv;
      __syncthreads();
      for (int k = j + 1 + warp; k < d; k += NW) {
        const double ljk = L[cj + k - j];
        const int ck = colstart(k, d);
        for (int i = k + lane; i < d; i += 32) L[ck + i - k] -= L[cj + i - j] * ljk;
      }
      __syncthreads();
    }
    // L⁻¹ column by column: warp per column, lanes over rows
    for (int j = warp; j < d; j += NW) {
      double y0 = (lane == j) ? 1.0 : 0.0, y1 = (lane + 32 == j) ? 1.0 : 0.0;
      for (int k = j; k < d; ++k) {
        const double yk = __shfl_sync(0xffffffffu, k < 32 ? y0 : y1, k & 31) * dinv[k];
        if (lane == k) y0 = yk;
        if (lane + 32 == k) y1 = yk;
        const int ck = colstart(k, d);
        if (lane > k && lane < d) y0 -= L[ck + lane - k] * yk;
        if (lane + 32 > k && lane + 32 < d) y1 -= L[ck + lane + 32 - k] * yk;
      }
      if (lane >= j && lane < d) Li[rowstart(lane) + j] = y0;
      if (lane + 32 >= j && lane + 32 < d) Li[rowstart(lane + 32) + j] = y1;
    }
    __syncthreads();
    if constexpr (sizeof(B) != sizeof(double)) {
      for (int e = threadIdx.x; e < P; e += TT) LiB[e] = B(Li[e]);
      __syncthreads();
    }
    return bcast0(logdet);
  }

  // W[n] = ||L⁻¹x_n||² = x_nᵀG⁻¹x_n: a half warp per datum, its lanes over
  // the rows i ≡ lane (mod 16) of L⁻¹
  __device__ void w_pass() {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = 2 * warp + (lane >> 4), part = lane & 15;
    for (int n0 = 0; n0 < N; n0 += XT) {
      const int nr = min(XT, N - n0);
      load_tile(n0, nr);
      B s = B(0);
      if (r < nr) {
        const B* xr = Xt + r * (d + 1);
        for (int i = part; i < d; i += 16) {
          const B* li = LiB + rowstart(i);
          B y = B(0);
          for (int k = 0; k <= i; ++k) y += li[k] * xr[k];
          s += y * y;
        }
      }
#pragma unroll
      for (int o = 8; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (part == 0 && r < nr) W[n0 + r] = s;
    }
    __syncthreads();
  }

  // y = L⁻¹b (into yv); returns ||y||² (every thread); x = L⁻ᵀy when x != 0
  __device__ double solve(const double* b, double* yv, double* x) {
    __syncthreads();  // b complete
    for (int i = threadIdx.x; i < d; i += TT) {
      const double* li = Li + rowstart(i);
      double s = 0.0;
      for (int k = 0; k <= i; ++k) s += li[k] * b[k];
      yv[i] = s;
    }
    __syncthreads();
    double qq = 0.0;
    for (int i = threadIdx.x; i < d; i += TT) qq += yv[i] * yv[i];
    const double quad = bsum(qq);
    if (x) {
      for (int k = threadIdx.x; k < d; k += TT) {
        double s = 0.0;
        for (int i = k; i < d; ++i) s += Li[rowstart(i) + k] * yv[i];
        x[k] = s;
      }
      __syncthreads();
    }
    return quad;
  }

  // dK = ∂K/∂q = ½ Σ_n Λ'_n x_n [w_n − (x_nᵀu)²] at the per-datum arrays'
  // position (rmhmc/integrators.py:111-114 through metrics.py:60-74)
  __device__ void kinetic_dq(const double* u, double* dK) {
    __syncthreads();  // u complete
    for (int n = threadIdx.x; n < N; n += TT) {
      const T* x = X + (size_t)n * d;
      B s = B(0);
      for (int k = 0; k < d; ++k) s += B(u[k]) * B(x[k]);
      A[n] = B(0.5) * LP[n] * (W[n] - s * s);
    }
    col_reduce(A, dK, nullptr, 0.0);
  }

  // ∇ℓ into g from R (point() must have run at q)
  __device__ void grad(const double* q, double* g) { col_reduce(R, g, q, -pinv); }

  // ---- dense LMC pieces -------------------------------------------------
  // tr(G⁻¹∂_kG) = Σ_n Λ'_n w_n x_nk
  __device__ void grad_logdet(double* gld) {
    for (int n = threadIdx.x; n < N; n += TT) A[n] = LP[n] * W[n];
    col_reduce(A, gld, nullptr, 0.0);
  }
  // out = G v from the packed copy Gp
  __device__ void gv(const double* v, double* out) {
    __syncthreads();
    for (int i = threadIdx.x; i < d; i += TT) {
      double s = 0.0;
      for (int j = 0; j < i; ++j) s += Gp[colstart(j, d) + i - j] * v[j];
      const int ci = colstart(i, d);
      for (int j = i; j < d; ++j) s += Gp[ci + j - i] * v[j];
      out[i] = s;
    }
    __syncthreads();
  }
  // Om = Ω̃(q, v, h) = G + h/4 Σ_n Λ'_n (x_nᵀv) x_n x_nᵀ, LU-factored in place
  // with partial pivoting (piv); returns log|det Ω̃| (every thread)
  __device__ double omega_lu(const double* v, double h) {
    __syncthreads();
    for (int n = threadIdx.x; n < N; n += TT) {
      const T* x = X + (size_t)n * d;
      B s = B(0);
      for (int k = 0; k < d; ++k) s += B(v[k]) * B(x[k]);
      A[n] = LP[n] * s;
    }
    gram(A, 1, 0.0, 0.25 * h);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double lad = 0.0;  // thread 0's copy
    for (int k = 0; k < d; ++k) {
      if (warp == 0) {  // pivot: the first row of largest |Om[i][k]|, i >= k
        double m = -1.0;
        int p = k;
        for (int i = k + lane; i < d; i += 32) {
          const double a = fabs(Om[i * d + k]);
          if (a > m) {
            m = a;
            p = i;
          }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const double m2 = __shfl_xor_sync(0xffffffffu, m, o);
          const int p2 = __shfl_xor_sync(0xffffffffu, p, o);
          if (m2 > m || (m2 == m && p2 < p)) {
            m = m2;
            p = p2;
          }
        }
        if (lane == 0) piv[k] = p;
      }
      __syncthreads();
      const int p = piv[k];
      if (p != k)
        for (int j = threadIdx.x; j < d; j += TT) {
          const double t = Om[k * d + j];
          Om[k * d + j] = Om[p * d + j];
          Om[p * d + j] = t;
        }
      __syncthreads();
      const double ukk = Om[k * d + k];
      if (threadIdx.x == 0) lad += log(fabs(ukk));
      const double inv = 1.0 / ukk;
      for (int i = k + 1 + threadIdx.x; i < d; i += TT) Om[i * d + k] *= inv;
      __syncthreads();
      const int rows = d - k - 1;
      for (int t = threadIdx.x; t < rows * rows; t += TT) {
        const int i = k + 1 + t / rows, j = k + 1 + t % rows;
        Om[i * d + j] -= Om[i * d + k] * Om[k * d + j];
      }
      __syncthreads();
    }
    return bcast0(lad);
  }
  // b = Ω̃⁻¹ b with the factor of omega_lu (one warp: pivots, then
  // column-oriented substitutions)
  __device__ void lu_solve(double* b) {
    __syncthreads();
    if (threadIdx.x < 32) {
      const int lane = threadIdx.x;
      if (lane == 0)
        for (int k = 0; k < d; ++k) {
          const int p = piv[k];
          if (p != k) {
            const double t = b[k];
            b[k] = b[p];
            b[p] = t;
          }
        }
      __syncwarp();
      double y0 = lane < d ? b[lane] : 0.0, y1 = lane + 32 < d ? b[lane + 32] : 0.0;
      for (int k = 0; k < d; ++k) {  // unit lower
        const double yk = __shfl_sync(0xffffffffu, k < 32 ? y0 : y1, k & 31);
        if (lane > k && lane < d) y0 -= Om[lane * d + k] * yk;
        if (lane + 32 > k && lane + 32 < d) y1 -= Om[(lane + 32) * d + k] * yk;
      }
      for (int k = d - 1; k >= 0; --k) {  // upper
        const double xk =
            __shfl_sync(0xffffffffu, k < 32 ? y0 : y1, k & 31) / Om[k * d + k];
        if (lane == k) y0 = xk;
        if (lane + 32 == k) y1 = xk;
        if (lane < k) y0 -= Om[lane * d + k] * xk;
        if (lane + 32 < k) y1 -= Om[(lane + 32) * d + k] * xk;
      }
      if (lane < d) b[lane] = y0;
      if (lane + 32 < d) b[lane + 32] = y1;
    }
    __syncthreads();
  }
};

__device__ __forceinline__ bool fp_go(int n, int max_iters, double norm, double tol) {
  return (n < max_iters) && isfinite(norm) && (norm < 1e10) && (norm > tol);
}

// vector slots
enum { V_DINV = 0, V_Q, V_P, V_G, V_U, V_U0, V_DK, V_QS, V_PS, V_QN, V_PN, V_Y, V_V, V_VT, V_GLD,
       V_TMP };

template <typename T, typename B>
__global__ void __launch_bounds__(TT, 3) rmhmc_cta_kernel(const T* X, const T* Y, int N, int d,
                                                          double pvar, StepDev sp, T* pos, T* grad,
                                                          double* logdens, const T* z,
                                                          const double* uacc, InfoDev<T> info,
                                                          int C) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int c = blockIdx.x;
  if (c >= C) return;
  Cta<T, B> ch;
  ch.bind(smem, X, Y, N, d, pvar, false);
  double* vb = reinterpret_cast<double*>(smem) + cta_layout<B>(d, N, false).vec;
  double* q = ch.vec(vb, V_Q);
  double* p = ch.vec(vb, V_P);
  double* g = ch.vec(vb, V_G);
  double* u = ch.vec(vb, V_U);
  double* u0 = ch.vec(vb, V_U0);
  double* dK = ch.vec(vb, V_DK);
  double* qs = ch.vec(vb, V_QS);
  double* ps = ch.vec(vb, V_PS);
  double* qn = ch.vec(vb, V_QN);
  double* pn = ch.vec(vb, V_PN);
  double* yv = ch.vec(vb, V_Y);
  const double hh = 0.5 * sp.h;
  for (int i = threadIdx.x; i < d; i += TT) {
    q[i] = double(pos[(size_t)c * d + i]);
    g[i] = double(grad[(size_t)c * d + i]);
  }
  const double ld0 = logdens[c];
  __syncthreads();
  // momentum p = chol(G(q))·z (rmhmc/metrics.py:45-58, util.py:83)
  ch.point(q);
  double logdet = ch.metric_factor(false);
  for (int i = threadIdx.x; i < d; i += TT) {
    double s = 0.0;
    for (int k = 0; k <= i; ++k) s += ch.L[colstart(k, d) + i - k] * double(z[(size_t)c * d + k]);
    p[i] = s;
    if (info.momentum) info.momentum[(size_t)c * d + i] = T(s);
  }
  // hmc_energy (mcmc/metrics.py:160-166) with K of rmhmc/metrics.py:60-74
  const double H0 = -ld0 + 0.5 * ch.solve(p, yv, nullptr) + 0.5 * logdet + 0.5 * d * kLog2Pi;
  double ld = ld0;
  int iters = 0;
  bool conv_all = true;
  const bool gl = sp.integrator == GJ_GENERALIZED_LEAPFROG;
  if (gl && sp.L > 0) ch.w_pass();  // w_n, Λ'_n at q for the first momentum solve
  for (int step = 0; step < sp.L; ++step) {
    for (int i = threadIdx.x; i < d; i += TT) {
      qs[i] = q[i];
      ps[i] = p[i];
    }
    __syncthreads();
    if (gl) {
      // (1) p½ = p − h/2 [∂_qK(q, p½) − ∇ℓ(q)]; G(q), w, Λ' and ∇ℓ(q) fixed
      ch.solve(p, yv, u);
      ch.kinetic_dq(u, dK);
      for (int i = threadIdx.x; i < d; i += TT) pn[i] = ps[i] - hh * (dK[i] - g[i]);
      double nrm = ch.dist_inf(pn, p);
      int it = 0;
      while (fp_go(it, sp.max_iters, nrm, sp.tol)) {
        for (int i = threadIdx.x; i < d; i += TT) p[i] = pn[i];
        ch.solve(p, yv, u);
        ch.kinetic_dq(u, dK);
        for (int i = threadIdx.x; i < d; i += TT) pn[i] = ps[i] - hh * (dK[i] - g[i]);
        nrm = ch.dist_inf(pn, p);
        ++it;
      }
      conv_all = conv_all && isfinite(nrm) && nrm <= sp.tol;
      iters += it;
      for (int i = threadIdx.x; i < d; i += TT) p[i] = pn[i];
      // u0 = G(q)⁻¹ p½
      ch.solve(p, yv, u0);
      // (2) q' = q + h/2 [G⁻¹(q) + G⁻¹(q')] p½: the eager map at q uses u0
      for (int i = threadIdx.x; i < d; i += TT) qn[i] = qs[i] + hh * (u0[i] + u0[i]);
      nrm = ch.dist_inf(qn, qs);
      it = 0;
      while (fp_go(it, sp.max_iters, nrm, sp.tol)) {
        for (int i = threadIdx.x; i < d; i += TT) q[i] = qn[i];
        __syncthreads();
        ch.point(q);
        ch.metric_factor(false);
        ch.solve(p, yv, u);
        for (int i = threadIdx.x; i < d; i += TT) qn[i] = qs[i] + hh * (u0[i] + u[i]);
        nrm = ch.dist_inf(qn, q);
        ++it;
      }
      conv_all = conv_all && isfinite(nrm) && nrm <= sp.tol;
      iters += it;
      for (int i = threadIdx.x; i < d; i += TT) q[i] = qn[i];
      __syncthreads();
      // (3) p' = p½ − h/2 [∂_qK(q', p½) − ∇ℓ(q')]
      ld = ch.point(q);
      ch.grad(q, g);
      logdet = ch.metric_factor(false);
      ch.w_pass();
      ch.solve(p, yv, u);
      ch.kinetic_dq(u, dK);
      for (int i = threadIdx.x; i < d; i += TT) p[i] = p[i] - hh * (dK[i] - g[i]);
      __syncthreads();
    } else {
      // implicit midpoint (rmhmc/integrators.py:116-154): the map
      // (q, p) ↦ (q_s + h/2 G(q)⁻¹p, p_s − h/2 [∂_qK(q, p) − ∇ℓ(q)])
      auto map = [&](const double* qi, const double* pi, const double* qb, const double* pb,
                     double* qo, double* po) {
        ch.point(qi);
        ch.grad(qi, g);
        ch.metric_factor(false);
        ch.w_pass();
        ch.solve(pi, yv, u);
        ch.kinetic_dq(u, dK);
        for (int i = threadIdx.x; i < d; i += TT) {
          qo[i] = qb[i] + hh * u[i];
          po[i] = pb[i] - hh * (dK[i] - g[i]);
        }
      };
      map(qs, ps, qs, ps, qn, pn);  // eager first evaluation (:84)
      double nrm = nanmax(ch.dist_inf(qn, qs), ch.dist_inf(pn, ps));
      int it = 0;
      while (fp_go(it, sp.max_iters, nrm, sp.tol)) {
        for (int i = threadIdx.x; i < d; i += TT) {
          q[i] = qn[i];
          p[i] = pn[i];
        }
        __syncthreads();
        map(q, p, qs, ps, qn, pn);
        nrm = nanmax(ch.dist_inf(qn, q), ch.dist_inf(pn, p));
        ++it;
      }
      conv_all = conv_all && isfinite(nrm) && nrm <= sp.tol;
      iters += it;
      for (int i = threadIdx.x; i < d; i += TT) {
        q[i] = qn[i];
        p[i] = pn[i];
      }
      __syncthreads();
      map(q, p, q, p, qn, pn);  // explicit half step from the midpoint (:147-148)
      __syncthreads();
      for (int i = threadIdx.x; i < d; i += TT) {
        q[i] = qn[i];
        p[i] = pn[i];
      }
      __syncthreads();
      ld = ch.point(q);
      ch.grad(q, g);
    }
  }
  // the proposal's energy: the factor of G(q_L) (the generalized leapfrog's
  // last momentum update left it in place)
  if (!gl && sp.L > 0) logdet = ch.metric_factor(false);
  const double quad = ch.solve(p, yv, u);  // u = G(q_L)⁻¹p_L
  const double H1 = -ld + 0.5 * quad + 0.5 * logdet + 0.5 * d * kLog2Pi;
  for (int i = threadIdx.x; i < d; i += TT) {  // RMHMCInfo.proposal.state (flipped)
    if (info.prop_q) info.prop_q[(size_t)c * d + i] = T(q[i]);
    if (info.prop_v) info.prop_v[(size_t)c * d + i] = T(-u[i]);
  }
  const AcceptOut a = metropolis(H0, H1, uacc[c], sp.div_threshold);
  if (a.accept) {
    for (int i = threadIdx.x; i < d; i += TT) {
      pos[(size_t)c * d + i] = T(q[i]);
      grad[(size_t)c * d + i] = T(g[i]);
    }
  }
  if (threadIdx.x != 0) return;
  if (a.accept) logdens[c] = ld;
  if (info.acc_rate) info.acc_rate[c] = a.p_acc;
  if (info.accepted) info.accepted[c] = a.accept;
  if (info.divergent) info.divergent[c] = a.divergent;
  if (info.energy) info.energy[c] = H1;
  if (info.fp_iters) info.fp_iters[c] = iters;
  if (info.status)
    info.status[c] = (conv_all ? 0u : GJ_CHAIN_FP_NOT_CONVERGED) |
                     (isfinite(H1) ? 0u : GJ_CHAIN_NONFINITE) | (ch.bad ? GJ_CHAIN_NOT_SPD : 0u);
}

// half_step_fn (lmcmc/integrators.py:61-91) at q with G(q) in Gp, its factor,
// w and Λ' current; v and J in/out
template <typename T, typename B>
__device__ void lmc_half(Cta<T, B>& ch, double* v, double* vt, double* gld, const double* g,
                         double h, double* J) {
  const int d = ch.d;
  ch.grad_logdet(gld);
  const double lad1 = ch.omega_lu(v, h);
  ch.gv(v, vt);
  for (int i = threadIdx.x; i < d; i += TT) vt[i] -= 0.5 * h * (-g[i] + 0.5 * gld[i]);
  ch.lu_solve(vt);
  for (int i = threadIdx.x; i < d; i += TT) v[i] = vt[i];
  const double lad2 = ch.omega_lu(v, -h);
  *J = *J - lad1 + lad2;
}

template <typename T, typename B>
__global__ void __launch_bounds__(TT) lmc_cta_kernel(const T* X, const T* Y, int N, int d,
                                                     double pvar, StepDev sp, T* pos, T* grad,
                                                     double* logdens, double* vol, const T* z,
                                                     const double* uacc, InfoDev<T> info, int C) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int c = blockIdx.x;
  if (c >= C) return;
  Cta<T, B> ch;
  ch.bind(smem, X, Y, N, d, pvar, true);
  double* vb = reinterpret_cast<double*>(smem) + cta_layout<B>(d, N, true).vec;
  double* q = ch.vec(vb, V_Q);
  double* g = ch.vec(vb, V_G);
  double* v = ch.vec(vb, V_V);
  double* vt = ch.vec(vb, V_VT);
  double* gld = ch.vec(vb, V_GLD);
  double* yv = ch.vec(vb, V_Y);
  for (int i = threadIdx.x; i < d; i += TT) {
    q[i] = double(pos[(size_t)c * d + i]);
    g[i] = double(grad[(size_t)c * d + i]);
    yv[i] = double(z[(size_t)c * d + i]);
  }
  const double ld0 = logdens[c];
  const double J0 = vol[c];
  __syncthreads();
  ch.point(q);
  double logdet = ch.metric_factor(true);
  // velocity v = L⁻ᵀz (lmcmc/metrics.py:75-91)
  for (int k = threadIdx.x; k < d; k += TT) {
    double s = 0.0;
    for (int i = k; i < d; ++i) s += ch.Li[rowstart(i) + k] * yv[i];
    v[k] = s;
    if (info.momentum) info.momentum[(size_t)c * d + k] = T(s);
  }
  // K = −½ log det G + ½ vᵀGv (lmcmc/metrics.py:93-112); lmc_energy (:209-219)
  ch.gv(v, vt);
  double vgv = 0.0;
  for (int i = threadIdx.x; i < d; i += TT) vgv += v[i] * vt[i];
  const double H0 = -ld0 - 0.5 * logdet + 0.5 * ch.bsum(vgv) - J0;
  double ld = ld0, J = J0;
  if (sp.L > 0) ch.w_pass();
  for (int step = 0; step < sp.L; ++step) {  // lan_integrator.one_step (:93-144)
    lmc_half(ch, v, vt, gld, g, sp.h, &J);
    for (int i = threadIdx.x; i < d; i += TT) q[i] += sp.h * v[i];
    __syncthreads();
    ld = ch.point(q);
    ch.grad(q, g);
    logdet = ch.metric_factor(true);
    ch.w_pass();
    lmc_half(ch, v, vt, gld, g, sp.h, &J);
  }
  ch.gv(v, vt);
  vgv = 0.0;
  for (int i = threadIdx.x; i < d; i += TT) vgv += v[i] * vt[i];
  const double H1 = -ld - 0.5 * logdet + 0.5 * ch.bsum(vgv) - J;
  for (int i = threadIdx.x; i < d; i += TT) {  // LMCInfo.proposal.state: q_L, −v_L
    if (info.prop_q) info.prop_q[(size_t)c * d + i] = T(q[i]);
    if (info.prop_v) info.prop_v[(size_t)c * d + i] = T(-v[i]);
  }
  const AcceptOut a = metropolis(H0, H1, uacc[c], sp.div_threshold);
  if (a.accept) {
    for (int i = threadIdx.x; i < d; i += TT) {
      pos[(size_t)c * d + i] = T(q[i]);
      grad[(size_t)c * d + i] = T(g[i]);
    }
  }
  if (threadIdx.x != 0) return;
  if (a.accept) {
    logdens[c] = ld;
    vol[c] = J;
  }
  if (info.acc_rate) info.acc_rate[c] = a.p_acc;
  if (info.accepted) info.accepted[c] = a.accept;
  if (info.divergent) info.divergent[c] = a.divergent;
  if (info.energy) info.energy[c] = H1;
  if (info.fp_iters) info.fp_iters[c] = 0;
  if (info.status)
    info.status[c] = (isfinite(H1) ? 0u : GJ_CHAIN_NONFINITE) | (ch.bad ? GJ_CHAIN_NOT_SPD : 0u);
}

}  // namespace

size_t logreg_cta_smem(int d, int N, int mixed, int lmc) {
  return mixed ? cta_layout<float>(d, N, lmc != 0).bytes : cta_layout<double>(d, N, lmc != 0).bytes;
}

bool logreg_cta_supported(int d, int N, int mixed, int lmc) {
  if (d < 1 || d > 64 || N < 1) return false;
  return logreg_cta_smem(d, N, mixed, lmc) <= (size_t)227 * 1024;
}

template <typename T>
cudaError_t launch_logreg_cta(int sampler, const TargetDev& t, const StepDev& sp, T* pos, T* grad,
                              double* ld, double* vol, const T* z, const double* u,
                              const InfoDev<T>& info, int C, cudaStream_t st) {
  const int d = t.d, N = t.n;
  const bool lmc = sampler == GJ_SAMPLER_LMC;
  if (!logreg_cta_supported(d, N, sizeof(T) == 4, lmc)) return cudaErrorInvalidValue;
  const size_t smem = cta_layout<T>(d, N, lmc).bytes;
  const T* X = static_cast<const T*>(t.X);
  const T* Y = static_cast<const T*>(t.y);
  cudaError_t e;
  if (lmc) {
    e = cudaFuncSetAttribute(lmc_cta_kernel<T, T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    if (e != cudaSuccess) return e;
    lmc_cta_kernel<T, T><<<C, TT, smem, st>>>(X, Y, N, d, t.p0, sp, pos, grad, ld, vol, z, u, info,
                                              C);
  } else {
    e = cudaFuncSetAttribute(rmhmc_cta_kernel<T, T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    if (e != cudaSuccess) return e;
    rmhmc_cta_kernel<T, T><<<C, TT, smem, st>>>(X, Y, N, d, t.p0, sp, pos, grad, ld, z, u, info,
                                                C);
  }
  return cudaGetLastError();
}

template cudaError_t launch_logreg_cta<double>(int, const TargetDev&, const StepDev&, double*,
                                               double*, double*, double*, const double*,
                                               const double*, const InfoDev<double>&, int,
                                               cudaStream_t);
template cudaError_t launch_logreg_cta<float>(int, const TargetDev&, const StepDev&, float*, float*,
                                              double*, double*, const float*, const double*,
                                              const InfoDev<float>&, int, cudaStream_t);

}  // namespace gj
