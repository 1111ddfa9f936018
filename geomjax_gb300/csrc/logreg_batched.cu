// Batched dense-Fisher logistic-regression RMHMC (implicit midpoint) over all
// chains at once, mixed precision.
//
// Reference path: rmhmc/rmhmc.py:131-174 (kernel), rmhmc/integrators.py:53-156
// (fixed-point implicit midpoint), rmhmc/metrics.py:42-127 (Gaussian
// kinetic energy, Cholesky momentum, solve), mcmc/proposal.py:87-185
// (accept).  The reference differentiates K through the Cholesky of the
// user's metric; for the Fisher metric G = XᵀΛX + I/s² of logistic
// regression the same derivative is, per chain,
//     ∂K/∂β_k = ½ Σ_n Λ'_n x_nk [x_nᵀG⁻¹x_n − (x_nᵀu)²],  u = G⁻¹p.
//
// One fixed-point map evaluation for all C chains is five contractions over
// the data, each one a split-BF16 GEMM with FP32 accumulation (gemm.cuh):
//   (1) A = Q Xᵀ            [C x N]  epilogue: σ, Λ, Λ', r1 = y − σ
//   (2) Gvec = Λ Zᵀ          [C x P]  Gram, Z_n = upper triangle of x_n x_nᵀ
//   (3) per-chain FP64 Cholesky of G = Gvec + I/s², u = G⁻¹p, log det G,
//       G⁻¹ packed as Z-coefficients (FP32, split to BF16)
//   (4) S = U Xᵀ            [C x N]  s_cn = x_nᵀu_c
//   (5) W = Ginv Zᵀ          [C x N]  epilogue: r2 = Λ'(w − s²)
//   (6) [∇ℓ | 2∂K] = [r1; r2] X      [2C x d]
//   (7) update: (q, p) ← (q0 + h/2·u, p0 − h/2·(∂K − ∇ℓ)), ∞-norm in FP64,
//       per-chain convergence exactly as the vmapped lax.while_loop.
// Z and X are constants of the target, staged once as split-BF16 planes.
// FP64 is used for the metric Cholesky, log det and solves, the fixed-point
// norm and the Hamiltonian difference; the log density at the proposal is
// evaluated per chain in FP32 with an FP64 sum.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <type_traits>
#include <vector>

#include "chain_kernels.cuh"
#include "gemm.cuh"
#include "logreg_batched.cuh"

namespace gj {

namespace {
thread_local std::string g_err;

inline int roundup(int x, int m) { return (x + m - 1) / m * m; }

enum CholMode : int { CH_DRAW = 0, CH_EVAL = 1, CH_ENERGY = 2 };
// implicit midpoint: the eager and the iterated map evaluation, the explicit
// half step; generalized leapfrog: the momentum solve (eager, iterated), the
// position solve (eager, iterated), the explicit final momentum
enum UpdMode : int {
  UP_FP0 = 0, UP_FPN = 1, UP_EXPLICIT = 2,
  UP_GLP0 = 3, UP_GLPN = 4, UP_GLQ0 = 5, UP_GLQN = 6, UP_GLPX = 7
};
__host__ __device__ inline bool upd_iterated(int m) { return m == UP_FPN || m == UP_GLPN || m == UP_GLQN; }

// ---------------------------------------------------------------------------
// constants: X and Z = vech(x xᵀ) as split-BF16 planes
// ---------------------------------------------------------------------------
__global__ void build_consts_kernel(const float* X, int N, int d, int P, SplitMat Xb, SplitMat XTb,
                                    SplitMat Zb, SplitMat Zt) {
  const int n = blockIdx.x;
  if (n >= N) return;
  const float* x = X + (size_t)n * d;
  for (int j = threadIdx.x; j < d; j += blockDim.x) {
    split_store(Xb, n, j, x[j]);
    split_store(XTb, j, n, x[j]);
  }
  for (int idx = threadIdx.x; idx < P; idx += blockDim.x) {
    // idx -> (j, k), j <= k, row-major over the upper triangle
    int j = 0, rem = idx;
    while (rem >= d - j) {
      rem -= d - j;
      ++j;
    }
    const int k = j + rem;
    const float zz = x[j] * x[k];
    split_store(Zb, n, idx, zz);
    split_store(Zt, idx, n, zz);
  }
}

// ---------------------------------------------------------------------------
// per-chain metric factorisation (one warp per chain, shared memory)
// ---------------------------------------------------------------------------
struct CholArgs {
  int mode, C, d, P;
  double prior_inv;
  const float* Gv;
  int gv_ld;
  const float* z;      // DRAW
  double* p0;          // DRAW: p0 := L z
  double* pc;          // current momentum (FP64 iterate; DRAW writes it)
  double* u;           // [C, d] G⁻¹p (FP64)
  SplitMat Ub;         // split U for (4)
  SplitMat Giv;        // split packed G⁻¹ for (5)
  double* logdet;      // [C]
  double* quad;        // [C] ||L⁻¹p||² (DRAW: ||z||²)
  const uint8_t* active;  // EVAL: skip inactive chains (may be NULL)
  uint8_t* bad;        // [C] non-SPD flag (sticky)
  float* mom_info;     // DRAW: info.momentum (may be NULL)
  float* vel_info;     // ENERGY: the proposal velocity −G⁻¹p (may be NULL)
  double* Lout;        // DRAW / EVAL: the packed factor, kept for later solves (may be NULL)
  float* Lout32;       // DRAW / EVAL: the same in FP32 (may be NULL)
  int no_inverse;      // EVAL: stop after u = G⁻¹p (no L⁻¹, no packed G⁻¹)
  // EVAL with no_inverse, FP64, 3 <= d <= 64, one chain per warp
  // (chol_refined_kernel): u by an FP32 factor and FP64-residual refinement
  // (refined_solve_w32 / refined_solve), the FP64 factorisation only for the
  // chains whose refinement does not converge
  int refine;
  int* fallbacks;      // refined solves that fell back to FP64 (may be NULL)
  // EVAL with no_inverse: the generalized leapfrog's position update
  // q' = q0 + h/2 [G⁻¹(q0) + G⁻¹(q_k)] p½ (UP_GLQN of update_kernel) done
  // here with u = G⁻¹(q_k)p½, with its convergence test
  int q_update;
  const StepDev* spd;  // graph path: h / tol / max_iters (else hh, tol, max_iters)
  double hh, tol;
  int max_iters;
  const double* u0;    // G(q0)⁻¹p½
  const double* q0;
  double* qc;          // the position iterate
  SplitMat Qb;         // its split copy for the Xβ contraction
  double* norm;
  int* iters;
  int* iters_total;
  uint8_t* active_w;   // the active set (the array `active` reads)
  uint8_t* notconv;
  int* n_active;       // set while some chain iterates
};

// Chain packing.  The FP64 pipe issues one warp instruction for all 32 lanes
// whatever the active mask, so the factorisation packs several chains into a
// warp: a sub-group of `lpc` lanes owns one chain and every pivot, scaling
// and substitution step serves 32 / lpc chains per instruction.  The factor
// is held as a packed lower triangle in column-major order,
// L(i, k) at colstart(k) + i − k with colstart(k) = k·d − k(k−1)/2, which is
// also the index of the upper-triangle entry (k, i) in the row-major packed
// Gram output, so unpacking G is a plain copy.
//
// Shared memory per CTA: the pair table (packed index t → row i | col k << 16,
// 4 bytes each), then per chain: L (P F's), y, x, 1/L_jj (d F's each) and
// L⁻¹ packed like L (P floats).  The per-chain stride is a multiple of 8 bytes
// that is 4 (mod 16) doubles, so the 4 chains of a half-warp touching
// consecutive packed entries fall in distinct banks.
struct CholCfg {
  int cpw;       // chains per warp
  int lpc;       // lanes per chain (32 / cpw; 128 / 256: one chain per CTA of 4 / 8 warps)
  int warps;     // warps per CTA
  int chains;    // chains per CTA
  size_t stride; // bytes per chain
  size_t tab;    // bytes of the pair table
  size_t smem;   // dynamic shared memory per CTA
};

__host__ __device__ inline size_t chol_table_bytes(int d) {
  const size_t pairs = (size_t)d * (d + 1) / 2;
  return (pairs * sizeof(uint32_t) + 15) / 16 * 16;
}

__host__ __device__ inline size_t chol_chain_bytes(int d, size_t fsz) {
  const size_t pairs = (size_t)d * (d + 1) / 2;
  size_t b = pairs * fsz + 3 * (size_t)d * fsz + pairs * sizeof(float);
  size_t w = (b + 7) / 8;  // 8-byte words
  while (w % 16 != 4) ++w;
  return w * 8;
}

// cpw_req: requested chains per warp (1, 2, 4 or 8; 0 = automatic); reduced
// until a warp's chains fit in 40 KB.  Measured on GB300 at d = 25, 4096
// chains (leapfrog steps/s of the whole transition): FP64 1.64M / 1.96M /
// 2.06M / 1.74M and FP32 2.29M / 2.46M / 2.35M / 2.00M for 1 / 2 / 4 / 8
// chains per warp, so the automatic choice is 4 for FP64 (whose issue slots
// bound the factorisation) and 2 for FP32 (where latency does).  With few
// chains (C < 1024) the GPU is far from full and one warp's serial path sets
// the kernel's time, so the automatic choice is one chain per warp (all 32
// lanes on one chain's trailing updates).
inline CholCfg chol_config(int d, size_t fsz, int cpw_req = 0, int C = 1 << 30) {
  CholCfg c{};
  c.stride = chol_chain_bytes(d, fsz);
  c.tab = chol_table_bytes(d);
  c.cpw = cpw_req > 0 ? cpw_req : (C < 1024 ? 1 : (fsz == sizeof(double) ? 4 : 2));
  while (c.cpw > 1 && (size_t)c.cpw * c.stride > 40 * 1024) c.cpw >>= 1;
  c.lpc = 32 / c.cpw;
  c.warps = c.cpw >= 4 ? 1 : 4 / c.cpw;
  // as many of those warps as fit 200 KB (large d: one warp of one chain)
  while (c.warps > 1 && c.tab + (size_t)c.warps * c.cpw * c.stride > 200 * 1024) --c.warps;
  c.smem = c.tab + (size_t)c.warps * c.cpw * c.stride;
  c.chains = c.warps * c.cpw;
  // One chain per warp, and four such chains would not let two CTAs share an
  // SM (d >= 64): each warp alone on its scheduler leaves the other FP64
  // units idle and exposes every latency of the chain's d dependent column
  // steps.  Such a chain gets a CTA of four warps (its trailing updates
  // spread over 128 lanes), one chain per CTA.
  if (c.cpw == 1 && c.tab + 4 * c.stride > 113 * 1024) {
    c.lpc = 128;
    c.warps = 4;
    c.chains = 1;
    // when even one such chain's full layout leaves no room for a second
    // CTA (d >= ~110), the SM would hold four warps only: the chain gets eight
    if (c.tab + c.stride > 113 * 1024) {
      c.lpc = 256;
      c.warps = 8;
    }
    // the chain's FP32 L⁻¹ (the end of its block) lives in the pair table's
    // place (d = 128: 102 KB, two CTAs per SM)
    c.smem = c.tab + c.stride - (size_t)d * (d + 1) / 2 * sizeof(float);
  }
  return c;
}

// Reciprocal square root of a pivot, without a division, and the pivot's
// validity.  A usable FP64 pivot is positive, finite and at least 2^-1021
// (a Schur complement of Gram + I/s² is at least 1/s²); any other marks the
// chain as not positive definite and gives NaN.  The FP32 estimate of the
// truncated value (relative error below 2^-22 + 2^-24) is refined by one
// Newton step x·(3 − a·x²)/2 = x·fma(−a·x, x/2, 3/2), whose quadratic
// convergence leaves a relative error below 2^-42: three FP64 operations.
// Pivots outside the binary32 exponent range take 1/sqrt.
__device__ __forceinline__ double pivot_rsqrt(double a, bool& bad) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(a);
  const uint32_t hi = (uint32_t)(b >> 52);  // sign and biased exponent
  if (hi - 2u >= 0x7fdu) {  // negative, zero, below 2^-1021, infinite or NaN
    bad = true;
    return NAN;
  }
  const int e = (int)hi - 1023;
  if (e < -126 || e > 127) return 1.0 / sqrt(a);
  const float af = __uint_as_float(((uint32_t)(e + 127) << 23) | ((uint32_t)(b >> 29) & 0x7fffffu));
  const float xf = rsqrtf(af);
  const double x = double(xf), hx = double(0.5f * xf);
  return x * fma(-(a * x), hx, 1.5);
}
__device__ __forceinline__ float pivot_rsqrt(float a, bool& bad) {
  if (!(a > 0.f) || !isfinite(a)) {
    bad = true;
    return NAN;
  }
  float x = rsqrtf(a);
  return x * (1.5f - 0.5f * a * x * x);
}

// log det accumulation: the running product of the pivots as mantissa
// m ∈ [0.5, 1) times 2^e, renormalised by integer operations on the bits
// (m · pivot is normal for every usable pivot)
__device__ __forceinline__ void ld_accumulate(double& m, int& e, double piv) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(m * piv);
  e += (int)((b >> 52) & 0x7ffu) - 1022;
  m = __longlong_as_double((long long)((b & 0x800fffffffffffffull) | 0x3fe0000000000000ull));
}

__device__ __forceinline__ int colstart(int k, int d) { return k * d - (k * (k - 1)) / 2; }

// sum over the LPC lanes of a sub-group (LPC a power of two, sub-groups aligned)
template <int LPC>
__device__ __forceinline__ double group_sum(double v) {
#pragma unroll
  for (int o = LPC >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
template <int LPC>
__device__ __forceinline__ double group_max(double v) {
#pragma unroll
  for (int o = LPC >> 1; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
template <int LPC>
__device__ __forceinline__ float group_maxf(float v) {
#pragma unroll
  for (int o = LPC >> 1; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
template <int LPC>
__device__ __forceinline__ bool group_any(bool b) {
  int v = b ? 1 : 0;
#pragma unroll
  for (int o = LPC >> 1; o > 0; o >>= 1) v |= __shfl_xor_sync(0xffffffffu, v, o);
  return v != 0;
}

// A chain's barrier and reductions: its sub-group of a warp (LPC <= 32) or
// its whole CTA (LPC > 32, LPC / 32 warps; reductions through shared memory,
// warps added in order)
template <int LPC>
__device__ __forceinline__ void chain_sync() {
  if constexpr (LPC > 32)
    __syncthreads();
  else
    __syncwarp();
}
template <int LPC>
__device__ __forceinline__ double chain_sum(double v) {
  if constexpr (LPC <= 32) {
    return group_sum<LPC>(v);
  } else {
    __shared__ double red[LPC / 32];
    v = group_sum<32>(v);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
#pragma unroll
    for (int w = 0; w < LPC / 32; ++w) t += red[w];
    __syncthreads();
    return t;
  }
}
template <int LPC>
__device__ __forceinline__ double chain_max(double v) {
  if constexpr (LPC <= 32) {
    return group_max<LPC>(v);
  } else {
    __shared__ double red[LPC / 32];
    v = group_max<32>(v);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = red[0];
#pragma unroll
    for (int w = 1; w < LPC / 32; ++w) t = fmax(t, red[w]);
    __syncthreads();
    return t;
  }
}
template <int LPC>
__device__ __forceinline__ bool chain_any(bool b) {
  if constexpr (LPC <= 32) return group_any<LPC>(b);
  else return __syncthreads_or(b ? 1 : 0) != 0;
}

// Right-looking Cholesky of one chain's packed matrix L (T = double / float),
// in place: the strict lower triangle becomes the factor's, rdiag[j] =
// 1/L_jj, and the diagonal keeps the pivots (DRAW: L_jj).  log det G = log Π
// pivots is accumulated as mantissa pm · 2^pe (want_ld), so that one
// logarithm is taken per chain.  With `border` the right-hand side in y
// rides along as a bordered row: at step j, y_j is scaled with the pivot and
// y_k (k > j) updated in the same phase as the trailing triangle, so y ends
// as L⁻¹y without a separate serial forward substitution.  A non-positive
// or non-finite pivot sets `bad`.
template <typename T, int LPC>
__device__ __forceinline__ void factor_packed(T* L, T* rdiag, T* y, const uint32_t* tab, int d,
                                              int P, int sl, bool border, bool draw,
                                              bool want_ld, bool& bad, double& pm, int& pe) {
  constexpr bool kCta = LPC > 32;
  // The FP64 factorisation takes one column per step: its DFMA count bounds
  // it, and rank-2 blocking (one pass over the trailing triangle for two
  // columns) measured no faster for T = double.  For T = float, where
  // latency bounds the kernel, columns are taken two at a time: pivot j,
  // scale column j, update column j + 1 with it, pivot j + 1, scale column
  // j + 1, then one pass applies both columns to the trailing triangle.
  // pivot(j): 1/L_jj from the current diagonal, log det product, and the
  // bordered y_j (all lanes compute the same scalars; lane 0 of the chain
  // writes them)
  auto pivot = [&](int j, int cj) -> T {
    if constexpr (kCta) {
      // a CTA per chain: thread 0 alone takes the pivot (the FP64 pipe issues
      // each warp's copy of it at full cost) and publishes 1/L_jj; bad, pm
      // and pe, read only by thread 0 at the end, stay its own
      if (sl == 0) {
        const T djj = L[cj];
        const T inv = pivot_rsqrt(djj, bad);
        if (want_ld) ld_accumulate(pm, pe, double(djj));
        if (draw) L[cj] = djj * inv;  // L_jj, read only by p = L z
        rdiag[j] = inv;
        if (border) y[j] *= inv;
      }
      chain_sync<LPC>();
      const T inv = rdiag[j];
      for (int i = j + 1 + sl; i < d; i += LPC) L[cj + i - j] *= inv;
      chain_sync<LPC>();
      return inv;
    }
    const T djj = L[cj];
    const T inv = pivot_rsqrt(djj, bad);  // 1/L_jj
    if (want_ld) ld_accumulate(pm, pe, double(djj));
    chain_sync<LPC>();
    if (sl == 0) {
      if (draw) L[cj] = djj * inv;  // L_jj, read only by p = L z
      rdiag[j] = inv;
      if (border) y[j] *= inv;
    }
    for (int i = j + 1 + sl; i < d; i += LPC) L[cj + i - j] *= inv;
    chain_sync<LPC>();
    return inv;
  };
  constexpr bool kRank2 = sizeof(T) == sizeof(float);
  int cj = 0;  // colstart(j)
  for (int j = 0; j < d; j += kRank2 ? 2 : 1) {
    pivot(j, cj);
    const int cj1 = cj + (d - j);  // colstart(j + 1)
    if (!kRank2 || j + 1 == d) {
      // rank-1 step: bordered y and the trailing triangle with column j
      if (border) {
        const T yj = y[j];
        for (int k = j + 1 + sl; k < d; k += LPC) y[k] -= yj * L[cj + k - j];
      }
      const T* __restrict__ colj = L + cj - j;  // colj[i] = L(i, j)
      T* __restrict__ tr = L;
#pragma unroll 4
      for (int t = cj1 + sl; t < P; t += LPC) {
        const uint32_t ik = tab[t];
        tr[t] -= colj[ik & 0xffffu] * colj[ik >> 16];
      }
      cj = cj1;
      chain_sync<LPC>();
      continue;
    }
    // column j + 1 (rows j + 1 ..) and y_{j+1} reduced by column j
    {
      const T l10 = L[cj + 1];  // L(j + 1, j)
      for (int i = j + 1 + sl; i < d; i += LPC) L[cj1 + i - j - 1] -= L[cj + i - j] * l10;
      if (border && sl == 0) y[j + 1] -= y[j] * l10;
    }
    chain_sync<LPC>();
    pivot(j + 1, cj1);
    // trailing triangle (columns k >= j + 2): both columns are read-only
    // here and disjoint from the entries written
    const int cn = cj1 + (d - j - 1);  // colstart(j + 2)
    const T* __restrict__ c0 = L + cj - j;        // c0[i] = L(i, j)
    const T* __restrict__ c1 = L + cj1 - j - 1;   // c1[i] = L(i, j + 1)
    T* __restrict__ tr = L;
    if (border) {
      const T y0 = y[j], y1 = y[j + 1];
      for (int k = j + 2 + sl; k < d; k += LPC) y[k] -= y0 * c0[k] + y1 * c1[k];
    }
#pragma unroll 4
    for (int t = cn + sl; t < P; t += LPC) {
      const uint32_t ik = tab[t];
      const int i = (int)(ik & 0xffffu), k = (int)(ik >> 16);
      tr[t] -= c0[i] * c0[k] + c1[i] * c1[k];
    }
    cj = cn;
    chain_sync<LPC>();
  }
}

// y ← L⁻¹y on a factor from factor_packed (column-oriented, one column per
// step)
template <typename T, int LPC>
__device__ __forceinline__ void forward_subst(const T* L, const T* rdiag, T* y, int d, int sl) {
  int cj = 0;  // colstart(j)
  for (int j = 0; j < d; ++j) {
    const T yj = y[j] * rdiag[j];
    chain_sync<LPC>();
    if (sl == 0) y[j] = yj;
    for (int i = j + 1 + sl; i < d; i += LPC) y[i] -= L[cj + i - j] * yj;
    cj += d - j;
    chain_sync<LPC>();
  }
}

// x ← L⁻ᵀx, column-oriented backward substitution (row j of L is L(j, i) at
// colstart(i) + j − i)
template <typename T, int LPC>
__device__ __forceinline__ void backward_subst(const T* L, const T* rdiag, T* x, int d, int sl) {
  for (int j = d - 1; j >= 0; --j) {
    const T xj = x[j] * rdiag[j];
    chain_sync<LPC>();
    if (sl == 0) x[j] = xj;
    for (int i = sl; i < j; i += LPC) x[i] -= L[colstart(i, d) + j - i] * xj;
    chain_sync<LPC>();
  }
}

// Most corrections a refined solve applies before it gives the chain back to
// the FP64 factorisation (about as many FP64 instructions as that
// factorisation at d = 25, one chain per warp).
constexpr int kRefineMax = 8;

// The stopping rule of a refined solve, on norms relative to ‖x₀‖∞ (float32
// scalars: the rule needs a few bits of them): er = ‖dx_k‖/‖x₀‖, pr = the
// previous correction's (1 for the first).
// * Converged once the next step's predicted size er²/pr is below 2⁻⁴⁴: x is
//   then as accurate as an FP64 factorisation's solve of a well-conditioned G.
// * Corrections that stop shrinking (by at least half) have reached the
//   floor set by the FP64 residual's rounding, which is also the order of
//   an FP64 factorisation's solve error: converged when that floor is below
//   2⁻³⁶, failed above it (then the FP64 factorisation takes over; on
//   log-spaced spectra at d = 64 that starts between κ(G) = 1e6 and 3e6).
// * Failed when a correction is not finite.
// Returns 1 = converged (apply dx), 0 = apply dx and go on, −1 = failed.
__device__ __forceinline__ int refine_verdict(float er, float pr, bool nonfinite) {
  if (nonfinite) return -1;
  if (er * er <= 0x1p-44f * pr) return 1;
  if (er > 0.5f * pr) return er <= 0x1p-36f ? 1 : -1;
  return 0;
}

// x = G⁻¹p for a position iterate of the generalized leapfrog, one chain
// per sub-group of LPC <= 32 lanes (the refined kernels use it with one
// chain per warp for 32 < d <= 64), by mixed-precision iterative refinement
// (Wilkinson 1963, Moler 1967; Carson and Higham, SIAM J. Sci. Comput. 40,
// 2018): G = Gram + prior·I is factored in FP32 (Lf, rdf; the first solution
// from the bordered factorisation), then x += G₃₂⁻¹(p − G·x) with the
// residual formed in FP64 from the FP64 Gram (G, packed, without the prior)
// and the prior.  Each correction shrinks the error by about κ(G)·d·2⁻²⁴
// (refine_verdict stops it).  Returns false (x then unspecified) when the
// FP32 factorisation breaks down, the corrections fail or kRefineMax of them
// do not converge: the caller then factors G in FP64.  The loop runs the
// same number of times for all chains of the warp; a chain that has
// converged (or failed) applies no further corrections, so its x depends on
// its own data only.
template <int LPC>
__device__ bool refined_solve(const double* G, const float* gv, double prior, float* Lf,
                              float* rdf, float* wf, double* x, const uint32_t* tab,
                              const double* p, bool live, int d, int P, int sl) {
  const float priorf = float(prior);
  for (int t = sl; t < P; t += LPC) {
    const uint32_t ik = tab[t];
    const bool diag = (ik & 0xffffu) == (ik >> 16);
    Lf[t] = live ? gv[t] + (diag ? priorf : 0.f) : (diag ? 1.f : 0.f);
  }
  for (int i = sl; i < d; i += LPC) wf[i] = live ? float(p[i]) : 0.f;
  chain_sync<LPC>();
  bool bad = false;
  double pm = 1.0;
  int pe = 0;
  factor_packed<float, LPC>(Lf, rdf, wf, tab, d, P, sl, true, false, false, bad, pm, pe);
  backward_subst<float, LPC>(Lf, rdf, wf, d, sl);
  float xm = 0.f;
  for (int i = sl; i < d; i += LPC) {
    x[i] = double(wf[i]);
    bad |= !isfinite(wf[i]);
    xm = fmaxf(xm, fabsf(wf[i]));
  }
  bool ok = !chain_any<LPC>(bad);
  const float xn = group_maxf<LPC>(xm);  // ‖x₀‖∞
  bool conv = ok && xn == 0.f;           // p = 0: x = 0 exactly
  float pr = 1.f;                        // ‖dx₀‖ / ‖x₀‖
  for (int k = 0; k < kRefineMax && __any_sync(0xffffffffu, ok && !conv); ++k) {
    chain_sync<LPC>();
    // r = p − prior·x − Gram·x in FP64, row i walked along the Gram's packed
    // row: columns m < i down the packed columns, m >= i along column i (one
    // trip count for every lane)
    for (int i = sl; i < d; i += LPC) {
      double s = live ? fma(-prior, x[i], p[i]) : 0.0;
      const int ci = colstart(i, d) - i;
      int cm = 0;  // colstart(m)
      for (int m = 0; m < d; ++m) {
        s = fma(-G[m < i ? cm + i - m : ci + m], x[m], s);
        cm += d - m;
      }
      wf[i] = float(s);
    }
    chain_sync<LPC>();
    forward_subst<float, LPC>(Lf, rdf, wf, d, sl);
    backward_subst<float, LPC>(Lf, rdf, wf, d, sl);
    float em = 0.f;
    bool nf = false;
    for (int i = sl; i < d; i += LPC) {
      nf |= !isfinite(wf[i]);
      em = fmaxf(em, fabsf(wf[i]));
    }
    nf = chain_any<LPC>(nf);
    const float er = group_maxf<LPC>(em) / xn;
    if (ok && !conv) {  // uniform over the chain's lanes
      const int v = refine_verdict(er, pr, nf);
      if (v < 0) {
        ok = false;
      } else {
        for (int i = sl; i < d; i += LPC) x[i] += double(wf[i]);
        conv = v > 0;
        pr = er;
      }
    }
  }
  chain_sync<LPC>();
  return ok && conv;
}

// The same for one chain per warp and d <= 32, on registers: lane i holds
// row i of the FP32 factor (the column broadcasts of the factorisation and
// the substitutions are warp shuffles), its component of y, x and the
// residual; the strict lower triangle is also written by rows to Lrow
// (packed, d(d−1)/2 floats), from which the backward substitution reads its
// columns.  The rows of G come from the FP32 Gram gv of the chain (global
// memory), the residual from its FP64 copy G in shared memory and from x in
// xs (shared, FP64).  The warp holds one live chain.
__device__ __forceinline__ bool refined_solve_w32(const double* G, const float* gv, double prior,
                                                  float* Lrow, double* xs, const double* p, int d,
                                                  int lane) {
  constexpr unsigned kAll = 0xffffffffu;
  const int i = lane;
  const bool in = i < d;
  float row[32];  // row[k] = G₃₂(i, k), then L(i, k), for k <= i
#pragma unroll
  for (int k = 0; k < 32; ++k) {
    float g = 0.f;
    if (k <= i && in) g = gv[colstart(k, d) + i - k];
    if (k == i && in) g += float(prior);
    row[k] = g;
  }
  const double pi = in ? p[i] : 0.0;
  float y = float(pi);
  float rinv = 0.f;  // 1 / L_ii
  bool bad = false;
  // right-looking, one column per step, with the bordered y = L⁻¹p
#pragma unroll
  for (int j = 0; j < 32; ++j) {
    if (j < d) {  // uniform
      const float inv = pivot_rsqrt(__shfl_sync(kAll, row[j], j), bad);
      const float lij = row[j] * inv;  // L(i, j) for i > j
      const float yj = __shfl_sync(kAll, y, j) * inv;
      if (i == j) {
        rinv = inv;
        y = yj;
      } else if (i > j) {
        row[j] = lij;
        y -= lij * yj;
      }
#pragma unroll
      for (int k = j + 1; k < 32; ++k) {
        if (k < d) {
          const float lkj = __shfl_sync(kAll, lij, k);
          if (i >= k) row[k] -= lij * lkj;
        }
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 31; ++k)
    if (k < i && in) Lrow[i * (i - 1) / 2 + k] = row[k];
  __syncwarp();
  auto forward = [&](float v) -> float {  // L⁻¹v
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      if (j < d) {
        const float vj = __shfl_sync(kAll, v * rinv, j);
        if (i == j) v = vj;
        else if (i > j) v -= row[j] * vj;
      }
    }
    return v;
  };
  auto backward = [&](float v) -> float {  // L⁻ᵀv, columns of L from Lrow
#pragma unroll
    for (int j = 31; j >= 0; --j) {
      if (j < d) {
        const float vj = __shfl_sync(kAll, v * rinv, j);
        if (i == j) v = vj;
        else if (i < j) v -= Lrow[j * (j - 1) / 2 + i] * vj;
      }
    }
    return v;
  };
  const float w = backward(y);  // x₀ = G₃₂⁻¹p
  double xi = double(w);
  if (in) xs[i] = xi;
  bool ok = !__any_sync(kAll, bad || !isfinite(w));
  const float xn = group_maxf<32>(fabsf(w));
  bool conv = ok && xn == 0.f;
  float pr = 1.f;
  for (int k = 0; k < kRefineMax && ok && !conv; ++k) {  // uniform: one chain
    __syncwarp();
    // r_i = p_i − prior·x_i − Σ_m Gram(i, m)·x_m in FP64 (packed row walk as
    // in refined_solve)
    double s = fma(-prior, xi, pi);
    if (in) {
      const int ci = colstart(i, d) - i;
      int cm = 0;
      for (int m = 0; m < d; ++m) {
        s = fma(-G[m < i ? cm + i - m : ci + m], xs[m], s);
        cm += d - m;
      }
    }
    const float dx = backward(forward(in ? float(s) : 0.f));
    const bool nf = __any_sync(kAll, !isfinite(dx));
    const float er = group_maxf<32>(fabsf(dx)) / xn;
    const int v = refine_verdict(er, pr, nf);
    if (v < 0) {
      ok = false;
    } else {
      xi += double(dx);
      conv = v > 0;
      pr = er;
      __syncwarp();
      if (in) xs[i] = xi;
    }
  }
  __syncwarp();
  return ok && conv;
}

// block bx of the factorisation (chol_kernel, or an item of a grouped launch)
// LPC = 128 / 256: one chain per CTA of four / eight warps (large d, where
// one warp per chain leaves most of an SM's FP64 units idle); its barrier is
// the CTA's.
// REF: the instantiation that serves the refined solves (CholArgs::refine;
// double, LPC = 32: chol_refined_kernel); the others compile without their
// code, so the FP64 factorisation keeps its registers and occupancy.
template <typename F, int LPC, bool REF = false>  // factorisation type, lanes per chain
__device__ __forceinline__ void chol_body(const CholArgs& a, int stride, int bx) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr bool kCta = LPC > 32;
  constexpr int CPW = kCta ? 1 : 32 / LPC;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nwarps = blockDim.x >> 5;
  const int sub = kCta ? 0 : lane / LPC, sl = kCta ? (int)threadIdx.x : lane % LPC;
  const int c = kCta ? bx : (bx * nwarps + warp) * CPW + sub;
  const int d = a.d;
  const int P = a.P;
  uint32_t* tab = reinterpret_cast<uint32_t*>(smem_raw);
  unsigned char* base =
      smem_raw + chol_table_bytes(d) + (size_t)(kCta ? 0 : warp * CPW + sub) * stride;
  F* L = reinterpret_cast<F*>(base);  // packed lower, column-major
  F* y = L + P;
  F* xv = y + d;
  F* rdiag = xv + d;  // 1 / L_jj
  // L⁻¹, packed like L; a CTA's single chain keeps it in the pair table's
  // place (the table is not read after the factorisation and its bytes)
  float* Li = kCta ? reinterpret_cast<float*>(smem_raw) : reinterpret_cast<float*>(rdiag + d);
  for (int k = threadIdx.x; k < d; k += blockDim.x) {
    int off = colstart(k, d);
    for (int i = k; i < d; ++i, ++off) tab[off] = (uint32_t)i | ((uint32_t)k << 16);
  }
  __syncthreads();
  pdl_wait();
  const bool live = c < a.C && !(a.mode == CH_EVAL && a.active && !a.active[c]);
  if (__all_sync(0xffffffffu, !live)) return;  // uniform per warp
  // G = Gvec + I/s²: the packed layouts coincide; idle slots get the identity.
  // The refined solves of the position iterates keep the Gram alone (their
  // residuals add the prior) and add the prior before an FP64 fallback.
  constexpr bool kRefinable = REF && !kCta && sizeof(F) == sizeof(double);
  const bool refine = kRefinable && a.refine;
  for (int t = sl; t < P; t += LPC) {
    const uint32_t ik = tab[t];
    const bool diag = (ik & 0xffffu) == (ik >> 16);
    F g;
    if (live) {
      g = F(a.Gv[(size_t)c * a.gv_ld + t]);
      if (diag && !refine) g += F(a.prior_inv);
    } else {
      g = diag ? F(1) : F(0);
    }
    L[t] = g;
  }
  chain_sync<LPC>();
  const bool border = a.mode != CH_DRAW;
  bool bad = false;
  // log det G is needed for the energies (DRAW at the start, ENERGY at the
  // proposal); the map evaluations (EVAL) skip it
  const bool want_ld = a.mode != CH_EVAL;
  double pm = 1.0;
  int pe = 0;
  // The position iterates (a.refine: chol_refined_kernel, F = double,
  // LPC = 32, 3 <= d <= 64) solve by mixed-precision refinement: FP32 factor,
  // FP64 residuals (refined_solve_w32 for d <= 32, else refined_solve), the
  // result in xv.  A warp factors in FP64 when one of its chains needs it;
  // the chains already solved park x in L⁻¹'s area meanwhile (free here; P
  // floats hold d doubles for d >= 3).
  bool fp64 = true;   // this warp runs the FP64 factorisation
  bool kept = false;  // this chain's refined x is final
  if constexpr (kRefinable) {
    if (refine) {  // uniform
      const float* gv = live ? a.Gv + (size_t)c * a.gv_ld : nullptr;
      const double* pc = live ? a.pc + (size_t)c * d : nullptr;
      bool w32 = false;
      if constexpr (LPC == 32) w32 = d <= 32;
      if (w32) {
        kept = refined_solve_w32(L, gv, a.prior_inv, Li, xv, pc, d, sl);
      } else {
        float* rdf = reinterpret_cast<float*>(rdiag);  // 2d floats in rdiag's d doubles
        kept = refined_solve<LPC>(L, gv, a.prior_inv, Li, rdf, rdf + d, xv, tab, pc, live, d, P,
                                  sl);
      }
      fp64 = __any_sync(0xffffffffu, !kept);
      if (!kept && live && sl == 0 && a.fallbacks) atomicAdd(a.fallbacks, 1);
      if (fp64) {
        if (kept) {
          double* park = reinterpret_cast<double*>(Li);
          for (int i = sl; i < d; i += LPC) park[i] = xv[i];
        }
        if (live)
          for (int i = sl; i < d; i += LPC) L[colstart(i, d)] += F(a.prior_inv);
        chain_sync<LPC>();
      }
    }
  }
  if (fp64) {
    if (border) {
      for (int i = sl; i < d; i += LPC) y[i] = live ? F(a.pc[(size_t)c * d + i]) : F(0);
    }
    factor_packed<F, LPC>(L, rdiag, y, tab, d, P, sl, border, a.mode == CH_DRAW, want_ld, bad,
                          pm, pe);
  }
  pdl_trigger();  // the factorisation is done; the successor may be scheduled
  if (fp64) {
    if (sl == 0 && live) {
      if (want_ld) a.logdet[c] = bad ? NAN : log(pm) + pe * 0.69314718055994530942;
      if (bad) a.bad[c] = 1;
    }
    if ((a.Lout || a.Lout32) && live) {  // the factor at this position serves the
      // momentum solves, with 1/L_jj in place of the diagonal (the solves multiply)
      for (int t = sl; t < P; t += LPC) {
        const uint32_t ik = tab[t];
        const int i = (int)(ik & 0xffffu), k = (int)(ik >> 16);
        const double v = i == k ? double(rdiag[i]) : double(L[t]);
        if (a.Lout) a.Lout[(size_t)c * P + t] = v;
        if (a.Lout32) a.Lout32[(size_t)c * P + t] = float(v);
      }
    }
    // right-hand side: DRAW p = L z (and L⁻¹p = z); otherwise y = L⁻¹ p by
    // column-oriented forward substitution
    if (a.mode == CH_DRAW) {
      for (int i = sl; i < d; i += LPC) y[i] = live ? F(a.z[(size_t)c * d + i]) : F(0);
      chain_sync<LPC>();
      double zz = 0.0;
      for (int i = sl; i < d; i += LPC) {
        F sacc = 0;
        int ck = 0;
        for (int k = 0; k <= i; ++k) {
          sacc += L[ck + i - k] * y[k];
          ck += d - k;
        }
        if (live) {
          a.p0[(size_t)c * d + i] = double(sacc);
          a.pc[(size_t)c * d + i] = double(sacc);
          if (a.mom_info) a.mom_info[(size_t)c * d + i] = float(sacc);
        }
        zz += double(y[i]) * double(y[i]);
      }
      zz = chain_sum<LPC>(zz);
      if (sl == 0 && live) a.quad[c] = zz;
    } else {  // y = L⁻¹p was formed with the factor
      if (a.mode == CH_ENERGY) {
        double q = 0.0;
        for (int i = sl; i < d; i += LPC) q += double(y[i]) * double(y[i]);
        q = chain_sum<LPC>(q);
        if (sl == 0 && live) a.quad[c] = q;
        if (!a.vel_info) return;  // uniform: the proposal velocity was not asked for
      }
    }
    chain_sync<LPC>();
    // u = L⁻ᵀ y
    for (int i = sl; i < d; i += LPC) xv[i] = y[i];
    chain_sync<LPC>();
    backward_subst<F, LPC>(L, rdiag, xv, d, sl);
    if (a.mode == CH_ENERGY) {  // flip_momentum: the proposal carries −G⁻¹p
      if (live)
        for (int i = sl; i < d; i += LPC) a.vel_info[(size_t)c * d + i] = float(-xv[i]);
      return;
    }
    if (kept) {  // this chain's refined x (the warp factored for another chain)
      const double* park = reinterpret_cast<const double*>(Li);
      for (int i = sl; i < d; i += LPC) xv[i] = F(park[i]);
    }
  }
  if (live) {
    for (int i = sl; i < d; i += LPC) {
      a.u[(size_t)c * d + i] = double(xv[i]);
      // the position iterates (no inverse) use u alone; the split copy
      // feeds the S contraction of full evaluations
      if (!a.no_inverse) split_store(a.Ub, c, i, float(xv[i]));
    }
  }
  if (a.no_inverse) {  // uniform: the position solve needs u only
    if (a.q_update) {
      const double hh = a.spd ? 0.5 * a.spd->h : a.hh;
      const double tol = a.spd ? a.spd->tol : a.tol;
      const int max_iters = a.spd ? a.spd->max_iters : a.max_iters;
      double nrm = 0.0;
      bool nan = false;
      if (live) {
        for (int i = sl; i < d; i += LPC) {
          const size_t o = (size_t)c * d + i;
          const double qn = a.q0[o] + hh * (a.u0[o] + double(xv[i]));
          const double e = qn - a.qc[o];
          nan |= isnan(e);
          nrm = fmax(nrm, fabs(e));
          a.qc[o] = qn;
          split_store(a.Qb, c, i, float(qn));
        }
      }
      nrm = chain_max<LPC>(nrm);
      if (chain_any<LPC>(nan)) nrm = NAN;
      bool act = false;
      if (live) {
        const int it = a.iters[c] + 1;
        act = (it < max_iters) && isfinite(nrm) && (nrm < 1e10) && (nrm > tol);
        if (sl == 0) {
          a.iters[c] = it;
          a.norm[c] = nrm;
          a.active_w[c] = act;
          a.iters_total[c] += 1;
          if (!act && !(isfinite(nrm) && nrm <= tol)) a.notconv[c] = 1;
        }
      }
      if (__any_sync(0xffffffffu, act) && lane == 0) *a.n_active = 1;
    }
    return;
  }
  // L⁻¹ in FP32 by forward substitution of the identity, all columns at
  // once: row k is final once scaled, then rows i > k are reduced by it
  if constexpr (kCta) {
    chain_sync<LPC>();  // the table's last readers are done: L⁻¹ takes its place
    for (int t = sl; t < P; t += LPC) Li[t] = 0.f;
    chain_sync<LPC>();
    for (int cc = sl; cc < d; cc += LPC) Li[colstart(cc, d)] = 1.f;
  } else {
    for (int t = sl; t < P; t += LPC) {
      const uint32_t ik = tab[t];
      Li[t] = (ik & 0xffffu) == (ik >> 16) ? 1.f : 0.f;
    }
  }
  chain_sync<LPC>();
  // two rows at a time: rows k and k + 1 are made final (row k scaled; row
  // k + 1 reduced by row k, then scaled), then rows i > k + 1 are reduced
  // by both in one pass
  int ck = 0;  // colstart(k)
  for (int k = 0; k < d; k += 2) {
    const float ikk = float(rdiag[k]);
    for (int cc = sl; cc <= k; cc += LPC) Li[colstart(cc, d) + k - cc] *= ikk;
    chain_sync<LPC>();
    const int ck1 = ck + (d - k);  // colstart(k + 1)
    if (k + 1 == d) break;
    const float l10 = float(L[ck + 1]);  // L(k + 1, k)
    const float ik1 = float(rdiag[k + 1]);
    for (int cc = sl; cc <= k + 1; cc += LPC) {
      const int o = colstart(cc, d);
      const float v = (cc <= k) ? Li[o + k + 1 - cc] - l10 * Li[o + k - cc] : Li[o];
      Li[o + k + 1 - cc] = v * ik1;
    }
    chain_sync<LPC>();
    if constexpr (kCta) {
      // a CTA's chain: warps over the columns cc of L⁻¹, lanes over the rows
      // (each row a serial loop over the columns leaves most threads idle at
      // d = 128 and exposes every load's latency).  Columns k and k + 1 of L
      // are converted to FP32 once, into y's and x's space (free by now)
      float* lc = reinterpret_cast<float*>(y);  // lc[i] = L(i, k), lc[d + i] = L(i, k + 1)
      for (int i = k + 2 + sl; i < d; i += LPC) {
        lc[i] = float(L[ck + i - k]);
        lc[d + i] = float(L[ck1 + i - k - 1]);
      }
      chain_sync<LPC>();
      const int nw = LPC / 32, w = sl >> 5, ln = sl & 31;
      for (int cc = w; cc <= k + 1; cc += nw) {
        const int o = colstart(cc, d) - cc;  // Li(m, cc) at o + m
        const float a0 = cc <= k ? Li[o + k] : 0.f;  // Li(k, cc); Li(k, k + 1) = 0
        const float a1 = Li[o + k + 1];              // Li(k + 1, cc)
        for (int i = k + 2 + ln; i < d; i += 32) Li[o + i] -= lc[i] * a0 + lc[d + i] * a1;
      }
    } else {
      for (int i = k + 2 + sl; i < d; i += LPC) {
        const float li0 = float(L[ck + i - k]);       // L(i, k)
        const float li1 = float(L[ck1 + i - k - 1]);  // L(i, k + 1)
        int cc0 = 0;  // colstart(cc)
        for (int cc = 0; cc <= k; ++cc) {
          Li[cc0 + i - cc] -= li0 * Li[cc0 + k - cc] + li1 * Li[cc0 + k + 1 - cc];
          cc0 += d - cc;
        }
        Li[cc0 + i - k - 1] -= li1 * Li[cc0];  // cc = k + 1: Li(k, k + 1) = 0
      }
    }
    ck = ck1 + (d - k - 1);
    chain_sync<LPC>();
  }
  // G⁻¹ = L⁻ᵀL⁻¹ packed as Z-coefficients (row-major upper triangle, whose
  // index for (k, i), k <= i, is the packed index t of (i, k)); the
  // off-diagonal coefficients are doubled
  if (!live) return;
  if constexpr (kCta) {
    // a CTA's chain: the same per-thread dot products over entries t = sl +
    // LPC·u, with (i, k) walked along the packed columns (the pair table's
    // place holds L⁻¹ now); the walk stops at the last column
    int i = 0, k = 0;  // (i, k) of entry t
    auto advance = [&](int delta) {
      while (delta > 0 && k < d) {
        const int left = d - i;  // entries of column k from row i on
        if (delta < left) {
          i += delta;
          delta = 0;
        } else {
          delta -= left;
          ++k;
          i = k;
        }
      }
    };
    advance(sl);
    for (int t = sl; t < P; t += LPC) {
      const float* li = Li + colstart(i, d) - i;  // li[m] = L⁻¹(m, i)
      const float* lk = Li + colstart(k, d) - k;  // lk[m] = L⁻¹(m, k)
      float sacc = 0.f;
      for (int m = i; m < d; ++m) sacc += lk[m] * li[m];
      split_store(a.Giv, c, t, (i == k) ? sacc : 2.f * sacc);
      advance(LPC);
    }
  } else {
    for (int t = sl; t < P; t += LPC) {
      const uint32_t ik = tab[t];
      const int i = (int)(ik & 0xffffu), k = (int)(ik >> 16);
      const float* li = Li + colstart(i, d) - i;  // li[m] = L⁻¹(m, i)
      const float* lk = Li + colstart(k, d) - k;  // lk[m] = L⁻¹(m, k)
      float sacc = 0.f;
      for (int m = i; m < d; ++m) sacc += lk[m] * li[m];
      split_store(a.Giv, c, t, (i == k) ? sacc : 2.f * sacc);
    }
  }
}

template <typename F, int LPC>
__global__ void chol_kernel(CholArgs a, int stride) {
  chol_body<F, LPC>(a, stride, (int)blockIdx.x);
}
// The refined solves (CholArgs::refine): one chain per warp, CTAs of four
// warps.  (A register bound of 64 or 72 per thread made ptxas spill.)
__global__ void chol_refined_kernel(CholArgs a, int stride) {
  chol_body<double, 32, true>(a, stride, (int)blockIdx.x);
}

// a grouped launch of factorisations: one item per posterior
struct CholItem {
  CholArgs a;
  int stride;
};
template <typename F, int LPC>
__global__ void chol_grouped_kernel(const CholItem* __restrict__ items,
                                    const int* __restrict__ prefix, int n) {
  const int i = group_item(prefix, n, (int)blockIdx.x);
  chol_body<F, LPC>(items[i].a, items[i].stride, (int)blockIdx.x - __ldg(prefix + i));
}
__global__ void chol_refined_grouped_kernel(const CholItem* __restrict__ items,
                                const int* __restrict__ prefix, int n) {
  const int i = group_item(prefix, n, (int)blockIdx.x);
  chol_body<double, 32, true>(items[i].a, items[i].stride,
                              (int)blockIdx.x - __ldg(prefix + i));
}

template <typename F>
cudaError_t chol_launch(const CholCfg& cf, size_t smem, dim3 grid, const CholArgs& a, bool pdl,
                        cudaStream_t st) {
  const dim3 th(32 * cf.warps);
  const int stride = (int)cf.stride;
  if constexpr (sizeof(F) == sizeof(double)) {
    if (a.refine)  // the host sets it with one chain per warp only
      return cf.lpc == 32 && cf.warps <= 4
                 ? launch_k(pdl, chol_refined_kernel, grid, th, smem, st, a, stride)
                 : cudaErrorInvalidValue;
  }
  switch (cf.lpc) {
    case 4: return launch_k(pdl, chol_kernel<F, 4>, grid, th, smem, st, a, stride);
    case 8: return launch_k(pdl, chol_kernel<F, 8>, grid, th, smem, st, a, stride);
    case 16: return launch_k(pdl, chol_kernel<F, 16>, grid, th, smem, st, a, stride);
    case 128: return launch_k(pdl, chol_kernel<F, 128>, grid, th, smem, st, a, stride);
    case 256: return launch_k(pdl, chol_kernel<F, 256>, grid, th, smem, st, a, stride);
    default: return launch_k(pdl, chol_kernel<F, 32>, grid, th, smem, st, a, stride);
  }
}

template <typename F>
cudaError_t chol_set_smem(int smax) {
  cudaError_t e = cudaSuccess, r;
  const void* grouped[8] = {(const void*)chol_grouped_kernel<F, 4>,
                            (const void*)chol_grouped_kernel<F, 8>,
                            (const void*)chol_grouped_kernel<F, 16>,
                            (const void*)chol_grouped_kernel<F, 32>,
                            (const void*)chol_grouped_kernel<F, 128>,
                            (const void*)chol_kernel<F, 128>,
                            (const void*)chol_grouped_kernel<F, 256>,
                            (const void*)chol_kernel<F, 256>};
  for (const void* k : grouped) {
    r = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smax);
    if (r != cudaSuccess) e = r;
  }
  r = cudaFuncSetAttribute(chol_kernel<F, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax);
  if (r != cudaSuccess) e = r;
  r = cudaFuncSetAttribute(chol_kernel<F, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax);
  if (r != cudaSuccess) e = r;
  r = cudaFuncSetAttribute(chol_kernel<F, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax);
  if (r != cudaSuccess) e = r;
  r = cudaFuncSetAttribute(chol_kernel<F, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax);
  if (r != cudaSuccess) e = r;
  if constexpr (sizeof(F) == sizeof(double)) {  // the refined solves' instantiation
    r = cudaFuncSetAttribute(chol_refined_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smax);
    if (r != cudaSuccess) e = r;
    r = cudaFuncSetAttribute(chol_refined_grouped_kernel,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, smax);
    if (r != cudaSuccess) e = r;
  }
  return e;
}

// ---------------------------------------------------------------------------
// fixed-point update (one thread per chain)
// ---------------------------------------------------------------------------
struct UpdArgs {
  int mode, C, d;
  double hh, prior_inv, tol;
  int max_iters;
  const StepDev* spd;  // when set (graph path), h / tol / max_iters are read from it
  const float* Gout;  // [2C, ldo] per K slice
  int ldo;
  int gs;          // K slices of the gradient contraction (summed here)
  size_t gstride;  // elements between slices
  // when set (the momentum updates of the generalized leapfrog after fused
  // evaluations): the r₂·X rows come from these g2s N-tile partials,
  // [tile][C][ldo], g2stride elements apart, instead of Gout's rows [C, 2C)
  const float* G2;
  int g2s;
  size_t g2stride;
  const double* u;
  const double* u0;           // generalized leapfrog: G(q0)⁻¹p½
  double *q0, *p0, *qc, *pc;  // FP64 fixed-point iterates
  float* qf;                  // FP32 copy of the position after each step
  double* norm;
  int* iters;
  int* iters_total;
  uint8_t* active;
  uint8_t* notconv;
  SplitMat Qb;
  int* n_active;
};

// the gradient contraction's K slices added in slice order (FP32, as one
// unsplit accumulation would hold them)
__device__ __forceinline__ float slice_sum(const float* p, size_t off, int ns, size_t stride) {
  float v = p[off];
  for (int s = 1; s < ns; ++s) v += p[off + (size_t)s * stride];
  return v;
}

// one warp per chain, lanes over coordinates.  *n_active is only a flag
// (> 0 while some chain iterates): one plain store per block that has an
// active chain, instead of an atomic per chain on one address.
__device__ __forceinline__ void update_body(const UpdArgs& a, int bx) {
  pdl_wait();
  const int lane = threadIdx.x & 31;
  const int c = (bx * blockDim.x + threadIdx.x) >> 5;
  bool act = false;
  if (a.mode >= UP_GLP0) {  // generalized leapfrog (grid-uniform)
    if (c < a.C && !(upd_iterated(a.mode) && !a.active[c])) {  // warp-uniform
      const int d = a.d;
      const double hh = a.spd ? 0.5 * a.spd->h : a.hh;
      const double tol = a.spd ? a.spd->tol : a.tol;
      const int max_iters = a.spd ? a.spd->max_iters : a.max_iters;
      double nrm = 0.0;
      bool nan = false;
      for (int i = lane; i < d; i += 32) {
        const size_t o = (size_t)c * d + i;
        const double q = a.qc[o];
        if (a.mode == UP_GLQ0 || a.mode == UP_GLQN) {
          // q' = q0 + h/2 [G⁻¹(q0) + G⁻¹(q_k)] p½; the eager map uses q_k = q0
          const double uk = a.mode == UP_GLQ0 ? a.u0[o] : a.u[o];
          const double qn = a.q0[o] + hh * (a.u0[o] + uk);
          const double e = qn - q;
          nan |= isnan(e);
          nrm = fmax(nrm, fabs(e));
          a.qc[o] = qn;
          split_store(a.Qb, c, i, float(qn));
        } else {
          // ∂_qH = ∂_qK − ∇ℓ at the current position
          const double g =
              double(slice_sum(a.Gout, (size_t)c * a.ldo + i, a.gs, a.gstride)) - q * a.prior_inv;
          const double dK =
              0.5 * double(slice_sum(a.Gout, (size_t)(a.C + c) * a.ldo + i, a.gs, a.gstride));
          if (a.mode == UP_GLPX) {  // p' = p½ − h/2 ∂_qH(q', p½)
            const double pn = a.pc[o] - hh * (dK - g);
            a.pc[o] = pn;
            a.p0[o] = pn;
            a.q0[o] = q;
            a.qf[o] = float(q);
          } else {  // p½ = p0 − h/2 ∂_qH(q0, p_k)
            const double pn = a.p0[o] - hh * (dK - g);
            const double e = pn - a.pc[o];
            nan |= isnan(e);
            nrm = fmax(nrm, fabs(e));
            a.pc[o] = pn;
          }
        }
      }
      if (a.mode != UP_GLPX) {
        nrm = warp_max(nrm);
        nan = __any_sync(0xffffffffu, nan);
        if (nan) nrm = NAN;
        const int it = upd_iterated(a.mode) ? a.iters[c] + 1 : 0;
        act = (it < max_iters) && isfinite(nrm) && (nrm < 1e10) && (nrm > tol);
        if (lane == 0) {
          a.iters[c] = it;
          a.norm[c] = nrm;
          a.active[c] = act;
          if (upd_iterated(a.mode)) a.iters_total[c] += 1;
          if (!act && !(isfinite(nrm) && nrm <= tol)) a.notconv[c] = 1;
        }
      }
    }
    if (a.mode == UP_GLPX) return;
    if (__syncthreads_or(act) && threadIdx.x == 0) *a.n_active = 1;
    return;
  }
  if (c < a.C && !(a.mode == UP_FPN && !a.active[c])) {  // warp-uniform
    const int d = a.d;
    const double hh = a.spd ? 0.5 * a.spd->h : a.hh;
    const double tol = a.spd ? a.spd->tol : a.tol;
    const int max_iters = a.spd ? a.spd->max_iters : a.max_iters;
    const double* qs = (a.mode == UP_EXPLICIT) ? a.qc : a.q0;
    const double* ps = (a.mode == UP_EXPLICIT) ? a.pc : a.p0;
    double nrm = 0.0;
    bool nan = false;
    for (int i = lane; i < d; i += 32) {
      const size_t o = (size_t)c * d + i;
      const double q = a.qc[o];
      const double g =
          double(slice_sum(a.Gout, (size_t)c * a.ldo + i, a.gs, a.gstride)) - q * a.prior_inv;
      const double dK =
          0.5 * double(slice_sum(a.Gout, (size_t)(a.C + c) * a.ldo + i, a.gs, a.gstride));
      const double qn = qs[o] + hh * a.u[o];
      const double pn = ps[o] - hh * (dK - g);
      const double e1 = qn - q, e2 = pn - a.pc[o];
      nan |= isnan(e1) || isnan(e2);
      nrm = fmax(nrm, fmax(fabs(e1), fabs(e2)));
      a.qc[o] = qn;
      a.pc[o] = pn;
      split_store(a.Qb, c, i, float(qn));
      if (a.mode == UP_EXPLICIT) {
        a.q0[o] = qn;
        a.p0[o] = pn;
        a.qf[o] = float(qn);
      }
    }
    if (a.mode != UP_EXPLICIT) {
      nrm = warp_max(nrm);
      nan = __any_sync(0xffffffffu, nan);
      if (nan) nrm = NAN;
      const int it = (a.mode == UP_FP0) ? 0 : a.iters[c] + 1;
      act = (it < max_iters) && isfinite(nrm) && (nrm < 1e10) && (nrm > tol);
      if (lane == 0) {
        a.iters[c] = it;
        a.norm[c] = nrm;
        a.active[c] = act;
        if (a.mode == UP_FPN) a.iters_total[c] += 1;
        if (!act && !(isfinite(nrm) && nrm <= tol)) a.notconv[c] = 1;
      }
    }
  }
  if (a.mode == UP_EXPLICIT) return;  // uniform over the grid
  if (__syncthreads_or(act) && threadIdx.x == 0) *a.n_active = 1;
}

// u = G⁻¹·rhs with a stored factor (packed column-major lower, L(i, k) at
// colstart(k) + i − k, the diagonal holding 1/L_jj): forward then backward
// substitution, both column-oriented (no reductions: each step broadcasts
// one solved component and the lanes update their rows), one warp per chain
// with lanes over rows (E slots: d <= 32·E).  FP64 divisions and FP64 warp
// reductions cost tens of FP64 instructions each on this part, so neither
// appears here.  y holds the right-hand side on entry (rows lane + 32k) and
// the solution on exit.
template <typename T, int E>
__device__ __forceinline__ void factor_solve(const T* __restrict__ Lc, int d, int lane, T (&y)[E]) {
  auto get = [&](const T(&v)[E], int j) {
    T x = T(0);
#pragma unroll
    for (int k = 0; k < E; ++k)
      if (k == (j >> 5)) x = v[k];
    return __shfl_sync(0xffffffffu, x, j & 31);
  };
  int cj = 0;  // colstart(j)
  for (int j = 0; j < d; ++j) {  // L y = rhs, column j eliminated from the rows below
    const T yj = get(y, j) * Lc[cj];
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int i = lane + 32 * k;
      if (i == j) y[k] = yj;
      else if (i > j && i < d) y[k] -= Lc[cj + i - j] * yj;
    }
    cj += d - j;
  }
  // Lᵀ x = y: x_j final once rows below are done; then row j of L (L(j, i),
  // i < j, at colstart(i) + j − i) updates the components above
  for (int j = d - 1; j >= 0; --j) {
    cj -= d - j;
    const T xj = get(y, j) * Lc[cj];
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int i = lane + 32 * k;
      if (i == j) y[k] = xj;
      else if (i < j) y[k] -= Lc[i * d - i * (i - 1) / 2 + j - i] * xj;
    }
  }
}

// For d <= 32 (E = 1) a warp first copies its chain's factor (at most 528
// entries) into shared memory with coalesced loads: the backward pass reads
// rows of L, whose entries lie in different columns, and those gathers cost
// a wavefront per cache line from L1 but about one from shared memory.
template <typename T, int E>
struct FactorStage {
  __device__ __forceinline__ const T* operator()(const T* g, int, int) const { return g; }
};
template <typename T>
struct FactorStage<T, 1> {
  T* buf;  // this warp's 528 entries
  __device__ __forceinline__ const T* operator()(const T* g, int P, int lane) const {
    for (int t = lane; t < P; t += 32) buf[t] = g[t];
    __syncwarp();
    return buf;
  }
};
constexpr int kSolveWarps = 8;     // warps per block of the solve kernels
constexpr int kStageEntries = 528; // packed entries of a factor with d = 32

// Inactive chains (active set, flag 0) are skipped.
template <typename T, int E>
__device__ __forceinline__ void solve_body(int C, int d, int P, const T* __restrict__ Lf,
                                           const double* __restrict__ rhs, double* u,
                                           const SplitMat& Ub, int split, const uint8_t* active,
                                           int bx) {
  __shared__ T stage[E == 1 ? kSolveWarps * kStageEntries : 1];
  pdl_wait();
  const int lane = threadIdx.x & 31;
  const int c = (bx * blockDim.x + threadIdx.x) >> 5;
  if (c >= C || (active && !active[c])) return;  // warp-uniform
  FactorStage<T, E> sg;
  if constexpr (E == 1) sg.buf = stage + (threadIdx.x >> 5) * kStageEntries;
  const T* Lc = sg(Lf + (size_t)c * P, P, lane);
  T y[E];
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const int i = lane + 32 * k;
    y[k] = i < d ? T(rhs[(size_t)c * d + i]) : T(0);
  }
  factor_solve<T, E>(Lc, d, lane, y);
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const int i = lane + 32 * k;
    if (i < d) {
      if (u) u[(size_t)c * d + i] = double(y[k]);
      if (split) split_store(Ub, c, i, float(y[k]));
    }
  }
}

// The generalized leapfrog's momentum update (UP_GLP0 / UP_GLPN of
// update_kernel) fused with the next momentum evaluation's solve: a chain
// still iterating solves u = G(q0)⁻¹p½ with its new iterate on the FP32
// factor kept at q0 and stores the split copy of u for the S contraction.
// Converged chains solve nothing, so the loop body that follows needs no
// solve of its own.
template <int E>
__device__ __forceinline__ void glp_update_solve_body(const UpdArgs& a,
                                                      const float* __restrict__ Lf, int P,
                                                      const SplitMat& Ub, int bx) {
  __shared__ float stage[E == 1 ? kSolveWarps * kStageEntries : 1];
  pdl_wait();
  const int lane = threadIdx.x & 31;
  const int c = (bx * blockDim.x + threadIdx.x) >> 5;
  bool act = false;
  if (c < a.C && !(a.mode == UP_GLPN && !a.active[c])) {  // warp-uniform
    const int d = a.d;
    const double hh = a.spd ? 0.5 * a.spd->h : a.hh;
    const double tol = a.spd ? a.spd->tol : a.tol;
    const int max_iters = a.spd ? a.spd->max_iters : a.max_iters;
    double nrm = 0.0;
    bool nan = false;
    float y[E];
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int i = lane + 32 * k;
      y[k] = 0.f;
      if (i < d) {
        // p½ = p0 − h/2 ∂_qH(q0, p_k), ∂_qH = ∂_qK − ∇ℓ(q0)
        const size_t o = (size_t)c * d + i;
        const double g = double(slice_sum(a.Gout, (size_t)c * a.ldo + i, a.gs, a.gstride)) -
                         a.qc[o] * a.prior_inv;
        const double dK =
            0.5 * double(a.G2 ? slice_sum(a.G2, (size_t)c * a.ldo + i, a.g2s, a.g2stride)
                              : slice_sum(a.Gout, (size_t)(a.C + c) * a.ldo + i, a.gs, a.gstride));
        const double pn = a.p0[o] - hh * (dK - g);
        const double e = pn - a.pc[o];
        nan |= isnan(e);
        nrm = fmax(nrm, fabs(e));
        a.pc[o] = pn;
        y[k] = float(pn);
      }
    }
    nrm = warp_max(nrm);
    nan = __any_sync(0xffffffffu, nan);
    if (nan) nrm = NAN;
    const int it = a.mode == UP_GLPN ? a.iters[c] + 1 : 0;
    act = (it < max_iters) && isfinite(nrm) && (nrm < 1e10) && (nrm > tol);
    if (lane == 0) {
      a.iters[c] = it;
      a.norm[c] = nrm;
      a.active[c] = act;
      if (a.mode == UP_GLPN) a.iters_total[c] += 1;
      if (!act && !(isfinite(nrm) && nrm <= tol)) a.notconv[c] = 1;
    }
    if (act) {  // warp-uniform
      FactorStage<float, E> sg;
      if constexpr (E == 1) sg.buf = stage + (threadIdx.x >> 5) * kStageEntries;
      const float* Lc = sg(Lf + (size_t)c * P, P, lane);
      factor_solve<float, E>(Lc, d, lane, y);
#pragma unroll
      for (int k = 0; k < E; ++k) {
        const int i = lane + 32 * k;
        if (i < d) split_store(Ub, c, i, y[k]);
      }
    }
  }
  if (__syncthreads_or(act) && threadIdx.x == 0) *a.n_active = 1;
}

struct BeginArgs {
  int C, d;
  const float* pos;
  double *q0, *qc;
  float* qf;
  SplitMat Qb;
  int* iters_total;
  uint8_t *notconv, *bad;
};

__device__ __forceinline__ void begin_body(const BeginArgs& a, int bx) {
  const int C = a.C, d = a.d;
  const float* pos = a.pos;
  double *q0 = a.q0, *qc = a.qc;
  float* qf = a.qf;
  const SplitMat& Qb = a.Qb;
  int* iters_total = a.iters_total;
  uint8_t *notconv = a.notconv, *bad = a.bad;
  const int c = bx * blockDim.x + threadIdx.x;
  if (c >= C) return;
  for (int i = 0; i < d; ++i) {
    const float q = pos[(size_t)c * d + i];
    q0[(size_t)c * d + i] = q;
    qc[(size_t)c * d + i] = q;
    qf[(size_t)c * d + i] = q;
    split_store(Qb, c, i, q);
  }
  iters_total[c] = 0;
  notconv[c] = 0;
  bad[c] = 0;
}

// Accept: H = −ℓ + ½pᵀG⁻¹p + ½ log det G + d/2 log 2π (rmhmc/metrics.py:60-74,
// mcmc/metrics.py:160-166), ℓ at the proposal = data row sums + the prior.
struct AcceptArgs {
  int C, d;
  const double *ld0, *H0q, *logdet0, *ldsum, *quad1, *logdet1, *uacc;
  double div_thr;
  const StepDev* spd;
  double prior_var;
  const double* qc;
  const float* Gout;
  int ldo, gs;
  size_t gstride;
  float *pos, *grad;
  double* logdens;
  InfoDev<float> info;
  const int* iters_total;
  const uint8_t *notconv, *bad;
};

__device__ __forceinline__ void accept_body(const AcceptArgs& A, int bx) {
  const int C = A.C, d = A.d;
  const double *ld0 = A.ld0, *H0q = A.H0q, *logdet0 = A.logdet0, *ldsum = A.ldsum,
               *quad1 = A.quad1, *logdet1 = A.logdet1, *uacc = A.uacc;
  const double div_thr = A.div_thr;
  const StepDev* spd = A.spd;
  const double prior_var = A.prior_var;
  const double* qc = A.qc;
  const float* Gout = A.Gout;
  const int ldo = A.ldo, gs = A.gs;
  const size_t gstride = A.gstride;
  float *pos = A.pos, *grad = A.grad;
  double* logdens = A.logdens;
  const InfoDev<float>& info = A.info;
  const int* iters_total = A.iters_total;
  const uint8_t *notconv = A.notconv, *bad = A.bad;
  pdl_wait();
  const int c = bx * blockDim.x + threadIdx.x;
  if (c >= C) return;
  const double cst = 0.5 * d * kLog2Pi;
  double qq = 0.0;
  for (int i = 0; i < d; ++i) qq += qc[(size_t)c * d + i] * qc[(size_t)c * d + i];
  const double ld1 = ldsum[c] - 0.5 * qq / prior_var - 0.5 * d * (kLog2Pi + log(prior_var));
  const double H0 = -ld0[c] + 0.5 * H0q[c] + 0.5 * logdet0[c] + cst;
  const double H1 = -ld1 + 0.5 * quad1[c] + 0.5 * logdet1[c] + cst;
  const AcceptOut a = metropolis(H0, H1, uacc[c], spd ? spd->div_threshold : div_thr);
  if (info.prop_q)  // RMHMCInfo.proposal.state.position
    for (int i = 0; i < d; ++i) info.prop_q[(size_t)c * d + i] = float(qc[(size_t)c * d + i]);
  if (a.accept) {
    for (int i = 0; i < d; ++i) {
      const double q = qc[(size_t)c * d + i];
      pos[(size_t)c * d + i] = float(q);
      grad[(size_t)c * d + i] =
          float(double(slice_sum(Gout, (size_t)c * ldo + i, gs, gstride)) - q / prior_var);
    }
    logdens[c] = ld1;
  }
  if (info.acc_rate) info.acc_rate[c] = a.p_acc;
  if (info.accepted) info.accepted[c] = a.accept;
  if (info.divergent) info.divergent[c] = a.divergent;
  if (info.energy) info.energy[c] = H1;
  if (info.fp_iters) info.fp_iters[c] = iters_total[c];
  if (info.status)
    info.status[c] = (notconv[c] ? GJ_CHAIN_FP_NOT_CONVERGED : 0u) |
                     (isfinite(H1) ? 0u : GJ_CHAIN_NONFINITE) | (bad[c] ? GJ_CHAIN_NOT_SPD : 0u);
}

// The pipeline's per-chain kernels: ordinary launches, and grouped launches
// over items (one per posterior) in one grid.
__global__ void update_kernel(UpdArgs a) { update_body(a, (int)blockIdx.x); }
__global__ void update_grouped_kernel(const UpdArgs* __restrict__ items,
                                      const int* __restrict__ prefix, int n) {
  const int i = group_item(prefix, n, (int)blockIdx.x);
  update_body(items[i], (int)blockIdx.x - __ldg(prefix + i));
}

struct SolveItem {
  int C, d, P;
  const void* Lf;
  const double* rhs;
  double* u;
  SplitMat Ub;
  int split;
  const uint8_t* active;
};
template <typename T, int E>
__global__ void __launch_bounds__(32 * kSolveWarps)
    solve_kernel(int C, int d, int P, const T* __restrict__ Lf, const double* __restrict__ rhs,
                 double* u, SplitMat Ub, int split, const uint8_t* active) {
  solve_body<T, E>(C, d, P, Lf, rhs, u, Ub, split, active, (int)blockIdx.x);
}
template <typename T, int E>
__global__ void __launch_bounds__(32 * kSolveWarps)
    solve_grouped_kernel(const SolveItem* __restrict__ items, const int* __restrict__ prefix,
                         int n) {
  const int i = group_item(prefix, n, (int)blockIdx.x);
  const SolveItem& it = items[i];
  solve_body<T, E>(it.C, it.d, it.P, static_cast<const T*>(it.Lf), it.rhs, it.u, it.Ub, it.split,
                   it.active, (int)blockIdx.x - __ldg(prefix + i));
}

struct GlpItem {
  UpdArgs a;
  const float* Lf;
  int P;
  SplitMat Ub;
};
template <int E>
__global__ void __launch_bounds__(32 * kSolveWarps)
    glp_update_solve_kernel(UpdArgs a, const float* __restrict__ Lf, int P, SplitMat Ub) {
  glp_update_solve_body<E>(a, Lf, P, Ub, (int)blockIdx.x);
}
template <int E>
__global__ void __launch_bounds__(32 * kSolveWarps)
    glp_update_solve_grouped_kernel(const GlpItem* __restrict__ items,
                                    const int* __restrict__ prefix, int n) {
  const int i = group_item(prefix, n, (int)blockIdx.x);
  glp_update_solve_body<E>(items[i].a, items[i].Lf, items[i].P, items[i].Ub,
                           (int)blockIdx.x - __ldg(prefix + i));
}

__global__ void begin_kernel(BeginArgs a) { begin_body(a, (int)blockIdx.x); }
__global__ void begin_grouped_kernel(const BeginArgs* __restrict__ items,
                                     const int* __restrict__ prefix, int n) {
  const int i = group_item(prefix, n, (int)blockIdx.x);
  begin_body(items[i], (int)blockIdx.x - __ldg(prefix + i));
}

__global__ void accept_kernel(AcceptArgs a) { accept_body(a, (int)blockIdx.x); }
__global__ void accept_grouped_kernel(const AcceptArgs* __restrict__ items,
                                      const int* __restrict__ prefix, int n) {
  const int i = group_item(prefix, n, (int)blockIdx.x);
  accept_body(items[i], (int)blockIdx.x - __ldg(prefix + i));
}

// zero fill of `words` 4-byte words (a grouped launch's memsets)
struct ZeroItem {
  uint32_t* p;
  long long words;
};
constexpr int kZeroPerBlock = 4096;  // words per block of zero_grouped_kernel
__global__ void zero_grouped_kernel(const ZeroItem* __restrict__ items,
                                    const int* __restrict__ prefix, int n) {
  const int i = group_item(prefix, n, (int)blockIdx.x);
  const ZeroItem it = items[i];
  const long long w0 = (long long)((int)blockIdx.x - __ldg(prefix + i)) * kZeroPerBlock;
  for (long long w = w0 + threadIdx.x; w < it.words && w < w0 + kZeroPerBlock; w += blockDim.x)
    it.p[w] = 0u;
}

// Sets the WHILE condition of the fixed-point loop node: iterate while a
// chain is active, at most max_iters + 1 body executions per solve.
// The flag is cleared here for the next body, so the body holds only
// kernels (programmatic dependencies chain kernel to kernel).
__global__ void loop_cond_kernel(cudaGraphConditionalHandle h, int* n_active, int* trips,
                                 const StepDev* spd) {
  pdl_wait();
  const int t = *trips;
  *trips = t + 1;
  const bool more = (*n_active > 0) && (t <= spd->max_iters);
  *n_active = 0;
  cudaGraphSetConditional(h, more ? 1u : 0u);
}

template <typename Tp>
Tp* dalloc(size_t n, std::vector<void*>& owned, bool* ok) {
  void* p = nullptr;
  if (cudaMalloc(&p, n * sizeof(Tp) + 256) != cudaSuccess) {
    *ok = false;
    return nullptr;
  }
  cudaMemset(p, 0, n * sizeof(Tp) + 256);
  owned.push_back(p);
  return static_cast<Tp*>(p);
}

// K slices of the gradient contraction [r₁; r₂]·X at most (its output
// buffer holds this many partial products)
constexpr int kMaxGoutSlices = 4;

}  // namespace

struct LogregBatched {
  TargetDev t;
  int C, N, d, P, dpad, Npad, Pp;
  std::vector<void*> owned;
  // constants
  SplitMat Xb, XTb, Zb, Zt;
  // per-chain buffers
  SplitMat Qb, Ub, Lam, Giv, Rb;
  float *Lp, *S, *Gv, *Gout;
  double *q0, *p0, *qc, *pc;
  float *qf, *gnew;
  double *u, *norm, *logdet0, *quad0, *logdet1, *quad1, *ldnew;
  // generalized leapfrog (allocated on first use): the factor and
  // w = x_nᵀG⁻¹x_n at the step's start position, and G(q0)⁻¹p½
  double *Lf, *u0;
  float *W, *Lf32;
  // the momentum evaluations' fused r₂·X partials, [tile][C][dpad] for up
  // to g2_tiles N tiles (allocated with the other generalized-leapfrog
  // buffers)
  float* G2;
  int g2_tiles;
  int fuse_r2x;  // logreg_batched_set_fuse_r2x
  int refine;    // logreg_batched_set_refine_iterates
  int *iters, *iters_total, *n_active_d;
  int* n_active_h;  // pinned
  uint8_t *active, *notconv, *bad;
  int* tc_err;
  int* refine_fb;  // refined solves that fell back (profiling on)
  TcOperand *tXb, *tXTb, *tZb, *tZt, *tQb, *tUb, *tLam, *tGiv, *tRb;
  bool tc_ok;
  int chol_fp64;
  int chol_cpw;  // chains per warp in the factorisation (0 = automatic)
  int pdl;       // launch the pipeline's kernels as programmatic dependents
  int gsplit_req;  // K slices of the gradient contraction (0 = automatic)
  int auto_C;      // chains the automatic rules (K slices, chains per warp)
                   // size their grids for
  int sms;         // multiprocessors of the device
  int prof;
  // graph path: device step parameters, staging buffers, captured graph
  StepDev* spd;
  float *pos_s, *grad_s, *z_s, *mom_s, *propq_s, *propv_s;
  double *ld_s, *u_s, *acc_s, *energy_s;
  uint8_t *accepted_s, *divergent_s, *status_s;
  int* fpit_s;
  int* trips;
  cudaStream_t cap_main, cap_body;
  // Captured transitions, one per (number of steps, GEMM implementation,
  // factorisation set-up, proposal velocity wanted), least recently used
  // evicted beyond kMaxGraphs: a jittered trajectory length
  // (rmhmc/rmhmc.py:179-244) draws the number of steps per transition.
  struct Graph {
    int L, impl, cfg, prop;
    cudaGraphExec_t exec;
    unsigned long long used;
  };
  std::vector<Graph> graphs;
  unsigned long long graph_tick;
  std::vector<cudaEvent_t> ev;
  size_t ev_used;
  std::vector<cudaEvent_t> cev;  // the same around the factorisations
  size_t cev_used;
  std::vector<cudaEvent_t> rev;  // the same around the refined iterate solves
  size_t rev_used;
  LogregStats stats;
};

const char* logreg_batched_error() { return g_err.c_str(); }

LogregStats logreg_batched_stats(const LogregBatched* lb) { return lb->stats; }
void logreg_batched_set_chol_fp64(LogregBatched* lb, int on) { lb->chol_fp64 = on; }
void logreg_batched_set_chol_cpw(LogregBatched* lb, int cpw) { lb->chol_cpw = cpw; }
void logreg_batched_set_pdl(LogregBatched* lb, int on) { lb->pdl = on; }
void logreg_batched_set_gemm_ksplit(LogregBatched* lb, int k) { lb->gsplit_req = k; }
void logreg_batched_set_fuse_r2x(LogregBatched* lb, int on) { lb->fuse_r2x = on ? 1 : 0; }
void logreg_batched_set_refine_iterates(LogregBatched* lb, int on) { lb->refine = on ? 1 : 0; }
void logreg_batched_set_auto_chains(LogregBatched* lb, int C) { lb->auto_C = C > 0 ? C : lb->C; }

// K slices of the gradient contractions [r₁; r₂]·X (M = 2C) and r₂·X
// (M = C, the momentum evaluations of the generalized leapfrog), N = d,
// K = N observations: few output tiles (32 for M = C at 4096 chains and
// d <= 32) and a long K, so K is split until the M = C grid fills the SMs
// once, keeping at least 4 K blocks per slice.  The SIMT path does not
// split.
static int gout_split(const LogregBatched* lb, int impl) {
  if (impl != 2) return 1;
  const int kb = (lb->N + 63) / 64;
  int s;
  if (lb->gsplit_req > 0) {
    s = std::min(lb->gsplit_req, kMaxGoutSlices);
  } else {
    const int bn = lb->d <= 32 ? 32 : (lb->d <= 64 ? 64 : 128);
    const int tiles = ((lb->d + bn - 1) / bn) * ((lb->auto_C + 127) / 128);
    s = std::max(1, std::min(kMaxGoutSlices, lb->sms / std::max(tiles, 1)));
    while (s > 1 && kb / s < 4) --s;
  }
  while (s > 1 && !gemm_ksplit_valid(lb->N, s)) --s;
  return s;
}
void logreg_batched_set_profile(LogregBatched* lb, int on) { lb->prof = on; }

static SplitMat make_split(LogregBatched* lb, int rows, int kdim, int planes, bool* ok) {
  SplitMat s;
  s.rows = rows;
  s.kdim = kdim;
  s.ld = roundup(kdim, 64);
  s.rpad = roundup(rows, 128);
  s.planes = planes;
  s.p = dalloc<bf16>((size_t)planes * s.rpad * s.ld, lb->owned, ok);
  return s;
}

void logreg_batched_destroy(LogregBatched* lb) {
  if (!lb) return;
  TcOperand* ops[] = {lb->tXb, lb->tXTb, lb->tZb, lb->tZt, lb->tQb,
                      lb->tUb, lb->tLam, lb->tGiv, lb->tRb};
  for (TcOperand* o : ops)
    if (o) tc_operand_destroy(o);
  for (void* p : lb->owned) cudaFree(p);
  for (cudaEvent_t e : lb->ev) cudaEventDestroy(e);
  for (cudaEvent_t e : lb->cev) cudaEventDestroy(e);
  for (cudaEvent_t e : lb->rev) cudaEventDestroy(e);
  for (auto& g : lb->graphs) cudaGraphExecDestroy(g.exec);
  if (lb->cap_main) cudaStreamDestroy(lb->cap_main);
  if (lb->cap_body) cudaStreamDestroy(lb->cap_body);
  if (lb->n_active_h) cudaFreeHost(lb->n_active_h);
  delete lb;
}

int logreg_batched_create(const TargetDev& t, int C, LogregBatched** out) {
  *out = nullptr;
  if (t.d > 128) {
    g_err = "batched logistic-regression path supports d <= 128";
    return GJ_ENOTSUP;
  }
  LogregBatched* lb = new LogregBatched();
  lb->t = t;
  lb->C = C;
  lb->N = t.n;
  lb->d = t.d;
  lb->P = t.d * (t.d + 1) / 2;
  lb->chol_fp64 = 1;
  lb->chol_cpw = 0;
  lb->pdl = 0;
  lb->gsplit_req = 0;
  lb->fuse_r2x = 1;
  lb->refine = 1;
  lb->auto_C = C;
  lb->sms = 0;
  {
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess)
      cudaDeviceGetAttribute(&lb->sms, cudaDevAttrMultiProcessorCount, dev);
  }
  lb->prof = 0;
  lb->ev_used = 0;
  lb->cev_used = 0;
  lb->rev_used = 0;
  lb->graph_tick = 0;
  lb->cap_main = lb->cap_body = nullptr;
  lb->stats = LogregStats{};
  bool ok = true;
  const int N = lb->N, d = lb->d, P = lb->P;
  // Operands whose rounding feeds the fixed-point map at first order (Xβ,
  // x_nᵀu and the gradient contraction) use three planes, so the map is
  // FP32-smooth and converges to the absolute tolerance; the Gram and trace
  // operands enter through G⁻¹ only and use two.
  lb->Xb = make_split(lb, N, d, 3, &ok);
  lb->XTb = make_split(lb, d, N, 3, &ok);
  lb->Zb = make_split(lb, N, P, 2, &ok);
  lb->Zt = make_split(lb, P, N, 2, &ok);
  lb->Qb = make_split(lb, C, d, 3, &ok);
  lb->Ub = make_split(lb, C, d, 3, &ok);
  lb->Lam = make_split(lb, C, N, 2, &ok);
  lb->Giv = make_split(lb, C, P, 2, &ok);
  lb->Rb = make_split(lb, 2 * C, N, 3, &ok);
  lb->dpad = roundup(d, 8);
  lb->Npad = roundup(N, 8);
  lb->Pp = roundup(P, 8);
  lb->Lp = dalloc<float>((size_t)C * lb->Npad, lb->owned, &ok);
  lb->S = dalloc<float>((size_t)C * lb->Npad, lb->owned, &ok);
  lb->Gv = dalloc<float>((size_t)C * lb->Pp, lb->owned, &ok);
  lb->Gout = dalloc<float>((size_t)kMaxGoutSlices * 2 * C * lb->dpad, lb->owned, &ok);
  lb->q0 = dalloc<double>((size_t)C * d, lb->owned, &ok);
  lb->p0 = dalloc<double>((size_t)C * d, lb->owned, &ok);
  lb->qc = dalloc<double>((size_t)C * d, lb->owned, &ok);
  lb->pc = dalloc<double>((size_t)C * d, lb->owned, &ok);
  lb->qf = dalloc<float>((size_t)C * d, lb->owned, &ok);
  lb->gnew = dalloc<float>((size_t)C * d, lb->owned, &ok);
  lb->u = dalloc<double>((size_t)C * d, lb->owned, &ok);
  lb->norm = dalloc<double>(C, lb->owned, &ok);
  lb->logdet0 = dalloc<double>(C, lb->owned, &ok);
  lb->quad0 = dalloc<double>(C, lb->owned, &ok);
  lb->logdet1 = dalloc<double>(C, lb->owned, &ok);
  lb->quad1 = dalloc<double>(C, lb->owned, &ok);
  lb->ldnew = dalloc<double>(C, lb->owned, &ok);
  lb->iters = dalloc<int>(C, lb->owned, &ok);
  lb->iters_total = dalloc<int>(C, lb->owned, &ok);
  lb->n_active_d = dalloc<int>(1, lb->owned, &ok);
  lb->active = dalloc<uint8_t>(C, lb->owned, &ok);
  lb->notconv = dalloc<uint8_t>(C, lb->owned, &ok);
  lb->bad = dalloc<uint8_t>(C, lb->owned, &ok);
  lb->tc_err = dalloc<int>(1, lb->owned, &ok);
  lb->refine_fb = dalloc<int>(1, lb->owned, &ok);
  lb->spd = dalloc<StepDev>(1, lb->owned, &ok);
  lb->pos_s = dalloc<float>((size_t)C * d, lb->owned, &ok);
  lb->grad_s = dalloc<float>((size_t)C * d, lb->owned, &ok);
  lb->z_s = dalloc<float>((size_t)C * d, lb->owned, &ok);
  lb->mom_s = dalloc<float>((size_t)C * d, lb->owned, &ok);
  lb->propq_s = dalloc<float>((size_t)C * d, lb->owned, &ok);
  lb->propv_s = dalloc<float>((size_t)C * d, lb->owned, &ok);
  lb->ld_s = dalloc<double>(C, lb->owned, &ok);
  lb->u_s = dalloc<double>(C, lb->owned, &ok);
  lb->acc_s = dalloc<double>(C, lb->owned, &ok);
  lb->energy_s = dalloc<double>(C, lb->owned, &ok);
  lb->accepted_s = dalloc<uint8_t>(C, lb->owned, &ok);
  lb->divergent_s = dalloc<uint8_t>(C, lb->owned, &ok);
  lb->status_s = dalloc<uint8_t>(C, lb->owned, &ok);
  lb->fpit_s = dalloc<int>(C, lb->owned, &ok);
  lb->trips = dalloc<int>(1, lb->owned, &ok);
  if (cudaStreamCreateWithFlags(&lb->cap_main, cudaStreamNonBlocking) != cudaSuccess) ok = false;
  if (cudaStreamCreateWithFlags(&lb->cap_body, cudaStreamNonBlocking) != cudaSuccess) ok = false;
  if (cudaMallocHost(&lb->n_active_h, sizeof(int)) != cudaSuccess) ok = false;
  if (!ok) {
    g_err = "device allocation failed in the batched logistic-regression context";
    logreg_batched_destroy(lb);
    return GJ_ENOMEM;
  }
  build_consts_kernel<<<N, 128>>>(static_cast<const float*>(t.X), N, d, P, lb->Xb, lb->XTb, lb->Zb,
                                  lb->Zt);
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    g_err = std::string("building logistic-regression constants: ") + cudaGetErrorString(e);
    logreg_batched_destroy(lb);
    return GJ_ECUDA;
  }
  {
    // the largest layout any chains-per-warp choice can ask for.  The
    // kernel attribute is process-wide and shared by every context, so it
    // only ever grows (a context for a small d must not lower the limit a
    // larger context's captured launches rely on).
    static size_t s_chol_smem = 0;
    static std::mutex s_mu;  // contexts may be created from several threads
    std::lock_guard<std::mutex> lock(s_mu);
    size_t smax = 0;
    for (int cpw = 1; cpw <= 8; cpw *= 2) {
      smax = std::max(smax, chol_config(d, sizeof(double), cpw).smem);
      smax = std::max(smax, chol_config(d, sizeof(float), cpw).smem);
    }
    cudaError_t a1 = cudaSuccess, a2 = cudaSuccess;
    if (smax > s_chol_smem) {
      a1 = chol_set_smem<double>((int)smax);
      a2 = chol_set_smem<float>((int)smax);
      if (a1 == cudaSuccess && a2 == cudaSuccess) s_chol_smem = smax;
    }
    if (a1 != cudaSuccess || a2 != cudaSuccess) {
      g_err = "metric factorisation needs more shared memory than the device allows";
      logreg_batched_destroy(lb);
      return GJ_ENOTSUP;
    }
  }
  lb->tc_ok = false;
  if (tc_available() && gemm_tc_prepare() == cudaSuccess) {
    const char* err = nullptr;
    lb->tXb = tc_operand_create(lb->Xb, 0, &err);
    lb->tXTb = tc_operand_create(lb->XTb, 0, &err);
    lb->tZb = tc_operand_create(lb->Zb, 0, &err);
    lb->tZt = tc_operand_create(lb->Zt, 0, &err);
    lb->tQb = tc_operand_create(lb->Qb, 0, &err);
    lb->tUb = tc_operand_create(lb->Ub, 0, &err);
    lb->tLam = tc_operand_create(lb->Lam, 0, &err);
    lb->tGiv = tc_operand_create(lb->Giv, 0, &err);
    lb->tRb = tc_operand_create(lb->Rb, 0, &err);
    lb->tc_ok = lb->tXb && lb->tXTb && lb->tZb && lb->tZt && lb->tQb && lb->tUb && lb->tLam &&
                lb->tGiv && lb->tRb;
  }
  *out = lb;
  return GJ_OK;
}

namespace {

// A recorded launch of the pipeline.  A batch of posteriors records each
// posterior's transition as such a list (the same list for every posterior
// up to sizes and addresses), then replays the lists side by side: every
// op becomes one grouped launch over the posteriors' items (one per kernel
// variant present), every loop one conditional WHILE node for the batch.
enum OpKind : int {
  OP_GEMM,
  OP_CHOL,
  OP_SOLVE,
  OP_UPDATE,
  OP_GLPUS,
  OP_BEGIN,
  OP_ACCEPT,
  OP_ZERO,
  OP_FLAG_CLEAR,   // the active-chain flag := 0
  OP_TRIPS_CLEAR,  // the loop trip counter := 0
  OP_LOOP_BEGIN,   // condition kernel, then the WHILE node's body starts
  OP_LOOP_END      // condition kernel at the end of the body
};
struct Op {
  int kind = 0;
  int variant = 0;  // kernel template selector
  int blocks = 0;   // CTAs
  int threads = 0;
  size_t smem = 0;  // dynamic shared memory
  std::vector<unsigned char> item;  // the kernel's item (argument struct) bytes
};
struct Recorder {
  std::vector<Op> ops;
  int* flag = nullptr;   // the batch's active-chain flag, shared by its posteriors
  template <typename T>
  void push(int kind, int variant, int blocks, int threads, size_t smem, const T& it) {
    static_assert(std::is_trivially_copyable<T>::value, "items are copied as bytes");
    Op o;
    o.kind = kind;
    o.variant = variant;
    o.blocks = blocks;
    o.threads = threads;
    o.smem = smem;
    o.item.resize(sizeof(T));
    std::memcpy(o.item.data(), &it, sizeof(T));
    ops.push_back(std::move(o));
  }
  void mark(int kind) {
    Op o;
    o.kind = kind;
    ops.push_back(std::move(o));
  }
};

struct Runner {
  LogregBatched* lb;
  int impl;
  cudaStream_t st;
  cudaError_t err = cudaSuccess;
  const StepDev* spd = nullptr;  // graph path: step parameters in device memory
  StepDev hsp{};                 // host path: the step parameters
  Recorder* rec = nullptr;       // record instead of launching (grouped batches)
  // inside a fixed-point loop body: contractions skip the tiles whose chains
  // have all converged (their outputs are not read before the evaluation
  // after the loop, which recomputes them)
  bool loop_body = false;
  const uint8_t* rows_active() const { return loop_body ? lb->active : nullptr; }

  int* active_flag() const { return rec ? rec->flag : lb->n_active_d; }
  // zero `bytes` (a multiple of 4) at p
  void zero(void* p, size_t bytes) {
    if (rec) {
      ZeroItem z{static_cast<uint32_t*>(p), (long long)(bytes / 4)};
      rec->push(OP_ZERO, 0, (int)((z.words + kZeroPerBlock - 1) / kZeroPerBlock), 256, 0, z);
      return;
    }
    check(cudaMemsetAsync(p, 0, bytes, st));
  }
  // the transition's start: positions into the FP64 iterates and the split Q
  void begin(const float* pos) {
    LogregBatched& L = *lb;
    BeginArgs b{L.C, L.d, pos, L.q0, L.qc, L.qf, L.Qb, L.iters_total, L.notconv, L.bad};
    if (rec) {
      rec->push(OP_BEGIN, 0, (L.C + 127) / 128, 128, 0, b);
      return;
    }
    begin_kernel<<<(L.C + 127) / 128, 128, 0, st>>>(b);
    check(cudaGetLastError());
  }

  void gemm(const SplitMat& A, const TcOperand* ta, const SplitMat& B, const TcOperand* tb, int M,
            int N, int K, const Epi& e, int ksplit = 1, int a_row0 = 0) {
    if (err != cudaSuccess) return;
    GemmArgs g;
    g.A = A;
    g.B = B;
    g.M = M;
    g.N = N;
    g.K = K;
    g.epi = e;
    g.pdl = lb->pdl != 0;
    g.ksplit = ksplit;
    g.a_row0 = a_row0;
    if (rec) {
      GemmItem it;
      int variant = 0, blocks = 0;
      size_t smem = 0;
      g.pdl = false;
      err = impl == 2 ? gemm_tc_describe(g, ta, tb, lb->tc_err, &it, &variant, &blocks, &smem)
                      : cudaErrorNotSupported;
      if (err == cudaSuccess) rec->push(OP_GEMM, variant, blocks, 320, smem, it);
      lb->stats.gemm_launches++;
      lb->stats.gemm_flops += 2.0 * M * N * K;
      return;
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (lb->prof) {
      while (lb->ev.size() < lb->ev_used + 2) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) break;
        lb->ev.push_back(e);
      }
      if (lb->ev.size() >= lb->ev_used + 2) {
        e0 = lb->ev[lb->ev_used];
        e1 = lb->ev[lb->ev_used + 1];
        lb->ev_used += 2;
        cudaEventRecord(e0, st);
      }
    }
    if (impl == 2)
      err = gemm_tc(g, ta, tb, lb->tc_err, st);
    else
      err = gemm_simt(g, st);
    if (e1) cudaEventRecord(e1, st);
    lb->stats.gemm_launches++;
    lb->stats.gemm_flops += 2.0 * M * N * K;
  }
  void check(cudaError_t e) {
    if (err == cudaSuccess) err = e;
    lb->stats.other_launches++;
  }
  // rows [row0, row0 + M) of the gradient contraction [r₁; r₂]·X into the
  // same rows of Gout, in gsplit() K slices gstride() elements apart: all
  // 2C rows at a full evaluation, r₁·X (rows [0, C)) for the energy, r₂·X
  // (rows [C, 2C)) for the momentum evaluations of the generalized leapfrog,
  // whose r₁·X at the fixed position stays from the evaluation there
  int gsplit() const { return gout_split(lb, impl); }
  size_t gstride() const { return (size_t)2 * lb->C * lb->dpad; }
  void grad_gemm(int row0, int M) {
    LogregBatched& L = *lb;
    if (impl != 2 && row0 > 0) {  // the SIMT GEMM takes no row offset: all rows
      M += row0;
      row0 = 0;
    }
    Epi o{};
    o.mode = EPI_STORE;
    o.D = L.Gout + (size_t)row0 * L.dpad;
    o.ldd = L.dpad;
    o.d_slice = gstride();
    if (M == L.C) o.active_rows = rows_active();  // output row m is chain m
    gemm(L.Rb, L.tRb, L.XTb, L.tXTb, M, L.d, L.N, o, gsplit(), row0);
  }

  // metric at the current iterate: (1) and (2); with ld_acc the Xβ epilogue
  // also sums the data log likelihood per chain
  void metric_gram(double* ld_acc = nullptr, bool lam_only = false) {
    LogregBatched& L = *lb;
    Epi e{};
    e.mode = EPI_SIGMOID;
    e.ld_acc = ld_acc;
    e.lam_only = lam_only ? 1 : 0;
    e.y = static_cast<const float*>(L.t.y);
    e.lam = L.Lam;
    e.lp = L.Lp;
    e.lp_ld = L.Npad;
    e.r = L.Rb;
    e.active_rows = rows_active();
    gemm(L.Qb, L.tQb, L.Xb, L.tXb, L.C, L.N, L.d, e);
    Epi g{};
    g.mode = EPI_STORE;
    g.D = L.Gv;
    g.ldd = L.Pp;
    g.active_rows = rows_active();
    gemm(L.Lam, L.tLam, L.Zt, L.tZt, L.C, L.P, L.N, g);
  }

  void chol(int mode, const float* z, double* logdet, double* quad, float* mom_info,
            bool only_active = false, float* vel_info = nullptr, double* Lout = nullptr,
            bool no_inverse = false, float* Lout32 = nullptr, bool q_update = false) {
    LogregBatched& L = *lb;
    CholArgs a{};
    if (q_update) {
      a.q_update = 1;
      a.spd = spd;
      a.hh = 0.5 * hsp.h;
      a.tol = hsp.tol;
      a.max_iters = hsp.max_iters;
      a.u0 = L.u0;
      a.q0 = L.q0;
      a.qc = L.qc;
      a.Qb = L.Qb;
      a.norm = L.norm;
      a.iters = L.iters;
      a.iters_total = L.iters_total;
      a.active_w = L.active;
      a.notconv = L.notconv;
      a.n_active = L.n_active_d;
    }
    a.mode = mode;
    a.C = L.C;
    a.d = L.d;
    a.P = L.P;
    a.prior_inv = 1.0 / L.t.p0;
    a.Gv = L.Gv;
    a.gv_ld = L.Pp;
    a.z = z;
    a.p0 = L.p0;
    a.pc = L.pc;
    a.u = L.u;
    a.Ub = L.Ub;
    a.Giv = L.Giv;
    a.logdet = logdet;
    a.quad = quad;
    a.active = only_active ? L.active : nullptr;
    a.bad = L.bad;
    a.mom_info = mom_info;
    a.vel_info = vel_info;
    a.Lout = Lout;
    a.Lout32 = Lout32;
    a.no_inverse = no_inverse ? 1 : 0;
    CholCfg cf =
        chol_config(L.d, L.chol_fp64 ? sizeof(double) : sizeof(float), L.chol_cpw, L.auto_C);
    // the position iterates' solves by FP32 factor and FP64 refinement
    // (the L⁻¹ area parks d doubles: d >= 3)
    a.refine = (L.refine && no_inverse && q_update && L.chol_fp64 && cf.lpc <= 32 && L.d >= 3)
                   ? 1 : 0;
    // The refined solves issue few FP64 instructions (d per row and
    // correction) and are bound by the latency of their serial column steps,
    // so they take one chain per warp (four times the warps of the FP64
    // factorisation's automatic packing; GJ_OPT_CHOL_CHAINS_PER_WARP applies
    // to the FP64 factorisations), which also gives d <= 32 the register
    // form.  Measured with the shared-memory form on the generalized leapfrog
    // at N = 1000, d = 25, 4096 chains: 49 / 53 / 67 µs per launch at 1 / 2 /
    // 4 chains per warp, against 72 µs for the FP64 factorisation; 43 µs in
    // the register form.
    if (a.refine) {
      const CholCfg rc = chol_config(L.d, sizeof(double), 1, L.auto_C);
      if (rc.lpc == 32)  // always for d <= 64
        cf = rc;
      else
        a.refine = 0;
    }
    std::vector<cudaEvent_t>& evs = a.refine ? L.rev : L.cev;
    size_t& used = a.refine ? L.rev_used : L.cev_used;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (L.prof) {
      while (evs.size() < used + 2) {
        cudaEvent_t ev;
        if (cudaEventCreate(&ev) != cudaSuccess) break;
        evs.push_back(ev);
      }
      if (evs.size() >= used + 2) {
        e0 = evs[used];
        e1 = evs[used + 1];
        used += 2;
        cudaEventRecord(e0, st);
      }
    }
    const double dd = L.d;
    if (a.refine) {
      a.fallbacks = L.prof ? L.refine_fb : nullptr;
      L.stats.refine_launches++;
    } else {
      L.stats.chol_launches++;
      const double solves = (mode == CH_ENERGY && !vel_info) ? 1.0 : 2.0;
      L.stats.chol_flops += (double)L.C * (dd * dd * dd / 3.0 + solves * dd * dd);
    }
    const int per_cta = cf.chains;
    const dim3 grid((L.C + per_cta - 1) / per_cta);
    const size_t smem = cf.smem;
    if (rec) {
      if (a.q_update) a.n_active = rec->flag;
      CholItem it{a, (int)cf.stride};
      // variants: FP32 lpc, FP64 100 + lpc, refined solves 400 + lpc
      rec->push(OP_CHOL, (a.refine ? 400 : (L.chol_fp64 ? 100 : 0)) + cf.lpc, (int)grid.x,
                32 * cf.warps, smem, it);
      return;
    }
    // the dynamic shared-memory limit was raised at context creation
    check(L.chol_fp64 ? chol_launch<double>(cf, smem, grid, a, L.pdl, st)
                      : chol_launch<float>(cf, smem, grid, a, L.pdl, st));
    if (e1) cudaEventRecord(e1, st);
  }

  // (4)-(6) after the factorisation
  void trace_grad(float* w_out = nullptr) {
    LogregBatched& L = *lb;
    Epi s{};
    s.mode = EPI_STORE;
    s.D = L.S;
    s.ldd = L.Npad;
    s.active_rows = rows_active();
    gemm(L.Ub, L.tUb, L.Xb, L.tXb, L.C, L.N, L.d, s);
    Epi w{};
    w.mode = EPI_TRACE;
    w.active_rows = rows_active();
    w.w_out = w_out;
    w.S = L.S;
    w.s_ld = L.Npad;
    w.lp = L.Lp;
    w.lp_ld = L.Npad;
    w.r = L.Rb;
    w.r_off = L.C;
    gemm(L.Giv, L.tGiv, L.Zb, L.tZb, L.C, L.N, L.P, w);
    grad_gemm(0, 2 * L.C);
  }

  // ---- generalized leapfrog (Girolami and Calderhead 2011, eqs. 16-18)
  // out = G⁻¹·rhs with the factor stored at the step's start position
  // fp32: with the FP32 copy of the factor, for the momentum evaluations,
  // whose u reaches ∂_qK only through the split-BF16 product s = x_nᵀu
  // (FP32-level either way); the FP64 factor serves G(q0)⁻¹p½, which enters
  // the position iterates
  template <typename T>
  void solve_t(const T* Lf, const double* rhs, double* out, bool split, const uint8_t* act) {
    LogregBatched& L = *lb;
    // one warp per chain, kSolveWarps warps per block (the staging buffers)
    const dim3 th(32 * kSolveWarps), grid((unsigned)(((size_t)L.C + kSolveWarps - 1) / kSolveWarps));
    if (rec) {
      SolveItem it{L.C, L.d, L.P, Lf, rhs, out, L.Ub, split ? 1 : 0, act};
      const int E = L.d <= 32 ? 1 : (L.d <= 64 ? 2 : 4);
      rec->push(OP_SOLVE, (sizeof(T) == sizeof(double) ? 10 : 0) + E, (int)grid.x, (int)th.x, 0, it);
      return;
    }
    if (L.d <= 32)
      check(launch_k(L.pdl, solve_kernel<T, 1>, grid, th, 0, st, L.C, L.d, L.P, Lf, rhs, out,
                     L.Ub, split ? 1 : 0, act));
    else if (L.d <= 64)
      check(launch_k(L.pdl, solve_kernel<T, 2>, grid, th, 0, st, L.C, L.d, L.P, Lf, rhs, out,
                     L.Ub, split ? 1 : 0, act));
    else
      check(launch_k(L.pdl, solve_kernel<T, 4>, grid, th, 0, st, L.C, L.d, L.P, Lf, rhs, out,
                     L.Ub, split ? 1 : 0, act));
    L.stats.other_launches++;
  }
  void solve(const double* rhs, double* out, bool split, bool only_active, bool fp32 = false) {
    LogregBatched& L = *lb;
    const uint8_t* act = only_active ? L.active : nullptr;
    if (fp32)
      solve_t<float>(L.Lf32, rhs, out, split, act);
    else
      solve_t<double>(L.Lf, rhs, out, split, act);
  }
  // ∂_qH at the step's start position q0 for the current momentum: the
  // metric, its factor, Λ' and w = x_nᵀG⁻¹x_n are those of q0 (kept from
  // the evaluation that ended the previous step), so only u = G⁻¹p,
  // s = x_nᵀu and the two contractions are recomputed.  Inside the
  // fixed-point loop the solve is done by the momentum update before it
  // (glp_update_solve_kernel), so the loop body is p_contract() alone.
  void p_eval() {
    solve(lb->pc, nullptr, true, false, true);
    p_contract();
  }
  // the fused form: r₂·X in the S GEMM's epilogue, one partial per N tile
  int g2_tiles_used() const {
    const int bn = gemm_tc_bn(3, lb->N, lb->d);
    return (lb->N + bn - 1) / bn;
  }
  bool fused_r2x() const {
    return impl == 2 && lb->fuse_r2x && lb->d <= 32 && lb->G2 && lb->tXTb &&
           gemm_tc_bn(3, lb->N, lb->d) == 128 && g2_tiles_used() <= lb->g2_tiles;
  }
  // s = x_nᵀu and r₂ = Λ'(w − s²) from the split u, then r₂·X
  void p_contract() {
    LogregBatched& L = *lb;
    if (fused_r2x()) {
      Epi f{};
      f.mode = EPI_R2G;
      f.W = L.W;
      f.s_ld = L.Npad;
      f.lp = L.Lp;
      f.lp_ld = L.Npad;
      f.xt = L.tXTb;
      f.xt_rpad = L.XTb.rpad;
      f.x_d = L.d;
      f.g2 = L.G2;
      f.g2_ld = L.dpad;
      f.g2_slice = (size_t)L.C * L.dpad;
      f.active_rows = rows_active();
      gemm(L.Ub, L.tUb, L.Xb, L.tXb, L.C, L.N, L.d, f);
      L.stats.gemm_flops += 2.0 * L.C * L.N * L.d;  // the in-kernel r₂·X MMAs
      L.stats.evals++;
      // a grouped batch replays the posteriors' launch lists side by side:
      // an empty launch stands where the stored form has its r₂·X GEMM
      if (rec) rec->push(OP_GEMM, -1, 0, 320, 0, GemmItem{});
      return;
    }
    Epi s{};
    s.mode = EPI_R2W;
    s.W = L.W;
    s.s_ld = L.Npad;
    s.lp = L.Lp;
    s.lp_ld = L.Npad;
    s.r = L.Rb;
    s.r_off = L.C;
    s.active_rows = rows_active();
    gemm(L.Ub, L.tUb, L.Xb, L.tXb, L.C, L.N, L.d, s);
    grad_gemm(L.C, L.C);
    L.stats.evals++;
  }
  // u = G(q_k)⁻¹ p½ at the position iterate (the factorisation without the
  // inverse), and with it the position update and its convergence test
  // (the loop body has no separate update)
  void q_eval(bool only_active) {
    LogregBatched& L = *lb;
    metric_gram(nullptr, true);
    chol(CH_EVAL, nullptr, L.logdet1, L.quad1, nullptr, only_active, nullptr, nullptr, true,
         nullptr, true);
    L.stats.evals++;
  }
  // everything at (qc, pc), keeping the factor and w for the next momentum
  // solve
  void full_eval(int mode, const float* z, float* mom_info) {
    LogregBatched& L = *lb;
    metric_gram();
    if (mode == CH_DRAW)
      chol(CH_DRAW, z, L.logdet0, L.quad0, mom_info, false, nullptr, L.Lf, false, L.Lf32);
    else
      chol(CH_EVAL, nullptr, L.logdet1, L.quad1, nullptr, false, nullptr, L.Lf, false, L.Lf32);
    trace_grad(L.W);
    L.stats.evals++;
  }

  // energy at the proposal: ℓ row sums, Gram, log det and ||L⁻¹p||², ∇ℓ;
  // with vel_out, also the flipped proposal velocity −G⁻¹p
  void energy(float* vel_out) {
    LogregBatched& L = *lb;
    zero(L.ldnew, sizeof(double) * L.C);
    metric_gram(L.ldnew);
    chol(CH_ENERGY, nullptr, L.logdet1, L.quad1, nullptr, false, vel_out);
    grad_gemm(0, L.C);
  }

  void accept(const double* ld0, const double* u, double div_thr, float* pos, float* grad,
              double* logdens, const InfoDev<float>& info) {
    LogregBatched& L = *lb;
    const AcceptArgs A{L.C,      L.d,         ld0,          L.quad0,   L.logdet0, L.ldnew,
                       L.quad1,  L.logdet1,   u,            div_thr,   spd,       L.t.p0,
                       L.qc,     L.Gout,      L.dpad,       gsplit(),  gstride(), pos,
                       grad,     logdens,     info,         L.iters_total, L.notconv, L.bad};
    if (rec) {
      rec->push(OP_ACCEPT, 0, (L.C + 127) / 128, 128, 0, A);
      return;
    }
    accept_kernel<<<(L.C + 127) / 128, 128, 0, st>>>(A);
    check(cudaGetLastError());
  }

  void update(int mode, const StepDev& sp) {
    LogregBatched& L = *lb;
    UpdArgs a{};
    a.mode = mode;
    a.C = L.C;
    a.d = L.d;
    a.hh = 0.5 * sp.h;
    a.prior_inv = 1.0 / L.t.p0;
    a.tol = sp.tol;
    a.max_iters = sp.max_iters;
    a.Gout = L.Gout;
    a.ldo = L.dpad;
    a.gs = gsplit();
    a.gstride = gstride();
    if ((mode == UP_GLP0 || mode == UP_GLPN) && fused_r2x()) {
      a.G2 = L.G2;
      a.g2s = g2_tiles_used();
      a.g2stride = (size_t)L.C * L.dpad;
    }
    a.u = L.u;
    a.u0 = L.u0;
    a.q0 = L.q0;
    a.p0 = L.p0;
    a.qc = L.qc;
    a.pc = L.pc;
    a.qf = L.qf;
    a.norm = L.norm;
    a.iters = L.iters;
    a.iters_total = L.iters_total;
    a.active = L.active;
    a.notconv = L.notconv;
    a.Qb = L.Qb;
    a.n_active = active_flag();
    a.spd = spd;
    static_assert(32 * kSolveWarps == 256, "the fused update stages one factor per warp");
    const dim3 grid((unsigned)(((size_t)L.C * 32 + 255) / 256)), th(256);
    if (rec) {
      if (mode == UP_GLP0 || mode == UP_GLPN) {
        GlpItem it{a, L.Lf32, L.P, L.Ub};
        rec->push(OP_GLPUS, L.d <= 32 ? 1 : (L.d <= 64 ? 2 : 4), (int)grid.x, 256, 0, it);
      } else {
        rec->push(OP_UPDATE, 0, (int)grid.x, 256, 0, a);
      }
      return;
    }
    if (mode == UP_GLP0 || mode == UP_GLPN) {  // with the next evaluation's solve
      if (L.d <= 32)
        check(launch_k(L.pdl, glp_update_solve_kernel<1>, grid, th, 0, st, a, L.Lf32, L.P, L.Ub));
      else if (L.d <= 64)
        check(launch_k(L.pdl, glp_update_solve_kernel<2>, grid, th, 0, st, a, L.Lf32, L.P, L.Ub));
      else
        check(launch_k(L.pdl, glp_update_solve_kernel<4>, grid, th, 0, st, a, L.Lf32, L.P, L.Ub));
      return;
    }
    check(launch_k(L.pdl, update_kernel, grid, th, 0, st, a));
  }
};

}  // namespace

// the generalized leapfrog's buffers, allocated on its first use (never
// while a graph is being captured)
static int ensure_gl(LogregBatched* lb) {
  if (lb->Lf) return GJ_OK;
  bool ok = true;
  lb->Lf = dalloc<double>((size_t)lb->C * lb->P, lb->owned, &ok);
  lb->u0 = dalloc<double>((size_t)lb->C * lb->d, lb->owned, &ok);
  lb->W = dalloc<float>((size_t)lb->C * lb->Npad, lb->owned, &ok);
  lb->Lf32 = dalloc<float>((size_t)lb->C * lb->P, lb->owned, &ok);
  // the fused r₂·X partials: one per N tile, whose width is at least 64
  // for N > 64 (one tile for N <= 64)
  lb->g2_tiles = lb->N <= 64 ? 1 : (lb->N + 63) / 64;
  lb->G2 = dalloc<float>((size_t)lb->g2_tiles * lb->C * lb->dpad, lb->owned, &ok);
  if (!ok) {
    g_err = "device allocation failed for the generalized leapfrog's buffers";
    return GJ_ENOMEM;
  }
  return GJ_OK;
}

int logreg_batched_rmhmc_step(LogregBatched* lb, const StepDev& sp, float* pos, float* grad,
                              double* logdens, const float* z, const double* u,
                              const InfoDev<float>& info, int gemm_impl, cudaStream_t st) {
  if (gemm_impl == 2 && !lb->tc_ok) {
    g_err = "tcgen05 GEMM unavailable (no sm_100-family device or tensor-map encoder)";
    return GJ_ENOTSUP;
  }
  const bool gl = sp.integrator == GJ_GENERALIZED_LEAPFROG;
  if (gl) {
    const int rc = ensure_gl(lb);
    if (rc) return rc;
  }
  lb->stats = LogregStats{};
  lb->ev_used = 0;
  lb->cev_used = 0;
  lb->rev_used = 0;
  if (lb->prof) cudaMemsetAsync(lb->refine_fb, 0, sizeof(int), st);
  Runner R{lb, gemm_impl, st};
  R.hsp = sp;
  const int C = lb->C, d = lb->d;
  R.begin(pos);
  // a fixed-point solve driven from the host: the eager update, then body +
  // update while some chain is active (at most max_iters + 1 bodies); with
  // iterated < 0 the body updates the iterate itself
  auto host_solve = [&](int eager, auto body, int iterated) {
    R.check(cudaMemsetAsync(lb->n_active_d, 0, sizeof(int), st));
    R.update(eager, sp);
    for (int guard = 0;; ++guard) {
      R.check(cudaMemcpyAsync(lb->n_active_h, lb->n_active_d, sizeof(int),
                              cudaMemcpyDeviceToHost, st));
      R.check(cudaStreamSynchronize(st));
      if (R.err != cudaSuccess || *lb->n_active_h == 0 || guard > sp.max_iters) break;
      R.check(cudaMemsetAsync(lb->n_active_d, 0, sizeof(int), st));
      R.loop_body = true;
      body();
      R.loop_body = false;
      if (iterated >= 0) R.update(iterated, sp);
    }
  };
  for (int s = 0; gl && s < sp.L; ++s) {
    // (1) p½ = p − h/2 ∂_qH(q, p½) at the fixed position q: the first map
    // evaluation at (q, p) draws the momentum at s == 0
    if (s == 0)
      R.full_eval(CH_DRAW, z, info.momentum);
    else
      R.p_eval();
    host_solve(UP_GLP0, [&] { R.p_contract(); }, UP_GLPN);
    // (2) q' = q + h/2 [G⁻¹(q) + G⁻¹(q')] p½
    R.solve(lb->pc, lb->u0, false, false);
    host_solve(UP_GLQ0, [&] { R.q_eval(true); }, -1);
    // (3) p' = p½ − h/2 ∂_qH(q', p½), keeping the factor and w at q' for the
    // next step's momentum solve
    R.full_eval(CH_EVAL, nullptr, nullptr);
    R.update(UP_GLPX, sp);
  }
  for (int s = 0; !gl && s < sp.L; ++s) {
    // fixed-point evaluation #0 (rmhmc/integrators.py:84); at s == 0 it also
    // draws p = chol(G(q0))·z (rmhmc/metrics.py:45-58)
    R.metric_gram();
    if (s == 0)
      R.chol(CH_DRAW, z, lb->logdet0, lb->quad0, info.momentum);
    else
      R.chol(CH_EVAL, nullptr, lb->logdet1, lb->quad1, nullptr);
    R.trace_grad();
    R.check(cudaMemsetAsync(lb->n_active_d, 0, sizeof(int), st));
    R.update(UP_FP0, sp);
    int guard = 0;
    for (;;) {
      R.check(cudaMemcpyAsync(lb->n_active_h, lb->n_active_d, sizeof(int),
                              cudaMemcpyDeviceToHost, st));
      R.check(cudaStreamSynchronize(st));
      if (R.err != cudaSuccess) break;
      if (*lb->n_active_h == 0 || guard > sp.max_iters + 1) break;
      ++guard;
      R.loop_body = true;
      R.metric_gram();
      R.chol(CH_EVAL, nullptr, lb->logdet1, lb->quad1, nullptr, true);
      R.trace_grad();
      R.loop_body = false;
      R.check(cudaMemsetAsync(lb->n_active_d, 0, sizeof(int), st));
      R.update(UP_FPN, sp);
      lb->stats.evals++;
    }
    lb->stats.evals++;
    // explicit half step from the midpoint (rmhmc/integrators.py:147-148)
    R.metric_gram();
    R.chol(CH_EVAL, nullptr, lb->logdet1, lb->quad1, nullptr);
    R.trace_grad();
    R.update(UP_EXPLICIT, sp);
    lb->stats.evals++;
  }
  if (sp.L == 0) {
    // no trajectory: draw the momentum anyway for H0 = H1
    R.metric_gram();
    R.chol(CH_DRAW, z, lb->logdet0, lb->quad0, info.momentum);
  }
  // energy at the proposal (3-plane Xβ row sums, Gram, log det, ∇ℓ) and accept
  R.energy(info.prop_v);
  R.accept(logdens, u, sp.div_threshold, pos, grad, logdens, info);
  if (R.err == cudaSuccess && lb->prof && lb->ev_used) {
    R.check(cudaStreamSynchronize(st));
    double ns = 0.0;
    for (size_t i = 0; i + 1 < lb->ev_used; i += 2) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, lb->ev[i], lb->ev[i + 1]) == cudaSuccess) ns += 1e6 * ms;
    }
    lb->stats.gemm_ns = ns;
    double cns = 0.0;
    for (size_t i = 0; i + 1 < lb->cev_used; i += 2) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, lb->cev[i], lb->cev[i + 1]) == cudaSuccess) cns += 1e6 * ms;
    }
    lb->stats.chol_ns = cns;
    double rns = 0.0;
    for (size_t i = 0; i + 1 < lb->rev_used; i += 2) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, lb->rev[i], lb->rev[i + 1]) == cudaSuccess) rns += 1e6 * ms;
    }
    lb->stats.refine_ns = rns;
    int fb = 0;
    if (cudaMemcpy(&fb, lb->refine_fb, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess)
      lb->stats.refine_fallbacks = fb;
  }
  if (R.err != cudaSuccess) {
    g_err = std::string("batched logistic-regression step: ") + cudaGetErrorString(R.err);
    return GJ_ECUDA;
  }
  if (gemm_impl == 2) {
    int herr = 0;
    if (cudaMemcpyAsync(&herr, lb->tc_err, sizeof(int), cudaMemcpyDeviceToHost, st) ==
            cudaSuccess &&
        cudaStreamSynchronize(st) == cudaSuccess && herr != 0) {
      g_err = "tcgen05 GEMM wait timed out (code " + std::to_string(herr) + ")";
      cudaMemsetAsync(lb->tc_err, 0, sizeof(int), st);
      return GJ_ECUDA;
    }
  }
  return GJ_OK;
}

namespace {

__global__ void set_step_kernel(StepDev* dst, StepDev v) { *dst = v; }

int graph_fail(const char* what, cudaError_t e) {
  g_err = std::string("graph capture (") + what + "): " + cudaGetErrorString(e);
  return GJ_ECUDA;
}

constexpr size_t kMaxGraphs = 64;

// every setting a captured transition depends on, in mixed radix (each
// field below its radix: chol_cpw <= 8, tuning code < 128, K slices <= 4)
int graph_cfg(const LogregBatched* lb) {
  int k = lb->chol_fp64;
  k = k * 16 + lb->chol_cpw;
  k = k * 2 + lb->pdl;
  k = k * 128 + gemm_tc_tuning_code();
  k = k * 8 + lb->gsplit_req;
  k = k * 2 + lb->fuse_r2x;
  return k * 2 + lb->refine;
}

// Record one whole transition (all L steps, each fixed-point solve a
// conditional WHILE node) into the capture that stream s takes part in.  The
// kernels read and write the context's staging buffers; step parameters come
// from lb->spd.  With prop, the energy factorisation also writes the
// proposal velocity.  Returns the first error (the capture stays open).
// The transition's sequence of stages, shared by the capture of one
// posterior's graph and the recording of a grouped batch: add_solve(eager,
// body, iterated) emits one fixed-point solve (the eager update, then body +
// the iterated update while some chain is active).
template <typename AddSolve>
cudaError_t transition_script(Runner& R, LogregBatched* lb, int L, bool prop, bool gl,
                              AddSolve&& add_solve) {
  cudaError_t e = cudaSuccess;
  StepDev dummy{};
  R.begin(lb->pos_s);
  for (int st = 0; st < L && R.err == cudaSuccess && e == cudaSuccess; ++st) {
    if (gl) {
      // generalized leapfrog: momentum solve at the fixed position, position
      // solve, explicit final momentum (the factor and w at q' are kept for
      // the next step's momentum solve)
      if (st == 0)
        R.full_eval(CH_DRAW, lb->z_s, lb->mom_s);
      else
        R.p_eval();
      e = add_solve(UP_GLP0, [](Runner& B) { B.p_contract(); }, UP_GLPN);
      if (e != cudaSuccess) break;
      R.solve(lb->pc, lb->u0, false, false);
      e = add_solve(UP_GLQ0, [](Runner& B) { B.q_eval(true); }, -1);
      if (e != cudaSuccess) break;
      R.full_eval(CH_EVAL, nullptr, nullptr);
      R.update(UP_GLPX, dummy);
      continue;
    }
    R.metric_gram();
    if (st == 0)
      R.chol(CH_DRAW, lb->z_s, lb->logdet0, lb->quad0, lb->mom_s);
    else
      R.chol(CH_EVAL, nullptr, lb->logdet1, lb->quad1, nullptr);
    R.trace_grad();
    e = add_solve(UP_FP0, [lb](Runner& B) {
      B.metric_gram();
      B.chol(CH_EVAL, nullptr, lb->logdet1, lb->quad1, nullptr, true);
      B.trace_grad();
    }, UP_FPN);
    if (e != cudaSuccess) break;
    R.metric_gram();
    R.chol(CH_EVAL, nullptr, lb->logdet1, lb->quad1, nullptr);
    R.trace_grad();
    R.update(UP_EXPLICIT, dummy);
  }
  if (L == 0) {
    R.metric_gram();
    R.chol(CH_DRAW, lb->z_s, lb->logdet0, lb->quad0, lb->mom_s);
  }
  R.energy(prop ? lb->propv_s : nullptr);
  InfoDev<float> inf{};
  inf.acc_rate = lb->acc_s;
  inf.accepted = lb->accepted_s;
  inf.divergent = lb->divergent_s;
  inf.energy = lb->energy_s;
  inf.fp_iters = lb->fpit_s;
  inf.status = lb->status_s;
  inf.momentum = nullptr;
  inf.prop_q = lb->propq_s;
  R.accept(lb->ld_s, lb->u_s, 0.0, lb->pos_s, lb->grad_s, lb->ld_s, inf);
  if (e == cudaSuccess) e = R.err;
  return e;
}

cudaError_t capture_transition(LogregBatched* lb, int L, int impl, bool prop, bool gl,
                               cudaStream_t s) {
  Runner R{lb, impl, s};
  R.spd = lb->spd;
  StepDev dummy{};
  // one fixed-point solve: the eager update, then a conditional WHILE node
  // whose body is `body` + the iterated update (none when iterated < 0: the
  // body updates the iterate itself), repeated while some chain is active
  // (at most max_iters + 1 times)
  auto add_solve = [&](int eager, auto body, int iterated) -> cudaError_t {
    R.check(cudaMemsetAsync(lb->n_active_d, 0, sizeof(int), s));
    R.update(eager, dummy);
    R.check(cudaMemsetAsync(lb->trips, 0, sizeof(int), s));
    cudaStreamCaptureStatus cs;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    cudaError_t r = cudaStreamGetCaptureInfo(s, &cs, nullptr, &cg, &deps, nullptr, &nd);
    if (r != cudaSuccess) return r;
    cudaGraphConditionalHandle h;
    r = cudaGraphConditionalHandleCreate(&h, cg, 0, cudaGraphCondAssignDefault);
    if (r != cudaSuccess) return r;
    loop_cond_kernel<<<1, 1, 0, s>>>(h, lb->n_active_d, lb->trips, lb->spd);
    r = cudaStreamGetCaptureInfo(s, &cs, nullptr, &cg, &deps, nullptr, &nd);
    if (r != cudaSuccess) return r;
    cudaGraphNodeParams np{};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    r = cudaGraphAddNode(&node, cg, deps, nullptr, nd, &np);
    if (r != cudaSuccess) return r;
    cudaGraph_t bodyg = np.conditional.phGraph_out[0];
    r = cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
    if (r != cudaSuccess) return r;
    r = cudaStreamBeginCaptureToGraph(lb->cap_body, bodyg, nullptr, nullptr, 0,
                                      cudaStreamCaptureModeThreadLocal);
    if (r != cudaSuccess) return r;
    Runner B{lb, impl, lb->cap_body};
    B.spd = lb->spd;
    B.loop_body = true;
    body(B);
    B.loop_body = false;
    if (iterated >= 0) B.update(iterated, dummy);
    loop_cond_kernel<<<1, 1, 0, lb->cap_body>>>(h, lb->n_active_d, lb->trips, lb->spd);
    B.check(cudaGetLastError());
    cudaGraph_t bout = nullptr;
    r = cudaStreamEndCapture(lb->cap_body, &bout);
    if (r == cudaSuccess && B.err != cudaSuccess) r = B.err;
    return r;
  };
  return transition_script(R, lb, L, prop, gl, add_solve);
}

// Record one transition of one posterior as launches (grouped batches).
cudaError_t record_transition(LogregBatched* lb, int L, int impl, bool prop, bool gl,
                              Recorder* rec) {
  Runner R{lb, impl, nullptr};
  R.spd = lb->spd;
  R.rec = rec;
  StepDev dummy{};
  auto add_solve = [&](int eager, auto body, int iterated) -> cudaError_t {
    rec->mark(OP_FLAG_CLEAR);
    R.update(eager, dummy);
    rec->mark(OP_TRIPS_CLEAR);
    rec->mark(OP_LOOP_BEGIN);
    R.loop_body = true;
    body(R);
    R.loop_body = false;
    if (iterated >= 0) R.update(iterated, dummy);
    rec->mark(OP_LOOP_END);
    return R.err;
  };
  return transition_script(R, lb, L, prop, gl, add_solve);
}

// Capture one whole transition into *out (its own graph).
int build_graph(LogregBatched* lb, int L, int impl, bool prop, bool gl, cudaGraphExec_t* out) {
  *out = nullptr;
  cudaStream_t s = lb->cap_main;
  cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return graph_fail("begin", e);
  e = capture_transition(lb, L, impl, prop, gl, s);
  cudaGraph_t g = nullptr;
  const cudaError_t e2 = cudaStreamEndCapture(s, &g);
  if (e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return graph_fail("transition", e);
  }
  if (e2 != cudaSuccess) return graph_fail("end", e2);
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    *out = nullptr;
    return graph_fail("instantiate", e);
  }
  return GJ_OK;
}

// The captured transition for these settings, captured now if absent.
int find_graph(LogregBatched* lb, int L, int impl, bool prop, bool gl, cudaStream_t st,
               cudaGraphExec_t* out) {
  const int cfg = graph_cfg(lb) + (gl ? (1 << 20) : 0);
  for (auto& g : lb->graphs)
    if (g.L == L && g.impl == impl && g.cfg == cfg && g.prop == (int)prop) {
      g.used = ++lb->graph_tick;
      *out = g.exec;
      return GJ_OK;
    }
  // the capture streams must not see unfinished work of the caller's stream
  cudaStreamSynchronize(st);
  if (lb->graphs.size() >= kMaxGraphs) {
    size_t lru = 0;
    for (size_t i = 1; i < lb->graphs.size(); ++i)
      if (lb->graphs[i].used < lb->graphs[lru].used) lru = i;
    cudaGraphExecDestroy(lb->graphs[lru].exec);
    lb->graphs.erase(lb->graphs.begin() + lru);
  }
  cudaGraphExec_t ex = nullptr;
  const int rc = build_graph(lb, L, impl, prop, gl, &ex);
  if (rc) return rc;
  lb->graphs.push_back({L, impl, cfg, (int)prop, ex, ++lb->graph_tick});
  *out = ex;
  return GJ_OK;
}

template <typename Tp>
void copy_out(Tp* dst, const Tp* src, size_t n, cudaStream_t st, cudaError_t* err) {
  if (!dst || *err != cudaSuccess) return;
  *err = cudaMemcpyAsync(dst, src, n * sizeof(Tp), cudaMemcpyDeviceToDevice, st);
}

}  // namespace

int logreg_batched_rmhmc_step_graph(LogregBatched* lb, const StepDev& sp, float* pos, float* grad,
                                    double* logdens, const float* z, const double* u,
                                    const InfoDev<float>& info, int gemm_impl, cudaStream_t st) {
  if (gemm_impl == 2 && !lb->tc_ok) {
    g_err = "tcgen05 GEMM unavailable (no sm_100-family device or tensor-map encoder)";
    return GJ_ENOTSUP;
  }
  const bool gl = sp.integrator == GJ_GENERALIZED_LEAPFROG;
  if (gl) {
    const int rg = ensure_gl(lb);
    if (rg) return rg;
  }
  cudaGraphExec_t gexec = nullptr;
  const int rc = find_graph(lb, sp.L, gemm_impl, info.prop_v != nullptr, gl, st, &gexec);
  if (rc) return rc;
  const int C = lb->C, d = lb->d;
  lb->stats = LogregStats{};
  set_step_kernel<<<1, 1, 0, st>>>(lb->spd, sp);
  cudaError_t e = cudaGetLastError();
  copy_out(lb->pos_s, pos, (size_t)C * d, st, &e);
  copy_out(lb->grad_s, grad, (size_t)C * d, st, &e);
  copy_out(lb->ld_s, logdens, (size_t)C, st, &e);
  copy_out(lb->z_s, z, (size_t)C * d, st, &e);
  copy_out(lb->u_s, u, (size_t)C, st, &e);
  if (e == cudaSuccess) e = cudaGraphLaunch(gexec, st);
  copy_out(pos, lb->pos_s, (size_t)C * d, st, &e);
  copy_out(grad, lb->grad_s, (size_t)C * d, st, &e);
  copy_out(logdens, lb->ld_s, (size_t)C, st, &e);
  copy_out(info.acc_rate, lb->acc_s, (size_t)C, st, &e);
  copy_out(info.accepted, lb->accepted_s, (size_t)C, st, &e);
  copy_out(info.divergent, lb->divergent_s, (size_t)C, st, &e);
  copy_out(info.energy, lb->energy_s, (size_t)C, st, &e);
  copy_out(info.fp_iters, lb->fpit_s, (size_t)C, st, &e);
  copy_out(info.status, lb->status_s, (size_t)C, st, &e);
  copy_out(info.momentum, lb->mom_s, (size_t)C * d, st, &e);
  copy_out(info.prop_q, lb->propq_s, (size_t)C * d, st, &e);
  copy_out(info.prop_v, lb->propv_s, (size_t)C * d, st, &e);
  if (e != cudaSuccess) {
    g_err = std::string("graph step: ") + cudaGetErrorString(e);
    return GJ_ECUDA;
  }
  lb->stats.other_launches = 1;  // one graph launch (its kernels are counted by the caller)
  return GJ_OK;
}

static __global__ void split_rows_kernel(const float* X, int R, int K, SplitMat S) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= (size_t)R * K) return;
  split_store(S, (int)(i / K), (int)(i % K), X[i]);
}

int gemm_split_test(int impl, int planes, int M, int N, int K, const float* A, const float* B,
                    float* D, cudaStream_t st) {
  if (M < 1 || N < 1 || K < 1 || !A || !B || !D || (planes != 2 && planes != 3)) {
    g_err = "bad GEMM test arguments";
    return GJ_EINVAL;
  }
  LogregBatched tmp;
  bool ok = true;
  SplitMat a = make_split(&tmp, M, K, planes, &ok);
  SplitMat b = make_split(&tmp, N, K, planes, &ok);
  int* err = dalloc<int>(1, tmp.owned, &ok);
  int rc = GJ_OK;
  if (!ok) {
    g_err = "device allocation failed";
    rc = GJ_ENOMEM;
  }
  TcOperand *ta = nullptr, *tb = nullptr;
  if (!rc) {
    cudaDeviceSynchronize();  // the scratch memsets run on the legacy stream
    split_rows_kernel<<<(unsigned)(((size_t)M * K + 255) / 256), 256, 0, st>>>(A, M, K, a);
    split_rows_kernel<<<(unsigned)(((size_t)N * K + 255) / 256), 256, 0, st>>>(B, N, K, b);
    GemmArgs g;
    g.A = a;
    g.B = b;
    g.M = M;
    g.N = N;
    g.K = K;
    g.epi = Epi{};
    g.epi.mode = EPI_STORE;
    g.epi.D = D;
    g.epi.ldd = N;
    cudaError_t e = cudaSuccess;
    if (impl == 2) {
      const char* msg = "tcgen05 unavailable";
      if (tc_available() && gemm_tc_prepare() == cudaSuccess) {
        ta = tc_operand_create(a, 0, &msg);
        tb = tc_operand_create(b, 0, &msg);
      }
      if (!ta || !tb) {
        g_err = msg;
        rc = GJ_ENOTSUP;
      } else {
        e = gemm_tc(g, ta, tb, err, st);
      }
    } else {
      e = gemm_simt(g, st);
    }
    if (!rc) {
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      int herr = 0;
      if (e == cudaSuccess) e = cudaMemcpy(&herr, err, sizeof(int), cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) {
        g_err = std::string("GEMM test: ") + cudaGetErrorString(e);
        rc = GJ_ECUDA;
      } else if (herr) {
        g_err = "tcgen05 GEMM wait timed out (code " + std::to_string(herr) + ")";
        rc = GJ_ECUDA;
      }
    }
  }
  if (ta) tc_operand_destroy(ta);
  if (tb) tc_operand_destroy(tb);
  for (void* p : tmp.owned) cudaFree(p);
  tmp.owned.clear();
  return rc;
}

// ---------------------------------------------------------------------------
// A batch of posteriors as one CUDA graph.  Every posterior's whole
// transition (its conditional WHILE nodes included) is recorded as an
// independent branch of one graph, so one launch advances every chain of
// every posterior and the graph executor runs the branches concurrently as
// the SMs allow.  One gather kernel before the launch copies the batch's
// ragged state and draws into the posteriors' staging buffers and sets their
// step parameters; one scatter kernel after it copies the results back.
// Neither the batch's array addresses nor the step size are baked into the
// graph, so one capture serves every call with the same number of steps,
// integrator, GEMM path and factorisation set-up.
// ---------------------------------------------------------------------------
namespace {

struct BatchStage {  // one posterior's staging buffers and its place in the batch arrays
  float *pos_s, *grad_s, *z_s, *mom_s, *propq_s, *propv_s;
  double *ld_s, *u_s, *acc_s, *energy_s;
  uint8_t *accepted_s, *divergent_s, *status_s;
  int* fpit_s;
  StepDev* spd;
  long long vec_off;  // the posterior's [C, d] block in the ragged vectors
  int d;
};

__global__ void batch_gather_kernel(const BatchStage* S, int C, StepDev sp, const float* pos,
                                    const float* grad, const double* ld, const float* z,
                                    const double* u) {
  const BatchStage st = S[blockIdx.x];
  const size_t nv = (size_t)C * st.d, o = (size_t)st.vec_off, co = (size_t)blockIdx.x * C;
  for (size_t i = threadIdx.x; i < nv; i += blockDim.x) {
    st.pos_s[i] = pos[o + i];
    st.grad_s[i] = grad[o + i];
    st.z_s[i] = z[o + i];
  }
  for (int i = threadIdx.x; i < C; i += blockDim.x) {
    st.ld_s[i] = ld[co + i];
    st.u_s[i] = u[co + i];
  }
  if (threadIdx.x == 0) *st.spd = sp;
}

__global__ void batch_scatter_kernel(const BatchStage* S, int C, float* pos, float* grad,
                                     double* ld, InfoDev<float> info) {
  const BatchStage st = S[blockIdx.x];
  const size_t nv = (size_t)C * st.d, o = (size_t)st.vec_off, co = (size_t)blockIdx.x * C;
  for (size_t i = threadIdx.x; i < nv; i += blockDim.x) {
    pos[o + i] = st.pos_s[i];
    grad[o + i] = st.grad_s[i];
    if (info.momentum) info.momentum[o + i] = st.mom_s[i];
    if (info.prop_q) info.prop_q[o + i] = st.propq_s[i];
    if (info.prop_v) info.prop_v[o + i] = st.propv_s[i];
  }
  for (int i = threadIdx.x; i < C; i += blockDim.x) {
    ld[co + i] = st.ld_s[i];
    if (info.acc_rate) info.acc_rate[co + i] = st.acc_s[i];
    if (info.accepted) info.accepted[co + i] = st.accepted_s[i];
    if (info.divergent) info.divergent[co + i] = st.divergent_s[i];
    if (info.energy) info.energy[co + i] = st.energy_s[i];
    if (info.fp_iters) info.fp_iters[co + i] = st.fpit_s[i];
    if (info.status) info.status[co + i] = st.status_s[i];
  }
}

constexpr size_t kMaxBatchGraphs = 8;
constexpr int kMaxBuckets = 256;  // grouped batches: most buckets of posteriors

// One grouped launch: the items of the posteriors whose op has this kernel
// variant and block size, in device memory.
struct GroupLaunch {
  int kind, variant, threads, n, blocks;
  size_t smem;
  const void* items;
  const int* prefix;
};


}  // namespace

struct LogregBatchGraph {
  std::vector<LogregBatched*> lbs;
  int C = 0;
  BatchStage* stages = nullptr;  // device [B]
  cudaStream_t cap_root = nullptr;
  cudaStream_t cap_body = nullptr;  // grouped: the WHILE bodies' capture
  cudaEvent_t fork = nullptr, join = nullptr;
  int grouped = 0;       // logreg_batch_graph_set_grouped
  int buckets = 0;       // grouped: buckets of posteriors (0 = automatic)
  int* flag = nullptr;   // grouped: each bucket's active-chain flag and trip counter
                         // (kMaxBuckets pairs, allocated once: captured graphs keep them)
  std::vector<cudaStream_t> bucket_main, bucket_body;  // grouped: capture streams
  struct Pending {  // a recorded bucket, between its recording and its capture
    std::vector<std::vector<GroupLaunch>> plan;
    std::vector<int> kinds;
    int* flag;
    int* trips;
  };
  std::vector<Pending> pending;
  std::vector<unsigned char> staging;  // grouped: the items of a capture, uploaded at once
  struct Entry {
    int L, impl, cfg, prop;
    cudaGraphExec_t exec;
    unsigned long long used;
    std::vector<void*> bufs;  // grouped: the launches' items and prefix sums
  };
  std::vector<Entry> graphs;
  unsigned long long tick = 0;
};

static void free_entry(LogregBatchGraph::Entry& g) {
  cudaGraphExecDestroy(g.exec);
  for (void* p : g.bufs) cudaFree(p);
  g.bufs.clear();
}

void logreg_batch_graph_set_grouped(LogregBatchGraph* bg, int on, int buckets) {
  bg->grouped = on ? 1 : 0;
  bg->buckets = buckets > 0 ? buckets : 0;
}

void logreg_batch_graph_destroy(LogregBatchGraph* bg) {
  if (!bg) return;
  for (auto& g : bg->graphs) free_entry(g);
  if (bg->stages) cudaFree(bg->stages);
  if (bg->flag) cudaFree(bg->flag);
  for (cudaStream_t x : bg->bucket_main) cudaStreamDestroy(x);
  for (cudaStream_t x : bg->bucket_body) cudaStreamDestroy(x);
  if (bg->cap_body) cudaStreamDestroy(bg->cap_body);
  if (bg->cap_root) cudaStreamDestroy(bg->cap_root);
  if (bg->fork) cudaEventDestroy(bg->fork);
  if (bg->join) cudaEventDestroy(bg->join);
  delete bg;
}

int logreg_batch_graph_create(LogregBatched* const* lbs, int B, int C, const size_t* vec_off,
                              LogregBatchGraph** out) {
  *out = nullptr;
  LogregBatchGraph* bg = new (std::nothrow) LogregBatchGraph();
  if (!bg) {
    g_err = "host allocation failed";
    return GJ_ENOMEM;
  }
  bg->lbs.assign(lbs, lbs + B);
  bg->C = C;
  std::vector<BatchStage> hs(B);
  for (int b = 0; b < B; ++b) {
    LogregBatched* lb = lbs[b];
    if (lb->C != C) {
      logreg_batch_graph_destroy(bg);
      g_err = "every posterior of a batch graph has the same chain count";
      return GJ_EINVAL;
    }
    BatchStage& st = hs[b];
    st.pos_s = lb->pos_s;
    st.grad_s = lb->grad_s;
    st.z_s = lb->z_s;
    st.mom_s = lb->mom_s;
    st.propq_s = lb->propq_s;
    st.propv_s = lb->propv_s;
    st.ld_s = lb->ld_s;
    st.u_s = lb->u_s;
    st.acc_s = lb->acc_s;
    st.energy_s = lb->energy_s;
    st.accepted_s = lb->accepted_s;
    st.divergent_s = lb->divergent_s;
    st.status_s = lb->status_s;
    st.fpit_s = lb->fpit_s;
    st.spd = lb->spd;
    st.vec_off = (long long)vec_off[b];
    st.d = lb->d;
  }
  cudaError_t e = cudaMalloc(&bg->stages, sizeof(BatchStage) * (size_t)B);
  if (e == cudaSuccess)
    e = cudaMemcpy(bg->stages, hs.data(), sizeof(BatchStage) * (size_t)B, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&bg->cap_root, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&bg->cap_body, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&bg->flag, 2 * sizeof(int) * kMaxBuckets);
  if (e == cudaSuccess) e = cudaMemset(bg->flag, 0, 2 * sizeof(int) * kMaxBuckets);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&bg->fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&bg->join, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    logreg_batch_graph_destroy(bg);
    g_err = std::string("batch graph set-up: ") + cudaGetErrorString(e);
    return GJ_ECUDA;
  }
  *out = bg;
  return GJ_OK;
}

namespace {

// Record every posterior's transition as one branch of one graph.
int batch_capture(LogregBatchGraph* bg, int L, int impl, bool prop, bool gl,
                  cudaGraphExec_t* out) {
  *out = nullptr;
  cudaStream_t root = bg->cap_root;
  cudaError_t e = cudaStreamBeginCapture(root, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return graph_fail("batch begin", e);
  e = cudaEventRecord(bg->fork, root);
  for (size_t b = 0; b < bg->lbs.size() && e == cudaSuccess; ++b) {
    LogregBatched* lb = bg->lbs[b];
    e = cudaStreamWaitEvent(lb->cap_main, bg->fork, 0);  // the branch starts at the fork
    if (e == cudaSuccess) e = capture_transition(lb, L, impl, prop, gl, lb->cap_main);
    if (e == cudaSuccess) e = cudaEventRecord(bg->join, lb->cap_main);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(root, bg->join, 0);  // and joins the root
  }
  cudaGraph_t g = nullptr;
  const cudaError_t e2 = cudaStreamEndCapture(root, &g);
  if (e != cudaSuccess || e2 != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return graph_fail("batch capture", e != cudaSuccess ? e : e2);
  }
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    *out = nullptr;
    return graph_fail("batch instantiate", e);
  }
  return GJ_OK;
}

cudaError_t launch_group(const GroupLaunch& g, cudaStream_t s) {
  if (g.blocks < 1) return cudaSuccess;
  const dim3 grid((unsigned)g.blocks), th((unsigned)g.threads);
  const int* pf = g.prefix;
  const int n = g.n;
  switch (g.kind) {
    case OP_GEMM:
      return gemm_tc_grouped(g.variant, static_cast<const GemmItem*>(g.items), pf, n, g.blocks,
                             g.smem, s);
    case OP_CHOL: {
      const CholItem* it = static_cast<const CholItem*>(g.items);
      switch (g.variant) {
        case 104: chol_grouped_kernel<double, 4><<<grid, th, g.smem, s>>>(it, pf, n); break;
        case 108: chol_grouped_kernel<double, 8><<<grid, th, g.smem, s>>>(it, pf, n); break;
        case 116: chol_grouped_kernel<double, 16><<<grid, th, g.smem, s>>>(it, pf, n); break;
        case 132: chol_grouped_kernel<double, 32><<<grid, th, g.smem, s>>>(it, pf, n); break;
        case 432: chol_refined_grouped_kernel<<<grid, th, g.smem, s>>>(it, pf, n); break;
        case 228: chol_grouped_kernel<double, 128><<<grid, th, g.smem, s>>>(it, pf, n); break;
        case 128: chol_grouped_kernel<float, 128><<<grid, th, g.smem, s>>>(it, pf, n); break;
        case 356: chol_grouped_kernel<double, 256><<<grid, th, g.smem, s>>>(it, pf, n); break;
        case 256: chol_grouped_kernel<float, 256><<<grid, th, g.smem, s>>>(it, pf, n); break;
        case 4: chol_grouped_kernel<float, 4><<<grid, th, g.smem, s>>>(it, pf, n); break;
        case 8: chol_grouped_kernel<float, 8><<<grid, th, g.smem, s>>>(it, pf, n); break;
        case 16: chol_grouped_kernel<float, 16><<<grid, th, g.smem, s>>>(it, pf, n); break;
        case 32: chol_grouped_kernel<float, 32><<<grid, th, g.smem, s>>>(it, pf, n); break;
        default: return cudaErrorInvalidValue;
      }
      break;
    }
    case OP_SOLVE: {
      const SolveItem* it = static_cast<const SolveItem*>(g.items);
      switch (g.variant) {
        case 1: solve_grouped_kernel<float, 1><<<grid, th, 0, s>>>(it, pf, n); break;
        case 2: solve_grouped_kernel<float, 2><<<grid, th, 0, s>>>(it, pf, n); break;
        case 4: solve_grouped_kernel<float, 4><<<grid, th, 0, s>>>(it, pf, n); break;
        case 11: solve_grouped_kernel<double, 1><<<grid, th, 0, s>>>(it, pf, n); break;
        case 12: solve_grouped_kernel<double, 2><<<grid, th, 0, s>>>(it, pf, n); break;
        case 14: solve_grouped_kernel<double, 4><<<grid, th, 0, s>>>(it, pf, n); break;
        default: return cudaErrorInvalidValue;
      }
      break;
    }
    case OP_GLPUS: {
      const GlpItem* it = static_cast<const GlpItem*>(g.items);
      switch (g.variant) {
        case 1: glp_update_solve_grouped_kernel<1><<<grid, th, 0, s>>>(it, pf, n); break;
        case 2: glp_update_solve_grouped_kernel<2><<<grid, th, 0, s>>>(it, pf, n); break;
        case 4: glp_update_solve_grouped_kernel<4><<<grid, th, 0, s>>>(it, pf, n); break;
        default: return cudaErrorInvalidValue;
      }
      break;
    }
    case OP_UPDATE:
      update_grouped_kernel<<<grid, th, 0, s>>>(static_cast<const UpdArgs*>(g.items), pf, n);
      break;
    case OP_BEGIN:
      begin_grouped_kernel<<<grid, th, 0, s>>>(static_cast<const BeginArgs*>(g.items), pf, n);
      break;
    case OP_ACCEPT:
      accept_grouped_kernel<<<grid, th, 0, s>>>(static_cast<const AcceptArgs*>(g.items), pf, n);
      break;
    case OP_ZERO:
      zero_grouped_kernel<<<grid, th, 0, s>>>(static_cast<const ZeroItem*>(g.items), pf, n);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

bool is_kernel_op(int kind) { return kind <= OP_ZERO; }

// One bucket of posteriors as grouped launches: every posterior's transition
// is recorded as a list of launches (the lists match op by op: same stages,
// same loops), then each op becomes one grid per kernel variant over the
// bucket's posteriors, and each fixed-point solve one WHILE node whose
// condition is the bucket's shared active-chain flag.  A posterior whose
// chains have all converged runs the loop's remaining bodies without
// changing state: the updates and factorisations skip inactive chains, and
// the contractions skip tiles with no active chain.  The items are staged
// here (batch_capture_grouped uploads them at once); emit_bucket records the
// launches into a capture.
// capture streams for nb buckets (their flags are allocated with the batch)
cudaError_t ensure_buckets(LogregBatchGraph* bg, int nb) {
  cudaError_t e = cudaSuccess;
  while ((int)bg->bucket_main.size() < nb && e == cudaSuccess) {
    cudaStream_t a = nullptr, b = nullptr;
    e = cudaStreamCreateWithFlags(&a, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b, cudaStreamNonBlocking);
    if (a) bg->bucket_main.push_back(a);
    if (b) bg->bucket_body.push_back(b);
  }
  return e;
}

cudaError_t capture_bucket(LogregBatchGraph* bg, const std::vector<int>& members, int* flag,
                           int* trips, int L, int impl, bool prop, bool gl) {
  const int B = (int)members.size();
  std::vector<Recorder> recs(B);
  for (int b = 0; b < B; ++b) {
    recs[b].flag = flag;
    const cudaError_t e = record_transition(bg->lbs[members[b]], L, impl, prop, gl, &recs[b]);
    if (e != cudaSuccess) return e;
  }
  const size_t nops = recs[0].ops.size();
  for (int b = 1; b < B; ++b) {
    bool same = recs[b].ops.size() == nops;
    for (size_t i = 0; same && i < nops; ++i)
      same = recs[b].ops[i].kind == recs[0].ops[i].kind &&
             recs[b].ops[i].item.size() == recs[0].ops[i].item.size();
    if (!same) return cudaErrorInvalidValue;  // the transitions differ in structure
  }
  // the grouped launches of every op, their items uploaded before the capture
  std::vector<std::vector<GroupLaunch>> plan(nops);
  for (size_t i = 0; i < nops; ++i) {
    if (!is_kernel_op(recs[0].ops[i].kind)) continue;
    std::vector<int> order(B);
    for (int b = 0; b < B; ++b) order[b] = b;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
      const Op &ox = recs[x].ops[i], &oy = recs[y].ops[i];
      return ox.variant != oy.variant ? ox.variant < oy.variant : ox.threads < oy.threads;
    });
    const size_t isz = recs[0].ops[i].item.size();
    for (size_t k = 0; k < order.size();) {
      const Op& o0 = recs[order[k]].ops[i];
      size_t k1 = k;
      std::vector<unsigned char> items;
      std::vector<int> prefix(1, 0);
      GroupLaunch g{o0.kind, o0.variant, o0.threads, 0, 0, 0, nullptr, nullptr};
      while (k1 < order.size() && recs[order[k1]].ops[i].variant == o0.variant &&
             recs[order[k1]].ops[i].threads == o0.threads) {
        const Op& o = recs[order[k1]].ops[i];
        items.insert(items.end(), o.item.begin(), o.item.end());
        prefix.push_back(prefix.back() + o.blocks);
        g.smem = std::max(g.smem, o.smem);
        ++k1;
      }
      g.n = (int)(k1 - k);
      g.blocks = prefix.back();
      // staged in the capture's one upload buffer; the offsets become device
      // addresses once it is allocated (64-byte aligned: items may hold
      // tensor maps)
      auto stage = [&](const void* src, size_t bytes) {
        std::vector<unsigned char>& h = bg->staging;
        const size_t off = (h.size() + 63) / 64 * 64;
        h.resize(off + bytes);
        std::memcpy(h.data() + off, src, bytes);
        return off;
      };
      g.items = reinterpret_cast<const void*>(stage(items.data(), items.size()));
      g.prefix = reinterpret_cast<const int*>(stage(prefix.data(), sizeof(int) * prefix.size()));
      plan[i].push_back(g);
      k = k1;
    }
  }
  bg->pending.push_back({std::move(plan), std::vector<int>(), flag, trips});
  auto& pk = bg->pending.back();
  pk.kinds.reserve(nops);
  for (size_t i = 0; i < nops; ++i) pk.kinds.push_back(recs[0].ops[i].kind);
  return cudaSuccess;
}

// Emit one recorded bucket into the capture stream s (loop bodies on sb).
cudaError_t emit_bucket(const LogregBatchGraph::Pending& pk, const StepDev* spd, cudaStream_t s,
                        cudaStream_t sb) {
  cudaStream_t cur = s;
  cudaError_t e = cudaSuccess;
  cudaGraphConditionalHandle h{};
  for (size_t i = 0; i < pk.kinds.size() && e == cudaSuccess; ++i) {
    const int kind = pk.kinds[i];
    if (is_kernel_op(kind)) {
      for (const GroupLaunch& g : pk.plan[i])
        if (e == cudaSuccess) e = launch_group(g, cur);
      continue;
    }
    if (kind == OP_FLAG_CLEAR) {
      e = cudaMemsetAsync(pk.flag, 0, sizeof(int), cur);
    } else if (kind == OP_TRIPS_CLEAR) {
      e = cudaMemsetAsync(pk.trips, 0, sizeof(int), cur);
    } else if (kind == OP_LOOP_BEGIN) {
      if (cur != s) return cudaErrorInvalidValue;  // loops do not nest
      cudaStreamCaptureStatus cs;
      cudaGraph_t cg = nullptr;
      const cudaGraphNode_t* deps = nullptr;
      size_t nd = 0;
      e = cudaStreamGetCaptureInfo(s, &cs, nullptr, &cg, &deps, nullptr, &nd);
      if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, cg, 0, cudaGraphCondAssignDefault);
      if (e != cudaSuccess) break;
      loop_cond_kernel<<<1, 1, 0, s>>>(h, pk.flag, pk.trips, spd);
      e = cudaStreamGetCaptureInfo(s, &cs, nullptr, &cg, &deps, nullptr, &nd);
      if (e != cudaSuccess) break;
      cudaGraphNodeParams np{};
      np.type = cudaGraphNodeTypeConditional;
      np.conditional.handle = h;
      np.conditional.type = cudaGraphCondTypeWhile;
      np.conditional.size = 1;
      cudaGraphNode_t node;
      e = cudaGraphAddNode(&node, cg, deps, nullptr, nd, &np);
      if (e == cudaSuccess)
        e = cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1,
                                                cudaStreamSetCaptureDependencies);
      if (e == cudaSuccess)
        e = cudaStreamBeginCaptureToGraph(sb, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal);
      cur = sb;
    } else if (kind == OP_LOOP_END) {
      if (cur != sb) return cudaErrorInvalidValue;
      loop_cond_kernel<<<1, 1, 0, cur>>>(h, pk.flag, pk.trips, spd);
      e = cudaGetLastError();
      cudaGraph_t bout = nullptr;
      const cudaError_t e2 = cudaStreamEndCapture(sb, &bout);
      if (e == cudaSuccess) e = e2;
      cur = s;
    }
  }
  if (cur != s) {  // an error inside a loop body: close its capture
    cudaGraph_t bout = nullptr;
    cudaStreamEndCapture(sb, &bout);
  }
  return e;
}

// The whole batch as grouped launches in buckets: the posteriors, sorted by
// (d, N), are cut into nb buckets of consecutive sizes; each bucket is one
// branch of the graph (its own loops and active-chain flag), so a bucket
// waits only for its own slowest chain and the branches overlap as the SMs
// allow.
int batch_capture_grouped(LogregBatchGraph* bg, int L, int impl, bool prop, bool gl,
                          cudaGraphExec_t* out, std::vector<void*>* bufs) {
  *out = nullptr;
  if (impl != 2) {
    g_err = "grouped batch launches need the tcgen05 GEMM path";
    return GJ_ENOTSUP;
  }
  const int B = (int)bg->lbs.size();
  // automatic: buckets of 16 posteriors (2048 posteriors: 128 buckets, the
  // measured optimum; fewer, larger buckets wait longer for their slowest
  // chain at every loop)
  const int want = bg->buckets > 0 ? bg->buckets : (B + 15) / 16;
  const int nb = std::max(1, std::min(std::min(want, B), kMaxBuckets));
  cudaError_t e = ensure_buckets(bg, nb);
  if (e != cudaSuccess) return graph_fail("bucket set-up", e);
  std::vector<int> order(B);
  for (int b = 0; b < B; ++b) order[b] = b;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    const LogregBatched *a = bg->lbs[x], *c = bg->lbs[y];
    return a->d != c->d ? a->d < c->d : a->N < c->N;
  });
  bg->pending.clear();
  bg->staging.clear();
  for (int k = 0; k < nb; ++k) {
    const int b0 = (int)((long long)B * k / nb), b1 = (int)((long long)B * (k + 1) / nb);
    std::vector<int> members(order.begin() + b0, order.begin() + b1);
    e = capture_bucket(bg, members, bg->flag + 2 * k, bg->flag + 2 * k + 1, L, impl, prop, gl);
    if (e != cudaSuccess) {
      bg->pending.clear();
      if (e == cudaErrorInvalidValue) {
        g_err = "grouped batch: the posteriors' transitions differ in structure";
        return GJ_EINVAL;
      }
      return graph_fail("batch record", e);
    }
  }
  {  // one upload of every launch's items and prefix sums
    void* dbuf = nullptr;
    e = cudaMalloc(&dbuf, std::max<size_t>(bg->staging.size(), 64));
    if (e == cudaSuccess) bufs->push_back(dbuf);
    if (e == cudaSuccess && !bg->staging.empty())
      e = cudaMemcpy(dbuf, bg->staging.data(), bg->staging.size(), cudaMemcpyHostToDevice);
    std::vector<unsigned char>().swap(bg->staging);
    if (e != cudaSuccess) {
      bg->pending.clear();
      return graph_fail("batch items", e);
    }
    unsigned char* d0 = static_cast<unsigned char*>(dbuf);
    for (auto& pk : bg->pending)
      for (auto& launches : pk.plan)
        for (GroupLaunch& g : launches) {
          g.items = d0 + reinterpret_cast<size_t>(g.items);
          g.prefix = reinterpret_cast<const int*>(d0 + reinterpret_cast<size_t>(g.prefix));
        }
  }
  const StepDev* spd = bg->lbs[0]->spd;  // every posterior gets the same step parameters
  cudaStream_t root = bg->cap_root;
  e = cudaStreamBeginCapture(root, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return graph_fail("grouped begin", e);
  e = cudaEventRecord(bg->fork, root);
  for (int k = 0; k < nb && e == cudaSuccess; ++k) {
    cudaStream_t sk = bg->bucket_main[k], sbk = bg->bucket_body[k];
    e = cudaStreamWaitEvent(sk, bg->fork, 0);
    if (e == cudaSuccess) e = emit_bucket(bg->pending[k], spd, sk, sbk);
    if (e == cudaSuccess) e = cudaEventRecord(bg->join, sk);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(root, bg->join, 0);
  }
  bg->pending.clear();
  cudaGraph_t g = nullptr;
  const cudaError_t e2 = cudaStreamEndCapture(root, &g);
  if (e != cudaSuccess || e2 != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return graph_fail("grouped capture", e != cudaSuccess ? e : e2);
  }
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    *out = nullptr;
    return graph_fail("grouped instantiate", e);
  }
  return GJ_OK;
}

}  // namespace

int logreg_batch_graph_step(LogregBatchGraph* bg, const StepDev& sp, float* pos, float* grad,
                            double* logdens, const float* z, const double* u,
                            const InfoDev<float>& info, int gemm_impl, cudaStream_t st) {
  const bool gl = sp.integrator == GJ_GENERALIZED_LEAPFROG;
  for (LogregBatched* lb : bg->lbs) {
    if (gemm_impl == 2 && !lb->tc_ok) {
      g_err = "tcgen05 GEMM unavailable (no sm_100-family device or tensor-map encoder)";
      return GJ_ENOTSUP;
    }
    if (gl) {
      const int rg = ensure_gl(lb);
      if (rg) return rg;
    }
    lb->stats = LogregStats{};
  }
  const bool prop = info.prop_v != nullptr;
  const int cfg = graph_cfg(bg->lbs[0]) + (gl ? (1 << 20) : 0) +
                  (bg->grouped ? (1 << 21) * (1 + std::min(bg->buckets, 255)) : 0);
  cudaGraphExec_t exec = nullptr;
  for (auto& g : bg->graphs)
    if (g.L == sp.L && g.impl == gemm_impl && g.cfg == cfg && g.prop == (int)prop) {
      g.used = ++bg->tick;
      exec = g.exec;
    }
  if (!exec) {
    // the capture streams must not see unfinished work of the caller's stream
    cudaStreamSynchronize(st);
    if (bg->graphs.size() >= kMaxBatchGraphs) {
      size_t lru = 0;
      for (size_t i = 1; i < bg->graphs.size(); ++i)
        if (bg->graphs[i].used < bg->graphs[lru].used) lru = i;
      free_entry(bg->graphs[lru]);
      bg->graphs.erase(bg->graphs.begin() + lru);
    }
    std::vector<void*> bufs;
    const int rc = bg->grouped
                       ? batch_capture_grouped(bg, sp.L, gemm_impl, prop, gl, &exec, &bufs)
                       : batch_capture(bg, sp.L, gemm_impl, prop, gl, &exec);
    if (rc) {
      for (void* p : bufs) cudaFree(p);
      return rc;
    }
    bg->graphs.push_back({sp.L, gemm_impl, cfg, (int)prop, exec, ++bg->tick, std::move(bufs)});
  }
  const int B = (int)bg->lbs.size();
  batch_gather_kernel<<<B, 256, 0, st>>>(bg->stages, bg->C, sp, pos, grad, logdens, z, u);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaGraphLaunch(exec, st);
  if (e == cudaSuccess) {
    batch_scatter_kernel<<<B, 256, 0, st>>>(bg->stages, bg->C, pos, grad, logdens, info);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    g_err = std::string("batch graph step: ") + cudaGetErrorString(e);
    return GJ_ECUDA;
  }
  return GJ_OK;
}

}  // namespace gj
