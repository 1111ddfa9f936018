// Cross-chain statistics of ChEES adaptation, computed on the device from the
// proposals a transition wrote (adaptation/chees_adaptation_riemanian.py:
// 145-190, adaptation/chees_adaptation_lmcmonge.py:151-236).
//
// From the proposed positions P, the proposed (flipped) velocities V and the
// initial positions I of C chains, with acceptance probabilities a and
// divergence flags:
//   harmonic  = 1 / mean(1/a over non-divergent chains)
//   P̃ = P − nanmean_c(P),  Ĩ = I − nanmean_c(I)
//   g_c       = (|P̃_c|² − |Ĩ_c|²) · (P̃_c · V_c)
//   gradient  = Σ a_c g_c / Σ a_c over non-divergent chains
// (the caller multiplies by jitter × trajectory length), and with a tangent
// D = ∂P/∂α² the same weighted mean of (|P̃_c|² − |Ĩ_c|²) · (P̃_c · D_c).
//
// Three launches, each with a fixed reduction order, so the result does not
// depend on scheduling: per-dimension means (32 dimensions × 8 chain lanes
// per CTA, coalesced rows), per-chain dots (one warp per chain), and one CTA
// that sums the per-chain terms.  All sums are in float64.
#include <cmath>

#include "common.cuh"

namespace gj {

namespace {

template <typename T>
__global__ void __launch_bounds__(256) chees_means_kernel(int C, int d, const T* __restrict__ P,
                                                          const T* __restrict__ I,
                                                          double* __restrict__ mean) {
  __shared__ double sp[8][32], si[8][32];
  __shared__ int np[8][32], ni[8][32];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int j = blockIdx.x * 32 + tx;
  double a = 0.0, b = 0.0;
  int na = 0, nb = 0;
  if (j < d) {
    for (int c = ty; c < C; c += 8) {
      const double x = double(P[(size_t)c * d + j]);
      const double y = double(I[(size_t)c * d + j]);
      if (!isnan(x)) {
        a += x;
        ++na;
      }
      if (!isnan(y)) {
        b += y;
        ++nb;
      }
    }
  }
  sp[ty][tx] = a;
  si[ty][tx] = b;
  np[ty][tx] = na;
  ni[ty][tx] = nb;
  __syncthreads();
  if (ty == 0 && j < d) {
    for (int k = 1; k < 8; ++k) {
      a += sp[k][tx];
      b += si[k][tx];
      na += np[k][tx];
      nb += ni[k][tx];
    }
    mean[j] = na ? a / na : NAN;  // nanmean of an all-NaN column is NaN
    mean[d + j] = nb ? b / nb : NAN;
  }
}

// part[c] = {a g, a, 1/a, 1, a g_α} for a non-divergent chain, zeros else
template <typename T>
__global__ void __launch_bounds__(256) chees_chain_kernel(int C, int d, const T* __restrict__ P,
                                                          const T* __restrict__ V,
                                                          const T* __restrict__ I,
                                                          const T* __restrict__ D,
                                                          const double* __restrict__ mean,
                                                          const double* __restrict__ acc,
                                                          const uint8_t* __restrict__ div,
                                                          double* __restrict__ part) {
  const int lane = threadIdx.x & 31;
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (c >= C) return;  // whole warp
  double pp = 0.0, ii = 0.0, pv = 0.0, pd = 0.0;
  for (int j = lane; j < d; j += 32) {
    const double p = double(P[(size_t)c * d + j]) - mean[j];
    const double q = double(I[(size_t)c * d + j]) - mean[d + j];
    pp += p * p;
    ii += q * q;
    pv += p * double(V[(size_t)c * d + j]);
    if (D) pd += p * double(D[(size_t)c * d + j]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    pp += __shfl_xor_sync(0xffffffffu, pp, o);
    ii += __shfl_xor_sync(0xffffffffu, ii, o);
    pv += __shfl_xor_sync(0xffffffffu, pv, o);
    pd += __shfl_xor_sync(0xffffffffu, pd, o);
  }
  if (lane == 0) {
    double* o = part + (size_t)c * 5;
    if (div && div[c]) {
      o[0] = o[1] = o[2] = o[3] = o[4] = 0.0;
    } else {
      const double a = acc[c];
      o[0] = a * (pp - ii) * pv;
      o[1] = a;
      o[2] = 1.0 / a;
      o[3] = 1.0;
      o[4] = a * (pp - ii) * pd;
    }
  }
}

__global__ void __launch_bounds__(256) chees_final_kernel(int C, const double* __restrict__ part,
                                                          double* __restrict__ out) {
  __shared__ double s[5][256];
  double r[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int c = threadIdx.x; c < C; c += 256)
    for (int k = 0; k < 5; ++k) r[k] += part[(size_t)c * 5 + k];
  for (int k = 0; k < 5; ++k) s[k][threadIdx.x] = r[k];
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int k = 0; k < 5; ++k) s[k][threadIdx.x] += s[k][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = s[3][0] / s[2][0];  // harmonic mean: n / Σ 1/a
    out[1] = s[0][0] / s[1][0];
    out[2] = s[4][0] / s[1][0];
  }
}

}  // namespace

size_t chees_workspace_bytes(int C, int d) { return sizeof(double) * (2 * (size_t)d + 5 * (size_t)C); }

template <typename T>
cudaError_t chees_statistics(int C, int d, const T* P, const T* V, const T* I, const T* D,
                             const double* acc, const uint8_t* div, double* work, double* out,
                             cudaStream_t st) {
  double* mean = work;
  double* part = work + 2 * (size_t)d;
  chees_means_kernel<T><<<(d + 31) / 32, 256, 0, st>>>(C, d, P, I, mean);
  chees_chain_kernel<T><<<(unsigned)(((size_t)C * 32 + 255) / 256), 256, 0, st>>>(
      C, d, P, V, I, D, mean, acc, div, part);
  chees_final_kernel<<<1, 256, 0, st>>>(C, part, out);
  return cudaGetLastError();
}

template cudaError_t chees_statistics<float>(int, int, const float*, const float*, const float*,
                                             const float*, const double*, const uint8_t*,
                                             double*, double*, cudaStream_t);
template cudaError_t chees_statistics<double>(int, int, const double*, const double*,
                                              const double*, const double*, const double*,
                                              const uint8_t*, double*, double*, cudaStream_t);

}  // namespace gj
