// SIMT FP32 implementation of the split-BF16 contraction (gemm.cuh).  It
// reconstructs the sum of the planes in FP32 (so it also carries the
// higher-order cross terms) and is the correctness cross-check of the
// tensor-core kernel, not the fast path.
#include "gemm.cuh"

namespace gj {

namespace {

constexpr int BM = 64, BN = 64, BK = 16;

__global__ void __launch_bounds__(256) gemm_simt_kernel(GemmArgs g) {
  __shared__ float As[BK][BM + 4];
  __shared__ float Bs[BK][BN + 4];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < g.K; k0 += BK) {
    for (int i = threadIdx.x; i < BM * BK; i += 256) {
      const int r = i / BK, k = i % BK;
      const int m = m0 + r, kk = k0 + k;
      float a = 0.f, b = 0.f;
      if (m < g.M && kk < g.K)
        for (int q = 0; q < g.A.planes; ++q)
          a += __bfloat162float(g.A.p[(size_t)(q * g.A.rpad + m) * g.A.ld + kk]);
      const int n = n0 + r;
      if (n < g.N && kk < g.K)
        for (int q = 0; q < g.B.planes; ++q)
          b += __bfloat162float(g.B.p[(size_t)(q * g.B.rpad + n) * g.B.ld + kk]);
      As[k][r] = a;
      Bs[k][r] = b;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < BK; ++k) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        a[i] = As[k][ty * 4 + i];
        b[i] = Bs[k][tx * 4 + i];
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int m = m0 + ty * 4 + i, n = n0 + tx * 4 + j;
      if (m < g.M && n < g.N) epi_apply(g.epi, m, n, acc[i][j]);
    }
}

}  // namespace

cudaError_t gemm_simt(const GemmArgs& g, cudaStream_t st) {
  if (g.M <= 0 || g.N <= 0) return cudaSuccess;
  // tcgen05 path only: K slices, A row offsets, the fused r2·X epilogue
  if (g.ksplit != 1 || g.a_row0 != 0 || g.epi.mode == EPI_R2G) return cudaErrorInvalidValue;
  dim3 grid((g.N + BN - 1) / BN, (g.M + BM - 1) / BM);
  gemm_simt_kernel<<<grid, 256, 0, st>>>(g);
  return cudaGetLastError();
}

}  // namespace gj
