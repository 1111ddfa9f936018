// Batched contractions of the dense-Fisher path: D[M, N] = A[M, K] · B[N, K]ᵀ
// with both operands stored K-major as split BF16 planes stacked along rows.
// Two planes (x0 + x1, 16 significant bits): the three-term product
// A0·B0 + A0·B1 + A1·B0.  Three planes (24 bits): the six terms with plane
// indices i + j <= 2.  FP32 accumulation either way.  Two implementations share the epilogues below:
// a SIMT FP32 kernel (gemm_simt.cu) and the tcgen05/TMA kernel (gemm_tc.cu).
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>

#include "common.cuh"

namespace gj {

using bf16 = __nv_bfloat16;

enum EpiMode : int { EPI_STORE = 0, EPI_SIGMOID = 1, EPI_TRACE = 2 };

// A split BF16 matrix, `rows` x `kdim`, as `planes` BF16 planes whose sum is
// the value: x0 = bf16(x), x1 = bf16(x − x0) and, with three planes,
// x2 = bf16(x − x0 − x1) (24 significant bits: every FP32 value exactly up
// to rounding of the last piece).  Plane k holds rows [k·rpad, (k+1)·rpad);
// row stride `ld` elements.  ld is a multiple of 64 and rpad a multiple of
// 128, and the padding is zero, so every 64-column x 128-row TMA box lies
// inside the allocation.
struct SplitMat {
  bf16* p;
  int rows;
  int kdim;
  int ld;
  int rpad;
  int planes;  // 2 or 3
};

__device__ __forceinline__ void split_store(const SplitMat& s, int r, int k, float x) {
  const bf16 b0 = __float2bfloat16_rn(x);
  const float r0 = x - __bfloat162float(b0);
  const bf16 b1 = __float2bfloat16_rn(r0);
  s.p[(size_t)r * s.ld + k] = b0;
  s.p[(size_t)(s.rpad + r) * s.ld + k] = b1;
  if (s.planes == 3)
    s.p[(size_t)(2 * s.rpad + r) * s.ld + k] = __float2bfloat16_rn(r0 - __bfloat162float(b1));
}

struct Epi {
  int mode;
  // EPI_STORE
  float* D;
  int ldd;
  // EPI_SIGMOID: a = x_nᵀβ_m  ->  Λ = σ(1−σ) into lam, Λ' = Λ(1−2σ) into lp,
  // r1 = y_n − σ into r (rows [0, C))
  const float* y;
  SplitMat lam;
  float* lp;
  int lp_ld;
  SplitMat r;
  // EPI_TRACE: w = x_nᵀG⁻¹x_n  ->  r2 = Λ'(w − s²) into r (rows [C, 2C)),
  // s = S[m, n] = x_nᵀu_m
  const float* S;
  int s_ld;
  int r_off;
  // EPI_SIGMOID, when set: ld_acc[m] += Σ_n [y_n a − log(1 + e^a)] (FP64 sum)
  double* ld_acc;
};

__device__ __forceinline__ float softplus(float a) {
  return a > 0.f ? a + log1pf(__expf(-a)) : log1pf(__expf(a));
}

__device__ __forceinline__ void epi_apply(const Epi& e, int m, int n, float v) {
  if (e.mode == EPI_STORE) {
    e.D[(size_t)m * e.ldd + n] = v;
  } else if (e.mode == EPI_SIGMOID) {
    if (e.ld_acc) atomicAdd(&e.ld_acc[m], double(e.y[n] * v - softplus(v)));
    const float sg = 1.f / (1.f + __expf(-v));
    const float lam = sg * (1.f - sg);
    split_store(e.lam, m, n, lam);
    e.lp[(size_t)m * e.lp_ld + n] = lam * (1.f - 2.f * sg);
    split_store(e.r, m, n, e.y[n] - sg);
  } else {
    const float s = e.S[(size_t)m * e.s_ld + n];
    const float r2 = e.lp[(size_t)m * e.lp_ld + n] * (v - s * s);
    split_store(e.r, e.r_off + m, n, r2);
  }
}

// 8 values of one row as split BF16: one 16-byte store into each plane
__device__ __forceinline__ void split_store8(const SplitMat& s, int r, int k, const float* x) {
  uint32_t w0[4], w1[4], w2[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(x[2 * j], x[2 * j + 1]);
    const float2 hf = __bfloat1622float2(h);
    const float ra = x[2 * j] - hf.x, rb = x[2 * j + 1] - hf.y;
    const __nv_bfloat162 m = __floats2bfloat162_rn(ra, rb);
    const float2 mf = __bfloat1622float2(m);
    const __nv_bfloat162 l = __floats2bfloat162_rn(ra - mf.x, rb - mf.y);
    w0[j] = *reinterpret_cast<const uint32_t*>(&h);
    w1[j] = *reinterpret_cast<const uint32_t*>(&m);
    w2[j] = *reinterpret_cast<const uint32_t*>(&l);
  }
  *reinterpret_cast<uint4*>(s.p + (size_t)r * s.ld + k) = make_uint4(w0[0], w0[1], w0[2], w0[3]);
  *reinterpret_cast<uint4*>(s.p + (size_t)(s.rpad + r) * s.ld + k) =
      make_uint4(w1[0], w1[1], w1[2], w1[3]);
  if (s.planes == 3)
    *reinterpret_cast<uint4*>(s.p + (size_t)(2 * s.rpad + r) * s.ld + k) =
        make_uint4(w2[0], w2[1], w2[2], w2[3]);
}

// Columns n0 .. n0+31 of row m (one tcgen05.ld chunk): vector loads/stores
// when the chunk is complete and the row strides allow 16-byte access,
// element-wise otherwise.
__device__ __forceinline__ void epi_row32(const Epi& e, int m, int n0, int N, const float* v) {
  const bool full = n0 + 32 <= N;
  if (e.mode == EPI_SIGMOID && e.ld_acc) {
    double acc = 0.0;
    for (int j = 0; j < 32; ++j)
      if (n0 + j < N) acc += double(e.y[n0 + j] * v[j] - softplus(v[j]));
    atomicAdd(&e.ld_acc[m], acc);
    Epi e2 = e;
    e2.ld_acc = nullptr;
    epi_row32(e2, m, n0, N, v);
    return;
  }
  if (!full || (e.mode == EPI_STORE && (e.ldd & 3)) ||
      (e.mode != EPI_STORE && ((e.lp_ld & 3) || (e.mode == EPI_TRACE && (e.s_ld & 3))))) {
    for (int j = 0; j < 32; ++j)
      if (n0 + j < N) epi_apply(e, m, n0 + j, v[j]);
    return;
  }
  if (e.mode == EPI_STORE) {
    float4* dst = reinterpret_cast<float4*>(e.D + (size_t)m * e.ldd + n0);
#pragma unroll
    for (int q = 0; q < 8; ++q) dst[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
  } else if (e.mode == EPI_SIGMOID) {
#pragma unroll
    for (int g = 0; g < 4; ++g) {
      float lam[8], lp[8], r1[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const float sg = 1.f / (1.f + __expf(-v[8 * g + j]));
        lam[j] = sg * (1.f - sg);
        lp[j] = lam[j] * (1.f - 2.f * sg);
        r1[j] = e.y[n0 + 8 * g + j] - sg;
      }
      split_store8(e.lam, m, n0 + 8 * g, lam);
      split_store8(e.r, m, n0 + 8 * g, r1);
      float4* lpd = reinterpret_cast<float4*>(e.lp + (size_t)m * e.lp_ld + n0 + 8 * g);
      lpd[0] = make_float4(lp[0], lp[1], lp[2], lp[3]);
      lpd[1] = make_float4(lp[4], lp[5], lp[6], lp[7]);
    }
  } else {
#pragma unroll
    for (int g = 0; g < 4; ++g) {
      const float4* sp = reinterpret_cast<const float4*>(e.S + (size_t)m * e.s_ld + n0 + 8 * g);
      const float4* lpp = reinterpret_cast<const float4*>(e.lp + (size_t)m * e.lp_ld + n0 + 8 * g);
      const float4 s0 = sp[0], s1 = sp[1], l0 = lpp[0], l1 = lpp[1];
      const float sv[8] = {s0.x, s0.y, s0.z, s0.w, s1.x, s1.y, s1.z, s1.w};
      const float lv[8] = {l0.x, l0.y, l0.z, l0.w, l1.x, l1.y, l1.z, l1.w};
      float r2[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) r2[j] = lv[j] * (v[8 * g + j] - sv[j] * sv[j]);
      split_store8(e.r, e.r_off + m, n0 + 8 * g, r2);
    }
  }
}

struct GemmArgs {
  SplitMat A;  // M x K
  SplitMat B;  // N x K
  int M, N, K;
  Epi epi;
  bool pdl = false;  // tcgen05 path: launch as a programmatic dependent
};

cudaError_t gemm_simt(const GemmArgs& g, cudaStream_t st);

// tcgen05 path: tensor maps are built once per operand buffer.
struct TcOperand {
  CUtensorMap map;    // 64 x 128-row boxes (A operands, B with 128-wide tiles)
  CUtensorMap map64;  // 64 x 64-row boxes (B with 64-wide tiles)
  CUtensorMap map32;  // 64 x 32-row boxes (B with 32-wide tiles)
  SplitMat s;
};
// Encodes the operand's tensor map in place (no allocation); false on error.
bool tc_operand_init(TcOperand* op, const SplitMat& s, const char** err);
TcOperand* tc_operand_create(const SplitMat& s, int box_rows, const char** err);
void tc_operand_destroy(TcOperand* op);
bool tc_available();
cudaError_t gemm_tc_prepare();  // raises the kernel's shared-memory limit (call before capture)
// Process-wide tile policy: bn_wide = 64 or 128 for N > 64 (0 = automatic);
// two_ctas = 1 limits the operand ring so that two CTAs share an SM, 0 keeps
// a deep ring, -1 = automatic.  Takes effect for launches (and graph
// captures) made after the call.
void gemm_tc_set_tuning(int bn_wide, int two_ctas);
// a small integer identifying the current tile policy (part of the key of
// captured graphs, whose launches keep the tiles they were captured with)
int gemm_tc_tuning_code();
cudaError_t gemm_tc(const GemmArgs& g, const TcOperand* a, const TcOperand* b, int* err_flag,
                    cudaStream_t st);

// noalloc.cu: the same contraction with the split planes in a static device
// array (no cudaMalloc / cudaFree); capacity in BF16 elements.
int gemm_split_noalloc(int impl, int planes, int M, int N, int K, const float* A, const float* B,
                       float* D, cudaStream_t st);
const char* gemm_noalloc_error();
size_t gemm_noalloc_capacity();

}  // namespace gj
