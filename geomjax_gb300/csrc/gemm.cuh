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

enum EpiMode : int { EPI_STORE = 0, EPI_SIGMOID = 1, EPI_TRACE = 2, EPI_R2W = 3, EPI_R2G = 4 };

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

struct TcOperand;

struct Epi {
  int mode;
  // EPI_STORE
  float* D;
  int ldd;
  // EPI_STORE with the K range split over gridDim.z CTAs (GemmArgs::ksplit):
  // slice z stores its partial product at D + z·d_slice (elements); the
  // consumer adds the slices in order
  size_t d_slice;
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
  // EPI_SIGMOID, when set: Λ alone (the metric at a position iterate of the
  // generalized leapfrog needs neither Λ' nor r₁)
  int lam_only;
  // EPI_TRACE, when set: w is also stored into w_out[m, n] (stride s_ld)
  float* w_out;
  // EPI_R2W: a = s = x_nᵀu_m  ->  r2 = Λ'(w − s²) into r (rows r_off + m),
  // w read from W[m, n] (stride s_ld): the momentum-only re-evaluation of
  // the generalized leapfrog, where w = x_nᵀG⁻¹x_n is fixed
  const float* W;
  // EPI_R2G (tcgen05 path only; three planes, 128-wide tiles, K <= 64):
  // EPI_R2W's r2, split into three BF16 planes in shared memory and
  // contracted with Xᵀ (the operand xt: x_d <= 32 rows, the observations
  // along K, plane pitch xt_rpad) by a second tcgen05 MMA in the same CTA
  // instead of being stored: the CTA of N tile t writes
  // g2[t·g2_slice + m·g2_ld + k] = Σ_{n in tile t} r2[m, n]·X[n, k] for
  // k < x_d (rounded up to a multiple of 4; 16-byte aligned rows); the
  // consumer adds the ⌈N / 128⌉ tile partials in tile order
  const TcOperand* xt;
  int xt_rpad;
  int x_d;
  float* g2;
  int g2_ld;
  size_t g2_slice;
  // tcgen05 path, when set: output row m (a chain) is wanted only while
  // active_rows[m] != 0, and a CTA whose 128 rows are all inactive does
  // nothing (the fixed-point loop bodies, whose converged chains' outputs
  // are not read again before the evaluation that follows the loop)
  const uint8_t* active_rows;
};

// σ(a), σ(−a) and log(1 + e^a) from one exponential, e = e^{−|a|}: neither
// sigmoid is formed as 1 − the other, which in float32 loses the relative
// accuracy of the small one (Λ = σ(a)σ(−a) at |a| = 7 would carry ~6e-5)
struct Sig {
  float sp, sm, e;  // e = e^{−|a|}
};
__device__ __forceinline__ Sig sig_pair(float a) {
  const float e = __expf(-fabsf(a));
  const float big = __fdividef(1.f, 1.f + e), small = e * big;
  Sig s;
  s.sp = a >= 0.f ? big : small;
  s.sm = a >= 0.f ? small : big;
  s.e = e;
  return s;
}
// log(1 + e^a) from the pair's e (only where the log density is summed)
__device__ __forceinline__ float sig_softplus(float a, const Sig& s) {
  return fmaxf(a, 0.f) + log1pf(s.e);
}

__device__ __forceinline__ void epi_apply(const Epi& e, int m, int n, float v) {
  if (e.mode == EPI_STORE) {
    e.D[(size_t)m * e.ldd + n] = v;
  } else if (e.mode == EPI_SIGMOID) {
    const Sig sg = sig_pair(v);
    const float yv = e.y[n];
    if (e.ld_acc) atomicAdd(&e.ld_acc[m], double(yv * v - sig_softplus(v, sg)));
    const float lam = sg.sp * sg.sm;
    split_store(e.lam, m, n, lam);
    if (e.lam_only) return;
    e.lp[(size_t)m * e.lp_ld + n] = lam * (sg.sm - sg.sp);
    split_store(e.r, m, n, yv * sg.sm - (1.f - yv) * sg.sp);
  } else if (e.mode == EPI_TRACE) {
    const float s = e.S[(size_t)m * e.s_ld + n];
    const float r2 = e.lp[(size_t)m * e.lp_ld + n] * (v - s * s);
    split_store(e.r, e.r_off + m, n, r2);
    if (e.w_out) e.w_out[(size_t)m * e.s_ld + n] = v;
  } else {  // EPI_R2W
    const float w = e.W[(size_t)m * e.s_ld + n];
    const float r2 = e.lp[(size_t)m * e.lp_ld + n] * (w - v * v);
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

struct GemmArgs {
  SplitMat A;  // M x K
  SplitMat B;  // N x K
  int M, N, K;
  Epi epi;
  bool pdl = false;  // tcgen05 path: launch as a programmatic dependent
  // tcgen05 path, EPI_STORE only: the K blocks split into this many
  // contiguous slices, one CTA per output tile and slice, so that a GEMM
  // with few output tiles and a long K fills the SMs.  Every slice must get
  // at least one K block (gemm_ksplit_valid).
  int ksplit = 1;
  // tcgen05 path: the A rows start at this row of each plane (output row m
  // is A row a_row0 + m); a_row0 + M must not exceed the planes' row pitch
  int a_row0 = 0;
};

// whether `ksplit` slices of ⌈K/64⌉ K blocks are all non-empty
inline bool gemm_ksplit_valid(int K, int ksplit) {
  const int kb = (K + 63) / 64;
  if (ksplit < 1 || ksplit > kb) return false;
  const int per = (kb + ksplit - 1) / ksplit;
  return (ksplit - 1) * per < kb;
}

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
// most K-range accumulators a CTA may use (1, 2 or 4; default 4): more
// ranges shorten the tensor core's low-rounding accumulation runs, and cost
// the epilogue one TMEM read per range
void gemm_tc_set_accumulators(int max_ranges);
cudaError_t gemm_tc(const GemmArgs& g, const TcOperand* a, const TcOperand* b, int* err_flag,
                    cudaStream_t st);
// the output tile width (32, 64 or 128) a launch with these planes, N and K
// takes under the current tile policy
int gemm_tc_bn(int planes, int N, int K);

// One contraction of a grouped launch: its tensor maps, epilogue, error
// flag and launch parameters (the ring depth, K-range accumulators and grid
// gemm_tc would use).  The tensor maps (64-byte aligned, so the item is)
// are read by the kernel from global memory.
struct GemmItem {
  CUtensorMap mapA, mapB, mapXT;
  Epi epi;
  int* err;
  int rpadA, rpadB, M, N, K, stages, a_row0, nacc, gx, gy, gz;
};
// The launch gemm_tc would make, described instead of made: the item, the
// kernel variant (planes, tile width, fused r2·X epilogue), the CTA count
// and the dynamic shared memory.  The same checks as gemm_tc.
cudaError_t gemm_tc_describe(const GemmArgs& g, const TcOperand* a, const TcOperand* b, int* err,
                             GemmItem* item, int* variant, int* blocks, size_t* smem);
// One grid over n described items of one variant; items and the prefix sums
// of their CTA counts (n + 1 entries, prefix[n] = blocks) in device memory.
cudaError_t gemm_tc_grouped(int variant, const GemmItem* items, const int* prefix, int n, int blocks,
                            size_t smem, cudaStream_t st);

// noalloc.cu: the same contraction with the split planes in a static device
// array (no cudaMalloc / cudaFree); capacity in BF16 elements.
int gemm_split_noalloc(int impl, int planes, int M, int N, int K, const float* A, const float* B,
                       float* D, cudaStream_t st);
const char* gemm_noalloc_error();
size_t gemm_noalloc_capacity();

}  // namespace gj
