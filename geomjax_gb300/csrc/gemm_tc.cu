// tcgen05 implementation of the split-BF16 contraction (gemm.cuh) for sm_103a.
//
// One CTA computes one 128 x BN output tile D = A·Bᵀ (both operands K-major,
// BN = 32, 64 or 128):
//   warp 0      TMA producer: per 64-wide K chunk, one 128 x 64 BF16 box per
//               plane of A and one BN x 64 box per plane of B (128B-swizzled)
//               into a ring of 1-4 stages sized at launch
//   warp 1      allocates NACC·max(32, BN) TMEM columns; one elected thread
//               issues tcgen05.mma.kind::f16 (BF16 x BF16 -> FP32, M = 128,
//               N = BN, K = 16): the plane products A_i·B_j with i + j <
//               planes per K step, and tcgen05.commit frees each stage /
//               signals the accumulators.  The K blocks are cut into NACC
//               contiguous ranges (1, 2 or 4), each with its own TMEM
//               accumulator, and the epilogue adds the NACC partial tiles in
//               FP32 registers: the tensor core's FP32 accumulation rounds
//               low (measured mean relative bias −4.5e-6 at K = 1000 and
//               −3.2e-5 at K = 5000 on positive operands, against ~0 for
//               round-to-nearest FP32 FMAs), and the bias grows with the
//               number of accumulation steps into one accumulator
//   warps 2-9   epilogue: tcgen05.ld 32x32b (warp w reads TMEM lanes
//               32·(w%4) .. +31 = output rows; the two warps of a lane
//               quarter take alternate 32-column chunks), staged once through
//               shared memory and processed as row segments (8 values of one
//               row per lane, 16-byte global accesses)
// The R2G instantiation (EPI_R2G: three planes, BN = 128, one K block) then
// contracts its r2 = Λ'(w − s²) with Xᵀ in the same CTA: r2 goes into the
// freed operand ring as swizzled BF16 planes, the producer warp TMA-loads
// the Xᵀ boxes, and one epilogue thread issues a second set of MMAs into 32
// more TMEM columns (see epi_r2g).
// Every mbarrier wait is bounded; on timeout the kernel records an error code
// in *err and skips the rest of its work, releasing TMEM before exit.
#include <cuda.h>

#include <algorithm>
#include <cstring>

#include "gemm.cuh"

namespace gj {

namespace {

constexpr int BM = 128, BK = 64;
constexpr int A_TILE_BYTES = BM * BK * 2;         // one 128 x 64 BF16 box
// NPL planes per operand, BN output columns per CTA (32, 64 or 128): a stage
// holds NPL A boxes (128 x 64) and NPL B boxes (BN x 64)
template <int NPL, int BN>
struct Cfg {
  static constexpr int B_TILE_BYTES = BN * BK * 2;
  static constexpr int STAGE_BYTES = NPL * (A_TILE_BYTES + B_TILE_BYTES);
  // up to 4 stages within the 227 KB a CTA may use
  static constexpr int FIT = (227 * 1024 - 1024 - 256) / STAGE_BYTES;
  static constexpr int MAX_STAGES = FIT < 4 ? FIT : 4;
  static constexpr int TMEM_COLS = BN < 32 ? 32 : BN;
  static constexpr int IDESC = (1 << 4) | (1 << 7) | (1 << 10) | ((BN >> 3) << 17) |
                               ((BM >> 4) << 24);
  static constexpr int smem(int stages) { return stages * STAGE_BYTES + 1024 + 256; }
};
constexpr long long WAIT_LIMIT = 1ll << 26;       // polls before giving up

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn get_encode() {
  static EncodeTiledFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

// bounded wait on the phase with the given parity; returns false on timeout
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  for (long long i = 0; i < WAIT_LIMIT; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if (i > 64) __nanosleep(32);
  }
  return false;
}

// Acquire a tensor map that the host copied into global memory (grouped
// launches), before the TMA unit reads it: the copy is not ordered with the
// tensor-map proxy otherwise; system scope for a host-side write.
__device__ __forceinline__ void tensormap_acquire(const CUtensorMap* m) {
  asm volatile("fence.proxy.tensormap::generic.acquire.sys [%0], 128;" ::"l"(m) : "memory");
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar,
                                            int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, "
      "%4}], [%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y)
      : "memory");
}

// K-major, 128B-swizzled shared-memory matrix descriptor (sm_100 format):
// start>>4 in [0,14), LBO>>4 in [16,30) (unused for swizzled K-major, 1),
// SBO>>4 in [32,46) = 1024 B between 8-row swizzle atoms, version 1 in
// [46,48), layout type 2 (SWIZZLE_128B) in [61,64).
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// instruction descriptor (Cfg::IDESC), kind::f16: D = F32 (bit 4), A = B = BF16
// (bits 7, 10), both K-major, N>>3 at [17,23), M>>4 at [24,29)
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
      "%12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, "
      "%30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Epilogue of one 32 x 32 chunk handled by one warp.  The accumulator rows
// (lane l holds row m_base + l, v[0..31] = columns n_base..+31) are staged
// once in the warp's shared-memory tile (stride 33: conflict-free both ways),
// then read back as row segments: in pass it (0..3) lane l takes row
// 8·it + l/4, columns 8·(l%4) .. +7.  Each lane then works on 8 consecutive
// values of one row, so every global access is 16 bytes per lane (one row
// of the chunk = 4 lanes) and few registers stay live.
__device__ __forceinline__ void stage_row(float* stg, int lane, const float* v) {
#pragma unroll
  for (int j = 0; j < 32; ++j) stg[lane * 33 + j] = v[j];
  __syncwarp();
}

__device__ __forceinline__ bool aligned16(const void* p, int ld) {
  return ((reinterpret_cast<uintptr_t>(p) & 15) == 0) && ((ld & 3) == 0);
}

__device__ __forceinline__ void load8(const float* src, int n, int N, bool vec, float* out) {
  if (vec) {
    const float4 a = __ldg(reinterpret_cast<const float4*>(src));
    const float4 b = __ldg(reinterpret_cast<const float4*>(src) + 1);
    out[0] = a.x; out[1] = a.y; out[2] = a.z; out[3] = a.w;
    out[4] = b.x; out[5] = b.y; out[6] = b.z; out[7] = b.w;
  } else {
#pragma unroll
    for (int k = 0; k < 8; ++k) out[k] = (n + k < N) ? __ldg(src + k) : 0.f;
  }
}

__device__ __forceinline__ void store8(float* dst, int n, int N, bool vec, const float* x) {
  if (vec) {
    reinterpret_cast<float4*>(dst)[0] = make_float4(x[0], x[1], x[2], x[3]);
    reinterpret_cast<float4*>(dst)[1] = make_float4(x[4], x[5], x[6], x[7]);
  } else {
#pragma unroll
    for (int k = 0; k < 8; ++k)
      if (n + k < N) dst[k] = x[k];
  }
}

__device__ __forceinline__ void split8(const SplitMat& S, int row, int n, int N, bool full,
                                       const float* x) {
  if (full) {
    split_store8(S, row, n, x);  // plane rows are 128-byte aligned, n a multiple of 8
  } else {
#pragma unroll
    for (int k = 0; k < 8; ++k)
      if (n + k < N) split_store(S, row, n + k, x[k]);
  }
}

__device__ __forceinline__ void epi_chunk(const Epi& e, float* stg, int lane, int m_base, int n_base,
                                          int M, int N, const float* v, int kslice) {
  stage_row(stg, lane, v);
  const int cc = (lane & 3) * 8;
  const int n = n_base + cc;
  const bool full = n + 8 <= N;
#pragma unroll 1
  for (int it = 0; it < 4; ++it) {
    const int rr = it * 8 + (lane >> 2);
    const int m = m_base + rr;
    float a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = stg[rr * 33 + cc + k];
    if (e.mode == EPI_STORE) {
      float* D = e.D + (size_t)kslice * e.d_slice;  // K slice (0 unless split)
      if (m < M) store8(D + (size_t)m * e.ldd + n, n, N, full && aligned16(D, e.ldd), a);
    } else if (e.mode == EPI_SIGMOID) {
      float yv[8], lam[8], lp[8], r1[8];
      load8(e.y + n, n, N, full && aligned16(e.y, 0), yv);
      double ld = 0.0;
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const Sig sg = sig_pair(a[k]);
        lam[k] = sg.sp * sg.sm;
        lp[k] = lam[k] * (sg.sm - sg.sp);
        r1[k] = yv[k] * sg.sm - (1.f - yv[k]) * sg.sp;  // y − σ(a)
        if (e.ld_acc && n + k < N) ld += double(yv[k] * a[k] - sig_softplus(a[k], sg));
      }
      if (m < M) {
        split8(e.lam, m, n, N, full, lam);
        if (!e.lam_only) {
          store8(e.lp + (size_t)m * e.lp_ld + n, n, N, full && aligned16(e.lp, e.lp_ld), lp);
          split8(e.r, m, n, N, full, r1);
        }
      }
      if (e.ld_acc) {  // the 4 lanes of a row, then one atomic per row and chunk
        ld += __shfl_xor_sync(0xffffffffu, ld, 1);
        ld += __shfl_xor_sync(0xffffffffu, ld, 2);
        if ((lane & 3) == 0 && m < M) atomicAdd(&e.ld_acc[m], ld);
      }
    } else if (e.mode == EPI_R2W) {  // a = s: r2 = Λ'(w − s²) with w stored
      if (m < M) {
        float wv[8], lv[8], r2[8];
        load8(e.W + (size_t)m * e.s_ld + n, n, N, full && aligned16(e.W, e.s_ld), wv);
        load8(e.lp + (size_t)m * e.lp_ld + n, n, N, full && aligned16(e.lp, e.lp_ld), lv);
#pragma unroll
        for (int k = 0; k < 8; ++k) r2[k] = lv[k] * (wv[k] - a[k] * a[k]);
        split8(e.r, e.r_off + m, n, N, full, r2);
      }
    } else {  // EPI_TRACE: r2 = Λ'(w − s²)
      if (m < M) {
        if (e.w_out) store8(e.w_out + (size_t)m * e.s_ld + n, n, N, full && aligned16(e.w_out, e.s_ld), a);
        float sv[8], lv[8], r2[8];
        load8(e.S + (size_t)m * e.s_ld + n, n, N, full && aligned16(e.S, e.s_ld), sv);
        load8(e.lp + (size_t)m * e.lp_ld + n, n, N, full && aligned16(e.lp, e.lp_ld), lv);
#pragma unroll
        for (int k = 0; k < 8; ++k) r2[k] = lv[k] * (a[k] - sv[k] * sv[k]);
        split8(e.r, e.r_off + m, n, N, full, r2);
      }
    }
  }
  __syncwarp();  // the tile is reused by the warp's next chunk
}

// One 32-column chunk of the accumulator for this warp's lane quarter (lane
// l = row 32·q + l), the NACC K-range partial tiles added in order.
__device__ __forceinline__ void load_acc(uint32_t tmem, int q, int c0, int nacc, int tmem_cols,
                                         float (&v)[32]) {
  const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0;
  {
    uint32_t r[32];
    tmem_ld32(ta, r);
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
  }
  // the other K ranges' partial tiles, added in order (round to nearest)
#pragma unroll 1
  for (int acc = 1; acc < nacc; ++acc) {
    uint32_t r[32];
    tmem_ld32(ta + (uint32_t)(acc * tmem_cols), r);
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] += __uint_as_float(r[j]);
  }
}

// EPI_R2G layout in the operand ring, free once the S accumulator is
// complete: the r2 tile of one 64-wide K half as three BF16 planes
// (128 rows x 64, 16 KB each, 128B-swizzled K-major like a TMA-loaded A
// box), then the six Xᵀ boxes (two K halves x three planes, 32 rows x 64).
constexpr int R2G_A_BYTES = 3 * A_TILE_BYTES;
constexpr int R2G_XT_BOX = 32 * BK * 2;
constexpr int R2G_SMEM = R2G_A_BYTES + 6 * R2G_XT_BOX;
constexpr uint32_t R2G_TMEM_COL = 128;  // the gradient accumulator's columns
constexpr uint32_t R2G_TMEM_ALLOC = 256;
constexpr uint32_t R2G_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((32u >> 3) << 17) |
                               ((uint32_t)(BM >> 4) << 24);  // M = 128, N = 32

// EPI_R2G, one epilogue warp (see Epi; BN = 128, 3 planes, one K block).
// For each 64-wide K half of the tile: lane l (tile row 32·q + l) forms
// r2 = Λ'(w − s²) over this warp's 32 columns of that half, splits it into
// three BF16 planes and stores them swizzled into the A tile; after a
// named barrier of the 256 epilogue threads one thread issues the plane
// products r2_i · Xᵀ_j (i + j <= 2) as tcgen05 MMAs, M = 128, N = 32,
// K = 64, into the TMEM columns after S's.  The second half waits for the
// first half's MMAs before overwriting the A tile.  Every epilogue thread
// reaches both barriers and all waits whatever the outcome of its own
// waits, and every wait is bounded.
__device__ __forceinline__ void epi_r2g(const Epi& e, unsigned char* base, uint64_t* xfull,
                                        uint64_t* gdone, uint32_t tmem, int warp, int lane,
                                        bool ok, int m0, int n0, int M, int N, int* err,
                                        int ntile) {
  const int q = warp & 3, half = (warp - 2) >> 2;
  const int row = q * 32 + lane;  // tile row of this lane
  const int m = m0 + row;
  unsigned char* At = base;
  const uint32_t a_s = smem_u32(At), x_s = smem_u32(base + R2G_A_BYTES);
#pragma unroll 1
  for (int kh = 0; kh < 2; ++kh) {
    const int c0 = 64 * kh + 32 * half;  // this warp's 32 columns
    if (kh == 1 && !mbar_wait(gdone, 0) && lane == 0) atomicExch(err, 5);
    float r2[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) r2[j] = 0.f;
    if (ok && n0 + c0 < N) {  // warp-uniform
      float sv[32];
      {
        uint32_t r[32];
        tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0, r);
#pragma unroll
        for (int j = 0; j < 32; ++j) sv[j] = __uint_as_float(r[j]);
      }
      if (m < M) {
        const int n = n0 + c0;
        const bool full = n + 32 <= N;
#pragma unroll
        for (int j8 = 0; j8 < 4; ++j8) {
          float wv[8], lv[8];
          const int nj = n + 8 * j8;
          load8(e.W + (size_t)m * e.s_ld + nj, nj, N, full && aligned16(e.W, e.s_ld), wv);
          load8(e.lp + (size_t)m * e.lp_ld + nj, nj, N, full && aligned16(e.lp, e.lp_ld), lv);
#pragma unroll
          for (int k = 0; k < 8; ++k) {
            const float s = sv[8 * j8 + k];
            r2[8 * j8 + k] = lv[k] * (wv[k] - s * s);
          }
        }
      }
    }
    // three planes, one 16-byte chunk (8 columns) per plane and store; the
    // 128B swizzle puts chunk c of row r at chunk c ^ (r mod 8)
#pragma unroll
    for (int j8 = 0; j8 < 4; ++j8) {
      uint32_t w0[4], w1[4], w2[4];
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const float xa = r2[8 * j8 + 2 * t], xb = r2[8 * j8 + 2 * t + 1];
        const __nv_bfloat162 h = __floats2bfloat162_rn(xa, xb);
        const float2 hf = __bfloat1622float2(h);
        const float ra = xa - hf.x, rb = xb - hf.y;
        const __nv_bfloat162 md = __floats2bfloat162_rn(ra, rb);
        const float2 mf = __bfloat1622float2(md);
        const __nv_bfloat162 lo = __floats2bfloat162_rn(ra - mf.x, rb - mf.y);
        w0[t] = *reinterpret_cast<const uint32_t*>(&h);
        w1[t] = *reinterpret_cast<const uint32_t*>(&md);
        w2[t] = *reinterpret_cast<const uint32_t*>(&lo);
      }
      const int chunk = (4 * half + j8) ^ (row & 7);
      unsigned char* p = At + row * 128 + chunk * 16;
      *reinterpret_cast<uint4*>(p) = make_uint4(w0[0], w0[1], w0[2], w0[3]);
      *reinterpret_cast<uint4*>(p + A_TILE_BYTES) = make_uint4(w1[0], w1[1], w1[2], w1[3]);
      *reinterpret_cast<uint4*>(p + 2 * A_TILE_BYTES) = make_uint4(w2[0], w2[1], w2[2], w2[3]);
    }
    // the tensor core reads shared memory through the async proxy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("bar.sync 1, 256;" ::: "memory");
    if (warp == 2 && lane == 0) {
      bool go = ok;
      if (kh == 0 && !mbar_wait(xfull, 0)) {
        atomicExch(err, 6);
        go = false;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (go) {
#pragma unroll
        for (int k = 0; k < BK / 16; ++k) {
          const uint64_t adv = (uint64_t)((k * 32) >> 4);
          uint64_t da[3], db[3];
#pragma unroll
          for (int p = 0; p < 3; ++p) {
            da[p] = make_desc(a_s + p * A_TILE_BYTES) + adv;
            db[p] = make_desc(x_s + (kh * 3 + p) * R2G_XT_BOX) + adv;
          }
          const uint32_t acc_t = tmem + R2G_TMEM_COL;
          mma_bf16(acc_t, da[0], db[0], R2G_IDESC, (kh > 0 || k > 0) ? 1u : 0u);
          mma_bf16(acc_t, da[0], db[1], R2G_IDESC, 1u);
          mma_bf16(acc_t, da[1], db[0], R2G_IDESC, 1u);
          mma_bf16(acc_t, da[0], db[2], R2G_IDESC, 1u);
          mma_bf16(acc_t, da[1], db[1], R2G_IDESC, 1u);
          mma_bf16(acc_t, da[2], db[0], R2G_IDESC, 1u);
        }
      }
      mma_commit(gdone);  // arrives also when nothing was issued
    }
    __syncwarp();
  }
  const bool done = __all_sync(0xffffffffu, mbar_wait(gdone, 1));
  if (!done && lane == 0) atomicExch(err, 7);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  uint32_t r[32];
  tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + R2G_TMEM_COL, r);
  if (ok && done && m < M) {  // the row's partial gradient for this N tile
    float* out = e.g2 + (size_t)ntile * e.g2_slice + (size_t)m * e.g2_ld;
    const int k4n = (e.x_d + 3) >> 2;
#pragma unroll
    for (int k4 = 0; k4 < 8; ++k4)
      if (k4 < k4n)
        reinterpret_cast<float4*>(out)[k4] =
            make_float4(__uint_as_float(r[4 * k4]), __uint_as_float(r[4 * k4 + 1]),
                        __uint_as_float(r[4 * k4 + 2]), __uint_as_float(r[4 * k4 + 3]));
  }
}

// STAGES (run time, 1 .. Cfg::MAX_STAGES) is the depth of the operand ring,
// chosen by the host so that two CTAs share an SM where that fits.
// NACC (run time, 1, 2 or 4) accumulators over contiguous K ranges; the
// host keeps NACC·TMEM_COLS·(CTAs per SM) within the SM's 512 columns.
// The CTA's work as a device function: block (bx, by, bz) of a grid with gz
// K slices, tensor maps by address (kernel parameters of gemm_tc_kernel, or
// the items of a grouped launch in global memory).
template <int NPL, int BN, bool R2G>  // R2G: the EPI_R2G epilogue
__device__ __forceinline__ void gemm_tc_body(const CUtensorMap* mapA, const CUtensorMap* mapB,
                                             const CUtensorMap* mapXT, int rpadA, int rpadB, int M,
                                             int N, int K, const Epi& epi, int* err, int STAGES,
                                             int a_row0, int NACC, int bx, int by, int bz, int gz,
                                             bool maps_in_global) {
  using C = Cfg<NPL, BN>;
  constexpr int STAGE_BYTES = C::STAGE_BYTES;
  constexpr int TMEM_COLS = C::TMEM_COLS;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // 1024-byte aligned tile ring (required by the 128B swizzle), then barriers
  unsigned char* base = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(base + STAGES * STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* accum = empty + STAGES;
  uint64_t* xfull = accum + 1;  // EPI_R2G: the Xᵀ boxes have landed
  uint64_t* gdone = accum + 2;  // EPI_R2G: a K half's gradient MMAs are complete
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(accum + 3);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = by * BM, n0 = bx * BN;
  // this CTA's contiguous range of K blocks (the whole K unless split)
  const int KB_all = (K + BK - 1) / BK;
  const int kper = (KB_all + gz - 1) / gz;
  const int kb_first = bz * kper;
  const int KB = max(0, min(KB_all, kb_first + kper) - kb_first);
  // a K slice with fewer K blocks than accumulators uses one per block, so
  // that no range is empty
  const int nacc = max(1, min(NACC, KB));

  if (warp == 0 && lane == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(accum, 1);
    mbar_init(xfull, 1);
    mbar_init(gdone, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // EPI_R2G adds 32 gradient columns after S's 128 (one accumulator)
  const uint32_t tmem_cols = R2G ? R2G_TMEM_ALLOC : (uint32_t)(TMEM_COLS * NACC);
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(tmem_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  // barriers and TMEM are set up; the operands and epilogue inputs come from
  // the preceding kernels
  pdl_wait();
  // a tile whose chains have all converged is skipped (whole CTA)
  bool work = true;
  if (epi.active_rows) {
    bool any = false;
    for (int r = (int)threadIdx.x; r < BM; r += (int)blockDim.x)
      any |= (m0 + r < M) && epi.active_rows[m0 + r] != 0;
    work = __syncthreads_or(any) != 0;
  }

  if (!work) {
    // nothing issued, nothing to wait for
  } else if (warp == 0) {
    if (lane == 0) {
      if (maps_in_global) {
        tensormap_acquire(mapA);
        tensormap_acquire(mapB);
        if (R2G) tensormap_acquire(mapXT);
      }
      for (int kb = 0; kb < KB; ++kb) {
        const int s = kb % STAGES;
        const uint32_t ph = (kb / STAGES) & 1;
        if (!mbar_wait(&empty[s], ph ^ 1)) {
          atomicExch(err, 1);
          break;
        }
        unsigned char* st = base + s * STAGE_BYTES;
        mbar_expect_tx(&full[s], STAGE_BYTES);
        const int x = (kb_first + kb) * BK;
#pragma unroll
        for (int q = 0; q < NPL; ++q) {
          tma_load_2d(st + q * A_TILE_BYTES, mapA, &full[s], x, q * rpadA + a_row0 + m0);
          tma_load_2d(st + NPL * A_TILE_BYTES + q * C::B_TILE_BYTES, mapB, &full[s], x,
                      q * rpadB + n0);
        }
      }
      if constexpr (R2G) {  // the Xᵀ boxes of the tile's two K halves, into
        // the ring once the S accumulator (its last reader) is complete
        if (mbar_wait(accum, 0)) {
          mbar_expect_tx(xfull, 6 * R2G_XT_BOX);
          for (int kh = 0; kh < 2; ++kh)
            for (int q = 0; q < 3; ++q)
              tma_load_2d(base + R2G_A_BYTES + (kh * 3 + q) * R2G_XT_BOX, mapXT, xfull,
                          n0 + 64 * kh, q * epi.xt_rpad);
        } else {
          atomicExch(err, 4);
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      bool ok = true;
      for (int kb = 0; kb < KB && ok; ++kb) {
        const int s = kb % STAGES;
        const uint32_t ph = (kb / STAGES) & 1;
        if (!mbar_wait(&full[s], ph)) {
          atomicExch(err, 2);
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t sa = smem_u32(base + s * STAGE_BYTES);
        uint64_t da[NPL], db[NPL];
#pragma unroll
        for (int q = 0; q < NPL; ++q) {
          da[q] = make_desc(sa + q * A_TILE_BYTES);
          db[q] = make_desc(sa + NPL * A_TILE_BYTES + q * C::B_TILE_BYTES);
        }
        constexpr uint32_t ID = (uint32_t)C::IDESC;
        // K range r = ⌊kb·nacc/KB⌋ accumulates into columns [r·TMEM_COLS, ..)
        const int r = (kb * nacc) / KB;
        const bool first = kb == (r * KB + nacc - 1) / nacc;  // the range's first K block
        const uint32_t acc_t = tmem + (uint32_t)(r * TMEM_COLS);
#pragma unroll
        for (int k = 0; k < BK / 16; ++k) {
          const uint64_t adv = (uint64_t)((k * 32) >> 4);  // 16 BF16 = 32 B along K
          // plane products with i + j <= NPL - 1 (the dropped ones are below
          // the last plane's resolution)
          mma_bf16(acc_t, da[0] + adv, db[0] + adv, ID, (!first || k > 0) ? 1u : 0u);
          mma_bf16(acc_t, da[0] + adv, db[1] + adv, ID, 1u);
          mma_bf16(acc_t, da[1] + adv, db[0] + adv, ID, 1u);
          if (NPL == 3) {
            mma_bf16(acc_t, da[0] + adv, db[NPL - 1] + adv, ID, 1u);
            mma_bf16(acc_t, da[1] + adv, db[1] + adv, ID, 1u);
            mma_bf16(acc_t, da[NPL - 1] + adv, db[0] + adv, ID, 1u);
          }
        }
        mma_commit(&empty[s]);
      }
      mma_commit(accum);  // also completes when nothing was issued
    }
  } else {
    // epilogue warps 2..9: TMEM lane quarter = warp % 4; the two warps of a
    // quarter take alternate 32-column chunks
    const int q = warp & 3;
    const int half = (warp - 2) >> 2;
    const bool ok = __all_sync(0xffffffffu, mbar_wait(accum, 0));
    if (!ok && lane == 0) atomicExch(err, 3);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if constexpr (R2G) {  // the host keeps K in one unsplit block (KB = 1)
      epi_r2g(epi, base, xfull, gdone, tmem, warp, lane, ok && KB > 0, m0, n0, M, N, err, bx);
    } else if (ok && KB > 0) {
      // the operand ring is free once the accumulator is complete: each
      // epilogue warp stages its chunks in its own 32 x 33 float tile
      float* stg = reinterpret_cast<float*>(base) + (warp - 2) * (32 * 33);
#pragma unroll 1
      for (int c0 = 32 * half; c0 < BN; c0 += 64) {
        if (n0 + c0 >= N) break;  // warp-uniform
        float v[32];
        load_acc(tmem, q, c0, nacc, TMEM_COLS, v);
        epi_chunk(epi, stg, lane, m0 + q * 32, n0 + c0, M, N, v, bz);
      }
    }
  }
  // the successor may be scheduled once every CTA is this far (its CTAs then
  // fill the SMs of this grid's finishing last wave)
  pdl_trigger();
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(tmem_cols)
                 : "memory");
  }
}

template <int NPL, int BN, bool R2G = false>
__global__ void __launch_bounds__(320, 2)
    gemm_tc_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                   const __grid_constant__ CUtensorMap mapXT, int rpadA, int rpadB, int M, int N,
                   int K, Epi epi, int* err, int STAGES, int a_row0, int NACC) {
  gemm_tc_body<NPL, BN, R2G>(&mapA, &mapB, &mapXT, rpadA, rpadB, M, N, K, epi, err, STAGES, a_row0,
                             NACC, (int)blockIdx.x, (int)blockIdx.y, (int)blockIdx.z,
                             (int)gridDim.z, false);
}

// Grouped launch: many independent contractions of one tile shape in one
// grid, each CTA finding its item (its own operands, tensor maps, epilogue
// and grid) by its block index.
template <int NPL, int BN, bool R2G>
__global__ void __launch_bounds__(320, 2)
    gemm_tc_grouped_kernel(const GemmItem* __restrict__ items, const int* __restrict__ prefix,
                           int n) {
  const int i = group_item(prefix, n, (int)blockIdx.x);
  const GemmItem& it = items[i];
  const int local = (int)blockIdx.x - __ldg(prefix + i);
  const int bx = local % it.gx, by = (local / it.gx) % it.gy, bz = local / (it.gx * it.gy);
  gemm_tc_body<NPL, BN, R2G>(&it.mapA, &it.mapB, &it.mapXT, it.rpadA, it.rpadB, it.M, it.N, it.K,
                             it.epi, it.err, it.stages, it.a_row0, it.nacc, bx, by, bz, it.gz,
                             true);
}

}  // namespace

bool tc_available() {
  int dev = 0, major = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess)
    return false;
  return major == 10 && get_encode() != nullptr;
}

bool tc_operand_init(TcOperand* op, const SplitMat& s, const char** err) {
  EncodeTiledFn enc = get_encode();
  if (!enc) {
    *err = "cuTensorMapEncodeTiled unavailable";
    return false;
  }
  if ((s.ld % 64) || (s.rpad % 128) || (reinterpret_cast<uintptr_t>(s.p) & 15) ||
      (s.planes != 2 && s.planes != 3)) {
    *err = "split matrix not padded for TMA";
    return false;
  }
  op->s = s;
  cuuint64_t dims[2] = {(cuuint64_t)s.ld, (cuuint64_t)s.planes * s.rpad};
  cuuint64_t strides[1] = {(cuuint64_t)s.ld * 2};
  cuuint32_t estr[2] = {1u, 1u};
  // boxes of 64 K-elements by 128, 64 and 32 rows (A tiles and the B tiles
  // of the three tile widths)
  CUtensorMap* maps[3] = {&op->map, &op->map64, &op->map32};
  const cuuint32_t rows[3] = {128u, 64u, 32u};
  for (int i = 0; i < 3; ++i) {
    cuuint32_t box[2] = {(cuuint32_t)BK, rows[i]};
    CUresult r = enc(maps[i], CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, s.p, dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
      *err = "cuTensorMapEncodeTiled failed";
      return false;
    }
  }
  return true;
}

TcOperand* tc_operand_create(const SplitMat& s, int, const char** err) {
  TcOperand* op = new TcOperand();
  if (!tc_operand_init(op, s, err)) {
    delete op;
    return nullptr;
  }
  return op;
}

void tc_operand_destroy(TcOperand* op) { delete op; }

namespace {

template <int NPL, int BN>
cudaError_t set_smem_limit() {
  const int bytes = Cfg<NPL, BN>::smem(Cfg<NPL, BN>::MAX_STAGES);
  cudaError_t e = cudaFuncSetAttribute(gemm_tc_kernel<NPL, BN, false>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(gemm_tc_grouped_kernel<NPL, BN, false>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if constexpr (NPL == 3 && BN == 128)
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(gemm_tc_grouped_kernel<NPL, BN, true>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if constexpr (NPL == 3 && BN == 128)  // the fused r2·X form (launched with these only)
    if (e == cudaSuccess) e = cudaFuncSetAttribute(gemm_tc_kernel<NPL, BN, true>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  return e;
}

}  // namespace

cudaError_t gemm_tc_prepare() {
  cudaError_t e = cudaSuccess;
  const cudaError_t r[6] = {set_smem_limit<2, 32>(), set_smem_limit<2, 64>(),
                            set_smem_limit<2, 128>(), set_smem_limit<3, 32>(),
                            set_smem_limit<3, 64>(), set_smem_limit<3, 128>()};
  for (cudaError_t x : r)
    if (x != cudaSuccess) e = x;
  return e;
}

namespace {

// Tile and pipeline choice (automatic unless forced by gemm_tc_set_tuning):
// * BN: the narrowest of 32 / 64 covering N; for N > 64, 64 for a two-plane
//   GEMM with at most 8 K blocks (more CTAs, two per SM), else 128;
// * stages: with 8 or more K blocks a 3-stage ring (one CTA per SM keeps
//   the TMA pipeline full); with fewer, as many as the K blocks need, cut
//   back towards the shared memory that lets two CTAs share an SM but never
//   below two stages when there are several K blocks.
// Measured per GEMM at N = 1000, d = 25, 4096 chains (µs, ncu launch list):
// trace (2 planes, 6 K blocks) 31.9 → 27.7 with BN = 64; Gram (2 planes,
// 16 K blocks) 18.4 → 16.7 and gradient (3 planes, 16 K blocks) 21.9 → 20.7
// with the 3-stage ring; Xβ and S (1 K block) best at BN = 128.
struct TcTuning {
  int bn_wide = 0;         // tile width for N > 64: 0 = automatic, 64 or 128
  int two_ctas = -1;       // -1 = automatic, 1 = prefer two CTAs per SM, 0 = deep ring
  int max_nacc = 4;        // most K-range accumulators per CTA: 1, 2 or 4
};
TcTuning g_tune;

constexpr int kTwoCtaSmem = 113 * 1024;

constexpr int variant_of(int npl, int bn, bool r2g) {
  return (npl - 2) * 6 + (bn == 32 ? 0 : (bn == 64 ? 1 : 2)) * 2 + (r2g ? 1 : 0);
}

// The launch parameters of one contraction with this tile shape.
template <int NPL, int BN>
cudaError_t plan_tc(const GemmArgs& g, const TcOperand* a, const TcOperand* b, int* err,
                    GemmItem* it, int* variant, size_t* smem) {
  using C = Cfg<NPL, BN>;
  const int kb = (g.K + BK - 1) / BK;
  int ns = std::max(1, std::min(C::MAX_STAGES, kb));
  const bool two = g_tune.two_ctas < 0 ? kb < 8 : g_tune.two_ctas != 0;
  if (two)  // keep two stages when there is more than one K block
    while (ns > 2 && C::smem(ns) > kTwoCtaSmem) --ns;
  else
    ns = std::min(ns, 3);
  const CUtensorMap& mb = BN == 128 ? b->map : (BN == 64 ? b->map64 : b->map32);
  // K-range accumulators: up to 4, at least 2 K blocks each, and within the
  // 512 TMEM columns of an SM for the CTAs that share it
  const int kb_cta = (kb + g.ksplit - 1) / g.ksplit;
  const int ctas = C::smem(ns) <= kTwoCtaSmem ? 2 : 1;
  int nacc = 1;
  while (nacc < g_tune.max_nacc && 2 * nacc * 2 <= kb_cta && 2 * nacc * C::TMEM_COLS * ctas <= 512)
    nacc *= 2;
  const bool r2g = g.epi.mode == EPI_R2G;
  it->mapA = a->map;
  it->mapB = mb;
  it->mapXT = mb;
  if (r2g) {
    // three planes, 128-wide tiles, one K block (one accumulator) and a
    // ring that holds the r2 tile and the Xᵀ boxes
    const TcOperand* xt = g.epi.xt;
    if (NPL != 3 || BN != 128 || kb != 1 || ns * C::STAGE_BYTES < R2G_SMEM || !xt ||
        xt->s.planes != 3 || xt->s.rows > 32 || g.epi.xt_rpad != xt->s.rpad)
      return cudaErrorInvalidValue;
    it->mapXT = xt->map32;
    nacc = 1;
  }
  it->epi = g.epi;
  it->err = err;
  it->rpadA = a->s.rpad;
  it->rpadB = b->s.rpad;
  it->M = g.M;
  it->N = g.N;
  it->K = g.K;
  it->stages = ns;
  it->a_row0 = g.a_row0;
  it->nacc = nacc;
  it->gx = (g.N + BN - 1) / BN;
  it->gy = (g.M + BM - 1) / BM;
  it->gz = g.ksplit;
  *variant = variant_of(NPL, BN, r2g);
  *smem = (size_t)C::smem(ns);
  return cudaSuccess;
}

template <int NPL, int BN>
cudaError_t launch_tc(const GemmArgs& g, const TcOperand* a, const TcOperand* b, int* err,
                      cudaStream_t st) {
  GemmItem it;
  int variant = 0;
  size_t smem = 0;
  const cudaError_t e = plan_tc<NPL, BN>(g, a, b, err, &it, &variant, &smem);
  if (e != cudaSuccess) return e;
  const dim3 grid(it.gx, it.gy, it.gz);
  if (g.epi.mode == EPI_R2G) {
    if constexpr (NPL == 3 && BN == 128)
      return launch_k(g.pdl, gemm_tc_kernel<NPL, BN, true>, grid, dim3(320), smem, st, it.mapA,
                      it.mapB, it.mapXT, it.rpadA, it.rpadB, g.M, g.N, g.K, g.epi, err, it.stages,
                      g.a_row0, 1);
    return cudaErrorInvalidValue;
  }
  return launch_k(g.pdl, gemm_tc_kernel<NPL, BN, false>, grid, dim3(320), smem, st, it.mapA,
                  it.mapB, it.mapB, it.rpadA, it.rpadB, g.M, g.N, g.K, g.epi, err, it.stages,
                  g.a_row0, it.nacc);
}

int tile_bn(int planes, int N, int K) {
  if (N <= 32) return 32;
  const int kb = (K + BK - 1) / BK;
  const bool narrow = g_tune.bn_wide == 0 ? (planes == 2 && kb <= 8) : g_tune.bn_wide == 64;
  return (N <= 64 || narrow) ? 64 : 128;
}

template <int NPL>
cudaError_t launch_tc_planes(const GemmArgs& g, const TcOperand* a, const TcOperand* b, int* err,
                             cudaStream_t st) {
  const int bn = tile_bn(NPL, g.N, g.K);
  if (bn == 32) return launch_tc<NPL, 32>(g, a, b, err, st);
  if (bn == 64) return launch_tc<NPL, 64>(g, a, b, err, st);
  return launch_tc<NPL, 128>(g, a, b, err, st);
}

template <int NPL>
cudaError_t plan_tc_planes(const GemmArgs& g, const TcOperand* a, const TcOperand* b, int* err,
                           GemmItem* it, int* variant, size_t* smem) {
  const int bn = tile_bn(NPL, g.N, g.K);
  if (bn == 32) return plan_tc<NPL, 32>(g, a, b, err, it, variant, smem);
  if (bn == 64) return plan_tc<NPL, 64>(g, a, b, err, it, variant, smem);
  return plan_tc<NPL, 128>(g, a, b, err, it, variant, smem);
}

}  // namespace

int gemm_tc_bn(int planes, int N, int K) { return tile_bn(planes, N, K); }

int gemm_tc_tuning_code() {
  return (g_tune.bn_wide / 64) * 3 + (g_tune.two_ctas + 1) + 16 * g_tune.max_nacc;
}

void gemm_tc_set_accumulators(int max_ranges) {
  g_tune.max_nacc = (max_ranges == 1 || max_ranges == 2) ? max_ranges : 4;
}

void gemm_tc_set_tuning(int bn_wide, int two_ctas) {
  g_tune.bn_wide = (bn_wide == 64 || bn_wide == 128) ? bn_wide : 0;
  g_tune.two_ctas = two_ctas < 0 ? -1 : (two_ctas ? 1 : 0);
}

namespace {

cudaError_t check_tc(const GemmArgs& g, const TcOperand* a, const TcOperand* b) {
  // every box must lie inside the padded planes
  if (g.a_row0 < 0 || g.a_row0 + g.M > a->s.rpad || g.N > b->s.rpad || g.K > a->s.ld ||
      g.K > b->s.ld || a->s.planes != b->s.planes)
    return cudaErrorInvalidValue;
  if (g.ksplit != 1 && (g.epi.mode != EPI_STORE || !gemm_ksplit_valid(g.K, g.ksplit) ||
                        (g.epi.d_slice & 3)))
    return cudaErrorInvalidValue;
  if (g.epi.mode == EPI_R2G &&
      (g.epi.x_d < 1 || g.epi.x_d > 32 || g.epi.g2_ld < 4 * ((g.epi.x_d + 3) / 4) ||
       (g.epi.g2_ld & 3) || (g.epi.g2_slice & 3) || !g.epi.g2 ||
       (reinterpret_cast<uintptr_t>(g.epi.g2) & 15) || g.ksplit != 1 || g.a_row0 != 0))
    return cudaErrorInvalidValue;
  return cudaSuccess;
}

}  // namespace

cudaError_t gemm_tc(const GemmArgs& g, const TcOperand* a, const TcOperand* b, int* err,
                    cudaStream_t st) {
  if (g.M <= 0 || g.N <= 0) return cudaSuccess;
  const cudaError_t e = check_tc(g, a, b);
  if (e != cudaSuccess) return e;
  return a->s.planes == 3 ? launch_tc_planes<3>(g, a, b, err, st)
                          : launch_tc_planes<2>(g, a, b, err, st);
}

cudaError_t gemm_tc_describe(const GemmArgs& g, const TcOperand* a, const TcOperand* b, int* err,
                             GemmItem* item, int* variant, int* blocks, size_t* smem) {
  if (g.M <= 0 || g.N <= 0) return cudaErrorInvalidValue;
  if (g.pdl) return cudaErrorInvalidValue;  // grouped launches are plain stream order
  cudaError_t e = check_tc(g, a, b);
  if (e != cudaSuccess) return e;
  e = a->s.planes == 3 ? plan_tc_planes<3>(g, a, b, err, item, variant, smem)
                       : plan_tc_planes<2>(g, a, b, err, item, variant, smem);
  if (e == cudaSuccess) *blocks = item->gx * item->gy * item->gz;
  return e;
}

cudaError_t gemm_tc_grouped(int variant, const GemmItem* items, const int* prefix, int n, int blocks,
                            size_t smem, cudaStream_t st) {
  if (n < 1 || blocks < 1) return cudaErrorInvalidValue;
  const dim3 grid((unsigned)blocks), th(320);
  switch (variant) {
    case variant_of(2, 32, false): gemm_tc_grouped_kernel<2, 32, false><<<grid, th, smem, st>>>(items, prefix, n); break;
    case variant_of(2, 64, false): gemm_tc_grouped_kernel<2, 64, false><<<grid, th, smem, st>>>(items, prefix, n); break;
    case variant_of(2, 128, false): gemm_tc_grouped_kernel<2, 128, false><<<grid, th, smem, st>>>(items, prefix, n); break;
    case variant_of(3, 32, false): gemm_tc_grouped_kernel<3, 32, false><<<grid, th, smem, st>>>(items, prefix, n); break;
    case variant_of(3, 64, false): gemm_tc_grouped_kernel<3, 64, false><<<grid, th, smem, st>>>(items, prefix, n); break;
    case variant_of(3, 128, false): gemm_tc_grouped_kernel<3, 128, false><<<grid, th, smem, st>>>(items, prefix, n); break;
    case variant_of(3, 128, true): gemm_tc_grouped_kernel<3, 128, true><<<grid, th, smem, st>>>(items, prefix, n); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace gj
