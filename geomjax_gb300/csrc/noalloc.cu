// The split-BF16 contraction D = A·Bᵀ without any device allocation.
//
// gj_gemm_split_bf16 (capi.cu) allocates its split-plane scratch with
// cudaMalloc on every call.  Some callers cannot do that: a kernel embedded in
// an XLA custom call runs while the framework's allocator owns nearly all
// device memory (a stray cudaMalloc can fail, or fragment the pool it
// reserved).  This file serves them from one file-scope device array that
// every GPU loading the library holds until the process exits.
//
// The array is shared by every call: overlapping calls on the GPU (two
// streams, or two host threads) race on it and must be serialised by the
// caller.  Each call rewrites every element it reads (the split kernel also
// writes the zero padding that the TMA boxes read, and the error word in the
// header is cleared first), so a call never sees the previous call's contents.
#include <atomic>
#include <mutex>
#include <string>

#include "gemm.cuh"

namespace gj {

namespace {

// 8 MiB of BF16 planes plus a 256-byte header holding the kernel's error flag
constexpr size_t kHeaderElems = 128;                 // 256 bytes
constexpr size_t kScratchElems = size_t(4) << 20;    // 4,194,304 BF16 elements
static __device__ __align__(256) bf16 g_scratch[kHeaderElems + kScratchElems];

// Largest M, N or K accepted before any rounding (the capacity check below
// rejects far smaller problems anyway; this bound keeps the rounding in range).
constexpr int kMaxDim = 1 << 24;

constexpr int kMaxDevices = 64;
// device address of g_scratch, per device; written once under g_setup_mu
std::atomic<bf16*> g_base[kMaxDevices];
std::mutex g_setup_mu;
thread_local std::string g_err;

inline int roundup(int x, int m) { return (x + m - 1) / m * m; }

// Split a row-major [R, K] float matrix into the planes of S, writing every
// element of the padded planes (zero outside R x K).
__global__ void split_padded_kernel(const float* X, int R, int K, SplitMat S) {
  const size_t total = (size_t)S.rpad * S.ld;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / S.ld), k = (int)(i % S.ld);
    if (r < R && k < K) {
      split_store(S, r, k, X[(size_t)r * K + k]);
    } else {
      for (int q = 0; q < S.planes; ++q) S.p[(size_t)(q * S.rpad + r) * S.ld + k] = bf16(0.f);
    }
  }
}

// Once per device, with that device current: the device address of the
// array (host code cannot use the symbol itself).
int setup(int* dev_out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    g_err = std::string("cudaGetDevice: ") + cudaGetErrorString(e);
    return GJ_ECUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    g_err = "device index beyond the no-allocation entry point's table";
    return GJ_ENOTSUP;
  }
  if (!g_base[dev].load(std::memory_order_acquire)) {
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_base[dev].load(std::memory_order_relaxed)) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_scratch);
      if (e != cudaSuccess || !p) {
        g_err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
        return GJ_ECUDA;
      }
      g_base[dev].store(static_cast<bf16*>(p), std::memory_order_release);
    }
  }
  *dev_out = dev;
  return GJ_OK;
}

}  // namespace

const char* gemm_noalloc_error() { return g_err.c_str(); }

size_t gemm_noalloc_capacity() { return kScratchElems; }

int gemm_split_noalloc(int impl, int planes, int M, int N, int K, const float* A, const float* B,
                       float* D, cudaStream_t st) {
  if (M < 1 || N < 1 || K < 1 || !A || !B || !D || (planes != 2 && planes != 3) ||
      (impl != 1 && impl != 2)) {
    g_err = "bad arguments (impl 1 or 2, planes 2 or 3, positive sizes, device arrays)";
    return GJ_EINVAL;
  }
  if (M > kMaxDim || N > kMaxDim || K > kMaxDim) {
    g_err = "problem exceeds the no-allocation scratch: planes * (ceil128(M) + ceil128(N)) * "
            "ceil64(K) must be <= 4194304";
    return GJ_EINVAL;
  }
  const int ld = roundup(K, 64);
  const size_t a_elems = (size_t)planes * roundup(M, 128) * ld;
  const size_t b_elems = (size_t)planes * roundup(N, 128) * ld;
  if (a_elems + b_elems > kScratchElems) {
    g_err = "problem exceeds the no-allocation scratch: planes * (ceil128(M) + ceil128(N)) * "
            "ceil64(K) must be <= 4194304";
    return GJ_EINVAL;
  }
  int dev = 0;
  int rc = setup(&dev);
  if (rc) return rc;
  // the tcgen05 operands are checked before anything is enqueued, so a
  // refused call leaves the stream untouched
  TcOperand ta, tb;
  bf16* base = g_base[dev].load(std::memory_order_acquire);
  int* err = reinterpret_cast<int*>(base);  // header
  SplitMat a{base + kHeaderElems, M, K, ld, roundup(M, 128), planes};
  SplitMat b{a.p + a_elems, N, K, ld, roundup(N, 128), planes};
  if (impl == 2) {
    const char* msg = "tcgen05 unavailable";
    if (!tc_available() || gemm_tc_prepare() != cudaSuccess || !tc_operand_init(&ta, a, &msg) ||
        !tc_operand_init(&tb, b, &msg)) {
      g_err = msg;
      return GJ_ENOTSUP;
    }
  }
  cudaError_t e = cudaMemsetAsync(err, 0, sizeof(int), st);
  if (e == cudaSuccess) {
    split_padded_kernel<<<304, 256, 0, st>>>(A, M, K, a);
    split_padded_kernel<<<304, 256, 0, st>>>(B, N, K, b);
    e = cudaGetLastError();
  }
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
  if (e == cudaSuccess) {
    if (impl == 2) {
      e = gemm_tc(g, &ta, &tb, err, st);
    } else {
      e = gemm_simt(g, st);
    }
  }
  int herr = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    g_err = std::string("no-allocation GEMM: ") + cudaGetErrorString(e);
    return GJ_ECUDA;
  }
  if (herr) {
    g_err = "tcgen05 GEMM wait timed out (code " + std::to_string(herr) + ")";
    return GJ_ECUDA;
  }
  return GJ_OK;
}

}  // namespace gj
