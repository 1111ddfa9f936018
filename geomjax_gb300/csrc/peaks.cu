// CUDA-core FMA throughput of this device (FP32 and FP64), the denominators
// of the rooflines of the kernels that run on those pipes: the metric
// factorisation (FP64) and the warp-per-chain Monge kernel (FP32).  The
// measured-peaks file of the pool holds only HBM bandwidth and BF16 tensor
// rates.
//
// Every thread runs 8 independent FMA chains x ← x·y + z for `iters`
// iterations (8 chains cover the pipe latency at the occupancy used), and
// stores its sum so nothing is eliminated.  Timed with CUDA events on the
// given stream after one untimed launch.
#include <cuda_runtime.h>

#include "common.cuh"

namespace gj {

namespace {

template <typename T>
__global__ void __launch_bounds__(256) fma_peak_kernel(T* out, int iters, T y, T z) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  T x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = T(tid & 7) * T(0.125) + T(k);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fma(x[k], y, z);
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  out[tid] = s;
}

template <typename T>
cudaError_t run(int blocks, int iters, T* out, cudaStream_t st, float* ms) {
  cudaEvent_t e0, e1;
  cudaError_t e = cudaEventCreate(&e0);
  if (e != cudaSuccess) return e;
  e = cudaEventCreate(&e1);
  if (e != cudaSuccess) {
    cudaEventDestroy(e0);
    return e;
  }
  // y slightly below 1 keeps the chains bounded for any iteration count
  fma_peak_kernel<T><<<blocks, 256, 0, st>>>(out, iters, T(0.999999), T(1e-3));
  cudaEventRecord(e0, st);
  fma_peak_kernel<T><<<blocks, 256, 0, st>>>(out, iters, T(0.999999), T(1e-3));
  cudaEventRecord(e1, st);
  e = cudaEventSynchronize(e1);
  if (e == cudaSuccess) e = cudaEventElapsedTime(ms, e0, e1);
  if (e == cudaSuccess) e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return e;
}

}  // namespace

cudaError_t fma_peak(int fp64, double* tflops, cudaStream_t st) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const int blocks = sms * 8;  // 2048 threads per SM
  const int iters = fp64 ? 1 << 11 : 1 << 15;
  void* out = nullptr;
  e = cudaMalloc(&out, (size_t)blocks * 256 * sizeof(double));
  if (e != cudaSuccess) return e;
  float ms = 0.f;
  e = fp64 ? run<double>(blocks, iters, static_cast<double*>(out), st, &ms)
           : run<float>(blocks, iters, static_cast<float*>(out), st, &ms);
  cudaFree(out);
  if (e != cudaSuccess) return e;
  const double flops = 2.0 * 8.0 * iters * (double)blocks * 256.0;
  *tflops = ms > 0.f ? flops / (ms * 1e-3) / 1e12 : 0.0;
  return cudaSuccess;
}

}  // namespace gj
