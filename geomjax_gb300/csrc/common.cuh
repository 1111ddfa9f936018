// Shared device/host helpers for the geomjax_gb300 kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/geomjax_gb300.h"

namespace gj {

constexpr double kLog2Pi = 1.8378770664093454835606594728112;

// Device-side view of a gj_target (passed by value to kernels).
struct TargetDev {
  int family;
  int metric;
  int d;
  int n;
  const void* X;
  const void* y;
  const void* s;
  double p0;
  double p1;
};

inline TargetDev to_dev(const gj_target& t) {
  TargetDev r;
  r.family = t.family;
  r.metric = t.metric;
  r.d = t.dim;
  r.n = t.n_data;
  r.X = t.X;
  r.y = t.y;
  r.s = t.s;
  r.p0 = t.p0;
  r.p1 = t.p1;
  return r;
}

// Step parameters in device-friendly form.
struct StepDev {
  double h;
  int L;
  int integrator;
  int max_iters;
  double tol;
  double div_threshold;
  double alpha2;
  const void* inv_mass;
  int alpha2_fix;
};

inline StepDev to_dev(const gj_step_params& p) {
  StepDev s;
  s.h = p.step_size;
  s.L = p.num_integration_steps;
  s.integrator = p.integrator;
  s.max_iters = p.max_iters;
  s.tol = p.tol;
  s.div_threshold = p.divergence_threshold;
  s.alpha2 = p.alpha2;
  s.inv_mass = p.inverse_mass;
  s.alpha2_fix = p.alpha2_fix;
  return s;
}

// Output pointers of one transition.
template <typename T>
struct InfoDev {
  double* acc_rate;
  uint8_t* accepted;
  uint8_t* divergent;
  double* energy;
  int32_t* fp_iters;
  uint8_t* status;
  T* momentum;
  T* prop_q;  // proposal position [C, d]
  T* prop_v;  // proposal velocity (flipped) [C, d]
};

// Output pointers of one NUTS transition
template <typename T>
struct NutsInfoDev {
  double* acc_rate;
  uint8_t* divergent;
  uint8_t* turning;
  double* energy;
  int32_t* doublings;
  int32_t* steps;
  int32_t* fp_iters;
  uint8_t* status;
  T* momentum;
  T* left_q;
  T* right_q;
};

template <typename T>
inline NutsInfoDev<T> to_dev(const gj_nuts_info* i) {
  NutsInfoDev<T> r{};
  if (i) {
    r.acc_rate = i->acceptance_rate;
    r.divergent = i->is_divergent;
    r.turning = i->is_turning;
    r.energy = i->energy;
    r.doublings = i->num_trajectory_expansions;
    r.steps = i->num_integration_steps;
    r.fp_iters = i->fp_iters;
    r.status = i->status;
    r.momentum = static_cast<T*>(i->momentum);
    r.left_q = static_cast<T*>(i->leftmost_position);
    r.right_q = static_cast<T*>(i->rightmost_position);
  }
  return r;
}

template <typename T>
inline InfoDev<T> to_dev(const gj_info* i) {
  InfoDev<T> r{};
  if (i) {
    r.acc_rate = i->acceptance_rate;
    r.accepted = i->is_accepted;
    r.divergent = i->is_divergent;
    r.energy = i->energy;
    r.fp_iters = i->fp_iters;
    r.status = i->status;
    r.momentum = static_cast<T*>(i->momentum);
    r.prop_q = static_cast<T*>(i->proposal_position);
    r.prop_v = static_cast<T*>(i->proposal_velocity);
  }
  return r;
}

// Metropolis accept of mcmc/proposal.py:87-121,168-185 in float64:
// w = H0 - H1 (NaN -> -inf), p = min(e^w, 1), accept = u < p.
struct AcceptOut {
  double w;
  double p_acc;
  bool accept;
  bool divergent;
};

__device__ __forceinline__ AcceptOut metropolis(double H0, double H1, double u, double div_thr) {
  AcceptOut a;
  double w = H0 - H1;
  if (isnan(w)) w = -INFINITY;
  a.w = w;
  a.p_acc = fmin(exp(w), 1.0);
  a.accept = u < a.p_acc;
  a.divergent = -w > div_thr;
  return a;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

template <typename T>
__device__ __forceinline__ T dexp(T x);
template <>
__device__ __forceinline__ float dexp<float>(float x) { return expf(x); }
template <>
__device__ __forceinline__ double dexp<double>(double x) { return exp(x); }

template <typename T>
__device__ __forceinline__ T dlog1pexp(T a) {  // log(1 + e^a), stable
  return a > T(0) ? a + log1p(exp(-a)) : log1p(exp(a));
}

template <typename T>
__device__ __forceinline__ T dsigmoid(T a) {
  return T(1) / (T(1) + exp(-a));
}

// Programmatic dependent launch.  A kernel launched with the PDL attribute
// may start while its predecessor in the stream (or graph) still runs: it
// must call pdl_wait() before touching global memory that other kernels
// read or write; pdl_wait() returns at once in a kernel launched without the
// attribute.  pdl_trigger() lets the successor's CTAs be scheduled; they are
// scheduled only once every CTA of this grid has triggered or exited, so a
// waiting successor never holds resources that this grid still needs.
// Kernels trigger late (after their main work): a trigger on entry let the
// successor's CTAs take SM slots the grid's own later waves needed.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;"); }

// Grouped launches run many independent launches of one kernel as one grid:
// item i owns blocks [prefix[i], prefix[i + 1]) (prefix[0] = 0, n items).
// Returns the item that holds block b (b < prefix[n]).
__device__ __forceinline__ int group_item(const int* __restrict__ prefix, int n, int b) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(prefix + mid) <= b)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

template <typename... KArgs, typename... Args>
inline cudaError_t launch_k(bool pdl, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                            cudaStream_t st, Args... args) {
  if (!pdl) {
    kernel<<<grid, block, smem, st>>>(args...);
    return cudaGetLastError();
  }
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

}  // namespace gj
