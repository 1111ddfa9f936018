// Host launchers of the per-chain kernels (chain_kernels.cu).
#pragma once

#include "common.cuh"

namespace gj {

template <typename T>
cudaError_t launch_rmhmc_chain(const TargetDev& t, const StepDev& sp, T* pos, T* grad, double* ld,
                               const T* z, const double* u, const InfoDev<T>& info, int C, int tpb,
                               cudaStream_t st);
// iterative NUTS with the dynamics of `sampler` (GJ_SAMPLER_*), thread per
// chain; u: [C, U] uniforms; vol: the volume adjustment (LMC samplers)
template <typename T>
cudaError_t launch_nuts(int sampler, const TargetDev& t, const StepDev& sp, int max_doublings,
                        int criterion, T* pos, T* grad, double* ld, double* vol, const T* z,
                        const double* u, int U, const NutsInfoDev<T>& info, int C, int tpb,
                        cudaStream_t st);
template <typename T>
cudaError_t launch_lmc_chain(const TargetDev& t, const StepDev& sp, T* pos, T* grad, double* ld,
                             double* vol, const T* z, const double* u, const InfoDev<T>& info,
                             int C, int tpb, cudaStream_t st);
template <typename T>
cudaError_t launch_monge_chain(const TargetDev& t, const StepDev& sp, T* pos, T* grad, double* ld,
                               double* vol, const T* z, const double* u, const InfoDev<T>& info,
                               int C, int tpb, cudaStream_t st);
template <typename T>
cudaError_t launch_logdensity_grad(const TargetDev& t, const T* q, double* ld, T* g, double* vol,
                                   int C, cudaStream_t st);
template <typename T>
cudaError_t launch_hvp(const TargetDev& t, const T* q, const T* u, T* out, int C, cudaStream_t st);
template <typename T>
cudaError_t launch_metric(const TargetDev& t, const T* q, T* out, int C, cudaStream_t st);
template <typename T>
cudaError_t launch_metric_vjp(const TargetDev& t, const T* q, const T* W, T* out, int C,
                              cudaStream_t st);

// differentiated generalized-leapfrog transition (traj_jvp.cu); shared
// memory per chain (one CTA) for d, N
size_t gl_trajectory_smem(int d, int N, int tangents);
cudaError_t launch_gl_trajectory_jvp(const double* X, const double* y, int N, int d,
                                     double prior_var, int C, const double* q0, const double* z,
                                     double h, double lam, int L, int Kp, int Kq, int tangents,
                                     double* out, cudaStream_t st);

// dense-Fisher logistic regression, one CTA per chain (logreg_cta.cu):
// RMHMC (either integrator) or dense LMC for d <= 64 while the chain's shared
// memory fits 227 KB; T = double is the plain FP64 form, T = float the mixed
// form (FP32 per-datum arithmetic, FP64 factor, solves and iterates)
size_t logreg_cta_smem(int d, int N, int mixed, int lmc);
bool logreg_cta_supported(int d, int N, int mixed, int lmc);
template <typename T>
cudaError_t launch_logreg_cta(int sampler, const TargetDev& t, const StepDev& sp, T* pos, T* grad,
                              double* ld, double* vol, const T* z, const double* u,
                              const InfoDev<T>& info, int C, cudaStream_t st);

// warp-per-chain LMC-Monge (monge_warp.cu): R = float (mixed form, float32
// state) or R = double (plain FP64 form)
template <typename R>
cudaError_t launch_monge_warp(const TargetDev& t, const StepDev& sp, R* pos, R* grad, double* ld,
                              double* vol, const R* z, const double* u, const InfoDev<R>& info,
                              int C, cudaStream_t st);
bool monge_warp_supported(const TargetDev& t);

// q_L and ∂q_L/∂α² of one LMC-Monge transition, forward mode in float64
// (monge_jvp.cu); qL may be NULL
bool monge_alpha2_jvp_supported(const TargetDev& t);
template <typename T>
cudaError_t launch_monge_alpha2_jvp(const TargetDev& t, const StepDev& sp, const T* pos,
                                    const T* z, T* qL, T* dq, int C, cudaStream_t st);

// FMA throughput of the CUDA cores in TFLOP/s (peaks.cu; synchronises)
cudaError_t fma_peak(int fp64, double* tflops, cudaStream_t st);

// ChEES cross-chain statistics (chees.cu): out[0] harmonic mean of the
// acceptance probabilities, out[1] the trajectory-length gradient, out[2]
// the α² gradient (0 without D); work holds chees_workspace_bytes(C, d)
size_t chees_workspace_bytes(int C, int d);
template <typename T>
cudaError_t chees_statistics(int C, int d, const T* P, const T* V, const T* I, const T* D,
                             const double* acc, const uint8_t* div, double* work, double* out,
                             cudaStream_t st);

}  // namespace gj
