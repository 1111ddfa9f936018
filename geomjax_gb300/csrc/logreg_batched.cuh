// Batched dense-Fisher logistic-regression RMHMC (implicit midpoint), mixed
// precision.  See logreg_batched.cu.
#pragma once

#include "common.cuh"

namespace gj {

struct LogregBatched;

int logreg_batched_create(const TargetDev& t, int C, LogregBatched** out);
void logreg_batched_destroy(LogregBatched* lb);
const char* logreg_batched_error();

// gemm_impl: 1 = SIMT FP32 GEMM over the BF16 hi/lo planes, 2 = tcgen05.
// chol_fp64: 1 = metric Cholesky / solves in float64 (default), 0 = float32.
int logreg_batched_rmhmc_step(LogregBatched* lb, const StepDev& sp, float* pos, float* grad,
                              double* logdens, const float* z, const double* u,
                              const InfoDev<float>& info, int gemm_impl, cudaStream_t st);

// Same transition as one CUDA-graph launch: every fixed-point solve is a
// conditional WHILE node driven by the device-side count of active chains
// (no host synchronisation inside the step).  One graph is captured per
// number of steps, GEMM implementation, factorisation set-up and whether the
// proposal velocity is asked for (up to 64, least recently used evicted), so
// a jittered number of steps per transition reuses its graphs; step size,
// tolerance, iteration cap and divergence threshold are read from device
// memory at run time.
int logreg_batched_rmhmc_step_graph(LogregBatched* lb, const StepDev& sp, float* pos, float* grad,
                                    double* logdens, const float* z, const double* u,
                                    const InfoDev<float>& info, int gemm_impl, cudaStream_t st);

// A batch of contexts (one per posterior, all with the same chain count)
// advanced by one CUDA-graph launch per transition: every posterior's whole
// transition an independent branch of the graph, or grouped launches over
// buckets of posteriors (logreg_batch_graph_set_grouped).  vec_off[b]: offset of
// posterior b's [C, d_b] block in the batch's ragged vectors; per-chain
// scalars are [B·C].  One gather kernel before the launch and one scatter
// kernel after it move the batch arrays in and out of the posteriors'
// staging buffers.  Up to 8 captured graphs are kept (by number of steps,
// GEMM path, factorisation set-up, integrator, proposal output and form).
struct LogregBatchGraph;
int logreg_batch_graph_create(LogregBatched* const* lbs, int B, int C, const size_t* vec_off,
                              LogregBatchGraph** out);
void logreg_batch_graph_destroy(LogregBatchGraph* bg);
// on = 1: the batch's graph holds grouped launches instead of one branch per
// posterior: the posteriors, sorted by size, are cut into `buckets` buckets
// (0 = automatic, 16 posteriors each); each bucket is a branch in which every stage of the transition
// is one grid (per kernel variant) over the bucket's posteriors and every
// fixed-point solve one WHILE node (tcgen05 GEMM path only).  on = 0
// (default): a branch per posterior.
void logreg_batch_graph_set_grouped(LogregBatchGraph* bg, int on, int buckets);
int logreg_batch_graph_step(LogregBatchGraph* bg, const StepDev& sp, float* pos, float* grad,
                            double* logdens, const float* z, const double* u,
                            const InfoDev<float>& info, int gemm_impl, cudaStream_t st);

// Last-step statistics of the batched path (host-side counters).
struct LogregStats {
  long long evals;           // fixed-point map evaluations issued (all chains)
  long long gemm_launches;   // GEMM kernels launched
  long long other_launches;  // other kernels launched
  double gemm_flops;         // algorithmic flops of the GEMMs issued
  double gemm_ns;            // GPU time of the GEMM launches (profiling on)
  long long chol_launches;   // metric factorisations launched
  double chol_flops;         // their algorithmic FP64 flops (d³/3 + 2d² per chain)
  double chol_ns;            // their GPU time (profiling on)
  long long refine_launches; // position-iterate solves by FP32 factor + FP64 refinement
  double refine_ns;          // their GPU time (profiling on)
  long long refine_fallbacks; // chains of those that fell back to FP64 (profiling on)
};
LogregStats logreg_batched_stats(const LogregBatched* lb);
void logreg_batched_set_chol_fp64(LogregBatched* lb, int on);
// chains per warp in the metric factorisation: 1, 2, 4, 8 or 0 (automatic)
void logreg_batched_set_chol_cpw(LogregBatched* lb, int cpw);
// 1: the pipeline's kernels are launched as programmatic dependents (their
// set-up overlaps the preceding kernel's tail); 0 (default): stream order
void logreg_batched_set_pdl(LogregBatched* lb, int on);
// K slices of the gradient contraction [r₁; r₂]·X on the tcgen05 path:
// 1 .. 4, or 0 (automatic: enough slices to fill the SMs once)
void logreg_batched_set_gemm_ksplit(LogregBatched* lb, int k);
// 1 (default): the generalized leapfrog's momentum evaluations contract
// r₂ = Λ'(w − s²) with X inside the S = U·Xᵀ GEMM's epilogue (tcgen05 path,
// d <= 32), one partial gradient per N tile; 0: r₂ is stored as split BF16
// planes and contracted by its own GEMM
void logreg_batched_set_fuse_r2x(LogregBatched* lb, int on);
// 1 = the generalized leapfrog's position iterates solve G⁻¹p by an FP32
// factorisation refined with FP64 residuals (default); 0 = FP64 factorisation
void logreg_batched_set_refine_iterates(LogregBatched* lb, int on);
// the chain count the automatic rules (K slices of the gradient contraction,
// chains per warp of the factorisation) size their grids for (default: the
// context's own; the chain groups of one sampler pass the sampler's total,
// so that results do not depend on the group count)
void logreg_batched_set_auto_chains(LogregBatched* lb, int C);
void logreg_batched_set_profile(LogregBatched* lb, int on);

// D[M, N] = A[M, K]·B[N, K]ᵀ through the split-BF16 GEMM `impl` (test hook;
// allocates scratch and synchronises the stream).
int gemm_split_test(int impl, int planes, int M, int N, int K, const float* A, const float* B,
                    float* D, cudaStream_t st);

}  // namespace gj
