/*
 * geomjax_gb300 — C ABI of the GB300-native sampler hot path.
 *
 * Every entry point replaces one call of the reference's pure-function kernel
 * API (williwilliams3/geomjax, Python/JAX):
 *
 *   gj_rmhmc_step     replaces kernel(rng_key, state, logdensity_fn, step_size,
 *                      metric_fn, num_integration_steps)
 *                      geomjax/rmhmc/rmhmc.py:131-174 (+ rmhmc_proposal :376-440)
 *   gj_lmcmonge_step  replaces kernel(rng_key, state, logdensity_fn, step_size,
 *                      inverse_mass_matrix, num_integration_steps, alpha2)
 *                      geomjax/lmcmonge/lmc.py:151-236 (+ lmc_proposal :472-536)
 *   gj_lmc_step       replaces kernel(rng_key, state, logdensity_fn, step_size,
 *                      metric_fn, num_integration_steps)
 *                      geomjax/lmcmc/lmc.py:135-180 (+ lmc_proposal :411-476)
 *   gj_init           replaces init(position, logdensity_fn)
 *                      geomjax/rmhmc/rmhmc.py:96-98, lmcmonge/lmc.py:101-109,
 *                      lmcmc/lmc.py:98-101 (value_and_grad at the position)
 *   gj_nuts_step       replaces the iterative NUTS kernels of rmhmc/nuts.py:78-161,
 *                      lmcmc/nuts.py and lmcmonge/nuts.py
 *   gj_logdensity_grad / gj_hvp / gj_metric
 *                      the operators the reference obtains by autodiff of the
 *                      user's logdensity_fn / metric_fn:
 *                      jax.value_and_grad (rmhmc/integrators.py:111),
 *                      util.hvp = jvp(grad f) (util.py:120-121),
 *                      metric_fn (rmhmc/metrics.py:42-58)
 *   gj_metric_vjp      the vector-Jacobian product of metric_fn that JAX
 *                      autodiff forms inside the kinetic-energy gradient
 *                      (rmhmc/integrators.py:111-114)
 *   gj_batch_*         a loop over posteriors around the rmhmc kernel,
 *                      posteriors of different sizes in one call
 *   gj_logreg_gl_transition_jvp
 *                      jax.jacfwd through a trajectory with respect to the
 *                      step size and a metric parameter
 *                      (adaptation/chees_adaptation_lmcmonge.py:497-519)
 *   gj_lmcmonge_alpha2_jvp
 *                      jax.jacfwd of the LMC-Monge proposal position with
 *                      respect to alpha2
 *                      (adaptation/chees_adaptation_lmcmonge.py:469-519)
 *   gj_chees_statistics, gj_chees_workspace_size
 *                      the cross-chain reductions of ChEES adaptation
 *                      (adaptation/chees_adaptation_riemanian.py:145-190,
 *                      chees_adaptation_lmcmonge.py:151-236)
 *   gj_gemm_split_bf16, gj_gemm_split_bf16_noalloc, gj_stats, gj_profile,
 *   gj_fma_peak, gj_set_option, gj_set_gemm_tiling, gj_set_gemm_accumulators
 *                      no reference counterpart: the split-BF16 contraction
 *                      as a test hook, measurement and tuning
 *
 * The reference's user-supplied Python callables become a registered device
 * target family (gj_target).  The reference draws its randomness from a JAX
 * key (key_momentum -> normal, key_integrator -> bernoulli,
 * rmhmc/rmhmc.py:158-161, mcmc/proposal.py:178); here the caller passes the
 * standard normals z[C, d] and the uniforms u[C] explicitly, and the accept
 * is u < min(exp(H0 - H1), 1) exactly as jax.random.bernoulli.
 *
 * Conventions
 *   - All array pointers are DEVICE pointers owned by the caller; row-major,
 *     chains first: position[C, d].  Per-chain scalars are float64.
 *   - precision GJ_FP64: every vector is float64 ("plain FP64 form").
 *     precision GJ_MIXED: vectors and target data are float32; FP64 is kept
 *     for the metric Cholesky/log-det/solves, the fixed-point convergence
 *     norm and the Hamiltonian difference.
 *   - Calls are stream-ordered on `stream` (a cudaStream_t, NULL = legacy
 *     default stream) and never synchronise the host, except where a
 *     comment says so.  A context is not thread-safe: one host thread per
 *     context.
 *   - Return value: a gj_status.  Numerical trouble never raises: it shows up
 *     per chain (NaN energy -> rejected, divergence flag, fixed-point
 *     non-convergence bit in gj_info.status), as in the reference.
 */
#ifndef GEOMJAX_GB300_H
#define GEOMJAX_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  GJ_OK = 0,
  GJ_EINVAL = 1,   /* bad shape / pointer / enum value */
  GJ_ENOTSUP = 2,  /* combination not built (e.g. dense metric above the size limit) */
  GJ_ECUDA = 3,    /* a CUDA runtime call failed; see gj_last_error() */
  GJ_ENOMEM = 4
} gj_status;

typedef enum { GJ_FUNNEL = 1, GJ_LOGREG = 2, GJ_HIERGAUSS = 3 } gj_family;

typedef enum {
  GJ_METRIC_DIAG_FISHER = 1,  /* funnel: diag(e^-v .., 1/s^2 + (D-1)/2) */
  GJ_METRIC_DENSE_FISHER = 2, /* logreg: X^T Lambda X + I/s^2 ; hier: arrowhead Fisher */
  GJ_METRIC_PULLBACK = 3,     /* funnel: J^-T J^-1 (examples/funnel/main.py:41-54) */
  GJ_METRIC_IDENTITY = 4      /* G = I (tests/test_samplers.py:25) */
} gj_metric_kind;

typedef enum { GJ_FP64 = 0, GJ_MIXED = 1 } gj_precision;

typedef enum { GJ_IMPLICIT_MIDPOINT = 0, GJ_GENERALIZED_LEAPFROG = 1 } gj_integrator;

typedef enum { GJ_SAMPLER_RMHMC = 0, GJ_SAMPLER_LMC = 1, GJ_SAMPLER_LMCMONGE = 2 } gj_sampler;

/* per-chain status bits (gj_info.status) */
#define GJ_CHAIN_FP_NOT_CONVERGED 0x1u /* a fixed-point solve stopped without reaching tol */
#define GJ_CHAIN_NONFINITE 0x2u        /* the proposal energy was NaN/Inf */
#define GJ_CHAIN_NOT_SPD 0x4u          /* a metric Cholesky met a non-positive pivot */

/* A registered target family plus its data (device pointers). */
typedef struct {
  int32_t family;  /* gj_family */
  int32_t metric;  /* gj_metric_kind */
  int32_t dim;     /* d */
  int32_t n_data;  /* logreg: N rows of X; hier: J groups; funnel: 0 */
  const void* X;   /* logreg: X[N, d] (float32 for GJ_MIXED, float64 for GJ_FP64) */
  const void* y;   /* logreg: labels[N]; hier: observations y[J] (same dtype as X) */
  const void* s;   /* hier: observation scales sigma[J] (same dtype); else NULL */
  double p0;       /* funnel: sigma (3); logreg: prior variance (100); hier: mu scale */
  double p1;       /* hier: v scale; otherwise unused */
} gj_target;

/* Chain state (device pointers).  Dtype of position/grad follows precision. */
typedef struct {
  void* position;            /* [C, d] */
  void* logdensity_grad;     /* [C, d] */
  double* logdensity;        /* [C] */
  double* volume_adjustment; /* [C] LMC / LMC-Monge only (may be NULL for RMHMC) */
  int32_t num_chains;        /* C */
} gj_chain_state;

/* Per-transition information (device pointers, each may be NULL). */
typedef struct {
  double* acceptance_rate; /* [C] min(exp(H0 - H1), 1) */
  uint8_t* is_accepted;    /* [C] */
  uint8_t* is_divergent;   /* [C] -(H0 - H1) > divergence_threshold */
  double* energy;          /* [C] H1, the proposal's energy */
  int32_t* fp_iters;       /* [C] fixed-point iterations summed over the trajectory */
  uint8_t* status;         /* [C] GJ_CHAIN_* bits */
  void* momentum;          /* [C, d] the drawn momentum (RMHMC) or velocity (LMC) */
  /* The proposal, written whether or not it is accepted: the end of the
   * trajectory after the flip (rmhmc/rmhmc.py:425-426,443-462,
   * lmcmonge/lmc.py:506-507, lmcmc/lmc.py:441-442), i.e. RMHMCInfo.proposal.state
   * / LMCInfo.proposal.state.  ChEES adaptation reads these
   * (adaptation/chees_adaptation_riemanian.py:161-190). */
  void* proposal_position; /* [C, d] q_L */
  void* proposal_velocity; /* [C, d] RMHMC: -G(q_L)^-1 p_L; LMC / LMC-Monge: -v_L */
} gj_info;

typedef struct {
  double step_size;
  int32_t num_integration_steps;
  int32_t integrator;          /* gj_integrator (RMHMC) */
  int32_t max_iters;           /* fixed-point iteration cap (reference default 100) */
  double tol;                  /* fixed-point tolerance (reference default 1e-6) */
  double divergence_threshold; /* reference default 1000 */
  double alpha2;               /* LMC-Monge alpha^2 (reference default 0.001) */
  const void* inverse_mass;    /* LMC-Monge diagonal inverse mass [d] (state dtype); NULL = ones */
  int32_t alpha2_fix;          /* LMC-Monge: 1 = multiply the Sherman-Morrison correction by
                                  alpha^2 (the reference omits it, lmcmonge/integrators.py:186-189) */
  int32_t reserved;
} gj_step_params;

/* Iterative NUTS (rmhmc/nuts.py:78-161, lmcmc/nuts.py, lmcmonge/nuts.py):
 * the trajectory doubles in a random direction until the generalized
 * U-turn criterion holds, a divergence occurs or max_num_doublings
 * expansions were made. */
typedef struct {
  double step_size;
  int32_t max_num_doublings;   /* reference default 10; at most 16 */
  int32_t integrator;          /* gj_integrator (RMHMC) */
  int32_t criterion;           /* stopping_criterion: 0 "euc" (default), 1 "bet", 2 "riem" */
  int32_t max_iters;           /* fixed-point iteration cap (RMHMC) */
  double tol;                  /* fixed-point tolerance (RMHMC) */
  double divergence_threshold; /* reference default 1000 */
  double alpha2;               /* LMC-Monge alpha^2 */
  const void* inverse_mass;    /* LMC-Monge diagonal inverse mass [d] (NULL = ones) */
  int32_t alpha2_fix;          /* LMC-Monge, as gj_step_params.alpha2_fix */
  int32_t reserved;
} gj_nuts_params;

/* NUTSInfo (rmhmc/nuts.py:37-75), device pointers, each may be NULL. */
typedef struct {
  double* acceptance_rate;            /* [C] exp(sum_log_p_accept) / num_integration_steps */
  uint8_t* is_divergent;              /* [C] */
  uint8_t* is_turning;                /* [C] */
  double* energy;                     /* [C] the sampled proposal's energy */
  int32_t* num_trajectory_expansions; /* [C] */
  int32_t* num_integration_steps;     /* [C] states in the trajectory */
  int32_t* fp_iters;                  /* [C] fixed-point iterations over the trajectory */
  uint8_t* status;                    /* [C] GJ_CHAIN_* bits */
  void* momentum;                     /* [C, d] the drawn momentum (RMHMC) or velocity (LMC) */
  void* leftmost_position;            /* [C, d] trajectory_leftmost_state.position */
  void* rightmost_position;           /* [C, d] trajectory_rightmost_state.position */
} gj_nuts_info;

typedef struct gj_ctx gj_ctx;

/* Version and last error message of the calling thread. */
int32_t gj_version(void);
const char* gj_last_error(void);

/* A context binds one target, sampler and precision to a chain count and owns
 * the device workspaces of the batched paths.  It allocates device memory
 * (cudaMalloc) at creation and on the first step that needs a workspace;
 * gj_destroy frees it.  The target's data pointers must outlive the context. */
int32_t gj_create(const gj_target* target, int32_t sampler, int32_t precision,
                  int32_t num_chains, gj_ctx** out);
int32_t gj_destroy(gj_ctx* ctx);

/* Selects the implementation of the dense-Fisher logistic-regression paths.
 * RMHMC: 0 = automatic (GJ_MIXED: batched tensor-core pipeline; GJ_FP64: one
 * CTA per chain), 1 = batched pipeline with the SIMT FP32 GEMM, 2 = batched
 * pipeline with the tcgen05 BF16 hi/lo GEMM, 3 = one thread per chain
 * (d <= 32), 4 = one CTA per chain in either precision (d <= 64; shared
 * memory of (d(d+1) + 16d + 274)·8 + (4N + max(N, 16d) + 16(d+1))·sizeof(T)
 * bytes, plus d(d+1)/2·4 in GJ_MIXED, at most 227 KB, else GJ_ENOTSUP).
 * Dense LMC: 3 = one thread per chain (d <= 32), any other value = one CTA
 * per chain (d <= 64; also d(d+1)/2 + d² doubles and d ints of shared
 * memory). */
int32_t gj_set_option(gj_ctx* ctx, int32_t key, int64_t value);
#define GJ_OPT_LOGREG_PATH 1
/* threads per block of the per-chain kernels: 32, 64, 96 or 128 (default) */
#define GJ_OPT_THREADS_PER_BLOCK 2
/* batched path loop driver: 0 = one CUDA-graph launch per transition with
 * conditional WHILE nodes for the fixed-point solves (default), 1 = host
 * loop that reads the active-chain count back after every iteration */
#define GJ_OPT_LOOP 3
/* batched path metric factorisation: 1 = float64 Cholesky / log det /
 * solves (default), 0 = float32 */
#define GJ_OPT_CHOL_FP64 4
/* batched path metric factorisation: chains sharing one warp (1, 2, 4 or 8;
 * 0 = automatic).  The factorisation's FP64 instructions issue once per warp
 * whatever the lanes in use, so packing chains divides its FP64 work, while
 * fewer warps hide less latency. */
#define GJ_OPT_CHOL_CHAINS_PER_WARP 5
/* batched path: independent chain groups (1 .. 8; 0 = automatic = 1).  In
 * graph mode each group's transition is its own CUDA graph on its own
 * stream, forked from and joined to the caller's stream, so that one group's
 * FP64 factorisation may overlap another group's GEMMs.  Results are
 * bit-identical for any group count. */
#define GJ_OPT_CHAIN_GROUPS 6
/* batched path: 1 = launch the pipeline's kernels with programmatic
 * dependent launch (each kernel's set-up overlaps its predecessor's last
 * wave; it waits on the predecessor before touching global memory),
 * 0 (default) = ordinary stream order.  On GB300 at d = 25, 4096 chains,
 * PDL measured 2.28M against 2.53M leapfrog steps/s without it. */
#define GJ_OPT_PDL 7
/* batched path, tcgen05 GEMMs: K slices of the gradient contraction
 * [r1; r2]·X (M = 2 x chains, N = d, K = observations), 1 .. 4, or 0
 * (automatic, default: as many as fill the SMs once with at least 4 K
 * blocks per slice).  Slice z writes its partial product to its own buffer
 * and the consumers add the slices in order, so results do not depend on
 * scheduling. */
#define GJ_OPT_GEMM_KSPLIT 8
/* batches of posteriors (gj_batch_set_option): 2 (default) = one CUDA graph
 * per transition of grouped launches: the posteriors, in buckets of similar
 * size (GJ_OPT_BATCH_BUCKETS), each bucket a branch of the graph, every stage
 * of the transition one grid (per kernel variant) over the bucket's
 * posteriors, whose blocks find their posterior in a list of per-posterior
 * items, and every fixed-point solve one WHILE node per bucket (tcgen05 GEMM
 * path); 1 = one CUDA graph per transition holding every posterior's
 * transition as its own branch; 0 = one graph per posterior, spread over the
 * batch's stream pool.  Each mode is launched once per transition (plus one
 * gather and one scatter kernel), and results are bit-identical in every
 * mode. */
#define GJ_OPT_BATCH_GRAPH 9
/* LMC-Monge (funnel and hierarchical Gaussian, d <= 256): 1 (default) = one
 * warp per chain in either precision (float64 throughout for GJ_FP64),
 * 0 = one thread per chain */
#define GJ_OPT_MONGE_WARP 10
/* batched path, tcgen05 GEMMs, d <= 32 and N > 64 (contexts and batches):
 * 1 (default) = the generalized leapfrog's momentum evaluations contract
 * r2 = Λ'(w − s²) with X inside the CTA of the S = U·Xᵀ GEMM (r2 as three
 * BF16 planes in shared memory, a second tcgen05 MMA against the Xᵀ tile,
 * one partial gradient per N tile, added in tile order by the momentum
 * update); 0 = r2 is stored as three BF16 planes in global memory and
 * contracted by its own tensor-core GEMM */
#define GJ_OPT_FUSE_R2X 11
/* batches with GJ_OPT_BATCH_GRAPH = 2 (gj_batch_set_option): the posteriors,
 * sorted by (d, N), are cut into this many buckets of consecutive sizes,
 * 1 .. 256 (0 = automatic: 16 posteriors per bucket); each bucket is one branch of the graph with its
 * own grouped launches and fixed-point loops, so a bucket waits only for its
 * own slowest chain and the branches overlap */
#define GJ_OPT_BATCH_BUCKETS 12
/* batched path, generalized leapfrog: 1 = each position iterate's solve
 * u = G(q_k)⁻¹p½ by mixed-precision iterative refinement (default): G is
 * factored in float32 and u corrected with float64 residuals p − G·u until
 * it is as accurate as a float64 factorisation's solve; a chain whose
 * refinement does not converge is factored in float64.  The full
 * evaluations (kept factor, log det) always factor in float64.  0 = every
 * factorisation in float64.  Applies with GJ_OPT_CHOL_FP64 = 1 for
 * 3 <= d <= 64 (where a chain's factorisation runs within one warp). */
#define GJ_OPT_REFINE_ITERATES 13

/* value_and_grad of the log density at state->position; zeroes
 * volume_adjustment when present. */
int32_t gj_init(gj_ctx* ctx, gj_chain_state* state, void* stream);

int32_t gj_rmhmc_step(gj_ctx* ctx, const gj_step_params* params, gj_chain_state* state,
                      const void* z, const double* u, gj_info* info, void* stream);
int32_t gj_lmcmonge_step(gj_ctx* ctx, const gj_step_params* params, gj_chain_state* state,
                         const void* z, const double* u, gj_info* info, void* stream);
int32_t gj_lmc_step(gj_ctx* ctx, const gj_step_params* params, gj_chain_state* state,
                    const void* z, const double* u, gj_info* info, void* stream);

/* One iterative-NUTS transition of every chain of a context, with the
 * context's dynamics: RMHMC (rmhmc/nuts.py:112-159, iterative_nuts_proposal
 * :253-348), dense LMC (lmcmc/nuts.py) or LMC-Monge (lmcmonge/nuts.py, the
 * kernel named nutslmc there); one thread per chain, d <= 32.  The state
 * (with the volume adjustment for the LMC samplers) moves to the sampled
 * proposal.  z: [C, d] momentum / velocity normals; uniforms: [C, uniforms_per_chain] float64 with
 * uniforms_per_chain >= 2M + 2^M - 1 (M = max_num_doublings), laid out per
 * chain as u[k] the direction of expansion k (+1 iff u < 1/2), u[M + k] the
 * biased merge of expansion k, u[2M + 2^k - 1 + j] the progressive sample
 * of step j (>= 1) of expansion k -- the draws the reference takes from its
 * split keys. */
int32_t gj_nuts_step(gj_ctx* ctx, const gj_nuts_params* params, gj_chain_state* state,
                     const void* z, const double* uniforms, int32_t uniforms_per_chain,
                     gj_nuts_info* info, void* stream);

/* Counters of the last step on this context: out[0] fixed-point map
 * evaluations, out[1] GEMM launches, out[2] other kernel launches,
 * out[3] algorithmic GEMM flops, out[4] GPU time of the GEMM launches in
 * nanoseconds (only while profiling is on), out[5] metric factorisations
 * launched, out[6] their algorithmic FP64 flops (d³/3 + 2d² per chain, d³/3
 * + d² for an energy evaluation), out[7] their GPU time in nanoseconds
 * (profiling on), out[8] position-iterate solves by FP32 factorisation and
 * FP64 refinement (GJ_OPT_REFINE_ITERATES; not counted in out[5..7]),
 * out[9] their GPU time in nanoseconds (profiling on), out[10] the chains
 * of those solves that fell back to the FP64 factorisation (profiling on).
 * Returns the number written (<= n, at most 11).  No counterpart in the reference (measurement only). */
int32_t gj_stats(gj_ctx* ctx, int64_t* out, int32_t n);
/* FMA throughput of this device's CUDA cores, in TFLOP/s (2 flops per FMA):
 * float64 for GJ_FP64, float32 for GJ_MIXED.  Eight independent FMA chains
 * per thread, 2048 threads per SM, timed with CUDA events on `stream`
 * (allocates a scratch buffer and synchronises).  The roofline denominator
 * of the FP64 metric factorisation and of the FP32 Monge kernel; no
 * counterpart in the reference (measurement only). */
int32_t gj_fma_peak(int32_t precision, double* tflops, void* stream);

/* 1 = bracket every GEMM launch with CUDA events so gj_stats reports their
 * GPU time (the step then synchronises at its end); 0 = off (default).
 * No counterpart in the reference (measurement only). */
int32_t gj_profile(gj_ctx* ctx, int32_t on);

/* Test hook of the batched contraction (no counterpart in the reference):
 * D[M, N] = A[M, K] · B[N, K]ᵀ for float32 device arrays A, B, D, computed
 * from `planes` (2 or 3) split-BF16 planes per operand with FP32
 * accumulation by impl 1 (SIMT) or impl 2 (tcgen05).  Allocates and frees
 * device scratch; synchronises the stream. */
int32_t gj_gemm_split_bf16(int32_t impl, int32_t planes, int32_t M, int32_t N, int32_t K,
                           const float* A, const float* B, float* D, void* stream);

/* The same contraction as gj_gemm_split_bf16, for callers that cannot
 * allocate device memory: a JAX/XLA custom call, whose framework has
 * reserved nearly all device memory for its own pool, so that a cudaMalloc
 * of its own can fail or fragment that pool.  It calls no cudaMalloc,
 * cudaFree or allocating library routine: its split planes live in one
 * static device array of 8 MiB (4,194,304 BF16 elements) that every GPU
 * loading the library holds until the process exits.  Limit: planes *
 * (ceil128(M) + ceil128(N)) * ceil64(K) <= 4194304, otherwise GJ_EINVAL.
 * All calls share the array: calls that overlap on the GPU (other streams or
 * host threads) race on it and must be serialised by the caller; every call
 * rewrites all of the array it reads.  The first call on each device looks
 * up the array's device address (cudaGetSymbolAddress) with that device
 * current; make that first call before any stream capture.  Ends with a
 * synchronisation of the stream (it reads the kernel's error word back).
 * No counterpart in the reference. */
int32_t gj_gemm_split_bf16_noalloc(int32_t impl, int32_t planes, int32_t M, int32_t N,
                                   int32_t K, const float* A, const float* B, float* D,
                                   void* stream);

/* Operator-level entry points (no context).  q, grad, u, out: [C, d];
 * logdensity: [C] float64; metric_out: [C, d] (diagonal metrics) or
 * [C, d, d] (dense), dtype of the precision. */
int32_t gj_logdensity_grad(const gj_target* target, int32_t precision, int32_t num_chains,
                           const void* q, double* logdensity, void* grad, void* stream);
int32_t gj_hvp(const gj_target* target, int32_t precision, int32_t num_chains, const void* q,
               const void* u, void* out, void* stream);
int32_t gj_metric(const gj_target* target, int32_t precision, int32_t num_chains,
                  const void* q, void* metric_out, void* stream);

/* Adjoint (vector-Jacobian product) of the metric operator:
 * out[c, k] = Σ_ab W[c, a, b] ∂G_ab/∂q_k at q[c] (W is [C, d] for diagonal
 * metrics).  Replaces jax.vjp of the user's metric_fn; the adjoints of the
 * log density and of its gradient are gj_logdensity_grad and gj_hvp. */
int32_t gj_metric_vjp(const gj_target* target, int32_t precision, int32_t num_chains,
                      const void* q, const void* w, void* out, void* stream);

/* ---- batches of independent posteriors ----------------------------------
 * A batch holds B dense-Fisher logistic-regression posteriors of any sizes
 * (n_data and dim may differ; dim <= 128), each sampled by C RMHMC chains
 * through the batched mixed-precision pipeline (either integrator).  By
 * default one CUDA graph holds every posterior's transition as an
 * independent branch, and one launch per transition advances them all
 * (GJ_OPT_BATCH_GRAPH; the graph is captured at the first step with a given
 * number of steps and kept); otherwise each posterior's transition is its
 * own graph, spread round-robin over num_streams streams forked from and
 * joined to the caller's stream.
 * The reference samples one posterior per kernel call; a batch is the
 * vmapped loop over posteriors a user would write around it.
 *
 * Layout: per-chain scalars (logdensity, u, info arrays but momentum) are
 * [B*C], posterior b's chains at rows [b*C, (b+1)*C).  Vectors (position,
 * logdensity_grad, z, info.momentum) are ragged: posterior b's [C, d_b]
 * block starts at C * (d_0 + ... + d_{b-1}).  state->num_chains = B*C.
 * Targets' X and y must stay valid while the batch lives. */
typedef struct gj_batch gj_batch;
int32_t gj_batch_create(const gj_target* targets, int32_t num_posteriors,
                        int32_t chains_per_posterior, int32_t num_streams, gj_batch** out);
int32_t gj_batch_destroy(gj_batch* batch);
/* GJ_OPT_CHOL_FP64, GJ_OPT_CHOL_CHAINS_PER_WARP and GJ_OPT_GEMM_KSPLIT, for
 * every posterior; GJ_OPT_BATCH_GRAPH for the batch */
int32_t gj_batch_set_option(gj_batch* batch, int32_t key, int64_t value);
int32_t gj_batch_rmhmc_step(gj_batch* batch, const gj_step_params* params, gj_chain_state* state,
                            const float* z, const double* u, gj_info* info, void* stream);

/* Process-wide tile policy of the tcgen05 split-BF16 GEMMs: output tile
 * width for N > 64 (0 = automatic per shape, or 64 / 128; narrower N always
 * takes 32 or 64) and whether the operand ring is cut back so that two CTAs
 * share an SM (1), kept up to three stages (0) or chosen per shape (-1,
 * default).  Applies to the launches made after the call; a context keeps
 * one captured graph per policy, so changing it (as the autotuner of
 * geomjax_gb300.autotune does) captures anew. */
int32_t gj_set_gemm_tiling(int32_t tile_n_wide, int32_t two_ctas_per_sm);

/* Process-wide: the most K-range accumulators a tcgen05 GEMM CTA uses (1, 2
 * or 4; default 4).  The K blocks of a CTA are cut into up to that many
 * contiguous ranges, each accumulated in its own TMEM tile and added in FP32
 * registers by the epilogue: the tensor core's FP32 accumulation rounds low
 * and its bias grows with the accumulation run (−4.5e-6 relative over
 * K = 1000 and −3.2e-5 over K = 5000 with one range).  Like
 * gj_set_gemm_tiling it applies to later launches and graph captures.  No
 * counterpart in the reference (accuracy / speed tuning). */
int32_t gj_set_gemm_accumulators(int32_t max_ranges);

/* Derivatives of one RMHMC transition with the generalized leapfrog, for a
 * GJ_LOGREG target with float64 data: with respect to the step size h and
 * the metric regulariser λ (G = XᵀΛX + λI; the prior variance stays
 * target->p0), by forward-mode tangent propagation through the whole
 * discrete trajectory.  Each fixed-point half step runs exactly kp (momentum)
 * / kq (position) iterations so the differentiated map is fixed.  q0, z:
 * [C, d] float64 start positions and momentum normals.  out[C, 6] =
 * (p_accept, ∂p_accept/∂h, ∂p_accept/∂λ, ΔH = H1 − H0, ∂ΔH/∂h, ∂ΔH/∂λ);
 * tangents = 0 computes the values only (the tangent slots are zero).
 * One CTA per chain holds the chain's factor, vectors and per-datum arrays
 * in shared memory: d <= 64, and (d(d+1)/2 + 10d + 3N + 256)·24 bytes plus a
 * 16-row tile of X must fit 227 KB (N <= 2000 at d = 64; GJ_ENOTSUP beyond).
 * Replaces the reference's jax.jacfwd through a trajectory
 * (adaptation/chees_adaptation_lmcmonge.py:497-519). */
int32_t gj_logreg_gl_transition_jvp(const gj_target* target, int32_t num_chains, const double* q0,
                                    const double* z, double step_size, double metric_reg,
                                    int32_t num_integration_steps, int32_t kp, int32_t kq,
                                    int32_t tangents, double* out, void* stream);

/* Proposal position q_L of one LMC-Monge transition and its derivative
 * ∂q_L/∂α², by forward-mode propagation of d/dα² through the velocity draw,
 * the normalising constant and every half_step_omega (float64 throughout,
 * whatever the precision of the arrays).  Replaces
 * jax.jacfwd(trajectory_proposal_position, argnums=0) of
 * adaptation/chees_adaptation_lmcmonge.py:469-519.  params gives the step
 * size, the number of steps, alpha2, the inverse mass (NULL = ones) and
 * alpha2_fix as for gj_lmcmonge_step; position and z are the transition's
 * start and normals, [C, d] in the precision's vector dtype, as are the
 * outputs (proposal_position may be NULL).  Targets: GJ_FUNNEL and
 * GJ_HIERGAUSS, d <= 256 (GJ_ENOTSUP otherwise). */
int32_t gj_lmcmonge_alpha2_jvp(const gj_target* target, int32_t precision, int32_t num_chains,
                               const gj_step_params* params, const void* position, const void* z,
                               void* proposal_position, void* proposal_alpha2_tangent,
                               void* stream);

/* ChEES cross-chain statistics of one transition
 * (adaptation/chees_adaptation_riemanian.py:145-190 and
 * chees_adaptation_lmcmonge.py:151-236), from the proposal the step wrote
 * into gj_info (proposal_position P, proposal_velocity V) and the positions
 * I the transition started from, all [C, d] in the precision's vector dtype:
 *   out[0] = 1 / mean(1 / acceptance_rate) over non-divergent chains
 *   out[1] = Σ a_c g_c / Σ a_c over non-divergent chains, with
 *            g_c = (|P̃_c|² − |Ĩ_c|²)(P̃_c · V_c), P̃ = P − nanmean over chains,
 *            Ĩ = I − nanmean over chains
 *   out[2] = the same weighted mean with V replaced by the tangent
 *            D = ∂P/∂α² (0 when proposal_alpha2_tangent is NULL)
 * The reference multiplies out[1] and out[2] by jitter × trajectory length.
 * is_divergent may be NULL (no chain divergent).  out: 3 doubles of DEVICE
 * memory; workspace: gj_chees_workspace_size(C, d) bytes of device memory.
 * Deterministic (fixed reduction order). */
int64_t gj_chees_workspace_size(int32_t num_chains, int32_t dim);
int32_t gj_chees_statistics(int32_t precision, int32_t num_chains, int32_t dim,
                            const void* proposal_position, const void* proposal_velocity,
                            const void* initial_position, const void* proposal_alpha2_tangent,
                            const double* acceptance_rate, const uint8_t* is_divergent,
                            void* workspace, double* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GEOMJAX_GB300_H */
