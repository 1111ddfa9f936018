// extern "C" boundary (include/geomjax_gb300.h): argument checks, context,
// dispatch to the per-chain kernels, the warp-per-chain LMC-Monge kernel and
// the batched dense-Fisher logistic-regression RMHMC pipeline.
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "chain_kernels.cuh"
#include "gemm.cuh"
#include "logreg_batched.cuh"

namespace {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, const char* a = "") {
  char buf[512];
  std::snprintf(buf, sizeof(buf), fmt, a);
  g_last_error = buf;
  return code;
}

int cuda_status(cudaError_t e, const char* where) {
  if (e == cudaSuccess) return GJ_OK;
  char buf[512];
  std::snprintf(buf, sizeof(buf), "%s: %s", where, cudaGetErrorString(e));
  g_last_error = buf;
  return GJ_ECUDA;
}

int check_target(const gj_target* t, int precision) {
  if (!t) return fail(GJ_EINVAL, "target is NULL");
  if (precision != GJ_FP64 && precision != GJ_MIXED) return fail(GJ_EINVAL, "bad precision");
  if (t->dim < 1) return fail(GJ_EINVAL, "dim must be >= 1");
  switch (t->family) {
    case GJ_FUNNEL:
      if (t->dim < 2) return fail(GJ_EINVAL, "funnel needs dim >= 2");
      if (t->metric != GJ_METRIC_DIAG_FISHER && t->metric != GJ_METRIC_PULLBACK &&
          t->metric != GJ_METRIC_IDENTITY)
        return fail(GJ_EINVAL, "funnel metric must be diag, pullback or identity");
      if (!(t->p0 > 0)) return fail(GJ_EINVAL, "funnel sigma must be > 0");
      break;
    case GJ_LOGREG:
      if (t->n_data < 1 || !t->X || !t->y) return fail(GJ_EINVAL, "logreg needs X[N, d] and y[N]");
      if (t->metric != GJ_METRIC_DENSE_FISHER && t->metric != GJ_METRIC_IDENTITY)
        return fail(GJ_EINVAL, "logreg metric must be dense Fisher or identity");
      if (!(t->p0 > 0)) return fail(GJ_EINVAL, "logreg prior variance must be > 0");
      break;
    case GJ_HIERGAUSS:
      if (t->n_data < 1 || t->dim != t->n_data + 2 || !t->y || !t->s)
        return fail(GJ_EINVAL, "hierarchical Gaussian needs dim = J + 2, y[J], sigma[J]");
      if (t->metric != GJ_METRIC_DENSE_FISHER && t->metric != GJ_METRIC_IDENTITY)
        return fail(GJ_EINVAL, "hier metric must be dense Fisher or identity");
      if (!(t->p0 > 0) || !(t->p1 > 0)) return fail(GJ_EINVAL, "hier scales must be > 0");
      break;
    default:
      return fail(GJ_EINVAL, "unknown target family");
  }
  return GJ_OK;
}

int check_state(const gj_chain_state* s, int C, bool need_vol) {
  if (!s || !s->position || !s->logdensity_grad || !s->logdensity)
    return fail(GJ_EINVAL, "chain state has a NULL array");
  if (s->num_chains != C) return fail(GJ_EINVAL, "state.num_chains differs from the context's");
  if (need_vol && !s->volume_adjustment)
    return fail(GJ_EINVAL, "LMC state needs volume_adjustment");
  return GJ_OK;
}

int check_params(const gj_step_params* p) {
  if (!p) return fail(GJ_EINVAL, "params is NULL");
  if (p->num_integration_steps < 0) return fail(GJ_EINVAL, "num_integration_steps < 0");
  if (!(p->step_size == p->step_size)) return fail(GJ_EINVAL, "step_size is NaN");
  if (p->max_iters < 0) return fail(GJ_EINVAL, "max_iters < 0");
  return GJ_OK;
}

}  // namespace

struct gj_ctx {
  gj_target target;
  int sampler;
  int precision;
  int C;
  int logreg_path;  // GJ_OPT_LOGREG_PATH
  int tpb;
  int profile;
  int loop_mode;  // GJ_OPT_LOOP
  int chol_fp64;  // GJ_OPT_CHOL_FP64
  int chol_cpw;   // GJ_OPT_CHOL_CHAINS_PER_WARP
  int groups;     // GJ_OPT_CHAIN_GROUPS (0 = automatic)
  int pdl;        // GJ_OPT_PDL
  int ksplit;     // GJ_OPT_GEMM_KSPLIT (0 = automatic)
  int monge_warp; // GJ_OPT_MONGE_WARP
  int fuse_r2x;   // GJ_OPT_FUSE_R2X
  int refine;     // GJ_OPT_REFINE_ITERATES
  // batched dense-Fisher path: one context per chain group; in graph mode
  // the groups' transitions run on their own streams, forked from and joined
  // to the caller's stream by events, so one group's factorisation can share
  // the GPU with another group's GEMMs
  std::vector<gj::LogregBatched*> lbs;
  std::vector<cudaStream_t> gstreams;
  std::vector<cudaEvent_t> gevents;  // [0] fork, [1 + g] join of group g
};

namespace {

void destroy_groups(gj_ctx* ctx) {
  for (gj::LogregBatched* lb : ctx->lbs) gj::logreg_batched_destroy(lb);
  for (cudaStream_t s : ctx->gstreams) cudaStreamDestroy(s);
  for (cudaEvent_t e : ctx->gevents) cudaEventDestroy(e);
  ctx->lbs.clear();
  ctx->gstreams.clear();
  ctx->gevents.clear();
}

// automatic group count: one.  On GB300 at d = 25, 4096 chains, 1 / 2 / 4
// groups measured 2.52M / 2.48M / 2.52M leapfrog steps/s: each group's
// kernels fill the GPU, so the graphs do not overlap.
int resolve_groups(const gj_ctx* ctx) {
  const int g = ctx->groups > 0 ? ctx->groups : 1;
  return g < ctx->C ? g : ctx->C;
}

void group_range(const gj_ctx* ctx, int G, int g, int* c0, int* n) {
  const int per = (ctx->C + G - 1) / G;
  *c0 = g * per;
  const int rest = ctx->C - *c0;
  *n = rest < per ? (rest > 0 ? rest : 0) : per;
}

template <typename T>
gj::InfoDev<T> info_offset(gj::InfoDev<T> i, size_t c0, int d) {
  if (i.acc_rate) i.acc_rate += c0;
  if (i.accepted) i.accepted += c0;
  if (i.divergent) i.divergent += c0;
  if (i.energy) i.energy += c0;
  if (i.fp_iters) i.fp_iters += c0;
  if (i.status) i.status += c0;
  if (i.momentum) i.momentum += c0 * d;
  if (i.prop_q) i.prop_q += c0 * d;
  if (i.prop_v) i.prop_v += c0 * d;
  return i;
}

int ensure_groups(gj_ctx* ctx, const gj::TargetDev& t) {
  const int G = resolve_groups(ctx);
  if ((int)ctx->lbs.size() == G) return GJ_OK;
  destroy_groups(ctx);
  for (int g = 0; g < G; ++g) {
    int c0, n;
    group_range(ctx, G, g, &c0, &n);
    gj::LogregBatched* lb = nullptr;
    const int rc = gj::logreg_batched_create(t, n, &lb);
    if (rc) {
      destroy_groups(ctx);
      return fail(rc, "%s", gj::logreg_batched_error());
    }
    gj::logreg_batched_set_profile(lb, ctx->profile);
    gj::logreg_batched_set_chol_fp64(lb, ctx->chol_fp64);
    gj::logreg_batched_set_chol_cpw(lb, ctx->chol_cpw);
    gj::logreg_batched_set_pdl(lb, ctx->pdl);
    gj::logreg_batched_set_gemm_ksplit(lb, ctx->ksplit);
    gj::logreg_batched_set_fuse_r2x(lb, ctx->fuse_r2x);
    gj::logreg_batched_set_refine_iterates(lb, ctx->refine);
    // every group makes the automatic choices of the whole context, so that
    // results do not depend on the group count
    gj::logreg_batched_set_auto_chains(lb, ctx->C);
    ctx->lbs.push_back(lb);
  }
  if (G > 1) {
    for (int g = 0; g < G; ++g) {
      cudaStream_t s;
      if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
        destroy_groups(ctx);
        return fail(GJ_ECUDA, "stream creation failed");
      }
      ctx->gstreams.push_back(s);
    }
    for (int e = 0; e < G + 1; ++e) {
      cudaEvent_t ev;
      if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
        destroy_groups(ctx);
        return fail(GJ_ECUDA, "event creation failed");
      }
      ctx->gevents.push_back(ev);
    }
  }
  return GJ_OK;
}

}  // namespace

extern "C" {

int32_t gj_version(void) { return 100; }

const char* gj_last_error(void) { return g_last_error.c_str(); }

int32_t gj_create(const gj_target* target, int32_t sampler, int32_t precision,
                  int32_t num_chains, gj_ctx** out) {
  if (!out) return fail(GJ_EINVAL, "out is NULL");
  *out = nullptr;
  int st = check_target(target, precision);
  if (st) return st;
  if (sampler < GJ_SAMPLER_RMHMC || sampler > GJ_SAMPLER_LMCMONGE)
    return fail(GJ_EINVAL, "bad sampler");
  if (num_chains < 1) return fail(GJ_EINVAL, "num_chains must be >= 1");
  gj_ctx* c = new (std::nothrow) gj_ctx();
  if (!c) return fail(GJ_ENOMEM, "host allocation failed");
  c->target = *target;
  c->sampler = sampler;
  c->precision = precision;
  c->C = num_chains;
  c->logreg_path = 0;
  c->tpb = 64;
  c->profile = 0;
  c->loop_mode = 0;
  c->chol_fp64 = 1;
  c->chol_cpw = 0;
  c->groups = 0;
  c->pdl = 0;
  c->ksplit = 0;
  c->monge_warp = 1;
  c->fuse_r2x = 1;
  c->refine = 1;
  *out = c;
  return GJ_OK;
}

int32_t gj_destroy(gj_ctx* ctx) {
  if (!ctx) return GJ_OK;
  destroy_groups(ctx);
  delete ctx;
  return GJ_OK;
}

int32_t gj_set_option(gj_ctx* ctx, int32_t key, int64_t value) {
  if (!ctx) return fail(GJ_EINVAL, "ctx is NULL");
  if (key == GJ_OPT_LOGREG_PATH) {
    if (value < 0 || value > 4) return fail(GJ_EINVAL, "logreg path must be 0..4");
    ctx->logreg_path = (int)value;
    return GJ_OK;
  }
  if (key == GJ_OPT_LOOP) {
    if (value < 0 || value > 1) return fail(GJ_EINVAL, "loop mode must be 0 (graph) or 1 (host)");
    ctx->loop_mode = (int)value;
    return GJ_OK;
  }
  if (key == GJ_OPT_CHOL_FP64) {
    if (value < 0 || value > 1) return fail(GJ_EINVAL, "factorisation precision flag must be 0 or 1");
    ctx->chol_fp64 = (int)value;
    for (gj::LogregBatched* lb : ctx->lbs) gj::logreg_batched_set_chol_fp64(lb, ctx->chol_fp64);
    return GJ_OK;
  }
  if (key == GJ_OPT_CHOL_CHAINS_PER_WARP) {
    if (value != 0 && value != 1 && value != 2 && value != 4 && value != 8)
      return fail(GJ_EINVAL, "chains per warp must be 0 (automatic), 1, 2, 4 or 8");
    ctx->chol_cpw = (int)value;
    for (gj::LogregBatched* lb : ctx->lbs) gj::logreg_batched_set_chol_cpw(lb, ctx->chol_cpw);
    return GJ_OK;
  }
  if (key == GJ_OPT_PDL) {
    if (value < 0 || value > 1) return fail(GJ_EINVAL, "PDL flag must be 0 or 1");
    ctx->pdl = (int)value;
    for (gj::LogregBatched* lb : ctx->lbs) gj::logreg_batched_set_pdl(lb, ctx->pdl);
    return GJ_OK;
  }
  if (key == GJ_OPT_GEMM_KSPLIT) {
    if (value < 0 || value > 4) return fail(GJ_EINVAL, "K slices must be 0 (automatic) .. 4");
    ctx->ksplit = (int)value;
    for (gj::LogregBatched* lb : ctx->lbs) gj::logreg_batched_set_gemm_ksplit(lb, ctx->ksplit);
    return GJ_OK;
  }
  if (key == GJ_OPT_FUSE_R2X) {
    if (value < 0 || value > 1) return fail(GJ_EINVAL, "fused r2·X flag must be 0 or 1");
    ctx->fuse_r2x = (int)value;
    for (gj::LogregBatched* lb : ctx->lbs) gj::logreg_batched_set_fuse_r2x(lb, ctx->fuse_r2x);
    return GJ_OK;
  }
  if (key == GJ_OPT_REFINE_ITERATES) {
    if (value < 0 || value > 1) return fail(GJ_EINVAL, "refined iterate flag must be 0 or 1");
    ctx->refine = (int)value;
    for (gj::LogregBatched* lb : ctx->lbs) gj::logreg_batched_set_refine_iterates(lb, ctx->refine);
    return GJ_OK;
  }
  if (key == GJ_OPT_MONGE_WARP) {
    if (value < 0 || value > 1) return fail(GJ_EINVAL, "LMC-Monge warp flag must be 0 or 1");
    ctx->monge_warp = (int)value;
    return GJ_OK;
  }
  if (key == GJ_OPT_CHAIN_GROUPS) {
    if (value < 0 || value > 8) return fail(GJ_EINVAL, "chain groups must be 0 (automatic) .. 8");
    ctx->groups = (int)value;
    destroy_groups(ctx);  // rebuilt at the next step
    return GJ_OK;
  }
  if (key == GJ_OPT_THREADS_PER_BLOCK) {
    // the per-chain kernels are compiled for at most 128 threads per block
    if (value < 32 || value > 128 || (value % 32))
      return fail(GJ_EINVAL, "threads per block must be 32, 64, 96 or 128");
    ctx->tpb = (int)value;
    return GJ_OK;
  }
  return fail(GJ_EINVAL, "unknown option");
}

int32_t gj_init(gj_ctx* ctx, gj_chain_state* s, void* stream) {
  if (!ctx) return fail(GJ_EINVAL, "ctx is NULL");
  int st = check_state(s, ctx->C, false);
  if (st) return st;
  const gj::TargetDev t = gj::to_dev(ctx->target);
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  if (ctx->precision == GJ_FP64)
    e = gj::launch_logdensity_grad<double>(t, (const double*)s->position, s->logdensity,
                                           (double*)s->logdensity_grad, s->volume_adjustment,
                                           ctx->C, cs);
  else
    e = gj::launch_logdensity_grad<float>(t, (const float*)s->position, s->logdensity,
                                          (float*)s->logdensity_grad, s->volume_adjustment,
                                          ctx->C, cs);
  return cuda_status(e, "gj_init");
}

int32_t gj_rmhmc_step(gj_ctx* ctx, const gj_step_params* p, gj_chain_state* s, const void* z,
                      const double* u, gj_info* info, void* stream) {
  if (!ctx) return fail(GJ_EINVAL, "ctx is NULL");
  if (ctx->sampler != GJ_SAMPLER_RMHMC) return fail(GJ_EINVAL, "context is not an RMHMC context");
  int st = check_params(p);
  if (!st) st = check_state(s, ctx->C, false);
  if (st) return st;
  if (!z || !u) return fail(GJ_EINVAL, "z and u must be device arrays");
  if (p->integrator != GJ_IMPLICIT_MIDPOINT && p->integrator != GJ_GENERALIZED_LEAPFROG)
    return fail(GJ_EINVAL, "bad integrator");
  const gj::TargetDev t = gj::to_dev(ctx->target);
  const gj::StepDev sp = gj::to_dev(*p);
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  // dense-Fisher logistic regression in mixed precision: batched pipeline
  // (paths 0, 1, 2; 3 is one thread per chain, 4 one CTA per chain)
  if (ctx->precision == GJ_MIXED && t.family == GJ_LOGREG && t.metric == GJ_METRIC_DENSE_FISHER &&
      ctx->logreg_path != 3 && ctx->logreg_path != 4) {
    int rc = ensure_groups(ctx, t);
    if (rc) return rc;
    const int gemm = (ctx->logreg_path == 1) ? 1 : 2;
    // host-driven loop while profiling (events around each GEMM) or on request
    const bool graph = ctx->loop_mode == 0 && !ctx->profile;
    const int G = (int)ctx->lbs.size();
    const bool fork = graph && G > 1;
    if (fork && cudaEventRecord(ctx->gevents[0], cs) != cudaSuccess)
      return fail(GJ_ECUDA, "event record failed");
    const int d = t.d;
    for (int g = 0; g < G; ++g) {
      int c0, n;
      group_range(ctx, G, g, &c0, &n);
      cudaStream_t gsm = fork ? ctx->gstreams[g] : cs;
      if (fork && cudaStreamWaitEvent(gsm, ctx->gevents[0], 0) != cudaSuccess)
        return fail(GJ_ECUDA, "stream wait failed");
      float* pos = (float*)s->position + (size_t)c0 * d;
      float* grad = (float*)s->logdensity_grad + (size_t)c0 * d;
      double* ld = s->logdensity + c0;
      const float* zg = (const float*)z + (size_t)c0 * d;
      const double* ug = u + c0;
      const gj::InfoDev<float> ig = info_offset(gj::to_dev<float>(info), c0, d);
      rc = graph ? gj::logreg_batched_rmhmc_step_graph(ctx->lbs[g], sp, pos, grad, ld, zg, ug, ig,
                                                       gemm, gsm)
                 : gj::logreg_batched_rmhmc_step(ctx->lbs[g], sp, pos, grad, ld, zg, ug, ig, gemm,
                                                 gsm);
      if (rc) return fail(rc, "%s", gj::logreg_batched_error());
      if (fork && cudaEventRecord(ctx->gevents[1 + g], gsm) != cudaSuccess)
        return fail(GJ_ECUDA, "event record failed");
    }
    if (fork)
      for (int g = 0; g < G; ++g)
        if (cudaStreamWaitEvent(cs, ctx->gevents[1 + g], 0) != cudaSuccess)
          return fail(GJ_ECUDA, "stream wait failed");
    return GJ_OK;
  }
  cudaError_t e;
  // dense-Fisher logistic regression, one CTA per chain: the plain FP64 form
  // by default (path 0), either precision on request (path 4)
  if (t.family == GJ_LOGREG && t.metric == GJ_METRIC_DENSE_FISHER &&
      (ctx->logreg_path == 4 || (ctx->logreg_path == 0 && ctx->precision == GJ_FP64))) {
    const bool mixed = ctx->precision == GJ_MIXED;
    if (!gj::logreg_cta_supported(t.d, t.n, mixed, 0))
      return fail(GJ_ENOTSUP, "CTA-per-chain logistic regression needs d <= 64 and the chain's "
                              "shared memory within 227 KB");
    if (!mixed)
      e = gj::launch_logreg_cta<double>(GJ_SAMPLER_RMHMC, t, sp, (double*)s->position,
                                        (double*)s->logdensity_grad, s->logdensity, nullptr,
                                        (const double*)z, u, gj::to_dev<double>(info), ctx->C, cs);
    else
      e = gj::launch_logreg_cta<float>(GJ_SAMPLER_RMHMC, t, sp, (float*)s->position,
                                       (float*)s->logdensity_grad, s->logdensity, nullptr,
                                       (const float*)z, u, gj::to_dev<float>(info), ctx->C, cs);
    return cuda_status(e, "gj_rmhmc_step");
  }
  if (t.d > 32) return fail(GJ_ENOTSUP, "per-chain RMHMC supports d <= 32");
  if (ctx->precision == GJ_FP64)
    e = gj::launch_rmhmc_chain<double>(t, sp, (double*)s->position, (double*)s->logdensity_grad,
                                       s->logdensity, (const double*)z, u,
                                       gj::to_dev<double>(info), ctx->C, ctx->tpb, cs);
  else
    e = gj::launch_rmhmc_chain<float>(t, sp, (float*)s->position, (float*)s->logdensity_grad,
                                      s->logdensity, (const float*)z, u, gj::to_dev<float>(info),
                                      ctx->C, ctx->tpb, cs);
  return cuda_status(e, "gj_rmhmc_step");
}

int32_t gj_nuts_step(gj_ctx* ctx, const gj_nuts_params* p, gj_chain_state* s, const void* z,
                     const double* uniforms, int32_t uniforms_per_chain, gj_nuts_info* info,
                     void* stream) {
  if (!ctx) return fail(GJ_EINVAL, "ctx is NULL");
  if (!p) return fail(GJ_EINVAL, "params is NULL");
  if (p->max_num_doublings < 1 || p->max_num_doublings > 16)
    return fail(GJ_EINVAL, "max_num_doublings must be 1..16");
  if (p->criterion < 0 || p->criterion > 2) return fail(GJ_EINVAL, "criterion must be 0, 1 or 2");
  if (p->integrator != GJ_IMPLICIT_MIDPOINT && p->integrator != GJ_GENERALIZED_LEAPFROG)
    return fail(GJ_EINVAL, "bad integrator");
  if (!(p->step_size == p->step_size) || p->max_iters < 0)
    return fail(GJ_EINVAL, "bad step size or iteration cap");
  const int M = p->max_num_doublings;
  if (uniforms_per_chain < 2 * M + (1 << M) - 1)
    return fail(GJ_EINVAL, "uniforms_per_chain must be >= 2M + 2^M - 1");
  const bool lmc_like = ctx->sampler != GJ_SAMPLER_RMHMC;
  int st = check_state(s, ctx->C, lmc_like);
  if (st) return st;
  if (!z || !uniforms) return fail(GJ_EINVAL, "z and uniforms must be device arrays");
  const gj::TargetDev t = gj::to_dev(ctx->target);
  if (t.d > 32) return fail(GJ_ENOTSUP, "NUTS supports d <= 32");
  gj::StepDev sp{};
  sp.h = p->step_size;
  sp.L = 0;
  sp.integrator = p->integrator;
  sp.max_iters = p->max_iters;
  sp.tol = p->tol;
  sp.div_threshold = p->divergence_threshold;
  sp.alpha2 = p->alpha2;
  sp.inv_mass = p->inverse_mass;
  sp.alpha2_fix = p->alpha2_fix;
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  if (ctx->precision == GJ_FP64)
    e = gj::launch_nuts<double>(ctx->sampler, t, sp, M, p->criterion, (double*)s->position,
                                (double*)s->logdensity_grad, s->logdensity, s->volume_adjustment,
                                (const double*)z, uniforms, uniforms_per_chain,
                                gj::to_dev<double>(info), ctx->C, ctx->tpb, cs);
  else
    e = gj::launch_nuts<float>(ctx->sampler, t, sp, M, p->criterion, (float*)s->position,
                               (float*)s->logdensity_grad, s->logdensity, s->volume_adjustment,
                               (const float*)z, uniforms, uniforms_per_chain,
                               gj::to_dev<float>(info), ctx->C, ctx->tpb, cs);
  return cuda_status(e, "gj_nuts_step");
}

int32_t gj_lmc_step(gj_ctx* ctx, const gj_step_params* p, gj_chain_state* s, const void* z,
                    const double* u, gj_info* info, void* stream) {
  if (!ctx) return fail(GJ_EINVAL, "ctx is NULL");
  if (ctx->sampler != GJ_SAMPLER_LMC) return fail(GJ_EINVAL, "context is not an LMC context");
  int st = check_params(p);
  if (!st) st = check_state(s, ctx->C, true);
  if (st) return st;
  if (!z || !u) return fail(GJ_EINVAL, "z and u must be device arrays");
  const gj::TargetDev t = gj::to_dev(ctx->target);
  const gj::StepDev sp = gj::to_dev(*p);
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  // dense-Fisher logistic regression: one CTA per chain (d <= 64), unless the
  // thread-per-chain kernel is asked for (path 3)
  if (t.family == GJ_LOGREG && t.metric == GJ_METRIC_DENSE_FISHER && ctx->logreg_path != 3) {
    const bool mixed = ctx->precision == GJ_MIXED;
    if (!gj::logreg_cta_supported(t.d, t.n, mixed, 1))
      return fail(GJ_ENOTSUP, "CTA-per-chain dense LMC needs d <= 64 and the chain's shared "
                              "memory within 227 KB");
    if (!mixed)
      e = gj::launch_logreg_cta<double>(GJ_SAMPLER_LMC, t, sp, (double*)s->position,
                                        (double*)s->logdensity_grad, s->logdensity,
                                        s->volume_adjustment, (const double*)z, u,
                                        gj::to_dev<double>(info), ctx->C, cs);
    else
      e = gj::launch_logreg_cta<float>(GJ_SAMPLER_LMC, t, sp, (float*)s->position,
                                       (float*)s->logdensity_grad, s->logdensity,
                                       s->volume_adjustment, (const float*)z, u,
                                       gj::to_dev<float>(info), ctx->C, cs);
    return cuda_status(e, "gj_lmc_step");
  }
  if (t.d > 32) return fail(GJ_ENOTSUP, "dense LMC supports d <= 32");
  if (ctx->precision == GJ_FP64)
    e = gj::launch_lmc_chain<double>(t, sp, (double*)s->position, (double*)s->logdensity_grad,
                                     s->logdensity, s->volume_adjustment, (const double*)z, u,
                                     gj::to_dev<double>(info), ctx->C, ctx->tpb, cs);
  else
    e = gj::launch_lmc_chain<float>(t, sp, (float*)s->position, (float*)s->logdensity_grad,
                                    s->logdensity, s->volume_adjustment, (const float*)z, u,
                                    gj::to_dev<float>(info), ctx->C, ctx->tpb, cs);
  return cuda_status(e, "gj_lmc_step");
}

int32_t gj_lmcmonge_step(gj_ctx* ctx, const gj_step_params* p, gj_chain_state* s, const void* z,
                         const double* u, gj_info* info, void* stream) {
  if (!ctx) return fail(GJ_EINVAL, "ctx is NULL");
  if (ctx->sampler != GJ_SAMPLER_LMCMONGE)
    return fail(GJ_EINVAL, "context is not an LMC-Monge context");
  int st = check_params(p);
  if (!st) st = check_state(s, ctx->C, true);
  if (st) return st;
  if (!z || !u) return fail(GJ_EINVAL, "z and u must be device arrays");
  const gj::TargetDev t = gj::to_dev(ctx->target);
  const gj::StepDev sp = gj::to_dev(*p);
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  if (ctx->monge_warp && gj::monge_warp_supported(t)) {  // one warp per chain
    if (ctx->precision == GJ_MIXED)
      e = gj::launch_monge_warp<float>(t, sp, (float*)s->position, (float*)s->logdensity_grad,
                                       s->logdensity, s->volume_adjustment, (const float*)z, u,
                                       gj::to_dev<float>(info), ctx->C, cs);
    else
      e = gj::launch_monge_warp<double>(t, sp, (double*)s->position, (double*)s->logdensity_grad,
                                        s->logdensity, s->volume_adjustment, (const double*)z, u,
                                        gj::to_dev<double>(info), ctx->C, cs);
    return cuda_status(e, "gj_lmcmonge_step");
  }
  if (t.d > 128) return fail(GJ_ENOTSUP, "per-chain LMC-Monge supports d <= 128");
  if (ctx->precision == GJ_FP64)
    e = gj::launch_monge_chain<double>(t, sp, (double*)s->position, (double*)s->logdensity_grad,
                                       s->logdensity, s->volume_adjustment, (const double*)z, u,
                                       gj::to_dev<double>(info), ctx->C, ctx->tpb, cs);
  else
    e = gj::launch_monge_chain<float>(t, sp, (float*)s->position, (float*)s->logdensity_grad,
                                      s->logdensity, s->volume_adjustment, (const float*)z, u,
                                      gj::to_dev<float>(info), ctx->C, ctx->tpb, cs);
  return cuda_status(e, "gj_lmcmonge_step");
}

int32_t gj_stats(gj_ctx* ctx, int64_t* out, int32_t n) {
  if (!ctx || !out || n < 0) return fail(GJ_EINVAL, "bad arguments");
  int64_t v[11] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (!ctx->lbs.empty()) {
    for (gj::LogregBatched* lb : ctx->lbs) {
      const gj::LogregStats s = gj::logreg_batched_stats(lb);
      v[0] += s.evals;
      v[1] += s.gemm_launches;
      v[2] += s.other_launches;
      v[3] += (int64_t)s.gemm_flops;
      v[4] += (int64_t)s.gemm_ns;
      v[5] += s.chol_launches;
      v[6] += (int64_t)s.chol_flops;
      v[7] += (int64_t)s.chol_ns;
      v[8] += s.refine_launches;
      v[9] += (int64_t)s.refine_ns;
      v[10] += s.refine_fallbacks;
    }
  } else {
    v[2] = 1;  // the per-chain and warp-per-chain paths launch one kernel per step
  }
  const int m = n < 11 ? n : 11;
  for (int i = 0; i < m; ++i) out[i] = v[i];
  return m;
}

int32_t gj_profile(gj_ctx* ctx, int32_t on) {
  if (!ctx) return fail(GJ_EINVAL, "ctx is NULL");
  ctx->profile = on ? 1 : 0;
  for (gj::LogregBatched* lb : ctx->lbs) gj::logreg_batched_set_profile(lb, ctx->profile);
  return GJ_OK;
}

int32_t gj_gemm_split_bf16(int32_t impl, int32_t planes, int32_t M, int32_t N, int32_t K,
                           const float* A, const float* B, float* D, void* stream) {
  if (impl != 1 && impl != 2) return fail(GJ_EINVAL, "impl must be 1 (SIMT) or 2 (tcgen05)");
  if (planes != 2 && planes != 3) return fail(GJ_EINVAL, "planes must be 2 or 3");
  int rc = gj::gemm_split_test(impl, planes, M, N, K, A, B, D, static_cast<cudaStream_t>(stream));
  if (rc) return fail(rc, "%s", gj::logreg_batched_error());
  return GJ_OK;
}

int32_t gj_gemm_split_bf16_noalloc(int32_t impl, int32_t planes, int32_t M, int32_t N, int32_t K,
                                   const float* A, const float* B, float* D, void* stream) {
  int rc = gj::gemm_split_noalloc(impl, planes, M, N, K, A, B, D, static_cast<cudaStream_t>(stream));
  if (rc) return fail(rc, "%s", gj::gemm_noalloc_error());
  return GJ_OK;
}

int32_t gj_logdensity_grad(const gj_target* target, int32_t precision, int32_t C, const void* q,
                           double* ld, void* grad, void* stream) {
  int st = check_target(target, precision);
  if (st) return st;
  if (C < 1 || !q || !ld || !grad) return fail(GJ_EINVAL, "bad arrays");
  const gj::TargetDev t = gj::to_dev(*target);
  if (t.d > 128) return fail(GJ_ENOTSUP, "operator kernels support d <= 128");
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  cudaError_t e = precision == GJ_FP64
                      ? gj::launch_logdensity_grad<double>(t, (const double*)q, ld, (double*)grad,
                                                           nullptr, C, cs)
                      : gj::launch_logdensity_grad<float>(t, (const float*)q, ld, (float*)grad,
                                                          nullptr, C, cs);
  return cuda_status(e, "gj_logdensity_grad");
}

int32_t gj_hvp(const gj_target* target, int32_t precision, int32_t C, const void* q,
               const void* u, void* out, void* stream) {
  int st = check_target(target, precision);
  if (st) return st;
  if (C < 1 || !q || !u || !out) return fail(GJ_EINVAL, "bad arrays");
  const gj::TargetDev t = gj::to_dev(*target);
  if (t.d > 128) return fail(GJ_ENOTSUP, "operator kernels support d <= 128");
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  cudaError_t e = precision == GJ_FP64
                      ? gj::launch_hvp<double>(t, (const double*)q, (const double*)u,
                                               (double*)out, C, cs)
                      : gj::launch_hvp<float>(t, (const float*)q, (const float*)u, (float*)out, C,
                                              cs);
  return cuda_status(e, "gj_hvp");
}

int32_t gj_metric(const gj_target* target, int32_t precision, int32_t C, const void* q,
                  void* out, void* stream) {
  int st = check_target(target, precision);
  if (st) return st;
  if (C < 1 || !q || !out) return fail(GJ_EINVAL, "bad arrays");
  const gj::TargetDev t = gj::to_dev(*target);
  if (t.d > 32) return fail(GJ_ENOTSUP, "metric operator supports d <= 32");
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  cudaError_t e = precision == GJ_FP64
                      ? gj::launch_metric<double>(t, (const double*)q, (double*)out, C, cs)
                      : gj::launch_metric<float>(t, (const float*)q, (float*)out, C, cs);
  return cuda_status(e, "gj_metric");
}

int32_t gj_metric_vjp(const gj_target* target, int32_t precision, int32_t C, const void* q,
                      const void* w, void* out, void* stream) {
  int st = check_target(target, precision);
  if (st) return st;
  if (C < 1 || !q || !w || !out) return fail(GJ_EINVAL, "bad arrays");
  const gj::TargetDev t = gj::to_dev(*target);
  if (t.d > 32) return fail(GJ_ENOTSUP, "metric adjoint supports d <= 32");
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  cudaError_t e = precision == GJ_FP64
                      ? gj::launch_metric_vjp<double>(t, (const double*)q, (const double*)w,
                                                      (double*)out, C, cs)
                      : gj::launch_metric_vjp<float>(t, (const float*)q, (const float*)w,
                                                     (float*)out, C, cs);
  return cuda_status(e, "gj_metric_vjp");
}

int32_t gj_logreg_gl_transition_jvp(const gj_target* target, int32_t C, const double* q0,
                                    const double* z, double step_size, double metric_reg,
                                    int32_t num_integration_steps, int32_t kp, int32_t kq,
                                    int32_t tangents, double* out, void* stream) {
  int st = check_target(target, GJ_FP64);
  if (st) return st;
  if (target->family != GJ_LOGREG) return fail(GJ_EINVAL, "the differentiated trajectory is for logistic regression");
  if (target->dim > 64) return fail(GJ_ENOTSUP, "the differentiated trajectory supports d <= 64");
  if (gj::gl_trajectory_smem(target->dim, (int)target->n_data, tangents) > 227 * 1024)
    return fail(GJ_ENOTSUP, "the differentiated trajectory's per-chain shared memory exceeds 227 KB "
                            "(d = 64 allows N <= 2000 with tangents)");
  if (C < 1 || !q0 || !z || !out || kp < 1 || kq < 1 || num_integration_steps < 0 ||
      !(metric_reg > 0) || !(step_size == step_size))
    return fail(GJ_EINVAL, "bad arguments");
  cudaError_t e = gj::launch_gl_trajectory_jvp(
      static_cast<const double*>(target->X), static_cast<const double*>(target->y), target->n_data,
      target->dim, target->p0, C, q0, z, step_size, metric_reg, num_integration_steps, kp, kq,
      tangents, out, static_cast<cudaStream_t>(stream));
  return cuda_status(e, "gj_logreg_gl_transition_jvp");
}

int32_t gj_fma_peak(int32_t precision, double* tflops, void* stream) {
  if (precision != GJ_FP64 && precision != GJ_MIXED) return fail(GJ_EINVAL, "bad precision");
  if (!tflops) return fail(GJ_EINVAL, "tflops is NULL");
  return cuda_status(gj::fma_peak(precision == GJ_FP64, tflops, static_cast<cudaStream_t>(stream)),
                     "gj_fma_peak");
}

// ---------------------------------------------------------------------------
// ChEES: the LMC-Monge proposal's derivative in α², cross-chain statistics
// ---------------------------------------------------------------------------
int32_t gj_lmcmonge_alpha2_jvp(const gj_target* target, int32_t precision, int32_t num_chains,
                               const gj_step_params* p, const void* position, const void* z,
                               void* proposal_position, void* proposal_alpha2_tangent,
                               void* stream) {
  int st = check_target(target, precision);
  if (!st) st = check_params(p);
  if (st) return st;
  const gj::TargetDev t = gj::to_dev(*target);
  if (!gj::monge_alpha2_jvp_supported(t))
    return fail(GJ_ENOTSUP, "the α² derivative supports the funnel and the hierarchical Gaussian, d <= 256");
  if (num_chains < 1 || !position || !z || !proposal_alpha2_tangent)
    return fail(GJ_EINVAL, "bad arguments");
  const gj::StepDev sp = gj::to_dev(*p);
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  if (precision == GJ_FP64)
    e = gj::launch_monge_alpha2_jvp<double>(t, sp, static_cast<const double*>(position),
                                            static_cast<const double*>(z),
                                            static_cast<double*>(proposal_position),
                                            static_cast<double*>(proposal_alpha2_tangent),
                                            num_chains, cs);
  else
    e = gj::launch_monge_alpha2_jvp<float>(t, sp, static_cast<const float*>(position),
                                           static_cast<const float*>(z),
                                           static_cast<float*>(proposal_position),
                                           static_cast<float*>(proposal_alpha2_tangent),
                                           num_chains, cs);
  return cuda_status(e, "gj_lmcmonge_alpha2_jvp");
}

int64_t gj_chees_workspace_size(int32_t num_chains, int32_t dim) {
  if (num_chains < 1 || dim < 1) return -1;
  return (int64_t)gj::chees_workspace_bytes(num_chains, dim);
}

int32_t gj_chees_statistics(int32_t precision, int32_t num_chains, int32_t dim,
                            const void* proposal_position, const void* proposal_velocity,
                            const void* initial_position, const void* proposal_alpha2_tangent,
                            const double* acceptance_rate, const uint8_t* is_divergent,
                            void* workspace, double* out, void* stream) {
  if (precision != GJ_FP64 && precision != GJ_MIXED) return fail(GJ_EINVAL, "bad precision");
  if (num_chains < 1 || dim < 1) return fail(GJ_EINVAL, "num_chains and dim must be >= 1");
  if (!proposal_position || !proposal_velocity || !initial_position || !acceptance_rate ||
      !workspace || !out)
    return fail(GJ_EINVAL, "a required array is NULL");
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  double* w = static_cast<double*>(workspace);
  cudaError_t e;
  if (precision == GJ_FP64)
    e = gj::chees_statistics<double>(num_chains, dim, static_cast<const double*>(proposal_position),
                                     static_cast<const double*>(proposal_velocity),
                                     static_cast<const double*>(initial_position),
                                     static_cast<const double*>(proposal_alpha2_tangent),
                                     acceptance_rate, is_divergent, w, out, cs);
  else
    e = gj::chees_statistics<float>(num_chains, dim, static_cast<const float*>(proposal_position),
                                    static_cast<const float*>(proposal_velocity),
                                    static_cast<const float*>(initial_position),
                                    static_cast<const float*>(proposal_alpha2_tangent),
                                    acceptance_rate, is_divergent, w, out, cs);
  return cuda_status(e, "gj_chees_statistics");
}

// ---------------------------------------------------------------------------
// batches of independent dense-Fisher logistic-regression posteriors
// ---------------------------------------------------------------------------
}  // extern "C"

struct gj_batch {
  int B, C, S;
  int one_graph;  // GJ_OPT_BATCH_GRAPH: 0 stream pool, 1 a branch per posterior, 2 grouped
  int buckets;    // GJ_OPT_BATCH_BUCKETS (0 = automatic)
  gj::LogregBatchGraph* bg;
  std::vector<gj::LogregBatched*> lbs;
  std::vector<int> dims;
  std::vector<size_t> pos_off;  // [B + 1] offsets of each posterior's [C, d_b] block
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> joins;
  cudaEvent_t fork;
};

namespace {

void batch_free(gj_batch* b) {
  gj::logreg_batch_graph_destroy(b->bg);
  for (gj::LogregBatched* lb : b->lbs) gj::logreg_batched_destroy(lb);
  for (cudaStream_t s : b->streams) cudaStreamDestroy(s);
  for (cudaEvent_t e : b->joins) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  delete b;
}

}  // namespace

extern "C" {

int32_t gj_batch_create(const gj_target* targets, int32_t num_posteriors,
                        int32_t chains_per_posterior, int32_t num_streams, gj_batch** out) {
  if (!out) return fail(GJ_EINVAL, "out is NULL");
  *out = nullptr;
  if (!targets || num_posteriors < 1) return fail(GJ_EINVAL, "need at least one target");
  if (chains_per_posterior < 1) return fail(GJ_EINVAL, "chains_per_posterior must be >= 1");
  if (num_streams < 1 || num_streams > 64) return fail(GJ_EINVAL, "num_streams must be 1..64");
  for (int b = 0; b < num_posteriors; ++b) {
    const gj_target& t = targets[b];
    int st = check_target(&t, GJ_MIXED);
    if (st) return st;
    if (t.family != GJ_LOGREG || t.metric != GJ_METRIC_DENSE_FISHER)
      return fail(GJ_EINVAL, "a batch holds dense-Fisher logistic-regression targets");
    if (t.dim > 128) return fail(GJ_ENOTSUP, "batched logistic regression supports d <= 128");
  }
  gj_batch* b = new (std::nothrow) gj_batch();
  if (!b) return fail(GJ_ENOMEM, "host allocation failed");
  b->B = num_posteriors;
  b->C = chains_per_posterior;
  b->one_graph = 2;
  b->buckets = 0;
  b->bg = nullptr;
  b->S = num_streams < num_posteriors ? num_streams : num_posteriors;
  b->fork = nullptr;
  b->pos_off.push_back(0);
  for (int i = 0; i < num_posteriors; ++i) {
    gj::LogregBatched* lb = nullptr;
    const int rc = gj::logreg_batched_create(gj::to_dev(targets[i]), b->C, &lb);
    if (rc) {
      const std::string msg = gj::logreg_batched_error();
      batch_free(b);
      return fail(rc, "%s", msg.c_str());
    }
    b->lbs.push_back(lb);
    b->dims.push_back(targets[i].dim);
    b->pos_off.push_back(b->pos_off.back() + (size_t)b->C * targets[i].dim);
  }
  bool ok = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) == cudaSuccess;
  for (int s = 0; s < b->S && ok; ++s) {
    cudaStream_t st;
    cudaEvent_t ev;
    ok = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess;
    if (ok) b->streams.push_back(st);
    ok = ok && cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) == cudaSuccess;
    if (ok) b->joins.push_back(ev);
  }
  if (!ok) {
    batch_free(b);
    return fail(GJ_ECUDA, "stream or event creation failed");
  }
  *out = b;
  return GJ_OK;
}

int32_t gj_batch_destroy(gj_batch* b) {
  if (b) batch_free(b);
  return GJ_OK;
}

int32_t gj_batch_set_option(gj_batch* b, int32_t key, int64_t value) {
  if (!b) return fail(GJ_EINVAL, "batch is NULL");
  if (key == GJ_OPT_CHOL_FP64) {
    if (value < 0 || value > 1) return fail(GJ_EINVAL, "factorisation precision flag must be 0 or 1");
    for (gj::LogregBatched* lb : b->lbs) gj::logreg_batched_set_chol_fp64(lb, (int)value);
    return GJ_OK;
  }
  if (key == GJ_OPT_CHOL_CHAINS_PER_WARP) {
    if (value != 0 && value != 1 && value != 2 && value != 4 && value != 8)
      return fail(GJ_EINVAL, "chains per warp must be 0 (automatic), 1, 2, 4 or 8");
    for (gj::LogregBatched* lb : b->lbs) gj::logreg_batched_set_chol_cpw(lb, (int)value);
    return GJ_OK;
  }
  if (key == GJ_OPT_GEMM_KSPLIT) {
    if (value < 0 || value > 4) return fail(GJ_EINVAL, "K slices must be 0 (automatic) .. 4");
    for (gj::LogregBatched* lb : b->lbs) gj::logreg_batched_set_gemm_ksplit(lb, (int)value);
    return GJ_OK;
  }
  if (key == GJ_OPT_FUSE_R2X) {
    if (value < 0 || value > 1) return fail(GJ_EINVAL, "fused r2·X flag must be 0 or 1");
    for (gj::LogregBatched* lb : b->lbs) gj::logreg_batched_set_fuse_r2x(lb, (int)value);
    return GJ_OK;
  }
  if (key == GJ_OPT_REFINE_ITERATES) {
    if (value < 0 || value > 1) return fail(GJ_EINVAL, "refined iterate flag must be 0 or 1");
    for (gj::LogregBatched* lb : b->lbs) gj::logreg_batched_set_refine_iterates(lb, (int)value);
    return GJ_OK;
  }
  if (key == GJ_OPT_BATCH_BUCKETS) {
    if (value < 0 || value > 256) return fail(GJ_EINVAL, "batch buckets must be 0 (automatic) .. 256");
    b->buckets = (int)value;
    if (b->bg) gj::logreg_batch_graph_set_grouped(b->bg, b->one_graph == 2, b->buckets);
    return GJ_OK;
  }
  if (key == GJ_OPT_BATCH_GRAPH) {
    if (value < 0 || value > 2) return fail(GJ_EINVAL, "batch graph mode must be 0, 1 or 2");
    b->one_graph = (int)value;
    if (b->bg) gj::logreg_batch_graph_set_grouped(b->bg, b->one_graph == 2, b->buckets);
    return GJ_OK;
  }
  return fail(GJ_EINVAL, "unknown batch option");
}

int32_t gj_batch_rmhmc_step(gj_batch* b, const gj_step_params* p, gj_chain_state* s,
                            const float* z, const double* u, gj_info* info, void* stream) {
  if (!b) return fail(GJ_EINVAL, "batch is NULL");
  int st = check_params(p);
  if (!st) st = check_state(s, b->B * b->C, false);
  if (st) return st;
  if (!z || !u) return fail(GJ_EINVAL, "z and u must be device arrays");
  if (p->integrator != GJ_IMPLICIT_MIDPOINT && p->integrator != GJ_GENERALIZED_LEAPFROG)
    return fail(GJ_EINVAL, "bad integrator");
  const gj::StepDev sp = gj::to_dev(*p);
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  const gj::InfoDev<float> inf = gj::to_dev<float>(info);
  if (b->one_graph) {  // one graph launch: grouped launches or a branch per posterior
    if (!b->bg) {
      const int rc = gj::logreg_batch_graph_create(b->lbs.data(), b->B, b->C, b->pos_off.data(),
                                                   &b->bg);
      if (rc) return fail(rc, "%s", gj::logreg_batched_error());
      gj::logreg_batch_graph_set_grouped(b->bg, b->one_graph == 2, b->buckets);
    }
    const int rc = gj::logreg_batch_graph_step(b->bg, sp, (float*)s->position,
                                               (float*)s->logdensity_grad, s->logdensity, z, u,
                                               inf, 2, cs);
    if (rc) return fail(rc, "%s", gj::logreg_batched_error());
    return GJ_OK;
  }
  if (cudaEventRecord(b->fork, cs) != cudaSuccess) return fail(GJ_ECUDA, "event record failed");
  for (int k = 0; k < b->S; ++k)
    if (cudaStreamWaitEvent(b->streams[k], b->fork, 0) != cudaSuccess)
      return fail(GJ_ECUDA, "stream wait failed");
  for (int i = 0; i < b->B; ++i) {
    const size_t po = b->pos_off[i], co = (size_t)i * b->C;
    gj::InfoDev<float> ig = info_offset(inf, co, 0);
    if (inf.momentum) ig.momentum = inf.momentum + po;
    if (inf.prop_q) ig.prop_q = inf.prop_q + po;
    if (inf.prop_v) ig.prop_v = inf.prop_v + po;
    const int rc = gj::logreg_batched_rmhmc_step_graph(
        b->lbs[i], sp, (float*)s->position + po, (float*)s->logdensity_grad + po,
        s->logdensity + co, z + po, u + co, ig, 2, b->streams[i % b->S]);
    if (rc) return fail(rc, "%s", gj::logreg_batched_error());
  }
  for (int k = 0; k < b->S; ++k) {
    if (cudaEventRecord(b->joins[k], b->streams[k]) != cudaSuccess ||
        cudaStreamWaitEvent(cs, b->joins[k], 0) != cudaSuccess)
      return fail(GJ_ECUDA, "event join failed");
  }
  return GJ_OK;
}

int32_t gj_set_gemm_accumulators(int32_t max_ranges) {
  if (max_ranges != 1 && max_ranges != 2 && max_ranges != 4)
    return fail(GJ_EINVAL, "K-range accumulators must be 1, 2 or 4");
  gj::gemm_tc_set_accumulators(max_ranges);
  return GJ_OK;
}

int32_t gj_set_gemm_tiling(int32_t tile_n_wide, int32_t two_ctas_per_sm) {
  if (tile_n_wide != 0 && tile_n_wide != 64 && tile_n_wide != 128)
    return fail(GJ_EINVAL, "tile width must be 0 (automatic), 64 or 128");
  if (two_ctas_per_sm < -1 || two_ctas_per_sm > 1)
    return fail(GJ_EINVAL, "two_ctas_per_sm must be -1 (automatic), 0 or 1");
  gj::gemm_tc_set_tuning(tile_n_wide, two_ctas_per_sm);
  return GJ_OK;
}

}  // extern "C"
