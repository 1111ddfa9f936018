// LMC on a Monge patch, one WARP per chain, float32 state (mixed precision).
//
// Restates lmcmonge/lmc.py:151-236 (kernel: L, normalised gradient, weighted
// gradient, two HVPs, velocity draw, momentum), lmc_proposal :472-536,
// lmcmonge/integrators.py:63-155 (lan_integrator.one_step) and :158-194
// (half_step_omega), lmcmonge/metrics.py:155-197,267-284.
//
// Layout: element i of a chain's d-vector lives in lane (i % 32), register
// slot (i / 32); E slots per lane cover d <= 32·E.  Position, gradient and z
// are read/written row-major [C, d] (lane-contiguous, coalesced).  Every dot
// product is a warp-shuffle reduction; no shared memory.  The velocity draw
// uses the O(d) closed-form Cholesky factor of diag(M⁻¹) − α²·w·wᵀ (rank-one
// modification, Gill, Golub, Murray & Saunders 1974) instead of the
// reference's dense d x d Cholesky (lmcmonge/metrics.py:162-166).
// FP64: the volume adjustment J across transitions (a transition's
// increments are summed in FP32), the log density at the proposal and the
// Hamiltonian difference; nothing in the step loop runs on the FP64 pipe.
#include "chain_kernels.cuh"

namespace gj {

namespace {

template <int E>
struct WVec {
  float x[E];
};

template <int E>
__device__ __forceinline__ float wdot(const WVec<E>& a, const WVec<E>& b) {
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < E; ++k) s = fmaf(a.x[k], b.x[k], s);
  return warp_sum(s);
}

// broadcast element i (runtime) of a warp vector to all lanes
template <int E>
__device__ __forceinline__ float wget(const WVec<E>& a, int i) {
  const int slot = i >> 5, lane = i & 31;
  float v = 0.f;
#pragma unroll
  for (int k = 0; k < E; ++k)
    if (k == slot) v = a.x[k];
  return __shfl_sync(0xffffffffu, v, lane);
}

// warp-level target: log density + gradient and HVP for funnel / hier.
// The scale constants are precomputed once per transition: on GB300 an FP64
// division or logarithm inside the step loop costs more than the whole FP32
// step (the FP64 pipe was 85 % busy with them in the loop).
struct WarpTarget {
  TargetDev t;
  int lane;
  float inv_a2, inv_b2;   // funnel: 1/σ² (a); hier: 1/σ_μ² (a), 1/σ_v² (b)
  double inv_a2d, inv_b2d;  // the same in FP64, for the log density
  double ld_const;          // the log density's constant terms
};

__device__ inline WarpTarget make_warp_target(const TargetDev& t, int lane) {
  WarpTarget W;
  W.t = t;
  W.lane = lane;
  if (t.family == GJ_FUNNEL) {
    W.inv_a2d = 1.0 / (t.p0 * t.p0);
    W.inv_b2d = 0.0;
    W.inv_a2 = float(W.inv_a2d);
    W.inv_b2 = 0.f;
    W.ld_const = -log(t.p0) - 0.5 * kLog2Pi - (t.d - 1) * 0.5 * kLog2Pi;
  } else {
    const int J = t.n;
    const float* sg = static_cast<const float*>(t.s);
    double c = 0.0;
    for (int i = lane; i < J; i += 32) c += -log(double(sg[i])) - 0.5 * kLog2Pi;
    c = warp_sum(c);
    W.inv_a2d = 1.0 / (t.p0 * t.p0);
    W.inv_b2d = 1.0 / (t.p1 * t.p1);
    W.inv_a2 = float(W.inv_a2d);
    W.inv_b2 = float(W.inv_b2d);
    W.ld_const = c - J * 0.5 * kLog2Pi - log(t.p0) - 0.5 * kLog2Pi - log(t.p1) - 0.5 * kLog2Pi;
  }
  return W;
}

// funnel: v = θ[d−1]
// The FP64 log density is formed only when need_ld (the proposal's, after
// the last step); the gradient is FP32.
template <int E>
__device__ double w_logdensity_grad(const WarpTarget& W, const WVec<E>& q, WVec<E>& g, float* sx_out,
                                    bool need_ld = true) {
  const TargetDev& t = W.t;
  const int d = t.d;
  if (t.family == GJ_FUNNEL) {
    const float v = wget<E>(q, d - 1);
    const float ev = expf(-v);
    float sx = 0.f;
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int i = W.lane + 32 * k;
      const float x = (i < d - 1) ? q.x[k] : 0.f;
      sx = fmaf(x, x, sx);
    }
    sx = warp_sum(sx);
    const float gv = -v * W.inv_a2 - 0.5f * float(d - 1) + 0.5f * ev * sx;
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int i = W.lane + 32 * k;
      g.x[k] = (i < d - 1) ? -q.x[k] * ev : ((i == d - 1) ? gv : 0.f);
    }
    *sx_out = sx;
    if (!need_ld) return 0.0;
    return W.ld_const - 0.5 * double(v) * double(v) * W.inv_a2d - 0.5 * double(ev) * double(sx) -
           (d - 1) * 0.5 * double(v);
  }
  // hierarchical Gaussian: θ = [θ_1..θ_J, μ, v]
  const int J = t.n;
  const float* y = static_cast<const float*>(t.y);
  const float* sg = static_cast<const float*>(t.s);
  const float mu = wget<E>(q, J), v = wget<E>(q, J + 1);
  const float ev = expf(-v);
  float sr = 0.f, srr = 0.f;
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const int i = W.lane + 32 * k;
    if (i < J) {
      const float r = q.x[k] - mu;
      const float e = y[i] - q.x[k];
      const float is2 = 1.f / (sg[i] * sg[i]);
      g.x[k] = e * is2 - r * ev;
      sr += r;
      srr = fmaf(r, r, srr);
    }
  }
  sr = warp_sum(sr);
  srr = warp_sum(srr);
  const float gmu = sr * ev - mu * W.inv_a2;
  const float gvv = 0.5f * ev * srr - 0.5f * J - v * W.inv_b2;
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const int i = W.lane + 32 * k;
    if (i == J) g.x[k] = gmu;
    if (i == J + 1) g.x[k] = gvv;
    if (i > J + 1) g.x[k] = 0.f;
  }
  *sx_out = srr;
  if (!need_ld) return 0.0;
  double se = 0.0;  // Σ (y_j − θ_j)² / σ_j², in FP64 as the initial log density
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const int i = W.lane + 32 * k;
    if (i < J) {
      const double e = double(y[i]) - double(q.x[k]);
      se += e * e / (double(sg[i]) * double(sg[i]));
    }
  }
  se = warp_sum(se);
  return W.ld_const - 0.5 * se - 0.5 * double(ev) * double(srr) - J * 0.5 * double(v) -
         0.5 * double(mu) * double(mu) * W.inv_a2d - 0.5 * double(v) * double(v) * W.inv_b2d;
}

// Hessian-vector product; `sx` is the Σx² (funnel) / Σr² (hier) of the
// last gradient evaluation at the same q.
template <int E>
__device__ void w_hvp(const WarpTarget& W, const WVec<E>& q, const WVec<E>& u, float sx, WVec<E>& out) {
  const TargetDev& t = W.t;
  const int d = t.d;
  if (t.family == GJ_FUNNEL) {
    const float v = wget<E>(q, d - 1);
    const float ev = expf(-v);
    const float uv = wget<E>(u, d - 1);
    float xu = 0.f;
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int i = W.lane + 32 * k;
      if (i < d - 1) xu = fmaf(q.x[k], u.x[k], xu);
    }
    xu = warp_sum(xu);
    const float ov = ev * xu + (-W.inv_a2 - 0.5f * ev * sx) * uv;
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int i = W.lane + 32 * k;
      out.x[k] = (i < d - 1) ? ev * (-u.x[k] + q.x[k] * uv) : ((i == d - 1) ? ov : 0.f);
    }
    return;
  }
  const int J = t.n;
  const float* sg = static_cast<const float*>(t.s);
  const float mu = wget<E>(q, J), v = wget<E>(q, J + 1);
  const float ev = expf(-v);
  const float um = wget<E>(u, J), uv = wget<E>(u, J + 1);
  float sr = 0.f, sut = 0.f, sru = 0.f;
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const int i = W.lane + 32 * k;
    if (i < J) {
      const float r = q.x[k] - mu;
      sr += r;
      sut += u.x[k];
      sru = fmaf(r, u.x[k], sru);
      out.x[k] = -(1.f / (sg[i] * sg[i]) + ev) * u.x[k] + ev * um + r * ev * uv;
    }
  }
  sr = warp_sum(sr);
  sut = warp_sum(sut);
  sru = warp_sum(sru);
  const float om = ev * sut + (-float(J) * ev - W.inv_a2) * um - ev * sr * uv;
  const float ovv = ev * sru - ev * sr * um + (-0.5f * ev * sx - W.inv_b2) * uv;
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const int i = W.lane + 32 * k;
    if (i == J) out.x[k] = om;
    if (i == J + 1) out.x[k] = ovv;
    if (i > J + 1) out.x[k] = 0.f;
  }
}

// half_step_omega (lmcmonge/integrators.py:158-194), im = diag(M⁻¹).  dJ
// accumulates this transition's volume-term increments in FP32 (each is
// ≈ 1e-3; 4 per step); the caller adds the sum to the FP64 J once.
template <int E>
__device__ void w_half(float a2, WVec<E>& v, float* dJ, const WVec<E>& gn, const WVec<E>& hv, float L,
                       const WVec<E>& im, const WVec<E>& Hdl, float eps, int fix) {
  WVec<E> dl_ig, igH;
#pragma unroll
  for (int k = 0; k < E; ++k) {
    dl_ig.x[k] = im.x[k] * gn.x[k];
    igH.x[k] = im.x[k] * Hdl.x[k];
  }
  // log|det1| and log|1 − ½εα²(Hdl·v)| as FP32 log1p of the small terms
  // (det1 is an FP32 value, so an FP64 logarithm adds nothing)
  const float x1 = 0.5f * eps * a2 * wdot<E>(hv, dl_ig);
  const float det1 = 1.f + x1;
  *dJ -= x1 > -1.f ? log1pf(x1) : logf(fabsf(det1));
  const float sL = sqrtf(L);
  // dphi·dl_ig with dphi = −dl + α² Hdl_ig / sL
  float pd = 0.f;
#pragma unroll
  for (int k = 0; k < E; ++k) pd = fmaf(-gn.x[k] + a2 * Hdl.x[k] / sL, dl_ig.x[k], pd);
  pd = warp_sum(pd);
  WVec<E> vt;
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const float dphi_ig = -dl_ig.x[k] + a2 * igH.x[k] / sL;
    vt.x[k] = v.x[k] - 0.5f * eps * sL * (dphi_ig - a2 * pd * dl_ig.x[k]);
  }
  float corr = 0.5f * eps * wdot<E>(vt, hv) / det1;
  if (fix) corr *= a2;
#pragma unroll
  for (int k = 0; k < E; ++k) v.x[k] = vt.x[k] - corr * dl_ig.x[k];
  const float x2 = -0.5f * eps * a2 * wdot<E>(Hdl, v);
  *dJ += x2 > -1.f ? log1pf(x2) : logf(fabsf(1.f + x2));
}

// inclusive warp scan (ascending lane order)
__device__ __forceinline__ float warp_incl_scan(float x, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const float y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  return x;
}
// inclusive warp scan in descending lane order (suffix sums)
__device__ __forceinline__ float warp_incl_rscan(float x, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const float y = __shfl_down_sync(0xffffffffu, x, o);
    if (lane + o < 32) x += y;
  }
  return x;
}

// three 256-thread CTAs per SM (at most 85 registers a thread): the kernel
// is bound by the latency of its warp reductions, and 24 warps per SM hide
// it better than 16 (D = 100 ran 0.28 ms per transition at 80 registers,
// 0.36 ms at the 120 the compiler picks unbounded)
template <int E>
__global__ void __launch_bounds__(256, 3) monge_warp_kernel(TargetDev t, StepDev sp, float* pos,
                                                         float* grad, double* logdens, double* vol,
                                                         const float* z, const double* uacc,
                                                         InfoDev<float> info, int C) {
  const int lane = threadIdx.x & 31;
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (c >= C) return;  // whole warp exits together
  const int d = t.d;
  const WarpTarget W = make_warp_target(t, lane);
  const float a2 = float(sp.alpha2);
  const float eps = float(sp.h);
  const float* imv = static_cast<const float*>(sp.inv_mass);
  WVec<E> q, g, im, gn, Hdl, hv, v;
  double slm_part = 0.0;
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const int i = lane + 32 * k;
    const bool in = i < d;
    q.x[k] = in ? pos[(size_t)c * d + i] : 0.f;
    g.x[k] = in ? grad[(size_t)c * d + i] : 0.f;
    im.x[k] = in ? (imv ? imv[i] : 1.f) : 0.f;
    if (in) slm_part += -double(logf(im.x[k]));  // cancels in H1 − H0
  }
  const double slm = warp_sum(slm_part);  // Σ log M
  const double ld0 = logdens[c];
  const double J0 = vol[c];
  float sx;
  // ---- setup (lmc.py:177-208)
  float L = 0.f;
#pragma unroll
  for (int k = 0; k < E; ++k) L = fmaf(im.x[k] * g.x[k], g.x[k], L);
  L = 1.f + a2 * warp_sum(L);
  float sL = sqrtf(L);
  {
    // Σx² at the current q for the HVPs (one extra gradient pass is avoided by
    // recomputing only the reduction)
    WVec<E> gtmp;
    (void)w_logdensity_grad<E>(W, q, gtmp, &sx, false);
  }
  WVec<E> dl_ig;
#pragma unroll
  for (int k = 0; k < E; ++k) {
    gn.x[k] = g.x[k] / sL;
    dl_ig.x[k] = im.x[k] * gn.x[k];
  }
  w_hvp<E>(W, q, dl_ig, sx, Hdl);
#pragma unroll
  for (int k = 0; k < E; ++k) Hdl.x[k] /= sL;
  // ---- velocity: closed-form factor (τ_j = 1/L + α² Σ_{k≥j} u_k², u = w/sqrt(M⁻¹))
  {
    WVec<E> u, zz;
    float tot_after = 0.f;  // Σ over slots > k of u²
    float tau[E], taun[E];
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int i = lane + 32 * k;
      u.x[k] = (i < d) ? dl_ig.x[k] * rsqrtf(im.x[k]) : 0.f;
      zz.x[k] = (i < d) ? z[(size_t)c * d + i] : 0.f;
    }
#pragma unroll
    for (int k = E - 1; k >= 0; --k) {
      const float u2 = u.x[k] * u.x[k];
      const float r = warp_incl_rscan(u2, lane);
      const float suf = r + tot_after;  // Σ_{j≥i}
      tau[k] = 1.f / L + a2 * suf;
      taun[k] = tau[k] - a2 * u2;
      tot_after += __shfl_sync(0xffffffffu, r, 0);
    }
    float pre_before = 0.f;  // Σ over slots < k
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int i = lane + 32 * k;
      const float tk = (i < d) ? u.x[k] * zz.x[k] * rsqrtf(tau[k] * taun[k]) : 0.f;
      const float incl = warp_incl_scan(tk, lane);
      const float pre = pre_before + incl - tk;  // Σ_{j<i}
      const float y = sqrtf(taun[k] / tau[k]) * zz.x[k] - a2 * u.x[k] * pre;
      v.x[k] = (i < d) ? sqrtf(im.x[k]) * y : 0.f;
      pre_before += __shfl_sync(0xffffffffu, incl, 31);
      if (info.momentum && i < d) info.momentum[(size_t)c * d + i] = v.x[k];
    }
  }
  w_hvp<E>(W, q, v, sx, hv);
#pragma unroll
  for (int k = 0; k < E; ++k) hv.x[k] /= sL;
  auto kinetic = [&](float Lc) -> double {  // lmcmonge/metrics.py:168-186
    float vmv = 0.f, vg = 0.f;
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const float m = (im.x[k] > 0.f) ? 1.f / im.x[k] : 0.f;
      vmv = fmaf(m * v.x[k], v.x[k], vmv);
      vg = fmaf(v.x[k], gn.x[k], vg);
    }
    vmv = warp_sum(vmv);
    vg = warp_sum(vg);
    return -0.5 * (log(double(Lc)) + slm) + 0.5 * double(vmv) +
           0.5 * double(Lc) * double(a2) * double(vg) * double(vg);
  };
  const double H0 = -ld0 + kinetic(L) - J0;
  double ld = ld0;
  float dJ = 0.f;  // this transition's volume-term increments
  for (int s = 0; s < sp.L; ++s) {  // lan_integrator.one_step
    w_half<E>(a2, v, &dJ, gn, hv, L, im, Hdl, eps, sp.alpha2_fix);
#pragma unroll
    for (int k = 0; k < E; ++k) q.x[k] = fmaf(eps, v.x[k], q.x[k]);
    ld = w_logdensity_grad<E>(W, q, g, &sx, s == sp.L - 1);
    float Ls = 0.f;
#pragma unroll
    for (int k = 0; k < E; ++k) Ls = fmaf(im.x[k] * g.x[k], g.x[k], Ls);
    L = 1.f + a2 * warp_sum(Ls);
    sL = sqrtf(L);
#pragma unroll
    for (int k = 0; k < E; ++k) {
      gn.x[k] = g.x[k] / sL;
      dl_ig.x[k] = im.x[k] * gn.x[k];
    }
    w_hvp<E>(W, q, v, sx, hv);
    w_hvp<E>(W, q, dl_ig, sx, Hdl);
#pragma unroll
    for (int k = 0; k < E; ++k) {
      hv.x[k] /= sL;
      Hdl.x[k] /= sL;
    }
    w_half<E>(a2, v, &dJ, gn, hv, L, im, Hdl, eps, sp.alpha2_fix);
    w_hvp<E>(W, q, v, sx, hv);
#pragma unroll
    for (int k = 0; k < E; ++k) hv.x[k] /= sL;
  }
  const double J = J0 + double(dJ);
  const double H1 = -ld + kinetic(L) - J;
  if (info.prop_q || info.prop_v) {  // LMCInfo.proposal.state: q_L and −v_L
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int i = lane + 32 * k;
      if (i < d) {
        if (info.prop_q) info.prop_q[(size_t)c * d + i] = q.x[k];
        if (info.prop_v) info.prop_v[(size_t)c * d + i] = -v.x[k];
      }
    }
  }
  const AcceptOut a = metropolis(H0, H1, uacc[c], sp.div_threshold);
  if (a.accept) {
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int i = lane + 32 * k;
      if (i < d) {
        pos[(size_t)c * d + i] = q.x[k];
        grad[(size_t)c * d + i] = gn.x[k] * sL;  // lmc.py:231
      }
    }
    if (lane == 0) {
      logdens[c] = ld;
      vol[c] = J;
    }
  }
  if (lane == 0) {
    if (info.acc_rate) info.acc_rate[c] = a.p_acc;
    if (info.accepted) info.accepted[c] = a.accept;
    if (info.divergent) info.divergent[c] = a.divergent;
    if (info.energy) info.energy[c] = H1;
    if (info.fp_iters) info.fp_iters[c] = 0;
    if (info.status) info.status[c] = isfinite(H1) ? 0u : GJ_CHAIN_NONFINITE;
  }
}

}  // namespace

bool monge_warp_supported(const TargetDev& t) {
  return (t.family == GJ_FUNNEL || t.family == GJ_HIERGAUSS) && t.d >= 2 && t.d <= 256;
}

cudaError_t launch_monge_warp(const TargetDev& t, const StepDev& sp, float* pos, float* grad,
                              double* ld, double* vol, const float* z, const double* u,
                              const InfoDev<float>& info, int C, cudaStream_t st) {
  const int tpb = 256;
  const dim3 grid((unsigned)(((size_t)C * 32 + tpb - 1) / tpb));
  if (t.d <= 32)
    monge_warp_kernel<1><<<grid, tpb, 0, st>>>(t, sp, pos, grad, ld, vol, z, u, info, C);
  else if (t.d <= 64)
    monge_warp_kernel<2><<<grid, tpb, 0, st>>>(t, sp, pos, grad, ld, vol, z, u, info, C);
  else if (t.d <= 128)
    monge_warp_kernel<4><<<grid, tpb, 0, st>>>(t, sp, pos, grad, ld, vol, z, u, info, C);
  else if (t.d <= 256)
    monge_warp_kernel<8><<<grid, tpb, 0, st>>>(t, sp, pos, grad, ld, vol, z, u, info, C);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

}  // namespace gj
