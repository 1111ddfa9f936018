// LMC on a Monge patch, one WARP per chain: float32 state (the mixed form) or
// float64 throughout (the plain form; R = double below).
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
// Mixed form (R = float) FP64: the volume adjustment J across transitions (a
// transition's increments are summed in FP32), the log density at the
// proposal and the Hamiltonian difference; nothing in its step loop runs on
// the FP64 pipe.  The plain form (R = double) is the same code in float64.
#include <cmath>

#include "chain_kernels.cuh"

namespace gj {

namespace {

// math on the kernel's real type R: the float forms call the float32
// functions explicitly (a bare rsqrt / log1p / log / fabs of a float may
// resolve to the double overload and run on the FP64 pipe)
__device__ __forceinline__ float m_exp(float x) { return expf(x); }
__device__ __forceinline__ double m_exp(double x) { return exp(x); }
__device__ __forceinline__ float m_log(float x) { return logf(x); }
__device__ __forceinline__ double m_log(double x) { return log(x); }
// log(1 + x) in float32 for the volume-term increments (|x| ~ 1e-3): the
// Taylor series x − x²/2 + x³/3 − x⁴/4 + x⁵/5 for |x| < 1e-2 (truncation
// ≤ x⁶/6 < 2e-13, below float32's resolution of the result), logf(1 + x)
// beyond (absolute error ~6e-8 there, a relative 6e-6 at most)
__device__ __forceinline__ float m_log1p(float x) {
  if (fabsf(x) < 1e-2f)
    return x * (1.f + x * (-0.5f + x * (1.f / 3.f + x * (-0.25f + x * 0.2f))));
  return logf(1.f + x);
}
__device__ __forceinline__ double m_log1p(double x) { return log1p(x); }
__device__ __forceinline__ float m_abs(float x) { return fabsf(x); }
__device__ __forceinline__ double m_abs(double x) { return fabs(x); }
__device__ __forceinline__ float m_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double m_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float m_rsqrt(float x) { return rsqrtf(x); }
__device__ __forceinline__ double m_rsqrt(double x) { return rsqrt(x); }
__device__ __forceinline__ float m_fma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double m_fma(double a, double b, double c) { return fma(a, b, c); }


template <int E, typename R>
struct WVec {
  R x[E];
};

template <int E, typename R>
__device__ __forceinline__ R wdot(const WVec<E, R>& a, const WVec<E, R>& b) {
  R s = R(0);
#pragma unroll
  for (int k = 0; k < E; ++k) s = m_fma(a.x[k], b.x[k], s);
  return warp_sum(s);
}

// broadcast element i (runtime) of a warp vector to all lanes
template <int E, typename R>
__device__ __forceinline__ R wget(const WVec<E, R>& a, int i) {
  const int slot = i >> 5, lane = i & 31;
  R v = R(0);
#pragma unroll
  for (int k = 0; k < E; ++k)
    if (k == slot) v = a.x[k];
  return __shfl_sync(0xffffffffu, v, lane);
}

// N independent warp sums in one butterfly: the N shuffles of a stage issue
// together, so the round costs the latency of one sum (every lane ends with
// the same, bit-identical totals: each stage adds a pair in both orders,
// which float addition makes equal)
template <int N, typename R>
__device__ __forceinline__ void warp_sum_n(R (&v)[N]) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    R t[N];
#pragma unroll
    for (int i = 0; i < N; ++i) t[i] = __shfl_xor_sync(0xffffffffu, v[i], o);
#pragma unroll
    for (int i = 0; i < N; ++i) v[i] += t[i];
  }
}

// warp-level target: log density + gradient and HVP for funnel / hier.
// The scale constants are precomputed once per transition: on GB300 an FP64
// division or logarithm inside the step loop costs more than the whole FP32
// step (the FP64 pipe was 85 % busy with them in the loop).
template <typename R>
struct WarpTarget {
  TargetDev t;
  int lane;
  R inv_a2, inv_b2;   // funnel: 1/σ² (a); hier: 1/σ_μ² (a), 1/σ_v² (b)
  double inv_a2d, inv_b2d;  // the same in FP64, for the log density
  double ld_const;          // the log density's constant terms
};

// The target's scale constants, computed once on the host: an FP64 division
// or logarithm costs every warp tens of FP64-pipe instructions (1/64 of the
// FP32 rate on GB300), which a transition of 16 steps cannot amortise.
struct WarpConst {
  double inv_a2d, inv_b2d;  // funnel: 1/σ²; hier: 1/σ_μ², 1/σ_v²
  double ld_const;          // the log density's constant terms but the hier σ_j sum
};

inline WarpConst warp_const_host(const TargetDev& t) {
  WarpConst k;
  if (t.family == GJ_FUNNEL) {
    k.inv_a2d = 1.0 / (t.p0 * t.p0);
    k.inv_b2d = 0.0;
    k.ld_const = -std::log(t.p0) - 0.5 * kLog2Pi - (t.d - 1) * 0.5 * kLog2Pi;
  } else {
    const int J = t.n;
    k.inv_a2d = 1.0 / (t.p0 * t.p0);
    k.inv_b2d = 1.0 / (t.p1 * t.p1);
    // J · (−½ log 2π) from the data terms and as many from the latent terms
    k.ld_const = -J * kLog2Pi - std::log(t.p0) - 0.5 * kLog2Pi - std::log(t.p1) - 0.5 * kLog2Pi;
  }
  return k;
}

template <typename R>
__device__ inline WarpTarget<R> make_warp_target(const TargetDev& t, const WarpConst& k, int lane) {
  WarpTarget<R> W;
  W.t = t;
  W.lane = lane;
  W.inv_a2d = k.inv_a2d;
  W.inv_b2d = k.inv_b2d;
  W.inv_a2 = R(k.inv_a2d);
  W.inv_b2 = R(k.inv_b2d);
  W.ld_const = k.ld_const;
  if (t.family != GJ_FUNNEL) {  // hier: −Σ_j log σ_j (the data's scales, on the device)
    const int J = t.n;
    const R* sg = static_cast<const R*>(t.s);
    R c = R(0);
    for (int i = lane; i < J; i += 32) c -= m_log(sg[i]);
    W.ld_const += double(warp_sum(c));
  }
  return W;
}

// funnel: v = θ[d−1]
// The FP64 log density is formed only when need_ld (the proposal's, after
// the last step); the gradient is FP32.  With Lout, the normalising constant
// L = 1 + α² Σ_i M⁻¹_i g_i² (lmcmonge/metrics.py:193-197) is formed from the
// same reduction round (its sum over the coordinates whose gradient is
// local, plus the one or two coordinates whose gradient needs the sums).
template <int E, typename R>
__device__ double w_logdensity_grad(const WarpTarget<R>& W, const WVec<E, R>& q, WVec<E, R>& g,
                                    R* sx_out, bool need_ld = true, const WVec<E, R>* im = nullptr,
                                    R a2 = R(0), R* Lout = nullptr) {
  const TargetDev& t = W.t;
  const int d = t.d;
  if (t.family == GJ_FUNNEL) {
    const R v = wget<E>(q, d - 1);
    const R ev = m_exp(-v);
    R p[2] = {R(0), R(0)};  // Σx², Σ M⁻¹x²
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int i = W.lane + 32 * k;
      const R x = (i < d - 1) ? q.x[k] : R(0);
      p[0] = m_fma(x, x, p[0]);
      if (Lout) p[1] = m_fma(im->x[k] * x, x, p[1]);
    }
    if (Lout)
      warp_sum_n<2>(p);
    else
      p[0] = warp_sum(p[0]);
    const R sx = p[0];
    const R gv = -v * W.inv_a2 - R(0.5) * R(d - 1) + R(0.5) * ev * sx;
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int i = W.lane + 32 * k;
      g.x[k] = (i < d - 1) ? -q.x[k] * ev : ((i == d - 1) ? gv : R(0));
    }
    if (Lout) *Lout = R(1) + a2 * (ev * ev * p[1] + wget<E>(*im, d - 1) * gv * gv);
    *sx_out = sx;
    if (!need_ld) return 0.0;
    return W.ld_const - 0.5 * double(v) * double(v) * W.inv_a2d - 0.5 * double(ev) * double(sx) -
           (d - 1) * 0.5 * double(v);
  }
  // hierarchical Gaussian: θ = [θ_1..θ_J, μ, v]
  const int J = t.n;
  const R* y = static_cast<const R*>(t.y);
  const R* sg = static_cast<const R*>(t.s);
  const R mu = wget<E>(q, J), v = wget<E>(q, J + 1);
  const R ev = m_exp(-v);
  R p[3] = {R(0), R(0), R(0)};  // Σr, Σr², Σ_{j<J} M⁻¹g_j²
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const int i = W.lane + 32 * k;
    if (i < J) {
      const R r = q.x[k] - mu;
      const R e = y[i] - q.x[k];
      const R is2 = R(1) / (sg[i] * sg[i]);
      g.x[k] = e * is2 - r * ev;
      p[0] += r;
      p[1] = m_fma(r, r, p[1]);
      if (Lout) p[2] = m_fma(im->x[k] * g.x[k], g.x[k], p[2]);
    }
  }
  if (Lout) {
    warp_sum_n<3>(p);
  } else {
    R p2[2] = {p[0], p[1]};
    warp_sum_n<2>(p2);
    p[0] = p2[0];
    p[1] = p2[1];
  }
  const R sr = p[0], srr = p[1];
  const R gmu = sr * ev - mu * W.inv_a2;
  const R gvv = R(0.5) * ev * srr - R(0.5) * J - v * W.inv_b2;
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const int i = W.lane + 32 * k;
    if (i == J) g.x[k] = gmu;
    if (i == J + 1) g.x[k] = gvv;
    if (i > J + 1) g.x[k] = R(0);
  }
  if (Lout)
    *Lout = R(1) + a2 * (p[2] + wget<E>(*im, J) * gmu * gmu + wget<E>(*im, J + 1) * gvv * gvv);
  *sx_out = srr;
  if (!need_ld) return 0.0;
  double se = 0.0;  // Σ (y_j − θ_j)² / σ_j², in FP64 as the initial log density
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const int i = W.lane + 32 * k;
    if (i < J) {
      const double e = double(y[i]) - double(q.x[k]);
      se += e * e * double(R(1) / (sg[i] * sg[i]));
    }
  }
  se = warp_sum(se);
  return W.ld_const - 0.5 * se - 0.5 * double(ev) * double(srr) - J * 0.5 * double(v) -
         0.5 * double(mu) * double(mu) * W.inv_a2d - 0.5 * double(v) * double(v) * W.inv_b2d;
}

// Metropolis accept (mcmc/proposal.py: p = min(1, e^{H0−H1}), accept when
// u < p) with the exponential in R: the energy difference is formed in
// float64, and in the float32 form e^w carries a relative error near 1e-7,
// so a decision changes only for a uniform within that of the threshold.
template <typename R>
__device__ __forceinline__ AcceptOut metropolis_r(double H0, double H1, double u, double div_thr) {
  if constexpr (sizeof(R) == 8) {
    return metropolis(H0, H1, u, div_thr);
  } else {
    AcceptOut a;
    float w = float(H0 - H1);
    if (isnan(w)) w = -INFINITY;
    a.w = w;
    a.p_acc = double(fminf(m_exp(w), 1.0f));
    a.accept = u < a.p_acc;
    a.divergent = -w > float(div_thr);
    return a;
  }
}

// Hessian-vector product; `sx` is the Σx² (funnel) / Σr² (hier) of the
// last gradient evaluation at the same q.
template <int E, typename R>
__device__ void w_hvp(const WarpTarget<R>& W, const WVec<E, R>& q, const WVec<E, R>& u, R sx, WVec<E, R>& out) {
  const TargetDev& t = W.t;
  const int d = t.d;
  if (t.family == GJ_FUNNEL) {
    const R v = wget<E>(q, d - 1);
    const R ev = m_exp(-v);
    const R uv = wget<E>(u, d - 1);
    R xu = R(0);
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int i = W.lane + 32 * k;
      if (i < d - 1) xu = m_fma(q.x[k], u.x[k], xu);
    }
    xu = warp_sum(xu);
    const R ov = ev * xu + (-W.inv_a2 - R(0.5) * ev * sx) * uv;
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int i = W.lane + 32 * k;
      out.x[k] = (i < d - 1) ? ev * (-u.x[k] + q.x[k] * uv) : ((i == d - 1) ? ov : R(0));
    }
    return;
  }
  const int J = t.n;
  const R* sg = static_cast<const R*>(t.s);
  const R mu = wget<E>(q, J), v = wget<E>(q, J + 1);
  const R ev = m_exp(-v);
  const R um = wget<E>(u, J), uv = wget<E>(u, J + 1);
  R sr = R(0), sut = R(0), sru = R(0);
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const int i = W.lane + 32 * k;
    if (i < J) {
      const R r = q.x[k] - mu;
      sr += r;
      sut += u.x[k];
      sru = m_fma(r, u.x[k], sru);
      out.x[k] = -(R(1) / (sg[i] * sg[i]) + ev) * u.x[k] + ev * um + r * ev * uv;
    }
  }
  sr = warp_sum(sr);
  sut = warp_sum(sut);
  sru = warp_sum(sru);
  const R om = ev * sut + (-R(J) * ev - W.inv_a2) * um - ev * sr * uv;
  const R ovv = ev * sru - ev * sr * um + (-R(0.5) * ev * sx - W.inv_b2) * uv;
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const int i = W.lane + 32 * k;
    if (i == J) out.x[k] = om;
    if (i == J + 1) out.x[k] = ovv;
    if (i > J + 1) out.x[k] = R(0);
  }
}

// Two Hessian-vector products at the same q (H·u1, H·u2) with one reduction
// round: the same arithmetic as two w_hvp calls.
template <int E, typename R>
__device__ void w_hvp2(const WarpTarget<R>& W, const WVec<E, R>& q, const WVec<E, R>& u1,
                       const WVec<E, R>& u2, R sx, WVec<E, R>& o1, WVec<E, R>& o2) {
  const TargetDev& t = W.t;
  const int d = t.d;
  if (t.family == GJ_FUNNEL) {
    const R v = wget<E>(q, d - 1);
    const R ev = m_exp(-v);
    const R uv1 = wget<E>(u1, d - 1), uv2 = wget<E>(u2, d - 1);
    R p[2] = {R(0), R(0)};
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int i = W.lane + 32 * k;
      if (i < d - 1) {
        p[0] = m_fma(q.x[k], u1.x[k], p[0]);
        p[1] = m_fma(q.x[k], u2.x[k], p[1]);
      }
    }
    warp_sum_n<2>(p);
    const R cv = -W.inv_a2 - R(0.5) * ev * sx;
    const R ov1 = ev * p[0] + cv * uv1, ov2 = ev * p[1] + cv * uv2;
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int i = W.lane + 32 * k;
      o1.x[k] = (i < d - 1) ? ev * (-u1.x[k] + q.x[k] * uv1) : ((i == d - 1) ? ov1 : R(0));
      o2.x[k] = (i < d - 1) ? ev * (-u2.x[k] + q.x[k] * uv2) : ((i == d - 1) ? ov2 : R(0));
    }
    return;
  }
  const int J = t.n;
  const R* sg = static_cast<const R*>(t.s);
  const R mu = wget<E>(q, J), v = wget<E>(q, J + 1);
  const R ev = m_exp(-v);
  const R um1 = wget<E>(u1, J), uv1 = wget<E>(u1, J + 1);
  const R um2 = wget<E>(u2, J), uv2 = wget<E>(u2, J + 1);
  R p[5] = {R(0), R(0), R(0), R(0), R(0)};  // Σr, Σu1, Σr·u1, Σu2, Σr·u2
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const int i = W.lane + 32 * k;
    if (i < J) {
      const R r = q.x[k] - mu;
      const R is2 = R(1) / (sg[i] * sg[i]);
      p[0] += r;
      p[1] += u1.x[k];
      p[2] = m_fma(r, u1.x[k], p[2]);
      p[3] += u2.x[k];
      p[4] = m_fma(r, u2.x[k], p[4]);
      o1.x[k] = -(is2 + ev) * u1.x[k] + ev * um1 + r * ev * uv1;
      o2.x[k] = -(is2 + ev) * u2.x[k] + ev * um2 + r * ev * uv2;
    }
  }
  warp_sum_n<5>(p);
  const R sr = p[0];
  const R om1 = ev * p[1] + (-R(J) * ev - W.inv_a2) * um1 - ev * sr * uv1;
  const R ovv1 = ev * p[2] - ev * sr * um1 + (-R(0.5) * ev * sx - W.inv_b2) * uv1;
  const R om2 = ev * p[3] + (-R(J) * ev - W.inv_a2) * um2 - ev * sr * uv2;
  const R ovv2 = ev * p[4] - ev * sr * um2 + (-R(0.5) * ev * sx - W.inv_b2) * uv2;
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const int i = W.lane + 32 * k;
    if (i == J) {
      o1.x[k] = om1;
      o2.x[k] = om2;
    }
    if (i == J + 1) {
      o1.x[k] = ovv1;
      o2.x[k] = ovv2;
    }
    if (i > J + 1) {
      o1.x[k] = R(0);
      o2.x[k] = R(0);
    }
  }
}

// half_step_omega (lmcmonge/integrators.py:158-194), im = diag(M⁻¹).  dJ
// accumulates this transition's volume-term increments in FP32 (each is
// ≈ 1e-3; 4 per step); the caller adds the sum to the FP64 J once.
//
// The reference's four dot products depend on one another (dφ·dl_ig, then
// v_tmp·Hv, then Hdl_ig·v'), so each would be its own warp reduction.  They
// are all linear in seven sums of the step's inputs, taken in one round:
//   S_dh = Σ hv·dl_ig, S_gd = Σ gn·dl_ig, S_Hd = Σ Hdl·dl_ig, S_vh = Σ v·hv,
//   S_gh = Σ igH·hv,  S_Hv = Σ Hdl·v,   S_HH = Σ Hdl·igH    (igH = M⁻¹Hdl)
// with dφ_ig = −dl_ig + α²·igH/√L and c1 = ½ε√L:
//   dφ·dl_ig  = −S_gd + α² S_Hd/√L
//   v_tmp·hv  = S_vh − c1 (−S_dh + α² S_gh/√L − α² (dφ·dl_ig) S_dh)
//   Hdl·v'    = S_Hv − c1 (−S_Hd + α² S_HH/√L − α² (dφ·dl_ig) S_Hd) − corr S_Hd
// (v' = v_tmp − corr·dl_ig); each leading sum dominates its correction, so
// the rewriting loses nothing to cancellation.
template <int E, typename R>
__device__ void w_half(R a2, WVec<E, R>& v, R* dJ, const WVec<E, R>& gn, const WVec<E, R>& hv, R L,
                       const WVec<E, R>& im, const WVec<E, R>& Hdl, R eps, int fix) {
  WVec<E, R> dl_ig, igH;
  R p[7] = {R(0), R(0), R(0), R(0), R(0), R(0), R(0)};
#pragma unroll
  for (int k = 0; k < E; ++k) {
    dl_ig.x[k] = im.x[k] * gn.x[k];
    igH.x[k] = im.x[k] * Hdl.x[k];
    p[0] = m_fma(hv.x[k], dl_ig.x[k], p[0]);
    p[1] = m_fma(gn.x[k], dl_ig.x[k], p[1]);
    p[2] = m_fma(Hdl.x[k], dl_ig.x[k], p[2]);
    p[3] = m_fma(v.x[k], hv.x[k], p[3]);
    p[4] = m_fma(igH.x[k], hv.x[k], p[4]);
    p[5] = m_fma(Hdl.x[k], v.x[k], p[5]);
    p[6] = m_fma(Hdl.x[k], igH.x[k], p[6]);
  }
  warp_sum_n<7>(p);
  // log|det1| and log|1 − ½εα²(Hdl·v)| as FP32 log1p of the small terms
  // (det1 is an FP32 value, so an FP64 logarithm adds nothing)
  const R x1 = R(0.5) * eps * a2 * p[0];
  const R det1 = R(1) + x1;
  *dJ -= x1 > -R(1) ? m_log1p(x1) : m_log(m_abs(det1));
  const R sL = m_sqrt(L);
  const R isL = R(1) / sL;  // one division, then products
  const R pd = -p[1] + a2 * isL * p[2];  // dφ·dl_ig
  const R c1 = R(0.5) * eps * sL;
  const R vt_hv = p[3] - c1 * (-p[0] + a2 * isL * p[4] - a2 * pd * p[0]);
  R corr = R(0.5) * eps * vt_hv / det1;
  if (fix) corr *= a2;
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const R dphi_ig = -dl_ig.x[k] + a2 * igH.x[k] * isL;
    const R vt = v.x[k] - c1 * (dphi_ig - a2 * pd * dl_ig.x[k]);
    v.x[k] = vt - corr * dl_ig.x[k];
  }
  const R hdl_v = p[5] - c1 * (-p[2] + a2 * isL * p[6] - a2 * pd * p[2]) - corr * p[2];
  const R x2 = -R(0.5) * eps * a2 * hdl_v;
  *dJ += x2 > -R(1) ? m_log1p(x2) : m_log(m_abs(R(1) + x2));
}

// inclusive warp scan (ascending lane order)
template <typename R>
__device__ __forceinline__ R warp_incl_scan(R x, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const R y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  return x;
}
// inclusive warp scan in descending lane order (suffix sums)
template <typename R>
__device__ __forceinline__ R warp_incl_rscan(R x, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const R y = __shfl_down_sync(0xffffffffu, x, o);
    if (lane + o < 32) x += y;
  }
  return x;
}

// three 256-thread CTAs per SM (at most 85 registers a thread): the kernel
// is bound by the latency of its warp reductions, and 24 warps per SM hide
// it better than 16 (D = 100 ran 0.28 ms per transition at 80 registers,
// 0.36 ms at the 120 the compiler picks unbounded)
template <int E, typename R>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 3 : 1) monge_warp_kernel(TargetDev t, WarpConst wc, StepDev sp, R* pos,
                                                         R* grad, double* logdens, double* vol,
                                                         const R* z, const double* uacc,
                                                         InfoDev<R> info, int C) {
  const int lane = threadIdx.x & 31;
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (c >= C) return;  // whole warp exits together
  const int d = t.d;
  const WarpTarget<R> W = make_warp_target<R>(t, wc, lane);
  const R a2 = R(sp.alpha2);
  const R eps = R(sp.h);
  const R* imv = static_cast<const R*>(sp.inv_mass);
  WVec<E, R> q, g, im, gn, Hdl, hv, v;
  R slm_part = R(0);
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const int i = lane + 32 * k;
    const bool in = i < d;
    q.x[k] = in ? pos[(size_t)c * d + i] : R(0);
    g.x[k] = in ? grad[(size_t)c * d + i] : R(0);
    im.x[k] = in ? (imv ? imv[i] : R(1)) : R(0);
    if (in) slm_part -= m_log(im.x[k]);  // cancels in H1 − H0
  }
  const double slm = double(warp_sum(slm_part));  // Σ log M
  const double ld0 = logdens[c];
  const double J0 = vol[c];
  R sx;
  // ---- setup (lmc.py:177-208)
  R L = R(0);
#pragma unroll
  for (int k = 0; k < E; ++k) L = m_fma(im.x[k] * g.x[k], g.x[k], L);
  L = R(1) + a2 * warp_sum(L);
  R sL = m_sqrt(L);
  R isL = R(1) / sL;
  {
    // Σx² at the current q for the HVPs (one extra gradient pass is avoided by
    // recomputing only the reduction)
    WVec<E, R> gtmp;
    (void)w_logdensity_grad<E>(W, q, gtmp, &sx, false);
  }
  WVec<E, R> dl_ig;
#pragma unroll
  for (int k = 0; k < E; ++k) {
    gn.x[k] = g.x[k] * isL;
    dl_ig.x[k] = im.x[k] * gn.x[k];
  }
  w_hvp<E>(W, q, dl_ig, sx, Hdl);
#pragma unroll
  for (int k = 0; k < E; ++k) Hdl.x[k] *= isL;
  // ---- velocity: closed-form factor (τ_j = 1/L + α² Σ_{k≥j} u_k², u = w/m_sqrt(M⁻¹))
  {
    WVec<E, R> u, zz;
    R tot_after = R(0);  // Σ over slots > k of u²
    R tau[E], taun[E];
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int i = lane + 32 * k;
      u.x[k] = (i < d) ? dl_ig.x[k] * m_rsqrt(im.x[k]) : R(0);
      zz.x[k] = (i < d) ? z[(size_t)c * d + i] : R(0);
    }
#pragma unroll
    for (int k = E - 1; k >= 0; --k) {
      const R u2 = u.x[k] * u.x[k];
      const R r = warp_incl_rscan(u2, lane);
      const R suf = r + tot_after;  // Σ_{j≥i}
      tau[k] = R(1) / L + a2 * suf;
      taun[k] = tau[k] - a2 * u2;
      tot_after += __shfl_sync(0xffffffffu, r, 0);
    }
    R pre_before = R(0);  // Σ over slots < k
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int i = lane + 32 * k;
      const R tk = (i < d) ? u.x[k] * zz.x[k] * m_rsqrt(tau[k] * taun[k]) : R(0);
      const R incl = warp_incl_scan(tk, lane);
      const R pre = pre_before + incl - tk;  // Σ_{j<i}
      const R y = m_sqrt(taun[k] / tau[k]) * zz.x[k] - a2 * u.x[k] * pre;
      v.x[k] = (i < d) ? m_sqrt(im.x[k]) * y : R(0);
      pre_before += __shfl_sync(0xffffffffu, incl, 31);
      if (info.momentum && i < d) info.momentum[(size_t)c * d + i] = v.x[k];
    }
  }
  w_hvp<E>(W, q, v, sx, hv);
#pragma unroll
  for (int k = 0; k < E; ++k) hv.x[k] *= isL;
  auto kinetic = [&](R Lc) -> double {  // lmcmonge/metrics.py:168-186
    R vmv = R(0), vg = R(0);
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const R m = (im.x[k] > R(0)) ? R(1) / im.x[k] : R(0);
      vmv = m_fma(m * v.x[k], v.x[k], vmv);
      vg = m_fma(v.x[k], gn.x[k], vg);
    }
    R p[2] = {vmv, vg};
    warp_sum_n<2>(p);
    vmv = p[0];
    vg = p[1];
    // in the state's type R: every factor is an R value, and each FP64
    // instruction costs 64 FP32 ones on GB300
    const R kin = R(0.5) * (vmv - m_log(Lc)) + R(0.5) * Lc * a2 * vg * vg;
    return double(kin) - 0.5 * slm;
  };
  const double H0 = -ld0 + kinetic(L) - J0;
  double ld = ld0;
  R dJ = R(0);  // this transition's volume-term increments
  for (int s = 0; s < sp.L; ++s) {  // lan_integrator.one_step
    w_half<E>(a2, v, &dJ, gn, hv, L, im, Hdl, eps, sp.alpha2_fix);
#pragma unroll
    for (int k = 0; k < E; ++k) q.x[k] = m_fma(eps, v.x[k], q.x[k]);
    ld = w_logdensity_grad<E>(W, q, g, &sx, s == sp.L - 1, &im, a2, &L);
    sL = m_sqrt(L);
    isL = R(1) / sL;
#pragma unroll
    for (int k = 0; k < E; ++k) {
      gn.x[k] = g.x[k] * isL;
      dl_ig.x[k] = im.x[k] * gn.x[k];
    }
    w_hvp2<E>(W, q, v, dl_ig, sx, hv, Hdl);
#pragma unroll
    for (int k = 0; k < E; ++k) {
      hv.x[k] *= isL;
      Hdl.x[k] *= isL;
    }
    w_half<E>(a2, v, &dJ, gn, hv, L, im, Hdl, eps, sp.alpha2_fix);
    w_hvp<E>(W, q, v, sx, hv);
#pragma unroll
    for (int k = 0; k < E; ++k) hv.x[k] *= isL;
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
  const AcceptOut a = metropolis_r<R>(H0, H1, uacc[c], sp.div_threshold);
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

template <typename R>
cudaError_t launch_monge_warp(const TargetDev& t, const StepDev& sp, R* pos, R* grad, double* ld,
                              double* vol, const R* z, const double* u, const InfoDev<R>& info,
                              int C, cudaStream_t st) {
  const int tpb = 256;
  const dim3 grid((unsigned)(((size_t)C * 32 + tpb - 1) / tpb));
  const WarpConst wc = warp_const_host(t);
  if (t.d <= 32)
    monge_warp_kernel<1, R><<<grid, tpb, 0, st>>>(t, wc, sp, pos, grad, ld, vol, z, u, info, C);
  else if (t.d <= 64)
    monge_warp_kernel<2, R><<<grid, tpb, 0, st>>>(t, wc, sp, pos, grad, ld, vol, z, u, info, C);
  else if (t.d <= 128)
    monge_warp_kernel<4, R><<<grid, tpb, 0, st>>>(t, wc, sp, pos, grad, ld, vol, z, u, info, C);
  else if (t.d <= 256)
    monge_warp_kernel<8, R><<<grid, tpb, 0, st>>>(t, wc, sp, pos, grad, ld, vol, z, u, info, C);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

template cudaError_t launch_monge_warp<float>(const TargetDev&, const StepDev&, float*, float*,
                                              double*, double*, const float*, const double*,
                                              const InfoDev<float>&, int, cudaStream_t);
template cudaError_t launch_monge_warp<double>(const TargetDev&, const StepDev&, double*, double*,
                                               double*, double*, const double*, const double*,
                                               const InfoDev<double>&, int, cudaStream_t);

}  // namespace gj
