// Derivative of the LMC-Monge proposal position with respect to α², by
// forward-mode tangent propagation through the whole transition.
//
// The reference's LMC-Monge ChEES adaptation takes
//   jax.jacfwd(trajectory_proposal_position, argnums=0)(alpha2, ...)
// (adaptation/chees_adaptation_lmcmonge.py:469-519): the proposal position
// q_L of one transition, as a function of α², differentiated through the
// velocity draw (the factor of diag(M⁻¹) − α²·w·wᵀ, lmcmonge/metrics.py:
// 155-166), the normalising constant L = 1 + α²∇ℓᵀM⁻¹∇ℓ and every
// half_step_omega (lmcmonge/integrators.py:158-194) of lan_integrator
// (:63-155).  Here every scalar of that computation carries one tangent
// component (Dual<1>: value and d/dα² in float64), so one pass gives q_L and
// ∂q_L/∂α² exactly (up to rounding) at about twice the cost of the primal.
//
// Layout: one warp per chain, element i of a d-vector in lane i % 32, slot
// i / 32, as the float32 warp kernel (monge_warp.cu); dot products and the
// closed-form factor's prefix / suffix sums are warp shuffles of both the
// value and the tangent.  The volume adjustment and the energy do not enter
// q_L and are not formed.  Targets: the funnel and the hierarchical
// Gaussian (closed-form gradient and HVP, written once over the dual type,
// so the HVP's own derivative along the trajectory comes out of the same
// code).
#include "chain_kernels.cuh"
#include "dual.cuh"

namespace gj {

namespace {

using S = Dual<1>;
constexpr unsigned kFull = 0xffffffffu;

template <int E>
struct DVec {
  S x[E];
};

__device__ __forceinline__ S shfl_xor(const S& a, int o) {
  S r;
  r.v = __shfl_xor_sync(kFull, a.v, o);
  r.t[0] = __shfl_xor_sync(kFull, a.t[0], o);
  return r;
}
__device__ __forceinline__ S shfl_idx(const S& a, int src) {
  S r;
  r.v = __shfl_sync(kFull, a.v, src);
  r.t[0] = __shfl_sync(kFull, a.t[0], src);
  return r;
}
__device__ __forceinline__ S dsum(S a) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a = a + shfl_xor(a, o);
  return a;
}
// inclusive scans over lanes, ascending (prefix) and descending (suffix)
__device__ __forceinline__ S dscan(S x, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    S y;
    y.v = __shfl_up_sync(kFull, x.v, o);
    y.t[0] = __shfl_up_sync(kFull, x.t[0], o);
    if (lane >= o) x = x + y;
  }
  return x;
}
__device__ __forceinline__ S drscan(S x, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    S y;
    y.v = __shfl_down_sync(kFull, x.v, o);
    y.t[0] = __shfl_down_sync(kFull, x.t[0], o);
    if (lane + o < 32) x = x + y;
  }
  return x;
}

template <int E>
__device__ __forceinline__ S dget(const DVec<E>& a, int i) {
  const int slot = i >> 5;
  S v;
#pragma unroll
  for (int k = 0; k < E; ++k)
    if (k == slot) v = a.x[k];
  return shfl_idx(v, i & 31);
}

template <int E>
__device__ __forceinline__ S ddot(const DVec<E>& a, const DVec<E>& b) {
  S s;
#pragma unroll
  for (int k = 0; k < E; ++k) s += a.x[k] * b.x[k];
  return dsum(s);
}

// gradient of the log density (the funnel: examples/funnel/main.py:28-54,
// v = θ[d−1]; the hierarchical Gaussian: θ = [θ_1..θ_J, μ, v])
template <typename T, int E>
__device__ void j_grad(const TargetDev& t, int lane, const DVec<E>& q, DVec<E>& g) {
  const int d = t.d;
  if (t.family == GJ_FUNNEL) {
    const double ia2 = 1.0 / (t.p0 * t.p0);
    const S v = dget<E>(q, d - 1);
    const S ev = exp(-v);
    S sx;
#pragma unroll
    for (int k = 0; k < E; ++k)
      if (lane + 32 * k < d - 1) sx += q.x[k] * q.x[k];
    sx = dsum(sx);
    const S gv = -v * ia2 - 0.5 * (d - 1) + 0.5 * ev * sx;
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int i = lane + 32 * k;
      g.x[k] = (i < d - 1) ? -q.x[k] * ev : ((i == d - 1) ? gv : S(0.0));
    }
    return;
  }
  const int J = t.n;
  const T* y = static_cast<const T*>(t.y);
  const T* sg = static_cast<const T*>(t.s);
  const S mu = dget<E>(q, J), v = dget<E>(q, J + 1);
  const S ev = exp(-v);
  S sr, srr;
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const int i = lane + 32 * k;
    if (i < J) {
      const S r = q.x[k] - mu;
      const double is2 = 1.0 / (double(sg[i]) * double(sg[i]));
      g.x[k] = (double(y[i]) - q.x[k]) * is2 - r * ev;
      sr += r;
      srr += r * r;
    }
  }
  sr = dsum(sr);
  srr = dsum(srr);
  const S gmu = sr * ev - mu / (t.p0 * t.p0);
  const S gv = 0.5 * ev * srr - 0.5 * J - v / (t.p1 * t.p1);
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const int i = lane + 32 * k;
    if (i == J) g.x[k] = gmu;
    if (i == J + 1) g.x[k] = gv;
    if (i > J + 1) g.x[k] = S(0.0);
  }
}

// Hessian-vector product of the log density (util.py:120-121)
template <typename T, int E>
__device__ void j_hvp(const TargetDev& t, int lane, const DVec<E>& q, const DVec<E>& u,
                      DVec<E>& out) {
  const int d = t.d;
  if (t.family == GJ_FUNNEL) {
    const S v = dget<E>(q, d - 1);
    const S ev = exp(-v);
    const S uv = dget<E>(u, d - 1);
    S sx, xu;
#pragma unroll
    for (int k = 0; k < E; ++k)
      if (lane + 32 * k < d - 1) {
        sx += q.x[k] * q.x[k];
        xu += q.x[k] * u.x[k];
      }
    sx = dsum(sx);
    xu = dsum(xu);
    const S ov = ev * xu + (-1.0 / (t.p0 * t.p0) - 0.5 * ev * sx) * uv;
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int i = lane + 32 * k;
      out.x[k] = (i < d - 1) ? ev * (q.x[k] * uv - u.x[k]) : ((i == d - 1) ? ov : S(0.0));
    }
    return;
  }
  const int J = t.n;
  const T* sg = static_cast<const T*>(t.s);
  const S mu = dget<E>(q, J), v = dget<E>(q, J + 1);
  const S ev = exp(-v);
  const S um = dget<E>(u, J), uv = dget<E>(u, J + 1);
  S sr, srr, sut, sru;
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const int i = lane + 32 * k;
    if (i < J) {
      const S r = q.x[k] - mu;
      const double is2 = 1.0 / (double(sg[i]) * double(sg[i]));
      sr += r;
      srr += r * r;
      sut += u.x[k];
      sru += r * u.x[k];
      out.x[k] = -(is2 + ev) * u.x[k] + ev * um + r * ev * uv;
    }
  }
  sr = dsum(sr);
  srr = dsum(srr);
  sut = dsum(sut);
  sru = dsum(sru);
  const S om = ev * sut + (-double(J) * ev - 1.0 / (t.p0 * t.p0)) * um - ev * sr * uv;
  const S ov = ev * sru - ev * sr * um + (-0.5 * ev * srr - 1.0 / (t.p1 * t.p1)) * uv;
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const int i = lane + 32 * k;
    if (i == J) out.x[k] = om;
    if (i == J + 1) out.x[k] = ov;
    if (i > J + 1) out.x[k] = S(0.0);
  }
}

// the velocity update of half_step_omega (lmcmonge/integrators.py:158-194)
template <int E>
__device__ void j_half(const S& a2, DVec<E>& v, const DVec<E>& gn, const DVec<E>& hv, const S& sL,
                       const double (&im)[E], const DVec<E>& Hdl, double eps, int fix) {
  DVec<E> dl_ig;
#pragma unroll
  for (int k = 0; k < E; ++k) dl_ig.x[k] = im[k] * gn.x[k];
  const S det1 = 1.0 + 0.5 * eps * a2 * ddot<E>(hv, dl_ig);
  S pd;
#pragma unroll
  for (int k = 0; k < E; ++k) pd += (-gn.x[k] + a2 * Hdl.x[k] / sL) * dl_ig.x[k];
  pd = dsum(pd);
  DVec<E> vt;
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const S dphi_ig = -dl_ig.x[k] + a2 * (im[k] * Hdl.x[k]) / sL;
    vt.x[k] = v.x[k] - 0.5 * eps * sL * (dphi_ig - a2 * pd * dl_ig.x[k]);
  }
  S corr = 0.5 * eps * ddot<E>(vt, hv) / det1;
  if (fix) corr = corr * a2;
#pragma unroll
  for (int k = 0; k < E; ++k) v.x[k] = vt.x[k] - corr * dl_ig.x[k];
}

template <typename T, int E>
__global__ void __launch_bounds__(128) monge_alpha2_jvp_kernel(TargetDev t, StepDev sp,
                                                               const T* __restrict__ pos,
                                                               const T* __restrict__ z, T* qL,
                                                               T* dq, int C) {
  const int lane = threadIdx.x & 31;
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (c >= C) return;  // whole warp
  const int d = t.d;
  const T* imv = static_cast<const T*>(sp.inv_mass);
  const S a2 = S::seed(sp.alpha2, 0);
  const double eps = sp.h;
  double im[E];
  DVec<E> q, g, gn, dl_ig, Hdl, hv, v;
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const int i = lane + 32 * k;
    const bool in = i < d;
    q.x[k] = S(in ? double(pos[(size_t)c * d + i]) : 0.0);
    im[k] = in ? (imv ? double(imv[i]) : 1.0) : 0.0;
  }
  // set-up (lmcmonge/lmc.py:177-208)
  j_grad<T, E>(t, lane, q, g);
  auto norm_const = [&]() {
    S s;
#pragma unroll
    for (int k = 0; k < E; ++k) s += im[k] * g.x[k] * g.x[k];
    return 1.0 + a2 * dsum(s);
  };
  S L = norm_const();
  S sL = sqrt(L);
#pragma unroll
  for (int k = 0; k < E; ++k) {
    gn.x[k] = g.x[k] / sL;
    dl_ig.x[k] = im[k] * gn.x[k];
  }
  j_hvp<T, E>(t, lane, q, dl_ig, Hdl);
#pragma unroll
  for (int k = 0; k < E; ++k) Hdl.x[k] = Hdl.x[k] / sL;
  // velocity: the closed-form factor of diag(M⁻¹) − α²·w·wᵀ with
  // u = w / sqrt(M⁻¹), τ_i = 1/L + α² Σ_{j≥i} u_j², τ'_i = τ_i − α² u_i²:
  // y_i = sqrt(τ'_i / τ_i) z_i − α² u_i Σ_{j<i} u_j z_j / sqrt(τ_j τ'_j),
  // v = sqrt(M⁻¹) ⊙ y (lmcmonge/metrics.py:155-166)
  {
    DVec<E> u, tau, taun;
    S tot_after;
#pragma unroll
    for (int k = E - 1; k >= 0; --k) {
      const int i = lane + 32 * k;
      u.x[k] = (i < d) ? dl_ig.x[k] / ::sqrt(im[k]) : S(0.0);
      const S u2 = u.x[k] * u.x[k];
      const S r = drscan(u2, lane);
      tau.x[k] = 1.0 / L + a2 * (r + tot_after);
      taun.x[k] = tau.x[k] - a2 * u2;
      tot_after += shfl_idx(r, 0);
    }
    S pre_before;
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int i = lane + 32 * k;
      const double zi = (i < d) ? double(z[(size_t)c * d + i]) : 0.0;
      const S tk = (i < d) ? u.x[k] * zi / sqrt(tau.x[k] * taun.x[k]) : S(0.0);
      const S incl = dscan(tk, lane);
      const S pre = pre_before + incl - tk;
      const S y = sqrt(taun.x[k] / tau.x[k]) * zi - a2 * u.x[k] * pre;
      v.x[k] = (i < d) ? ::sqrt(im[k]) * y : S(0.0);
      pre_before += shfl_idx(incl, 31);
    }
  }
  j_hvp<T, E>(t, lane, q, v, hv);
#pragma unroll
  for (int k = 0; k < E; ++k) hv.x[k] = hv.x[k] / sL;
  for (int s = 0; s < sp.L; ++s) {  // lan_integrator.one_step
    j_half<E>(a2, v, gn, hv, sL, im, Hdl, eps, sp.alpha2_fix);
#pragma unroll
    for (int k = 0; k < E; ++k) q.x[k] += eps * v.x[k];
    j_grad<T, E>(t, lane, q, g);
    L = norm_const();
    sL = sqrt(L);
#pragma unroll
    for (int k = 0; k < E; ++k) {
      gn.x[k] = g.x[k] / sL;
      dl_ig.x[k] = im[k] * gn.x[k];
    }
    j_hvp<T, E>(t, lane, q, v, hv);
    j_hvp<T, E>(t, lane, q, dl_ig, Hdl);
#pragma unroll
    for (int k = 0; k < E; ++k) {
      hv.x[k] = hv.x[k] / sL;
      Hdl.x[k] = Hdl.x[k] / sL;
    }
    j_half<E>(a2, v, gn, hv, sL, im, Hdl, eps, sp.alpha2_fix);
    j_hvp<T, E>(t, lane, q, v, hv);
#pragma unroll
    for (int k = 0; k < E; ++k) hv.x[k] = hv.x[k] / sL;
  }
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const int i = lane + 32 * k;
    if (i < d) {
      if (qL) qL[(size_t)c * d + i] = T(q.x[k].v);
      dq[(size_t)c * d + i] = T(q.x[k].t[0]);
    }
  }
}

template <typename T, int E>
void launch_e(const TargetDev& t, const StepDev& sp, const T* pos, const T* z, T* qL, T* dq, int C,
              cudaStream_t st) {
  const int tpb = 128;
  const dim3 grid((unsigned)(((size_t)C * 32 + tpb - 1) / tpb));
  monge_alpha2_jvp_kernel<T, E><<<grid, tpb, 0, st>>>(t, sp, pos, z, qL, dq, C);
}

}  // namespace

bool monge_alpha2_jvp_supported(const TargetDev& t) { return monge_warp_supported(t); }

template <typename T>
cudaError_t launch_monge_alpha2_jvp(const TargetDev& t, const StepDev& sp, const T* pos,
                                    const T* z, T* qL, T* dq, int C, cudaStream_t st) {
  if (t.d <= 32)
    launch_e<T, 1>(t, sp, pos, z, qL, dq, C, st);
  else if (t.d <= 64)
    launch_e<T, 2>(t, sp, pos, z, qL, dq, C, st);
  else if (t.d <= 128)
    launch_e<T, 4>(t, sp, pos, z, qL, dq, C, st);
  else if (t.d <= 256)
    launch_e<T, 8>(t, sp, pos, z, qL, dq, C, st);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

template cudaError_t launch_monge_alpha2_jvp<float>(const TargetDev&, const StepDev&, const float*,
                                                    const float*, float*, float*, int,
                                                    cudaStream_t);
template cudaError_t launch_monge_alpha2_jvp<double>(const TargetDev&, const StepDev&,
                                                     const double*, const double*, double*,
                                                     double*, int, cudaStream_t);

}  // namespace gj
