"""Benchmark of the geomjax sampler hot path on one GB300 (or N replicas).

Workload (default, ``--workload logreg``): Bayesian logistic regression,
X ∈ R^{1000×25} iid N(0,1) float32, β* ~ N(0, I), y ~ Bernoulli(σ(Xβ*)),
prior N(0, 100·I), RMHMC with the generalized leapfrog (implicit momentum
and position fixed-point half-steps, explicit final momentum step;
fixed-point tol 1e-6, at most 100 iterations; ``--integrator
implicit_midpoint`` runs the reference's own integrator instead, on every
arm) with the Fisher metric XᵀΛX + I/100, 4096 chains, 8 steps of 0.05 per
transition, mixed precision (FP32 state, split-BF16 tcgen05 contractions,
FP64 Cholesky / log det / accept).  Synthetic seeded data; the reference
publishes no dataset for this path.

A "step" is one transition of every chain.  ``value`` = leapfrog steps/s =
chains × integration steps × timed transitions / device seconds, with the
inputs (z, u) already resident; L2 is flushed (256 MB write) between timed
transitions.  ``e2e`` times the same transitions through the public API
with host buffers: H2D of z and u from pinned memory, the step, D2H of the
new positions and accept flags, every transition.

``--impl reference`` times the reference's algorithm on the host cores: the
reference itself is JAX, which is not installed here, so its float64 NumPy
restatement (``oracle/``) is timed on a bounded sample of chains.

Multi-GPU: chains are independent, so N ranks run N replicas with their own
chains (weak scaling, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

# hardware work queues for the stream pool of posterior batches (read when
# the CUDA context is created)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "min-ESS/s and leapfrog steps/s, batched mixed-precision vs plain FP64 CUDA, 1 GB300"

# DRAM bytes (read + write) per GEMM launch on the default logistic-regression
# workload (4096 chains), averaged over three consecutive GEMM launches of the
# generalized leapfrog's momentum loop (r₂·X, Xβ / S, r₂·X), from one
# cold-cache ncu capture (profiles/gemm_tc_logreg_N1000_d25_C4096_ncu.md).
# Reported only for that chain count.
NCU_TRAFFIC_PER_GEMM_LAUNCH = {("logistic_regression_N1000_d25_rmhmc_fisher_4096chains", 4096): 28.7e6}

WORKLOADS = {
    "logreg": dict(name="logistic_regression_N1000_d25_rmhmc_fisher_4096chains", N=1000, d=25,
                   C=4096, L=8, h=0.05, sampler="rmhmc"),
    "monge": dict(name="funnel_D100_lmcmonge_alpha1_8192chains", D=100, C=8192, L=16, h=0.02,
                  sampler="lmcmonge"),
    "funnel2d": dict(name="funnel_D2_rmhmc_diag_fisher_gl10_fp64_4chains", D=2, C=4, L=10, h=0.1,
                     max_iters=6, sampler="rmhmc_funnel"),
    "trajectory_grad": dict(name="logistic_regression_N2000_d64_gl20_dh_dlambda_1024chains", N=2000,
                            d=64, C=1024, L=20, h=0.02, lam=0.01, sampler="jvp"),
    # the uneven batch's largest posterior as one context (its factorisation
    # takes a CTA of four warps per chain); no plain or ESS arms (the plain
    # CTA-per-chain form stops at d = 64)
    "logreg_large": dict(name="logistic_regression_N5000_d128_rmhmc_fisher_1024chains", N=5000,
                         d=128, C=1024, L=8, h=0.02, sampler="rmhmc", comparisons=False),
    "uneven": dict(name="uneven_logreg_2048posteriors_N200-5000_d8-128_64chains", B=2048, C=64,
                   L=8, h=0.05, sampler="batch"),
    "nuts": dict(name="funnel_D2_nuts_rmhmc_diag_fisher_fp64_4096chains", D=2, C=4096, h=0.1,
                 M=6, sampler="nuts"),
}


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p, "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


_FMA = {}


def _fma_peak(fp64: bool):
    """CUDA-core FMA throughput measured on this device (gj_fma_peak), in
    TFLOP/s; None when the measurement fails."""
    key = "fp64" if fp64 else "fp32"
    if key not in _FMA:
        import ctypes

        import torch

        from geomjax_gb300 import _lib as L

        v = ctypes.c_double(0.0)
        rc = L.lib().gj_fma_peak(L.GJ_FP64 if fp64 else L.GJ_MIXED, ctypes.byref(v),
                                 ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        _FMA[key] = float(v.value) if rc == L.GJ_OK and v.value > 0 else None
    return _FMA[key]


# algorithmic flops of one LMC-Monge leapfrog step per chain and dimension
# (funnel, warp kernel): two half steps ≈ 42, position 2, gradient 3,
# normalising constant and weights 4, three HVPs 15, their scalings 3 (≈ 69,
# divisions counted once), frozen at 72 as the cost model states
MONGE_FLOPS_PER_DIM = 72


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 50 ms.

    ``start`` waits (at most 3 s) for nvidia-smi's first sample, so that the
    sampler runs when the timed region begins; ``stop`` keeps the samples that
    arrived after ``start`` returned (all of them if none did)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0, interval_ms=50):
        self.samples = []  # (arrival time, fields)
        self.proc = None
        self.gpu = gpu_index
        self.interval_ms = interval_ms
        self.t_mark = None

    def start(self, wait_s=3.0):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", str(self.interval_ms)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
            return
        t0 = time.perf_counter()
        while not self.samples and self.proc.poll() is None and time.perf_counter() - t0 < wait_s:
            time.sleep(0.005)
        self.t_mark = time.perf_counter()

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append((time.perf_counter(), [x.strip() for x in line.split(",")]))

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        timed = [s for t, s in self.samples if self.t_mark is not None and t >= self.t_mark]
        for s in timed or [s for _, s in self.samples]:
            try:
                sm.append(float(s[1]))
                mx = float(s[2])
                for n, v in zip(names, s[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
            except Exception:
                pass
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _barrier_max(x, ws):
    if ws == 1:
        return x
    from geomjax_gb300.distributed import max_over_ranks

    return max_over_ranks(x, device="cuda")


def run_ours(args, wl):
    import numpy as np
    import torch

    import geomjax_gb300 as gj
    from geomjax_gb300 import _lib as L
    from geomjax_gb300.data import logreg_data

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    C, Lsteps, h = wl["C"], wl["L"], wl["h"]
    L.check(L.lib().gj_set_gemm_tiling(args.gemm_tile_n, 0 if args.gemm_one_cta else
                                       (1 if args.gemm_two_cta else -1)))
    L.check(L.lib().gj_set_gemm_accumulators(args.gemm_accumulators))
    if wl["sampler"] == "rmhmc":
        X, y = logreg_data(wl["N"], wl["d"], seed=0)
        target = gj.logistic_regression(X, y, precision="mixed", device=dev)
        kern = gj.rmhmc.build_kernel(logreg_path=args.logreg_path, loop=args.loop,
                                     integrator=args.integrator, cholesky=args.cholesky,
                                     chol_chains_per_warp=args.chol_cpw,
                                     chain_groups=args.groups, pdl=args.pdl,
                                     gemm_ksplit=args.gemm_ksplit,
                                     fuse_r2x=not args.no_fuse_r2x,
                                     refine_iterates=not args.no_refine)
        d = wl["d"]
        extra = {}
        state = gj.rmhmc.init(torch.zeros(C, d) + 0.01 * torch.randn(C, d, generator=torch.Generator().manual_seed(rank)), target)
    elif wl["sampler"] == "rmhmc_funnel":
        d = wl["D"]
        target = gj.funnel(D=d, metric="diag", precision="fp64", device=dev)
        kern = gj.rmhmc.build_kernel(integrator="generalized_leapfrog", max_iters=wl["max_iters"])
        extra = {}
        state = gj.rmhmc.init(torch.ones(C, d, dtype=torch.float64), target)
    else:
        d = wl["D"]
        target = gj.funnel(D=d, precision="mixed", device=dev)
        kern = gj.lmcmonge.build_kernel()
        extra = dict(alpha2=1.0, inverse_mass=torch.ones(d, device=dev))
        state = gj.lmcmonge.init(torch.ones(C, d), target)
    K, W = args.steps, args.warmup
    gen = torch.Generator(device=dev)
    gen.manual_seed(1234 + rank)
    Z = torch.randn(K + W, C, d, generator=gen, device=dev, dtype=target.dtype)
    U = torch.rand(K + W, C, generator=gen, device=dev, dtype=torch.float64)
    info = kern.new_info(C, d, target, dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    tuned = None
    if args.autotune and wl["sampler"] == "rmhmc":  # before the warm-up, on a copy of the state
        res = gj.autotune(kern, target, state, h, Lsteps, transitions=3)
        tuned = {"best": res.best, "ms_per_transition": round(res.ms_per_transition, 3),
                 "candidates": len(res.table)}
    # warm-up
    for i in range(W):
        kern.step_inplace(target, state, Z[i], U[i], info, h, Lsteps, **extra)
    torch.cuda.synchronize()
    ctx = kern.context(target, C)
    trace = torch.empty(K, C, d, dtype=target.dtype, device=dev)
    acc_sum = torch.zeros(C, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    stats = np.zeros(11, dtype=np.int64)
    import ctypes

    buf = (ctypes.c_int64 * 11)()
    clocks = ClockSampler(local)
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    t_wall = time.perf_counter()
    for i in range(K):
        flush.zero_()
        evs[i][0].record(stream)
        kern.step_inplace(target, state, Z[W + i], U[W + i], info, h, Lsteps, **extra)
        evs[i][1].record(stream)
        trace[i].copy_(state.position)
        acc_sum += info["acceptance_rate"]
        n = ctx.lib.gj_stats(ctx.h, buf, 11)
        stats += np.array(buf[:11], dtype=np.int64)
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    # dominant-kernel timing: the same transitions with CUDA events around every
    # GEMM launch (profiling switches the batched path to its host-driven loop)
    prof = np.zeros(11, dtype=np.int64)
    if wl["sampler"] == "rmhmc":
        L.check(ctx.lib.gj_profile(ctx.h, 1))
        for i in range(min(K, 3)):
            flush.zero_()
            kern.step_inplace(target, state, Z[W + i], U[W + i], info, h, Lsteps, **extra)
            ctx.lib.gj_stats(ctx.h, buf, 11)
            prof += np.array(buf[:11], dtype=np.int64)
        L.check(ctx.lib.gj_profile(ctx.h, 0))
        torch.cuda.synchronize()
    dev_s = sum(a.elapsed_time(b) for a, b in evs) / 1e3
    dev_s = _barrier_max(dev_s, ws)
    steps_per_s = ws * C * Lsteps * K / dev_s
    min_ess = float("nan")
    if K >= 4:
        # ESS over every rank's chains (per-rank autocovariance sums; replicas
        # exchange nothing while sampling)
        from geomjax_gb300.distributed import global_min_ess

        min_ess = global_min_ess(trace, chain_axis=1, sample_axis=0)
    ess_cmp = None
    if (rank == 0 and args.ess_transitions > 0 and wl["sampler"] in ("rmhmc", "lmcmonge")
            and wl.get("comparisons", True)):
        # rank 0 only: the plain arm is a baseline, not part of the weak-scaled value
        ess_cmp = ess_comparison(args, wl, kern, target, state, info, extra, dev)
    # --- e2e through the public API with host buffers
    Zh = torch.empty(C, d, dtype=target.dtype).pin_memory()
    Uh = torch.empty(C, dtype=torch.float64).pin_memory()
    Ph = torch.empty(C, d, dtype=target.dtype).pin_memory()
    Ah = torch.empty(C, dtype=torch.uint8).pin_memory()
    g2 = torch.Generator().manual_seed(99 + rank)
    Zd = torch.empty(C, d, dtype=target.dtype, device=dev)
    Ud = torch.empty(C, dtype=torch.float64, device=dev)
    Zh.copy_(torch.randn(C, d, generator=g2).to(target.dtype))
    Uh.copy_(torch.rand(C, generator=g2, dtype=torch.float64))
    torch.cuda.synchronize()
    e2e_steps = max(1, min(K, 10))
    t0 = time.perf_counter()
    for i in range(e2e_steps):
        Zd.copy_(Zh, non_blocking=True)
        Ud.copy_(Uh, non_blocking=True)
        kern.step_inplace(target, state, Zd, Ud, info, h, Lsteps, **extra)
        Ph.copy_(state.position, non_blocking=True)
        Ah.copy_(info["is_accepted"], non_blocking=True)
        torch.cuda.current_stream().synchronize()
    e2e_s = _barrier_max(time.perf_counter() - t0, ws)
    e2e = ws * C * Lsteps * e2e_steps / e2e_s
    h2d = Zh.numel() * Zh.element_size() + Uh.numel() * 8
    d2h = Ph.numel() * Ph.element_size() + Ah.numel()
    peaks, src = _peaks()
    roof = None
    if wl["sampler"] == "rmhmc" and prof[4] > 0:
        achieved = prof[3] / (prof[4] * 1e-9) / 1e12  # TFLOP/s over the GEMM launches
        peak = float(peaks.get("bf16_tflops_sustained", peaks["bf16_tflops"]))
        roof = {"bound": "tensor", "kernel": "gemm_tc_kernel (split-BF16 tcgen05)",
                "achieved": round(achieved, 2), "peak": peak, "unit": "TFLOP/s",
                "frac": round(achieved / peak, 4), "peak_source": f"{src} bf16 sustained",
                "traffic": NCU_TRAFFIC_PER_GEMM_LAUNCH.get((wl["name"], C)),
                "traffic_unit": "bytes per GEMM launch (ncu dram read + write)",
                "gemm_ms_per_transition": round(prof[4] * 1e-6 / min(K, 3), 3),
                "gemm_launches_per_transition": int(prof[1] // min(K, 3)),
                "evals_per_transition": round(prof[0] / min(K, 3), 2)}
        if prof[7] > 0:
            # the FP64 metric factorisation, the other half of the time: its
            # algorithmic FP64 rate against the FP64 FMA throughput measured
            # on this device (the measured-peaks file has no FP64 figure)
            fp64 = prof[6] / (prof[7] * 1e-9) / 1e12
            p64 = _fma_peak(True)
            roof["fp64_kernel"] = {
                "kernel": "chol_kernel (FP64 Cholesky, log det, solves)", "achieved": round(fp64, 4),
                "peak": round(p64, 4) if p64 else 1.25, "unit": "TFLOP/s",
                "frac": round(fp64 / (p64 or 1.25), 4),
                "peak_source": ("measured FP64 FMA throughput (gj_fma_peak)" if p64
                                else "nominal GB300 FP64 (measurement failed)"),
                "nominal_peak": 1.25,
                "ms_per_transition": round(prof[7] * 1e-6 / min(K, 3), 3),
                "launches_per_transition": int(prof[5] // min(K, 3))}
        if prof[8] > 0:
            # the position iterates' solves by FP32 factor + FP64 refinement
            # (same kernel, not part of the FP64 rate above)
            roof["refined_iterate_solves"] = {
                "kernel": "chol_kernel (FP32 factor, FP64-residual refinement)",
                "ms_per_transition": round(prof[9] * 1e-6 / min(K, 3), 3),
                "launches_per_transition": int(prof[8] // min(K, 3)),
                "fp64_fallbacks_per_transition": round(float(prof[10]) / min(K, 3), 2)}
    elif wl["sampler"] == "lmcmonge":
        # the warp-per-chain Monge kernel runs on the FP32 pipe: algorithmic
        # flops (MONGE_FLOPS_PER_DIM·D per chain and step) against the FP32
        # FMA throughput measured on this device
        p32 = _fma_peak(False)
        achieved = MONGE_FLOPS_PER_DIM * wl["D"] * steps_per_s / 1e12
        if p32:
            roof = {"bound": "fp32", "kernel": "monge_warp_kernel (warp per chain, FP32)",
                    "achieved": round(achieved, 3), "peak": round(p32, 2), "unit": "TFLOP/s",
                    "frac": round(achieved / p32, 4),
                    "peak_source": "measured FP32 FMA throughput (gj_fma_peak)",
                    "flops_per_step_per_chain": MONGE_FLOPS_PER_DIM * wl["D"],
                    "traffic": None}
    out = {
        "metric": METRIC, "value": round(steps_per_s, 1), "unit": "leapfrog steps/s",
        "n_gpus": ws, "steps": K, "warmup": W, "ms_per_step": round(1e3 * dev_s / K, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"rmhmc": "f32+bf16x3+f64", "rmhmc_funnel": "f64"}.get(wl["sampler"], "f32"),
        "data": "synthetic (seeded)",
        "config": {"workload": wl["name"], "chains_per_gpu": C, "integration_steps": Lsteps,
                   "step_size": h, "precision": "fp64" if wl["sampler"] == "rmhmc_funnel" else "mixed",
                   "integrator": (args.integrator if wl["sampler"] == "rmhmc" else
                                  ("generalized_leapfrog" if wl["sampler"] == "rmhmc_funnel" else None)),
                   "loop": args.loop,
                   "cholesky": args.cholesky, "chol_chains_per_warp": args.chol_cpw or "auto",
                   "chain_groups": args.groups or "auto", "pdl": args.pdl, "gemm_tile_n": args.gemm_tile_n or "auto",
                   "gemm_ksplit": args.gemm_ksplit or "auto",
                   "fuse_r2x": not args.no_fuse_r2x,
                   "refine_iterates": not args.no_refine and args.cholesky == "fp64",
                   "gemm_accumulators": args.gemm_accumulators,
                   "gemm_ctas_per_sm": 1 if args.gemm_one_cta else (2 if args.gemm_two_cta else "auto"),
                   "l2": "flushed between timed steps (256 MB write)",
                   "parallelism": f"replicas x{ws}", "autotune": tuned},
        # min-ESS/s from the post-burn-in trace of ess_comparison when it ran
        # (the K timed transitions start out of equilibrium and are too short)
        "min_ess_per_s": (ess_cmp["mixed"]["min_ess_per_s"] if ess_cmp else
                          (round(min_ess / dev_s, 2) if K >= 4 else None)),
        "min_ess": (ess_cmp["mixed"]["min_ess"] if ess_cmp else
                    (round(min_ess, 2) if K >= 4 else None)),
        "ess_comparison": ess_cmp,
        "mean_acceptance": round(float(acc_sum.mean().item()) / K, 4),
        "e2e": {"value": round(e2e, 1), "unit": "leapfrog steps/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(K * (prof[1] + prof[2]) // max(1, min(K, 3))) if wl["sampler"] == "rmhmc" else K,
        "roofline": roof, "clocks": clk, "wall_s": round(t_wall, 3),
    }
    return out


def run_batch(args, wl):
    """Uneven batch: B logistic-regression posteriors with N and d
    log-uniform in [200, 5000] and [8, 128], C chains each, one transition =
    every posterior's CUDA graph on a pool of streams."""
    import numpy as np
    import torch

    from geomjax_gb300 import _lib as L
    from geomjax_gb300.batch import PosteriorBatch
    from geomjax_gb300.data import logreg_data, uneven_logreg_batch

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    B, C, Lsteps, h = wl["B"], wl["C"], wl["L"], wl["h"]
    L.check(L.lib().gj_set_gemm_tiling(args.gemm_tile_n, 0 if args.gemm_one_cta else
                                       (1 if args.gemm_two_cta else -1)))
    L.check(L.lib().gj_set_gemm_accumulators(args.gemm_accumulators))
    Ns, ds = uneven_logreg_batch(B, seed=rank)
    t_setup = time.perf_counter()
    data = [logreg_data(int(n), int(d), seed=1000 * rank + i) for i, (n, d) in enumerate(zip(Ns, ds))]
    pb = PosteriorBatch(data, C, num_streams=args.streams, device=dev, integrator=args.integrator,
                        one_graph=not args.batch_pool, grouped=not args.batch_branches,
                        buckets=args.batch_buckets)
    if args.cholesky == "fp32":
        pb.set_option(L.GJ_OPT_CHOL_FP64, 0)
    if args.chol_cpw:
        pb.set_option(L.GJ_OPT_CHOL_CHAINS_PER_WARP, args.chol_cpw)
    if args.no_refine:
        pb.set_option(L.GJ_OPT_REFINE_ITERATES, 0)
    del data
    g0 = torch.Generator().manual_seed(rank)
    state = pb.init([0.01 * torch.randn(C, int(d), generator=g0) for d in ds])
    n = int(pb.offsets[-1])
    K, W = args.steps, args.warmup
    gen = torch.Generator(device=dev)
    gen.manual_seed(1234 + rank)
    Z = torch.randn(K + W, n, generator=gen, device=dev, dtype=torch.float32)
    U = torch.rand(K + W, B * C, generator=gen, device=dev, dtype=torch.float64)
    info = pb.new_info()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    tuned = None
    if args.autotune:  # a short candidate list: one transition of the batch takes seconds
        res = gj.autotune_batch(pb, state, h, Lsteps, transitions=1,
                                tilings=((0, -1), (0, 1), (64, -1)), chol_chains_per_warp=(0, 2))
        tuned = {"best": res.best, "ms_per_transition": round(res.ms_per_transition, 3),
                 "candidates": len(res.table)}
    for i in range(W):
        pb.step_inplace(state, Z[i], U[i], info, h, Lsteps)
    torch.cuda.synchronize()
    t_setup = time.perf_counter() - t_setup
    stream = torch.cuda.current_stream()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    acc_sum = torch.zeros(B * C, dtype=torch.float64, device=dev)
    clocks = ClockSampler(local)
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    t_wall = time.perf_counter()
    for i in range(K):
        flush.zero_()
        evs[i][0].record(stream)
        pb.step_inplace(state, Z[W + i], U[W + i], info, h, Lsteps)
        evs[i][1].record(stream)
        acc_sum += info["acceptance_rate"]
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    dev_s = _barrier_max(sum(a.elapsed_time(b) for a, b in evs) / 1e3, ws)
    steps_per_s = ws * B * C * Lsteps * K / dev_s
    # e2e: host draws in, positions and accept flags out, every transition
    Zh = torch.randn(n, generator=torch.Generator().manual_seed(9)).pin_memory()
    Uh = torch.rand(B * C, dtype=torch.float64, generator=torch.Generator().manual_seed(8)).pin_memory()
    Ph = torch.empty(n, dtype=torch.float32).pin_memory()
    Ah = torch.empty(B * C, dtype=torch.uint8).pin_memory()
    Zd, Ud = torch.empty_like(Zh, device=dev), torch.empty_like(Uh, device=dev)
    e2e_steps = max(1, min(K, 5))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(e2e_steps):
        Zd.copy_(Zh, non_blocking=True)
        Ud.copy_(Uh, non_blocking=True)
        pb.step_inplace(state, Zd, Ud, info, h, Lsteps)
        Ph.copy_(state.position, non_blocking=True)
        Ah.copy_(info["is_accepted"], non_blocking=True)
        torch.cuda.current_stream().synchronize()
    e2e_s = _barrier_max(time.perf_counter() - t0, ws)
    return {
        "metric": "leapfrog steps/s over all chains of an uneven posterior batch, 1 GB300",
        "value": round(steps_per_s, 1), "unit": "leapfrog steps/s", "n_gpus": ws, "steps": K,
        "warmup": W, "ms_per_step": round(1e3 * dev_s / K, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+bf16x3+f64",
        "data": "synthetic (seeded)",
        "config": {"workload": wl["name"], "posteriors": B, "chains_per_posterior": C,
                   "integration_steps": Lsteps, "step_size": h, "streams": args.streams,
                   "launch": ("one graph per posterior on the stream pool" if args.batch_pool else
                              ("one CUDA graph per transition, every posterior a branch"
                               if args.batch_branches else
                               "one CUDA graph per transition of grouped launches: every stage "
                               "one grid over a bucket of posteriors, each bucket a branch")),
                   "cholesky": args.cholesky,
                   "refine_iterates": not args.no_refine and args.cholesky == "fp64",
                   "chol_chains_per_warp": args.chol_cpw or "auto",
                   "buckets": None if (args.batch_branches or args.batch_pool) else
                              (args.batch_buckets or "auto"),
                   "mean_N": float(np.mean(Ns)), "mean_d": float(np.mean(ds)),
                   "l2": "flushed between timed steps (256 MB write)",
                   "parallelism": f"replicas x{ws}", "autotune": tuned},
        "mean_acceptance": round(float(acc_sum.mean().item()) / K, 4),
        "e2e": {"value": round(ws * B * C * Lsteps * e2e_steps / e2e_s, 1), "unit": "leapfrog steps/s",
                "h2d_bytes_per_step": int(Zh.numel() * 4 + Uh.numel() * 8),
                "d2h_bytes_per_step": int(Ph.numel() * 4 + Ah.numel())},
        "graph_launches": K if not args.batch_pool else B * K,
        "gpu_launches": 3 * K if not args.batch_pool else None,
        "setup_s": round(t_setup, 1), "clocks": clk,
        "wall_s": round(t_wall, 3),
        "plain_fp64": (batch_plain_comparison(args, wl, Ns, ds, dev)
                       if rank == 0 and not args.no_plain else None),
    }


def batch_plain_comparison(args, wl, Ns, ds, dev, T=4):
    """The uneven batch's mixed pipeline against the plain FP64 form on the
    same sample of posteriors: the first `args.plain_posteriors` posteriors
    whose chains fit one CTA each (d <= 64 and the CTA's shared memory within
    227 KB).  The mixed arm is a PosteriorBatch of those posteriors; the plain
    arm runs each posterior's chains with the CTA-per-chain FP64 kernel, the
    posteriors on concurrent streams.  Both are timed with CUDA events over
    T transitions from the same start positions."""
    import numpy as np
    import torch

    import geomjax_gb300 as gj
    from geomjax_gb300.batch import PosteriorBatch
    from geomjax_gb300.data import logreg_data
    from geomjax_gb300.samplers import cta_supported

    C, Lsteps, h = wl["C"], wl["L"], wl["h"]
    pick = [i for i, (n, d) in enumerate(zip(Ns, ds)) if cta_supported(int(n), int(d), "fp64")]
    pick = pick[: args.plain_posteriors]
    if not pick:
        return None
    data = [logreg_data(int(Ns[i]), int(ds[i]), seed=1000 * 0 + i) for i in pick]
    g0 = torch.Generator().manual_seed(17)
    starts = [0.01 * torch.randn(C, int(ds[i]), generator=g0) for i in pick]
    gen = torch.Generator(device=dev)
    gen.manual_seed(18)
    tot = sum(int(ds[i]) for i in pick) * C
    Z = torch.randn(T, tot, generator=gen, device=dev)
    U = torch.rand(T, len(pick) * C, generator=gen, device=dev, dtype=torch.float64)
    stream = torch.cuda.current_stream()
    # mixed: the batched pipeline over the sample
    pb = PosteriorBatch(data, C, num_streams=args.streams, device=dev, integrator=wl["integrator"])
    st = pb.init(starts)
    info = pb.new_info()
    pb.step_inplace(st, Z[0], U[0], info, h, Lsteps)  # graph capture, untimed
    st = pb.init(starts)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for t in range(T):
        pb.step_inplace(st, Z[t], U[t], info, h, Lsteps)
    e1.record(stream)
    torch.cuda.synchronize()
    s_mixed = e0.elapsed_time(e1) / 1e3
    # plain FP64: one CTA per chain, a stream per posterior
    kern = gj.rmhmc.build_kernel(integrator=wl["integrator"])
    tgs = [gj.logistic_regression(X, y, precision="fp64", device=dev) for X, y in data]
    sts = [gj.rmhmc.init(q.double(), tg) for q, tg in zip(starts, tgs)]
    infos = [kern.new_info(C, tg.dim, tg, dev) for tg in tgs]
    streams = [torch.cuda.Stream(device=dev) for _ in range(min(len(pick), args.streams))]
    offs, o = [], 0
    for i in pick:
        offs.append(o)
        o += int(ds[i]) * C

    def plain_transition(t):
        ev = torch.cuda.Event()
        ev.record(stream)
        for k, (tg, st_, inf) in enumerate(zip(tgs, sts, infos)):
            s_ = streams[k % len(streams)]
            s_.wait_event(ev)
            with torch.cuda.stream(s_):
                z = Z[t, offs[k]:offs[k] + tg.dim * C].view(C, tg.dim).double()
                kern.step_inplace(tg, st_, z, U[t, k * C:(k + 1) * C], inf, h, Lsteps)
        for s_ in streams:
            stream.wait_stream(s_)

    plain_transition(0)  # untimed
    sts = [gj.rmhmc.init(q.double(), tg) for q, tg in zip(starts, tgs)]
    torch.cuda.synchronize()
    e0.record(stream)
    for t in range(T):
        plain_transition(t)
    e1.record(stream)
    torch.cuda.synchronize()
    s_plain = e0.elapsed_time(e1) / 1e3
    steps = len(pick) * C * Lsteps * T
    return {"posteriors": len(pick), "chains_per_posterior": C, "transitions": T,
            "sample": "the first posteriors of the batch with d <= 64 whose chains fit one CTA",
            "mean_N": float(np.mean([Ns[i] for i in pick])),
            "mean_d": float(np.mean([ds[i] for i in pick])),
            "mixed_leapfrog_steps_per_s": round(steps / s_mixed, 1),
            "plain_fp64_leapfrog_steps_per_s": round(steps / s_plain, 1),
            "plain_form": "one CTA per chain, float64 throughout, a stream per posterior",
            "steps_ratio": round(s_plain / s_mixed, 2)}


def run_nuts(args, wl):
    """Iterative NUTS with the RMHMC dynamics (rmhmc/nuts.py) on the funnel
    D = 2 with the diagonal Fisher metric, plain FP64, one thread per chain:
    every chain builds its own tree (up to 2^M states).  A "step" is one NUTS
    transition of every chain; the unit counts the integration steps the
    trees actually took."""
    import torch

    import geomjax_gb300 as gj

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    C, d, h, M = wl["C"], wl["D"], wl["h"], wl["M"]
    tg = gj.funnel(D=d, metric="diag", precision="fp64", device=dev)
    kern = gj.nutsrmhmc.build_kernel(integrator="generalized_leapfrog", max_iters=6)
    st = gj.nutsrmhmc.init(torch.ones(C, d, dtype=torch.float64), tg)
    gen = torch.Generator(device=dev)
    gen.manual_seed(31 + rank)
    K, W = args.steps, args.warmup
    for _ in range(W + 50):  # warm-up and burn-in
        st, _ = kern(gen, st, tg, h, M)
    trace = torch.empty(K, C, d, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(K)]
    nsteps = torch.zeros((), dtype=torch.int64, device=dev)
    clocks = ClockSampler(local)
    torch.cuda.synchronize()
    clocks.start()
    for i in range(K):
        evs[i][0].record(stream)
        st, info = kern(gen, st, tg, h, M)
        evs[i][1].record(stream)
        trace[i].copy_(st.position)
        nsteps += info.num_integration_steps.sum()
    torch.cuda.synchronize()
    clk = clocks.stop()
    dev_s = _barrier_max(sum(a.elapsed_time(b) for a, b in evs) / 1e3, ws)
    steps = float(nsteps.item())
    ess = gj.effective_sample_size(trace, chain_axis=1, sample_axis=0) if K >= 4 else None
    return {
        "metric": "leapfrog steps/s of iterative NUTS-RMHMC (integration steps the trees took), 1 GB300",
        "value": round(ws * steps / dev_s, 1), "unit": "leapfrog steps/s", "n_gpus": ws,
        "steps": K, "warmup": W, "ms_per_step": round(1e3 * dev_s / K, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded)",
        "config": {"workload": wl["name"], "chains": C, "step_size": h, "max_num_doublings": M,
                   "integrator": "generalized_leapfrog", "max_iters": 6,
                   "form": "one thread per chain, float64"},
        "mean_tree_steps": round(steps / (C * K), 2),
        "min_ess_per_s": (round(float(ess.min()) / dev_s, 2) if ess is not None else None),
        "gpu_launches": K, "clocks": clk,
    }


def run_jvp(args, wl):
    """Differentiated trajectory: per chain, p_accept and ΔH of one
    generalized-leapfrog transition of L steps with their derivatives with
    respect to the step size and the metric regulariser (float64 forward
    mode), through gj_logreg_gl_transition_jvp."""
    import torch

    from geomjax_gb300 import autodiff as AD
    from geomjax_gb300.data import logreg_data

    import geomjax_gb300 as gj

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    X, y = logreg_data(wl["N"], wl["d"], seed=0)
    tg = gj.logistic_regression(X, y, precision="fp64", device=dev)
    C, d = wl["C"], wl["d"]
    g0 = torch.Generator().manual_seed(rank)
    q0 = (0.05 * torch.randn(C, d, generator=g0, dtype=torch.float64)).to(dev)
    z = torch.randn(C, d, generator=g0, dtype=torch.float64).to(dev)
    K, W = args.steps, args.warmup
    for _ in range(W):
        AD.transition_jacobian(tg, q0, z, wl["h"], wl["lam"], wl["L"])
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    clocks = ClockSampler(local)
    clocks.start()
    for i in range(K):
        evs[i][0].record(stream)
        J = AD.transition_jacobian(tg, q0, z, wl["h"], wl["lam"], wl["L"])
        evs[i][1].record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    dev_s = _barrier_max(sum(a.elapsed_time(b) for a, b in evs) / 1e3, ws)
    t0 = time.perf_counter()
    Jh = AD.transition_jacobian(tg, q0, z, wl["h"], wl["lam"], wl["L"]).cpu()
    e2e_s = time.perf_counter() - t0
    # roofline: the dual-number Gram assemblies G = XᵀΛX (and its two
    # tangents), 1 + K_q = 7 per step, each N·d(d+1)/2 terms of one product
    # and three FMAs (7 FP64 flops): a lower bound on the kernel's
    # algorithmic FP64 work, against the FP64 FMA throughput measured here
    N, P = wl["N"], d * (d + 1) // 2
    grams = wl["L"] * (1 + 6)
    flops = grams * N * P * 7.0 * C
    achieved = flops / (dev_s / K) / 1e12
    p64 = _fma_peak(True)
    roof = {"bound": "fp64", "kernel": "gl_trajectory_kernel (CTA per chain, Dual<2> float64)",
            "achieved": round(achieved, 4), "peak": round(p64, 4) if p64 else 1.25,
            "unit": "TFLOP/s", "frac": round(achieved / (p64 or 1.25), 4),
            "peak_source": ("measured FP64 FMA throughput (gj_fma_peak)" if p64
                            else "nominal GB300 FP64 (measurement failed)"),
            "flops_counted": "Gram assemblies only: L*(1+K_q) * N * d(d+1)/2 * 7 per chain",
            "traffic": None}
    return {
        "metric": "differentiated leapfrog steps/s (d/dh and d/dlambda, float64 forward mode), 1 GB300",
        "value": round(ws * C * wl["L"] * K / dev_s, 1), "unit": "leapfrog steps/s", "n_gpus": ws,
        "steps": K, "warmup": W, "ms_per_step": round(1e3 * dev_s / K, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64 (dual numbers, 2 tangents)",
        "data": "synthetic (seeded)",
        "config": {"workload": wl["name"], "chains": C, "integration_steps": wl["L"],
                   "step_size": wl["h"], "metric_regulariser": wl["lam"],
                   "fixed_point_evaluations": "6 momentum + 6 position per step"},
        "mean_dDeltaH_dh": float(Jh[:, 4].mean()), "mean_dDeltaH_dlambda": float(Jh[:, 5].mean()),
        "mean_p_accept": float(Jh[:, 0].mean()),
        "e2e": {"value": round(ws * C * wl["L"] / e2e_s, 1), "unit": "leapfrog steps/s",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": int(Jh.numel() * 8)},
        "gpu_launches": K, "roofline": roof, "clocks": clk,
    }


def _moments_agreement(xm, xp, ess_p):
    """Per-coordinate agreement of two traces [T, C, d] of the same chains:
    |Δmean| and |Δvariance| in units of the plain trace's Monte Carlo
    standard errors (mean: sqrt(var/ESS); variance: sqrt((m4 − var²)/ESS))."""
    import torch

    a = xm.double().reshape(-1, xm.shape[-1])
    b = xp.double().reshape(-1, xp.shape[-1])
    ma, mb = a.mean(0), b.mean(0)
    va, vb = a.var(0), b.var(0)
    m4 = ((b - mb) ** 4).mean(0)
    se_m = torch.sqrt(vb / ess_p)
    se_v = torch.sqrt(torch.clamp(m4 - vb * vb, min=0.0) / ess_p)
    dm = (ma - mb).abs() / se_m
    dv = (va - vb).abs() / se_v
    return {"max_mean_dev_in_mcse": round(float(dm.max()), 4),
            "max_var_dev_in_mcse": round(float(dv.max()), 4),
            "coords_within_2_mcse": int(((dm < 2) & (dv < 2)).sum()), "coords": int(a.shape[1])}


def ess_comparison(args, wl, kern, target, state, info, extra, dev):
    """min-ESS/s of the batched mixed-precision form against the plain FP64
    form on the same posterior.  After a burn-in of the mixed chains, both
    arms run the same number of transitions from the same positions with
    common random numbers (the same z and u; z is drawn in float32), each
    transition timed with CUDA events on the launching stream and L2 flushed
    between transitions.  The plain arm samples the first `plain_chains`
    chains.  ESS is diagnostics.py:78-209 over each arm's trace."""
    import torch

    import geomjax_gb300 as gj

    T, burn = args.ess_transitions, args.ess_burnin
    C, d = state.position.shape
    Lsteps, h = wl["L"], wl["h"]
    gen = torch.Generator(device=dev)
    gen.manual_seed(777)
    for _ in range(burn):
        kern.step_inplace(target, state, torch.randn(C, d, generator=gen, device=dev,
                                                     dtype=target.dtype),
                          torch.rand(C, generator=gen, device=dev, dtype=torch.float64), info, h,
                          Lsteps, **extra)
    start = state.position.detach().clone()
    Z = torch.randn(T, C, d, generator=gen, device=dev, dtype=torch.float32)
    U = torch.rand(T, C, generator=gen, device=dev, dtype=torch.float64)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()

    def run(kern_, target_, st_, info_, extra_):
        n = st_.position.shape[0]
        tr = torch.empty(T, n, d, dtype=target_.dtype, device=dev)
        acc = torch.empty(T, n, dtype=torch.uint8, device=dev)
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(T)]
        torch.cuda.synchronize()
        for i in range(T):
            z = Z[i, :n].to(target_.dtype)
            flush.zero_()
            evs[i][0].record(stream)
            kern_.step_inplace(target_, st_, z, U[i, :n], info_, h, Lsteps, **extra_)
            evs[i][1].record(stream)
            tr[i].copy_(st_.position)
            acc[i].copy_(info_["is_accepted"])
        torch.cuda.synchronize()
        return tr, acc, sum(a.elapsed_time(b) for a, b in evs) / 1e3

    tr_m, acc_m, s_m = run(kern, target, state, info, extra)
    # the warp-per-chain Monge form needs every chain to fill the GPU (8192
    # chains are 1024 CTAs); the CTA-per-chain logistic form fills it with
    # plain_chains and costs ~60x more per chain
    Cp = C if wl["sampler"] == "lmcmonge" else min(C, args.plain_chains)
    if wl["sampler"] == "rmhmc":
        from geomjax_gb300.data import logreg_data

        X, y = logreg_data(wl["N"], wl["d"], seed=0)
        pt = gj.logistic_regression(X, y, precision="fp64", device=dev)
        pk = gj.rmhmc.build_kernel(integrator=wl["integrator"])  # one CTA per chain
        pst = gj.rmhmc.init(start[:Cp].double(), pt)
        pextra = {}
        form = "one CTA per chain, float64 throughout (data, state, Gram, factor, solves)"
    else:
        pt = gj.funnel(D=wl["D"], precision="fp64", device=dev)
        pk = gj.lmcmonge.build_kernel()  # one warp per chain
        pst = gj.lmcmonge.init(start[:Cp].double(), pt)
        pextra = dict(alpha2=1.0, inverse_mass=torch.ones(d, dtype=torch.float64, device=dev))
        form = "one warp per chain, float64 throughout"
    pinfo = pk.new_info(Cp, d, pt, dev)
    tr_p, acc_p, s_p = run(pk, pt, pst, pinfo, pextra)
    ess_m = gj.effective_sample_size(tr_m, chain_axis=1, sample_axis=0)
    ess_p = gj.effective_sample_size(tr_p, chain_axis=1, sample_axis=0)
    ess_m_sub = gj.effective_sample_size(tr_m[:, :Cp], chain_axis=1, sample_axis=0)
    mixed = {"chains": C, "min_ess": round(float(ess_m.min()), 2), "device_s": round(s_m, 4),
             "min_ess_per_s": round(float(ess_m.min()) / s_m, 2),
             "leapfrog_steps_per_s": round(C * Lsteps * T / s_m, 1)}
    plain = {"chains": Cp, "form": form, "min_ess": round(float(ess_p.min()), 2),
             "device_s": round(s_p, 4), "min_ess_per_s": round(float(ess_p.min()) / s_p, 2),
             "leapfrog_steps_per_s": round(Cp * Lsteps * T / s_p, 1)}
    agree = _moments_agreement(tr_m[:, :Cp], tr_p, ess_p)
    agree["accept_agreement"] = round(float((acc_m[:, :Cp] == acc_p).double().mean()), 6)
    agree["mixed_min_ess_same_chains"] = round(float(ess_m_sub.min()), 2)
    return {"transitions": T, "burn_in": burn,
            "draws": "common random numbers: the same z (float32) and u on both arms",
            "mixed": mixed, "plain_fp64": plain,
            "min_ess_ratio": round(mixed["min_ess_per_s"] / plain["min_ess_per_s"], 3),
            "posterior_agreement": agree}


def run_plain_fp64(args, wl):
    """The thread-per-chain FP64 form of the same workload: one thread per
    chain, every vector and the metric algebra in float64.  For the
    dense-Fisher workload it runs on a bounded sample of chains (each chain
    costs O(N·d²) FP64 per map evaluation in one thread); the min-ESS/s
    comparison uses the CTA-per-chain FP64 form instead (ess_comparison)."""
    import torch

    import geomjax_gb300 as gj
    from geomjax_gb300.data import logreg_data

    dev = torch.device("cuda", _dist()[2])
    Lsteps, h = wl["L"], wl["h"]
    if wl["sampler"] == "rmhmc":
        C = min(wl["C"], 256)
        X, y = logreg_data(wl["N"], wl["d"], seed=0)
        target = gj.logistic_regression(X, y, precision="fp64", device=dev)
        kern = gj.rmhmc.build_kernel(integrator=wl["integrator"], logreg_path="per_chain")
        d = wl["d"]
        extra = {}
        state = gj.rmhmc.init(0.01 * torch.randn(C, d, generator=torch.Generator().manual_seed(0),
                                                 dtype=torch.float64), target)
        K = 2
    else:
        C = wl["C"]
        d = wl["D"]
        target = gj.funnel(D=d, precision="fp64", device=dev)
        kern = gj.lmcmonge.build_kernel(warp=False)
        extra = dict(alpha2=1.0, inverse_mass=torch.ones(d, dtype=torch.float64, device=dev))
        state = gj.lmcmonge.init(torch.ones(C, d, dtype=torch.float64), target)
        K = args.steps
    gen = torch.Generator(device=dev)
    gen.manual_seed(4321)
    info = kern.new_info(C, d, target, dev)
    W = 1 if wl["sampler"] == "rmhmc" else args.warmup
    for i in range(W):
        kern.step_inplace(target, state, torch.randn(C, d, generator=gen, device=dev, dtype=torch.float64),
                          torch.rand(C, generator=gen, device=dev, dtype=torch.float64), info, h, Lsteps,
                          **extra)
    Z = torch.randn(K, C, d, generator=gen, device=dev, dtype=torch.float64)
    U = torch.rand(K, C, generator=gen, device=dev, dtype=torch.float64)
    stream = torch.cuda.current_stream()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    torch.cuda.synchronize()
    for i in range(K):
        evs[i][0].record(stream)
        kern.step_inplace(target, state, Z[i], U[i], info, h, Lsteps, **extra)
        evs[i][1].record(stream)
    torch.cuda.synchronize()
    dev_s = sum(a.elapsed_time(b) for a, b in evs) / 1e3
    # leapfrog steps/s only: its few transitions start out of equilibrium, so
    # an ESS of them would not be a min-ESS/s (ess_comparison has that)
    return {"value": round(C * Lsteps * K / dev_s, 1), "unit": "leapfrog steps/s", "chains": C,
            "transitions": K, "ms_per_step": round(1e3 * dev_s / K, 3),
            "form": "one thread per chain, float64 throughout"}


def cpu_baseline(wl, budget_s=12.0):
    """The float64 oracle on the host cores, on a bounded sample of chains."""
    import numpy as np

    from oracle import lmcmonge as O_monge
    from oracle import rmhmc as O_rm
    from oracle import targets as OT

    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    rng = np.random.Generator(np.random.PCG64(0))
    if wl["sampler"] == "rmhmc":
        X, y = OT.make_logreg_data(wl["N"], wl["d"], seed=0)
        ot = OT.LogisticRegression(X, y)
        d = wl["d"]

        def run(C):
            q = rng.standard_normal((C, d)) * 0.01
            s = O_rm.init(ot, q)
            t = time.perf_counter()
            O_rm.kernel(ot, s, rng.standard_normal((C, d)), rng.random(C), wl["h"], wl["L"],
                        integrator=wl["integrator"])
            return time.perf_counter() - t
    elif wl["sampler"] == "rmhmc_funnel":
        ot = OT.Funnel(D=wl["D"], metric="diag")
        d = wl["D"]

        def run(C):
            s = O_rm.init(ot, np.ones((C, d)))
            t = time.perf_counter()
            for _ in range(50):
                s, _ = O_rm.kernel(ot, s, rng.standard_normal((C, d)), rng.random(C), wl["h"],
                                   wl["L"], integrator="generalized_leapfrog", max_iters=wl["max_iters"])
            return (time.perf_counter() - t) / 50
    else:
        d = wl["D"]
        ot = OT.Funnel(D=d)

        def run(C):
            s = O_monge.init(ot, np.ones((C, d)))
            t = time.perf_counter()
            O_monge.kernel(ot, s, rng.standard_normal((C, d)), rng.random(C), wl["h"], np.ones(d),
                           wl["L"], alpha2=1.0)
            return time.perf_counter() - t
    C = 8
    t = run(C)
    while t < budget_s / 4 and C < wl["C"]:
        C = min(wl["C"], C * 4)
        t = run(C)
    return {"value": round(C * wl["L"] / t, 2), "unit": "leapfrog steps/s", "cores": cores,
            "kind": "port",
            "sample": f"{C} chains x 1 transition x {wl['L']} steps of the same workload, "
                      f"float64 NumPy oracle ({t:.1f} s)"}


def run_reference(args, wl):
    ws, rank, _ = _dist()
    if rank != 0:
        return None
    import numpy as np

    from oracle import lmcmonge as O_monge
    from oracle import rmhmc as O_rm
    from oracle import targets as OT

    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    rng = np.random.Generator(np.random.PCG64(0))
    if wl["sampler"] == "jvp":
        return {"impl": "reference", "unavailable": "the reference differentiates trajectories with "
                "JAX autodiff, and JAX is not installable here; the float64 oracle has no derivative"}
    if wl["sampler"] == "nuts":
        from oracle import nuts as O_nuts

        ot = OT.Funnel(D=wl["D"], metric="diag")
        d, C, M = wl["D"], 16, wl["M"]
        s = O_rm.init(ot, np.ones((C, d)))
        counted = {"n": 0}

        def step(s):
            s2, infos = O_nuts.kernel(ot, s, rng.standard_normal((C, d)),
                                      rng.random((C, O_nuts.num_uniforms(M))), wl["h"], M,
                                      integrator="generalized_leapfrog", max_iters=6)
            counted["n"] += int(sum(i.num_integration_steps for i in infos))
            return s2

        for _ in range(max(1, min(args.warmup, 2))):
            s = step(s)
        counted["n"] = 0
        t0 = time.perf_counter()
        for _ in range(args.steps):
            s = step(s)
        dt = time.perf_counter() - t0
        v = counted["n"] / dt
        return {
            "metric": "leapfrog steps/s of iterative NUTS-RMHMC (integration steps the trees took)",
            "value": round(v, 2), "unit": "leapfrog steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(1e3 * dt / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)", "impl": "reference",
            "config": {"workload": wl["name"], "chains_sampled": C},
            "cpu_baseline": {"value": round(v, 2), "unit": "leapfrog steps/s", "cores": cores,
                             "kind": "port", "sample": f"{C} chains per step, float64 NumPy "
                                                       "restatement in oracle/"},
            "e2e": {"value": round(v, 2), "unit": "leapfrog steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    if wl["sampler"] == "rmhmc_funnel":
        ot = OT.Funnel(D=wl["D"], metric="diag")
        d, C = wl["D"], wl["C"]
        s = O_rm.init(ot, np.ones((C, d)))

        def step(s):
            s2, _ = O_rm.kernel(ot, s, rng.standard_normal((C, d)), rng.random(C), wl["h"], wl["L"],
                                integrator="generalized_leapfrog", max_iters=wl["max_iters"])
            return s2
    elif wl["sampler"] == "rmhmc":
        X, y = OT.make_logreg_data(wl["N"], wl["d"], seed=0)
        ot = OT.LogisticRegression(X, y)
        d = wl["d"]
        C = 16
        s = O_rm.init(ot, rng.standard_normal((C, d)) * 0.01)

        def step(s):
            s2, _ = O_rm.kernel(ot, s, rng.standard_normal((C, d)), rng.random(C), wl["h"], wl["L"],
                                integrator=wl["integrator"])
            return s2
    elif wl["sampler"] == "batch":
        # a bounded sample of the uneven batch: 8 chains of each of the first
        # four posteriors, one after another as the reference would run them
        from geomjax_gb300.data import uneven_logreg_batch

        Ns, ds = uneven_logreg_batch(wl["B"], seed=0)
        C = 8
        posts = []
        for i in range(4):
            X, y = OT.make_logreg_data(int(Ns[i]), int(ds[i]), seed=1000 + i)
            ot_i = OT.LogisticRegression(X, y)
            posts.append((ot_i, int(ds[i]), O_rm.init(ot_i, rng.standard_normal((C, int(ds[i]))) * 0.01)))
        C = 8 * len(posts)

        def step(s):
            out = []
            for ot_i, d_i, s_i in s:
                s2, _ = O_rm.kernel(ot_i, s_i, rng.standard_normal((8, d_i)), rng.random(8),
                                    wl["h"], wl["L"], integrator=wl["integrator"])
                out.append((ot_i, d_i, s2))
            return out

        s = posts
    else:
        d = wl["D"]
        ot = OT.Funnel(D=d)
        C = 256
        s = O_monge.init(ot, np.ones((C, d)))

        def step(s):
            s2, _ = O_monge.kernel(ot, s, rng.standard_normal((C, d)), rng.random(C), wl["h"],
                                   np.ones(d), wl["L"], alpha2=1.0)
            return s2
    for _ in range(max(1, min(args.warmup, 2))):
        s = step(s)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        s = step(s)
    dt = time.perf_counter() - t0
    v = C * wl["L"] * args.steps / dt
    return {
        "metric": METRIC, "value": round(v, 2), "unit": "leapfrog steps/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * dt / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded)", "impl": "reference",
        "config": {"workload": wl["name"], "chains_sampled": C, "integration_steps": wl["L"],
                   "step_size": wl["h"],
                   "integrator": (wl["integrator"] if wl["sampler"] in ("rmhmc", "batch") else
                                  ("generalized_leapfrog" if wl["sampler"] == "rmhmc_funnel"
                                   else None))},
        "cpu_baseline": {"value": round(v, 2), "unit": "leapfrog steps/s", "cores": cores,
                         "kind": "port",
                         "sample": f"{C} chains per step (JAX reference not installable; float64 "
                                   f"NumPy restatement in oracle/)"},
        "e2e": {"value": round(v, 2), "unit": "leapfrog steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="logreg", choices=sorted(WORKLOADS))
    ap.add_argument("--logreg-path", default="tcgen05", choices=["auto", "simt", "tcgen05", "per_chain"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--integrator", default="generalized_leapfrog",
                    choices=["implicit_midpoint", "generalized_leapfrog"],
                    help="RMHMC integrator of the logistic-regression workloads")
    ap.add_argument("--autotune", action="store_true",
                    help="pick the GEMM tile policy and the factorisation's chains per warp by "
                         "timing the candidates before the warm-up (batched paths)")
    ap.add_argument("--no-plain", action="store_true",
                    help="skip the thread-per-chain plain FP64 arm")
    ap.add_argument("--ess-transitions", type=int, default=200,
                    help="transitions of the min-ESS/s comparison on each arm (0 = skip)")
    ap.add_argument("--ess-burnin", type=int, default=100,
                    help="untimed burn-in transitions of the mixed chains before it")
    ap.add_argument("--plain-chains", type=int, default=1024,
                    help="chains of the plain FP64 arm of the min-ESS/s comparison")
    ap.add_argument("--plain-posteriors", type=int, default=64,
                    help="posteriors of the uneven batch's plain FP64 comparison")
    ap.add_argument("--chains", type=int, default=None, help="override the chain count (small cases)")
    ap.add_argument("--loop", default="graph", choices=["graph", "host"],
                    help="fixed-point loop driver of the batched path (host: profilable by ncu)")
    ap.add_argument("--cholesky", default="fp64", choices=["fp64", "fp32"])
    ap.add_argument("--gemm-tile-n", type=int, default=0, choices=[0, 64, 128],
                    help="tcgen05 GEMM output tile width for N > 64 (0 = automatic)")
    ap.add_argument("--gemm-one-cta", action="store_true",
                    help="deep operand ring, one CTA per SM, for every GEMM")
    ap.add_argument("--gemm-two-cta", action="store_true",
                    help="operand ring cut back to two CTAs per SM for every GEMM")
    ap.add_argument("--gemm-accumulators", type=int, default=4, choices=[1, 2, 4],
                    help="most K-range TMEM accumulators per tcgen05 GEMM CTA")
    ap.add_argument("--gemm-ksplit", type=int, default=0, choices=[0, 1, 2, 3, 4],
                    help="K slices of the gradient contraction (0 = automatic)")
    ap.add_argument("--no-fuse-r2x", action="store_true",
                    help="store r2 and contract it by its own GEMM in the momentum evaluations "
                         "(default: r2·X inside the S GEMM's epilogue)")
    ap.add_argument("--no-refine", action="store_true",
                    help="factor the generalized leapfrog's position iterates in FP64 (default: "
                         "FP32 factor, solve refined with FP64 residuals)")
    ap.add_argument("--pdl", action="store_true",
                    help="launch the batched pipeline's kernels with programmatic dependent launch")
    ap.add_argument("--groups", type=int, default=0,
                    help="chain groups on concurrent streams (0 = automatic)")
    ap.add_argument("--streams", type=int, default=16, help="stream pool of the uneven batch")
    ap.add_argument("--batch-branches", action="store_true",
                    help="uneven batch: every posterior its own branch of the graph "
                         "(default: grouped launches over buckets of posteriors)")
    ap.add_argument("--batch-buckets", type=int, default=0,
                    help="uneven batch, grouped launches: buckets of posteriors (0 = automatic)")
    ap.add_argument("--batch-pool", action="store_true",
                    help="uneven batch: one graph per posterior on the stream pool instead of one "
                         "graph holding every posterior")
    ap.add_argument("--posteriors", type=int, default=None, help="override the uneven batch size")
    ap.add_argument("--chol-cpw", type=int, default=0, choices=[0, 1, 2, 4, 8],
                    help="chains per warp in the metric factorisation (0 = automatic)")
    args = ap.parse_args()
    wl = dict(WORKLOADS[args.workload])
    wl["integrator"] = args.integrator  # the logistic-regression workloads' RMHMC integrator
    if args.chains:
        wl["C"] = args.chains
        wl["name"] = wl["name"].rsplit("_", 1)[0] + f"_{args.chains}chains"
    if args.posteriors and "B" in wl:
        wl["B"] = args.posteriors
        wl["name"] = wl["name"].replace("2048posteriors", f"{args.posteriors}posteriors")
    ws, rank, local = _dist()
    if args.impl == "reference":
        out = run_reference(args, wl)
        if out is not None:
            print(json.dumps(out), flush=True)
        return
    if ws > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    if wl["sampler"] in ("batch", "jvp", "nuts"):
        out = {"batch": run_batch, "jvp": run_jvp, "nuts": run_nuts}[wl["sampler"]](args, wl)
        if rank == 0:
            print(json.dumps(out), flush=True)
        return
    out = run_ours(args, wl)
    if rank == 0:
        if out.get("ess_comparison"):
            cmp_ = out["ess_comparison"]
            out["plain_fp64"] = dict(cmp_["plain_fp64"], transitions=cmp_["transitions"])
            out["min_ess_ratio"] = cmp_["min_ess_ratio"]
        if (not args.no_plain and wl["sampler"] in ("rmhmc", "lmcmonge")
                and wl.get("comparisons", True)):
            # the thread-per-chain FP64 form, kept for continuity
            out["plain_fp64_thread_per_chain"] = run_plain_fp64(args, wl)
            out["steps_ratio_vs_thread_per_chain"] = round(
                out["value"] / out["plain_fp64_thread_per_chain"]["value"], 1)
        if not args.no_cpu_baseline:
            out["cpu_baseline"] = cpu_baseline(wl)
        print(json.dumps(out), flush=True)
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
