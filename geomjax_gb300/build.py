"""Build the CUDA shared library of geomjax_gb300 in-tree with nvcc for sm_103a.

``python -m geomjax_gb300.build`` or ``geomjax_gb300.build.build()``.  Each
translation unit is compiled in parallel; the result is
``geomjax_gb300/_build/libgeomjax_gb300.so``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libgeomjax_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "--expt-relaxed-constexpr", "-diag-suppress", "177,2190"]

# (source, extra defines) — chain_kernels.cu is compiled once per precision so
# the two halves build in parallel.
UNITS = [
    ("chain_kernels.cu", ["-DGJ_CHAIN_PREC=1"]),
    ("chain_kernels.cu", ["-DGJ_CHAIN_PREC=2"]),
    ("monge_warp.cu", []),
    ("logreg_cta.cu", []),
    ("logreg_batched.cu", []),
    ("gemm_simt.cu", []),
    ("gemm_tc.cu", []),
    ("capi.cu", []),
    ("noalloc.cu", []),
    ("traj_jvp.cu", []),
    ("chees.cu", []),
    ("monge_jvp.cu", []),
    ("peaks.cu", []),
]


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _compile(nvcc, src, defs, out, verbose):
    cmd = [nvcc, *ARCH, *FLAGS, *defs, "-c", os.path.join(CSRC, src), "-o", out]
    if verbose:
        cmd.append("-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return r.stderr


def sources_newer_than(path):
    if not os.path.exists(path):
        return True
    t = os.path.getmtime(path)
    for root, _, files in os.walk(CSRC):
        for f in files:
            if os.path.getmtime(os.path.join(root, f)) > t:
                return True
    inc = os.path.join(os.path.dirname(HERE), "include")
    for f in os.listdir(inc):
        if os.path.getmtime(os.path.join(inc, f)) > t:
            return True
    return False


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not sources_newer_than(LIB):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    objs = []
    jobs = []
    with cf.ThreadPoolExecutor(max_workers=min(len(UNITS), os.cpu_count() or 4)) as ex:
        for i, (src, defs) in enumerate(UNITS):
            out = os.path.join(BUILD, f"u{i}_{os.path.splitext(src)[0]}.o")
            objs.append(out)
            jobs.append((src, ex.submit(_compile, nvcc, src, defs, out, verbose)))
        logs = []
        for src, j in jobs:
            logs.append((src, j.result()))
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        for src, log in logs:
            sys.stderr.write(f"== {src}\n{log}\n")
    return LIB


if __name__ == "__main__":
    import time

    t0 = time.time()
    p = build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(p, f"{time.time() - t0:.1f}s")
