"""Build libfmf.so (the sm_103a CUDA library) in-tree with nvcc.

Each translation unit under csrc/ is compiled separately and in parallel, then
linked into ``fmf/_lib/libfmf.so``.  The drop-in kernels are compiled with
``-fmad=false`` so that every multiply and add is rounded separately, in the
reference's order; the fused step kernels (files named ``fused_*.cu``) and the
arithmetic-heavy adjoint kernels (``adj_mom.cu``, ``adj_visc.cu``,
``adj_transport.cu``, whose recomputed branch tests round operation by operation
through explicit intrinsics) let nvcc contract multiply-adds.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
OUT = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT, "libfmf.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _flags(name: str):
    base = ["-O3", "-lineinfo", "-std=c++17", "--extended-lambda", "-Xcompiler", "-fPIC",
            "-Xcompiler", "-O2"] + ARCH
    contract = name.startswith("fused_") or name in ("adj_mom.cu", "adj_visc.cu", "adj_transport.cu")
    base += ["-fmad=true"] if contract else ["-fmad=false"]
    return base


def _needs(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    deps.append(os.path.join(ROOT, "..", "include", "fmf_capi.h"))
    return any(os.path.exists(d) and os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra=None) -> str:
    os.makedirs(OUT, exist_ok=True)
    objdir = os.path.join(OUT, "obj")
    os.makedirs(objdir, exist_ok=True)
    nv = nvcc()
    jobs = []
    for f in sources():
        src = os.path.join(CSRC, f)
        obj = os.path.join(objdir, f[:-3] + ".o")
        if force or _needs(obj, src):
            cmd = [nv] + _flags(f) + (extra or []) + ["-c", src, "-o", obj]
            jobs.append((f, cmd))
    def run(job):
        f, cmd = job
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {f}:\n{r.stdout}\n{r.stderr}")
        return f, r.stderr
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for f, err in ex.map(run, jobs):
                if verbose and err.strip():
                    print(f, err, file=sys.stderr)
    objs = [os.path.join(objdir, f[:-3] + ".o") for f in sources()]
    if jobs or not os.path.exists(LIB):
        cmd = [nv] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
