"""Build libnekgpu.so in-tree: nvcc for sm_103a, one object per translation
unit compiled in parallel, then one shared library with the C ABI of
include/nekgpu.h.  No cmake, no torch extension machinery."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libnekgpu.so")
SOURCES = ["axhelm_f64.cu", "axhelm_f32.cu", "axhelm_tma.cu", "axhelm_df.cu", "tune.cu", "gs.cu", "pcg.cu", "mixed.cu", "split.cu", "perm.cu", "batch.cu", "adjoint.cu", "proj.cu", "multi.cu", "noalloc.cu", "geom.cu", "gmres.cu", "h1mg.cu", "amg.cu", "vecops.cu", "gradops.cu", "plan4.cu", "stress.cu", "dealias.cu", "capi.cu",
           "meshio.cpp", "h1mg_plan.cpp", "xxt.cpp", "amg_plan.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
# host-only sources: no contraction into fused multiply-adds, so that x86 and
# aarch64 hosts round the same way
HOST_FLAGS = ["-Xcompiler", "-ffp-contract=off"]


def _obj(src: str) -> str:
    return os.path.join(BUILD, os.path.splitext(src)[0] + ".o")


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(obj: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers += [os.path.join(ROOT, "include", h) for h in ("nekgpu.h", "nekmesh.h")]
    nv = nvcc()
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = _obj(src)
        if force or _stale(o, [s] + headers):
            extra = HOST_FLAGS if src.endswith(".cpp") else []
            jobs.append([nv, *ARCH, *FLAGS, *extra, "-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            futs = [ex.submit(subprocess.run, j, capture_output=True, text=True) for j in jobs]
            for j, f in zip(jobs, futs):
                r = f.result()
                if verbose and r.stdout:
                    print(r.stdout)
                if r.returncode != 0:
                    raise RuntimeError(f"nvcc failed: {' '.join(j)}\n{r.stdout}\n{r.stderr}")
    objs = [_obj(s) for s in SOURCES]
    if force or jobs or _stale(LIB, objs):
        r = subprocess.run([nv, *ARCH, "-shared", "-o", LIB, *objs], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
