"""Build libocelot_sc.so (sm_103a) in-tree with nvcc.

Each .cu translation unit compiles in parallel to an object file under
ocelot_gb300/_build/, then nvcc links them into ocelot_gb300/lib/libocelot_sc.so
with the CUDA runtime linked statically, so the library loads through ctypes
with or without PyTorch in the process.  A unit is recompiled only when it or
a header is newer than its object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libocelot_sc.so")

SOURCES = ["sc_api.cu", "sc_particles.cu", "sc_sort.cu", "sc_green.cu", "sc_fft.cu", "sc_tmap.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: no implicit contraction of a*b+c into FMAs.  Every kernel body
# is inlined into a plain and a batched kernel, and a + b*c + d*e can be
# contracted either way; without implicit contraction each body rounds the
# same in both, so a beam's result does not depend on how it was launched.
# The FMAs the kernels want are written out (fma, __fma_rn).
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "--expt-relaxed-constexpr", "-I", os.path.join(REPO, "include")]
if os.environ.get("OCELOT_SC_CHECKED") == "1":
    # index checks that record the first bad index in the device state
    FLAGS += ["-DSC_CHECKED"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libocelot_sc")


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(REPO, "include", "ocelot_sc.h"))
    return hs


def _stale(src: str, obj: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src, *deps])


def _compile(src: str, obj: str, verbose: bool):
    cmd = [nvcc(), *ARCH, *FLAGS, "-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
    return r.stderr if verbose else ""


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    deps = _headers()
    jobs = []
    objs = []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s.replace(".cu", ".o"))
        objs.append(obj)
        if force or verbose or _stale(src, obj, deps):
            jobs.append((src, obj))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for out in ex.map(lambda j: _compile(j[0], j[1], verbose), jobs):
                if out:
                    sys.stderr.write(out)
    if jobs or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
