"""Builds libmwblas_gb300.so (and the static libmwblas_gb300.a) from csrc/
with nvcc for sm_103a.

Each .cu translation unit is compiled in parallel into _build/, then linked
into a shared library next to this file and archived beside it. A unit is recompiled only when it or
any header in csrc/ or include/ is newer than its object.

Usage:  python build.py            (or call build() from Python)
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmwblas_gb300.so")
ARCHIVE = os.path.join(HERE, "libmwblas_gb300.a")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    # Each FP64 step of the error-free transforms must round on its own.
    "-fmad=false",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
    "-I" + INCLUDE,
]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newest_header() -> float:
    t = 0.0
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh")):
                t = max(t, os.path.getmtime(os.path.join(d, f)))
    return t


def _compile(nvcc: str, src: str, obj: str, verbose: bool) -> None:
    cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj]
    if os.environ.get("MWBLAS_PTXAS_VERBOSE"):
        cmd += ["-Xptxas", "-v"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip() and (verbose or os.environ.get("MWBLAS_PTXAS_VERBOSE")):
        print(r.stderr, file=sys.stderr)


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compiles (incrementally) and links the library; returns its path."""
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    hdr = _newest_header()
    units = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    todo = []
    objs = []
    for u in units:
        src = os.path.join(CSRC, u)
        obj = os.path.join(BUILD, u[:-3] + ".o")
        objs.append(obj)
        if not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), hdr):
            todo.append((src, obj))
    if todo:
        jobs = jobs or min(len(todo), os.cpu_count() or 4)
        with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
            futs = [ex.submit(_compile, nvcc, s, o, verbose) for s, o in todo]
            for f in futs:
                f.result()
    if todo or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        tmp = LIB + ".tmp"
        cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lpthread"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    if not os.path.exists(ARCHIVE) or os.path.getmtime(ARCHIVE) < max(os.path.getmtime(o) for o in objs):
        # the same objects as a static archive; a program links it with the
        # static CUDA runtime: -lmwblas_gb300 -lcudart_static -lstdc++ -lpthread -ldl -lrt
        tmp = ARCHIVE + ".tmp"
        if os.path.exists(tmp):
            os.remove(tmp)
        r = subprocess.run(["ar", "rcs", tmp, *objs], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"archive failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, ARCHIVE)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
