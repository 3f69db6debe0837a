"""Builds and runs the dual-link timing harness (tests/dual/dual_driver.c).

The reference compares implementations of the same BLAS inside ONE process:
each static archive's exported symbols get a per-leg prefix with objcopy
(benchmark/dual/BENCH_PROTOCOL.md:32-38, benchmark/dual/nsbuild.sh), so the
legs link together without clashes, and the driver times them back to back
on shared buffers. This script does the same for:

  gb300      libmwblas_gb300.a (epblas-parallel_gb300/build.py), every exported
             ABI name renamed gb_<name>;
  port       the C restatement of the reference's algorithms, oracle/ddoracle.c
             (its own or_* names need no renaming);
  reference  the reference's own double-double objects under oracle/_ref/mf/
             (built by `make -C oracle ref`, only where a checkout exists),
             archived and renamed ref_<name>.

It links the driver against the static CUDA runtime and prints the driver's
JSON lines (wall time per call for each leg, min over reps; the ratios;
the largest relative difference between the legs' results).

Usage: python tests/dual/run_dual.py [--reps R] [--gemm-n N] [--vec-n N]
"""
from __future__ import annotations

import argparse
import glob
import json
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
BUILD = os.path.join(HERE, "_build")
GB_ARCHIVE = os.path.join(ROOT, "epblas-parallel_gb300", "libmwblas_gb300.a")
REF_OBJS = os.path.join(ROOT, "oracle", "_ref", "mf")
ABI_NAME = re.compile(r"^[a-z][a-z0-9_]*$")   # the exported C names (C++ internals are mangled)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{' '.join(cmd)} failed:\n{r.stdout}\n{r.stderr}")
    return r.stdout


def exported_names(archive_or_objs):
    """Global defined ABI names of an archive (or a list of objects)."""
    paths = archive_or_objs if isinstance(archive_or_objs, list) else [archive_or_objs]
    out = _run(["nm", "-g", "--defined-only", *paths])
    names = set()
    for line in out.splitlines():
        parts = line.split()
        if len(parts) == 3 and parts[1] in "TDBR" and ABI_NAME.match(parts[2]):
            names.add(parts[2])
    return sorted(names)


def namespace(src_archive, prefix, out_archive):
    """objcopy --redefine-syms: every exported ABI name -> prefix + name."""
    names = exported_names(src_archive)
    mapfile = out_archive + ".map"
    with open(mapfile, "w") as f:
        for n in names:
            f.write(f"{n} {prefix}{n}\n")
    _run(["objcopy", f"--redefine-syms={mapfile}", src_archive, out_archive])
    return names


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    if not os.path.exists(GB_ARCHIVE):
        sys.path.insert(0, os.path.join(ROOT, "epblas-parallel_gb300"))
        import build as libbuild   # noqa: E402
        libbuild.build()
    gb_ns = os.path.join(BUILD, "lib_gb_ns.a")
    namespace(GB_ARCHIVE, "gb_", gb_ns)
    objs = [gb_ns]
    defs = []
    ref_objs = sorted(glob.glob(os.path.join(REF_OBJS, "*.o")))
    if ref_objs:
        ref_a = os.path.join(BUILD, "lib_ref.a")
        if os.path.exists(ref_a):
            os.remove(ref_a)
        _run(["ar", "rcs", ref_a, *ref_objs])
        ref_ns = os.path.join(BUILD, "lib_ref_ns.a")
        namespace(ref_a, "ref_", ref_ns)
        objs.append(ref_ns)
        defs.append("-DHAVE_REF")
    cc = shutil.which("gcc") or "cc"
    port_o = os.path.join(BUILD, "ddoracle.o")
    _run([cc, "-std=gnu11", "-O2", "-fopenmp", "-ffp-contract=off", "-c",
          os.path.join(ROOT, "oracle", "ddoracle.c"), "-o", port_o])
    drv_o = os.path.join(BUILD, "dual_driver.o")
    _run([cc, "-std=gnu11", "-O2", "-fopenmp", *defs, "-c", os.path.join(HERE, "dual_driver.c"), "-o", drv_o])
    exe = os.path.join(BUILD, "dual_driver")
    cuda_lib = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64")
    _run([shutil.which("g++") or "c++", drv_o, port_o, *objs, f"-L{cuda_lib}", "-lcudart_static", "-lpthread",
          "-ldl", "-lrt", "-lm", "-fopenmp", "-o", exe])
    return exe, bool(ref_objs)


def run(reps=10, gemm_n=1024, vec_n=1 << 22):
    exe, _ = build()
    out = _run([exe, str(reps), str(gemm_n), str(vec_n)])
    return [json.loads(line) for line in out.splitlines() if line.startswith("{")]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reps", type=int, default=10)
    ap.add_argument("--gemm-n", type=int, default=1024)
    ap.add_argument("--vec-n", type=int, default=1 << 22)
    a = ap.parse_args()
    for row in run(a.reps, a.gemm_n, a.vec_n):
        print(json.dumps(row))


if __name__ == "__main__":
    main()
