"""Generates tests/golden/ref_gemm_scalar.npz from the reference's scalar GEMM.

Runs in the development container only (it needs the reference sources):
`make -C oracle ref REF=<checkout>` builds the reference's double-double
sources twice, with its AVX2 block (libmwblas_ref.so) and without the SIMD
defines (libmwblas_ref_scalar.so): the second is the scalar micro-kernel
(mgemm_serial.cpp:355-407, non-SIMD branch) that the reference compiles to
where the AVX2 path is unavailable, as on an aarch64 host. Seeded GEMM inputs
are fed to mgemm_64_ of the scalar build; inputs and outputs are saved.

The fixture pins the oracle's port of that path (or_port_mgemm with
simd_order = 0), the CPU baseline timed on aarch64 hosts, bit for bit
(tests/test_oracle_pin.py). The scalar path computes every C element in one
fixed order whatever the OpenMP team, so one team size suffices.

Usage: python tests/golden/make_gemm_scalar.py
"""
from __future__ import annotations

import importlib.util
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "ref_gemm_scalar.npz")
SEED = 20261204
REF_SCALAR = os.path.join(ROOT, "oracle", "_ref", "libmwblas_ref_scalar.so")

# m, n, k, transa, transb, beta kind: crossing the MC = 64, KC = 128 and
# NC = 256 block edges of mgemm_serial.cpp:35-37, with padded leading dimensions
CASES = [
    (7, 5, 3, "N", "N", "rand"),
    (65, 33, 130, "N", "N", "rand"),
    (64, 40, 129, "T", "N", "zero"),
    (30, 70, 257, "N", "T", "one"),
    (70, 20, 140, "T", "T", "rand"),
    (5, 260, 20, "N", "N", "rand"),
    (129, 9, 64, "C", "N", "rand"),
]


def _load(name, path):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def main():
    mwb = _load("mwblas", os.path.join(ROOT, "epblas-parallel_gb300", "mwblas.py"))
    if not os.path.exists(REF_SCALAR):
        raise SystemExit("build the reference first: make -C oracle ref REF=<checkout of the reference>")
    ref = mwb.MWBlas(REF_SCALAR, extensions=False)
    rng = np.random.default_rng(SEED)
    data, meta = {}, []
    for ci, (m, n, k, ta, tb, bk) in enumerate(CASES):
        ar, ac = (m, k) if ta == "N" else (k, m)
        br, bc = (k, n) if tb == "N" else (n, k)
        lda, ldb, ldc = ar + 1, br + 2, m + 3
        A = mwb.dd_matrix(rng, ar, ac, lda)
        B = mwb.dd_matrix(rng, br, bc, ldb)
        C0 = mwb.dd_matrix(rng, m, n, ldc)
        al = mwb.random_dd(rng, ())
        be = {"rand": mwb.random_dd(rng, ()), "zero": np.zeros(2), "one": np.array([1.0, 0.0])}[bk]
        out = C0.copy()
        ref.mgemm(ta, tb, m, n, k, al, A, lda, B, ldb, be, out, ldc)
        key = f"g{ci}"
        data.update({key + "_A": A, key + "_B": B, key + "_C": C0, key + "_alpha": al, key + "_beta": be,
                     key + "_ref": out})
        meta.append(dict(key=key, m=m, n=n, k=k, ta=ta, tb=tb, lda=lda, ldb=ldb, ldc=ldc))
    data["meta_json"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(OUT, **data)
    print(f"wrote {OUT} ({len(meta)} cases)")


if __name__ == "__main__":
    main()
