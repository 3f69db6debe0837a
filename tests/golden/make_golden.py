"""Generates tests/golden/ref_vectors.npz from the reference itself.

Runs in the development container only (it needs the reference sources):
  1. `make -C oracle ref` builds the reference's own double-double sources
     (src/epblas-parallel/multifloats/*.cpp, against the clean-room shim in
     oracle/shim/) into oracle/_ref/libmwblas_ref.so and its __float128
     sources (src/epblas-parallel/kind16/*.c) into oracle/_ref/libkind16_ref.so.
  2. Seeded inputs are fed to both through their Fortran-style C ABI.
  3. Inputs and outputs are saved; the bit-exact level-1 routines are run
     once per OpenMP team size, each in a fresh process with OMP_NUM_THREADS
     set, because the reference's body/tail split follows the team.

The fixtures pin the CPU oracle (tests/test_oracle_pin.py) and give the GPU
parity tests the reference's own outputs.

Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import importlib.util
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "ref_vectors.npz")
TEAMS = (1, 3, 8)
SEED = 20240617


def _load(name, path):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


mwb = _load("mwblas", os.path.join(ROOT, "epblas-parallel_gb300", "mwblas.py"))
orc = _load("oracle", os.path.join(ROOT, "oracle", "oracle.py"))

REF_MW = os.path.join(ROOT, "oracle", "_ref", "libmwblas_ref.so")
REF_K16 = os.path.join(ROOT, "oracle", "_ref", "libkind16_ref.so")

L1_NS = (0, 1, 3, 5, 8, 13, 64, 2051)
L1_INCS = (1, -1, 2, -3)


def l1_inputs(rng):
    cases = []
    for n in L1_NS:
        for inc in L1_INCS:
            if inc != 1 and n > 64:
                continue
            cases.append((n, inc))
    data = {}
    for ci, (n, inc) in enumerate(cases):
        span = max(1, 1 + (n - 1) * abs(inc)) if n > 0 else 1
        data[f"l1_{ci}_x"] = mwb.random_dd(rng, (span,))
        data[f"l1_{ci}_y"] = mwb.random_dd(rng, (span,))
        data[f"l1_{ci}_cx"] = mwb.random_cdd(rng, (span,))
        data[f"l1_{ci}_alpha"] = mwb.random_dd(rng, ())
        data[f"l1_{ci}_calpha"] = mwb.random_cdd(rng, ())
    return cases, data


def run_l1(team_env: int) -> dict:
    """Child process: reference level-1 outputs under OMP_NUM_THREADS=team_env."""
    rng = np.random.default_rng(SEED)
    cases, data = l1_inputs(rng)
    ref = mwb.MWBlas(REF_MW, extensions=False)
    out = {}
    for ci, (n, inc) in enumerate(cases):
        x = data[f"l1_{ci}_x"].copy()
        ref.mscal(n, data[f"l1_{ci}_alpha"], x, inc)
        out[f"t{team_env}_mscal_{ci}"] = x
        cx = data[f"l1_{ci}_cx"].copy()
        ref.wscal(n, data[f"l1_{ci}_calpha"], cx, inc)
        out[f"t{team_env}_wscal_{ci}"] = cx
        cx = data[f"l1_{ci}_cx"].copy()
        ref.wmscal(n, data[f"l1_{ci}_alpha"], cx, inc)
        out[f"t{team_env}_wmscal_{ci}"] = cx
        y = data[f"l1_{ci}_y"].copy()
        ref.maxpy(n, data[f"l1_{ci}_alpha"], data[f"l1_{ci}_x"], inc, y, inc)
        out[f"t{team_env}_maxpy_{ci}"] = y
        if inc == 1 and n > 0:
            r = ref.mdot(n, data[f"l1_{ci}_x"], 1, data[f"l1_{ci}_y"], 1)
            out[f"t{team_env}_mdot_{ci}"] = np.array(r)
    return out


class K16:
    """The reference's kind16 (__float128) routines, arrays as raw quad buffers."""

    def __init__(self, o):
        self.o = o
        self.lib = C.CDLL(REF_K16)

    def q(self, x):
        return self.o.to_quad(x)

    def gemm(self, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, cplx=False):
        I = lambda v: C.byref(C.c_int64(v))
        qa, qb, qc = self.q(a), self.q(b), self.q(c)
        qal, qbe = self.q(alpha), self.q(beta)
        f = self.lib.xgemm_64_ if cplx else self.lib.qgemm_64_
        f(ta.encode(), tb.encode(), I(m), I(n), I(k), C.c_void_p(qal.ctypes.data), C.c_void_p(qa.ctypes.data), I(lda), C.c_void_p(qb.ctypes.data),
          I(ldb), C.c_void_p(qbe.ctypes.data), C.c_void_p(qc.ctypes.data), I(ldc))
        return self.o.from_quad(qc, c.shape)

    def syrk(self, uplo, trans, n, k, alpha, a, lda, beta, c, ldc, herk=False):
        I = lambda v: C.byref(C.c_int64(v))
        qa, qc, qal, qbe = self.q(a), self.q(c), self.q(alpha), self.q(beta)
        f = self.lib.xherk_64_ if herk else self.lib.qsyrk_64_
        f(uplo.encode(), trans.encode(), I(n), I(k), C.c_void_p(qal.ctypes.data), C.c_void_p(qa.ctypes.data), I(lda), C.c_void_p(qbe.ctypes.data),
          C.c_void_p(qc.ctypes.data), I(ldc))
        return self.o.from_quad(qc, c.shape)

    def trsm(self, side, uplo, ta, diag, m, n, alpha, a, lda, b, ldb):
        I = lambda v: C.byref(C.c_int64(v))
        qa, qb, qal = self.q(a), self.q(b), self.q(alpha)
        self.lib.qtrsm_64_(side.encode(), uplo.encode(), ta.encode(), diag.encode(), I(m), I(n), C.c_void_p(qal.ctypes.data),
                           C.c_void_p(qa.ctypes.data), I(lda), C.c_void_p(qb.ctypes.data), I(ldb))
        return self.o.from_quad(qb, b.shape)

    def gemv(self, trans, m, n, alpha, a, lda, x, incx, beta, y, incy):
        I = lambda v: C.byref(C.c_int64(v))
        qa, qx, qy, qal, qbe = self.q(a), self.q(x), self.q(y), self.q(alpha), self.q(beta)
        self.lib.qgemv_64_(trans.encode(), I(m), I(n), C.c_void_p(qal.ctypes.data), C.c_void_p(qa.ctypes.data), I(lda), C.c_void_p(qx.ctypes.data),
                           I(incx), C.c_void_p(qbe.ctypes.data), C.c_void_p(qy.ctypes.data), I(incy))
        return self.o.from_quad(qy, y.shape)

    def dot(self, n, x, incx, y, incy):
        # qdot_ returns __float128 by value; use a 1x1x n GEMM instead (exact same sum in binary128).
        one = np.array([1.0, 0.0]); zero = np.array([0.0, 0.0])
        c = np.zeros((1, 1, 2))
        xs = x[::incx] if incx > 0 else x[::incx]
        ys = y[::incy] if incy > 0 else y[::incy]
        return self.gemm("T", "N", 1, 1, n, one, np.ascontiguousarray(xs[:n]), n,
                         np.ascontiguousarray(ys[:n]), n, zero, c, 1)[0, 0]


def l3_cases(rng, data, k16, ref):
    meta = []

    def rscal():
        return mwb.random_dd(rng, ())

    def rcscal():
        return mwb.random_cdd(rng, ())

    # real GEMM: all trans, padded lds, general alpha/beta and beta = 0
    for ci, (ta, tb, m, n, k, pad) in enumerate([
            ("N", "N", 17, 13, 11, 3), ("N", "T", 9, 20, 33, 0), ("T", "N", 24, 7, 40, 5),
            ("T", "T", 31, 29, 5, 1), ("N", "N", 40, 24, 130, 0), ("C", "N", 5, 6, 7, 2)]):
        lda = (m if ta == "N" else k) + pad
        ldb = (k if tb == "N" else n) + pad
        ldc = m + pad
        A = mwb.dd_matrix(rng, m if ta == "N" else k, k if ta == "N" else m, lda)
        B = mwb.dd_matrix(rng, k if tb == "N" else n, n if tb == "N" else k, ldb)
        Cm = mwb.dd_matrix(rng, m, n, ldc)
        al, be = rscal(), (rscal() if ci % 2 == 0 else np.zeros(2))
        key = f"gemm_{ci}"
        data.update({key + "_A": A, key + "_B": B, key + "_C": Cm, key + "_alpha": al, key + "_beta": be})
        data[key + "_q"] = k16.gemm(ta, tb, m, n, k, al, A, lda, B, ldb, be, Cm.copy(), ldc)
        c2 = Cm.copy()
        ref.mgemm(ta, tb, m, n, k, al, A, lda, B, ldb, be, c2, ldc)
        data[key + "_ref"] = c2
        meta.append(dict(kind="gemm", key=key, ta=ta, tb=tb, m=m, n=n, k=k, lda=lda, ldb=ldb, ldc=ldc))

    # complex GEMM
    for ci, (ta, tb, m, n, k, pad) in enumerate([
            ("N", "N", 11, 9, 13, 2), ("N", "C", 8, 12, 17, 0), ("C", "T", 15, 6, 9, 1), ("T", "N", 7, 7, 20, 0)]):
        lda = (m if ta == "N" else k) + pad
        ldb = (k if tb == "N" else n) + pad
        ldc = m + pad
        A = mwb.dd_matrix(rng, m if ta == "N" else k, k if ta == "N" else m, lda, cplx_=True)
        B = mwb.dd_matrix(rng, k if tb == "N" else n, n if tb == "N" else k, ldb, cplx_=True)
        Cm = mwb.dd_matrix(rng, m, n, ldc, cplx_=True)
        al, be = rcscal(), (rcscal() if ci % 2 == 0 else np.zeros((2, 2)))
        key = f"wgemm_{ci}"
        data.update({key + "_A": A, key + "_B": B, key + "_C": Cm, key + "_alpha": al, key + "_beta": be})
        data[key + "_q"] = k16.gemm(ta, tb, m, n, k, al, A, lda, B, ldb, be, Cm.copy(), ldc, cplx=True)
        c2 = Cm.copy()
        ref.wgemm(ta, tb, m, n, k, al, A, lda, B, ldb, be, c2, ldc)
        data[key + "_ref"] = c2
        meta.append(dict(kind="wgemm", key=key, ta=ta, tb=tb, m=m, n=n, k=k, lda=lda, ldb=ldb, ldc=ldc))

    # SYRK / HERK
    for ci, (uplo, trans, n, k, pad) in enumerate([
            ("U", "N", 19, 7, 2), ("L", "T", 12, 25, 0), ("U", "T", 33, 9, 1), ("L", "N", 40, 30, 0)]):
        lda = (n if trans == "N" else k) + pad
        ldc = n + pad
        A = mwb.dd_matrix(rng, n if trans == "N" else k, k if trans == "N" else n, lda)
        Cm = mwb.dd_matrix(rng, n, n, ldc)
        al, be = rscal(), (rscal() if ci % 2 == 0 else np.zeros(2))
        key = f"syrk_{ci}"
        data.update({key + "_A": A, key + "_C": Cm, key + "_alpha": al, key + "_beta": be})
        data[key + "_q"] = k16.syrk(uplo, trans, n, k, al, A, lda, be, Cm.copy(), ldc)
        c2 = Cm.copy()
        ref.msyrk(uplo, trans, n, k, al, A, lda, be, c2, ldc)
        data[key + "_ref"] = c2
        meta.append(dict(kind="syrk", key=key, uplo=uplo, trans=trans, n=n, k=k, lda=lda, ldc=ldc))
    for ci, (uplo, trans, n, k, pad) in enumerate([
            ("U", "N", 14, 9, 1), ("L", "C", 11, 16, 0), ("L", "N", 24, 40, 2), ("U", "C", 9, 3, 0)]):
        lda = (n if trans == "N" else k) + pad
        ldc = n + pad
        A = mwb.dd_matrix(rng, n if trans == "N" else k, k if trans == "N" else n, lda, cplx_=True)
        Cm = mwb.dd_matrix(rng, n, n, ldc, cplx_=True)
        al, be = rscal(), (rscal() if ci % 2 == 0 else np.zeros(2))
        key = f"herk_{ci}"
        data.update({key + "_A": A, key + "_C": Cm, key + "_alpha": al, key + "_beta": be})
        data[key + "_q"] = k16.syrk(uplo, trans, n, k, al, A, lda, be, Cm.copy(), ldc, herk=True)
        c2 = Cm.copy()
        ref.wherk(uplo, trans, n, k, al, A, lda, be, c2, ldc)
        data[key + "_ref"] = c2
        meta.append(dict(kind="herk", key=key, uplo=uplo, trans=trans, n=n, k=k, lda=lda, ldc=ldc))

    # TRSM: diagonally dominant triangles (fuzz_mtrsm.fypp:67-117 recipe)
    ci = 0
    for side in ("L", "R"):
        for uplo in ("U", "L"):
            for ta in ("N", "T"):
                for diag in ("N", "U"):
                    m, n = (13, 6) if side == "L" else (7, 11)
                    if ci in (0, 8):
                        m, n = (130, 5) if side == "L" else (5, 130)
                    na = m if side == "L" else n
                    lda, ldb = na + 1, m + 2
                    A = mwb.dd_matrix(rng, na, na, lda)
                    A[..., 0] /= na
                    A[..., 1] /= na
                    for d in range(na):
                        A[d, d, 0] = 1.0 + rng.random()
                        A[d, d, 1] = 0.0
                    B = mwb.dd_matrix(rng, m, n, ldb)
                    al = rscal()
                    key = f"trsm_{ci}"
                    data.update({key + "_A": A, key + "_B": B, key + "_alpha": al})
                    data[key + "_q"] = k16.trsm(side, uplo, ta, diag, m, n, al, A, lda, B.copy(), ldb)
                    b2 = B.copy()
                    ref.mtrsm(side, uplo, ta, diag, m, n, al, A, lda, b2, ldb)
                    data[key + "_ref"] = b2
                    meta.append(dict(kind="trsm", key=key, side=side, uplo=uplo, ta=ta, diag=diag, m=m, n=n,
                                     lda=lda, ldb=ldb))
                    ci += 1

    # GEMV
    for ci, (trans, m, n, incx, incy, pad) in enumerate([
            ("N", 23, 17, 1, 1, 2), ("T", 19, 31, 1, 1, 0), ("N", 12, 9, 2, -1, 1), ("T", 40, 8, -3, 2, 0),
            ("N", 150, 40, 1, 1, 0)]):
        lda = m + pad
        A = mwb.dd_matrix(rng, m, n, lda)
        lx, ly = (n, m) if trans == "N" else (m, n)
        x = mwb.random_dd(rng, (1 + (lx - 1) * abs(incx),))
        y = mwb.random_dd(rng, (1 + (ly - 1) * abs(incy),))
        al, be = rscal(), (rscal() if ci % 2 == 0 else np.zeros(2))
        key = f"gemv_{ci}"
        data.update({key + "_A": A, key + "_x": x, key + "_y": y, key + "_alpha": al, key + "_beta": be})
        data[key + "_q"] = k16.gemv(trans, m, n, al, A, lda, x, incx, be, y.copy(), incy)
        y2 = y.copy()
        ref.mgemv(trans, m, n, al, A, lda, x, incx, be, y2, incy)
        data[key + "_ref"] = y2
        meta.append(dict(kind="gemv", key=key, trans=trans, m=m, n=n, lda=lda, incx=incx, incy=incy))

    # DOT (binary128 via a 1x1xn GEMM in kind16)
    for ci, n in enumerate((1, 7, 1000, 3000)):
        x = mwb.random_dd(rng, (n,))
        y = mwb.random_dd(rng, (n,))
        key = f"dot_{ci}"
        data.update({key + "_x": x, key + "_y": y})
        data[key + "_q"] = k16.dot(n, x, 1, y, 1)
        data[key + "_ref"] = np.array(ref.mdot(n, x, 1, y, 1))
        meta.append(dict(kind="dot", key=key, n=n))

    # I*AMAX with exact ties and lo-limb tie-breaks
    for ci, n in enumerate((2, 9, 33, 1000)):
        x = mwb.random_dd(rng, (n,))
        big = 2.0
        pos = rng.choice(n, size=min(3, n), replace=False)
        for t, p in enumerate(sorted(pos)):
            x[p, 0] = big if t % 2 == 0 else -big
            x[p, 1] = 0.0
        if n > 5:
            q = int(rng.integers(0, n))
            x[q, 0] = big
            x[q, 1] = 2.0 ** -60   # wins on the lo limb
        cx = mwb.random_cdd(rng, (n,))
        key = f"amax_{ci}"
        data.update({key + "_x": x, key + "_cx": cx})
        data[key + "_ref"] = np.array([ref.imamax(n, x, 1), ref.imamax(n, x, 1, cplx_=True) if False else 0])
        data[key + "_ref"][1] = ref.imamax(n, cx, 1, cplx_=True)
        meta.append(dict(kind="amax", key=key, n=n))
    return meta


def main():
    if len(sys.argv) > 2 and sys.argv[1] == "--l1-child":
        out = run_l1(int(sys.argv[2]))
        np.savez(sys.argv[3], **out)
        return
    orc.build(ref=True)
    o = orc.Oracle()
    data = {}
    rng = np.random.default_rng(SEED)
    cases, l1data = l1_inputs(rng)
    data.update(l1data)
    tmp = os.path.join(HERE, "_l1_tmp.npz")
    for t in TEAMS:
        env = dict(os.environ, OMP_NUM_THREADS=str(t))
        subprocess.run([sys.executable, __file__, "--l1-child", str(t), tmp], check=True, env=env)
        with np.load(tmp) as z:
            data.update({k: z[k] for k in z.files})
    os.remove(tmp)
    ref = mwb.MWBlas(REF_MW, extensions=False)
    k16 = K16(o)
    meta = l3_cases(np.random.default_rng(SEED + 1), data, k16, ref)
    data["meta_json"] = np.frombuffer(json.dumps(
        dict(seed=SEED, teams=TEAMS, l1_cases=cases, l3=meta)).encode(), dtype=np.uint8)
    np.savez_compressed(OUT, **data)
    print(f"wrote {OUT}: {len(data)} arrays, {os.path.getsize(OUT) / 1e6:.2f} MB")


if __name__ == "__main__":
    main()
