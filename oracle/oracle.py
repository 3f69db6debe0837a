"""ctypes wrapper of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline legs of bench.py, always as the checker or the timed CPU
baseline, never as the implementation under test.

Also holds the reference's normwise error metric
(test/.../fuzz_util_body.fypp:242-271, fuzz_gemm_real_body.fypp:90-98):
    err = max|C - C_ref| / max(max|C_ref|, op_norm),
    op_norm = |alpha| * k * max|A| * max|B| + |beta| * max|C0|.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

_i64 = C.c_int64
_p = C.c_void_p
_c = C.c_char


def build(ref: bool = False, ref_dir: str | None = None) -> None:
    """Builds liboracle.so (and, when `ref`, the reference libraries from the
    reference checkout at `ref_dir`, else at $EPBLAS_REFERENCE_DIR)."""
    targets = ["all"] + (["ref"] if ref else [])
    extra = []
    if ref:
        d = ref_dir or os.environ.get("EPBLAS_REFERENCE_DIR", "")
        if not d:
            raise RuntimeError("building the reference needs EPBLAS_REFERENCE_DIR (a checkout of the reference)")
        extra = [f"REF={d}"]
    subprocess.run(["make", "-s", "-C", HERE, f"-j{os.cpu_count() or 4}", *targets, *extra], check=True)


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, int):
        return a
    return a.ctypes.data


class DD2(C.Structure):
    """A double-double returned by value (two doubles, hi first)."""
    _fields_ = [("hi", C.c_double), ("lo", C.c_double)]


# generator -> number of pointer arguments
GENERATORS = {"mcabs1": 1, "mrotg": 4, "mrotmg": 5, "wrotg": 4}


class Oracle:
    def __init__(self, path: str = LIB):
        if not os.path.exists(path):
            build()
        self.lib = C.CDLL(path)
        L = self.lib
        sig = {
            "or_mscal": [_i64, _p, _p, _i64, _i64],
            "or_wscal": [_i64, _p, _p, _i64, _i64],
            "or_wmscal": [_i64, _p, _p, _i64, _i64],
            "or_maxpy": [_i64, _p, _p, _i64, _p, _i64, _i64],
            "or_copy": [_i64, _p, _i64, _p, _i64, C.c_int],
            "or_swap": [_i64, _p, _i64, _p, _i64, C.c_int],
            "or_qgemm": [_c, _c, _i64, _i64, _i64, _p, _p, _i64, _p, _i64, _p, _p, _i64, _i64, _p, _p, _p],
            "or_qwgemm": [_c, _c, _i64, _i64, _i64, _p, _p, _i64, _p, _i64, _p, _p, _i64, _i64, _p, _p, _p],
            "or_qsyrk": [_c, _c, _i64, _i64, _p, _p, _i64, _p, _p, _i64],
            "or_qherk": [_c, _c, _i64, _i64, _p, _p, _i64, _p, _p, _i64],
            "or_qtrsm": [_c, _c, _c, _c, _i64, _i64, _p, _p, _i64, _p, _i64],
            "or_qgemv": [_c, _i64, _i64, _p, _p, _i64, _p, _i64, _p, _p, _i64],
            "or_qdot": [_i64, _p, _i64, _p, _i64, _p],
            "or_qaxpy": [_i64, _p, _p, _p],
            "or_port_mgemm": [_c, _c, _i64, _i64, _i64, _p, _p, _i64, _p, _i64, _p, _p, _i64, C.c_int],
            "or_port_mdot": [_i64, _p, _p, _i64, _p],
            "or_dd_mul_fast": [_p, _p, _p, _i64],
            "or_dd_add_fast": [_p, _p, _p, _i64],
            "or_dd_mul_exact": [_p, _p, _p, _i64],
            "or_dd_add_exact": [_p, _p, _p, _i64],
            "or_dd_to_q": [_p, _p, _i64],
            "or_q_to_dd": [_p, _p, _i64],
        }
        for name, args in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = None
        for name in ("or_imamax", "or_iwamax"):
            f = getattr(L, name)
            f.argtypes = [_i64, _p, _i64]
            f.restype = _i64
        L.or_max_threads.restype = C.c_int
        for name, nargs in GENERATORS.items():
            f = getattr(L, "or_" + name)
            f.argtypes = [_p] * nargs
            f.restype = DD2 if name == "mcabs1" else None

    # scalar generators (mcabs1.cpp, mrotg.cpp, mrotmg.cpp, wrotg.cpp), with the
    # reference's argument order; float64 arrays are modified in place
    def generator(self, name, *bufs):
        r = getattr(self.lib, "or_" + name)(*[_ptr(b) for b in bufs])
        return np.array([r.hi, r.lo]) if name == "mcabs1" else None

    # bit-exact level 1 (arrays modified in place)
    def mscal(self, n, alpha, x, incx, team=1):
        a = np.asarray(alpha, dtype=np.float64).reshape(2).copy()
        self.lib.or_mscal(n, _ptr(a), _ptr(x), incx, team)

    def wscal(self, n, alpha, x, incx, team=1):
        a = np.asarray(alpha, dtype=np.float64).reshape(2, 2).copy()
        self.lib.or_wscal(n, _ptr(a), _ptr(x), incx, team)

    def wmscal(self, n, alpha, x, incx, team=1):
        a = np.asarray(alpha, dtype=np.float64).reshape(2).copy()
        self.lib.or_wmscal(n, _ptr(a), _ptr(x), incx, team)

    def maxpy(self, n, alpha, x, incx, y, incy, team=1):
        a = np.asarray(alpha, dtype=np.float64).reshape(2).copy()
        self.lib.or_maxpy(n, _ptr(a), _ptr(x), incx, _ptr(y), incy, team)

    def copy(self, n, x, incx, y, incy, elem=1):
        self.lib.or_copy(n, _ptr(x), incx, _ptr(y), incy, elem)

    def swap(self, n, x, incx, y, incy, elem=1):
        self.lib.or_swap(n, _ptr(x), incx, _ptr(y), incy, elem)

    def imamax(self, n, x, incx):
        return int(self.lib.or_imamax(n, _ptr(x), incx))

    def iwamax(self, n, x, incx):
        return int(self.lib.or_iwamax(n, _ptr(x), incx))

    # binary128 references (results rounded to DD)
    def qgemm(self, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, rows=None, cols=None):
        al = np.asarray(alpha, dtype=np.float64).reshape(2).copy()
        be = np.asarray(beta, dtype=np.float64).reshape(2).copy()
        if rows is None:
            self.lib.or_qgemm(ta.encode(), tb.encode(), m, n, k, _ptr(al), _ptr(a), lda, _ptr(b), ldb, _ptr(be),
                              _ptr(c), ldc, 0, None, None, None)
            return c
        rows = np.ascontiguousarray(rows, dtype=np.int64)
        cols = np.ascontiguousarray(cols, dtype=np.int64)
        out = np.zeros((len(rows), 2))
        self.lib.or_qgemm(ta.encode(), tb.encode(), m, n, k, _ptr(al), _ptr(a), lda, _ptr(b), ldb, _ptr(be),
                          _ptr(c), ldc, len(rows), _ptr(rows), _ptr(cols), _ptr(out))
        return out

    def qwgemm(self, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, rows=None, cols=None):
        al = np.asarray(alpha, dtype=np.float64).reshape(2, 2).copy()
        be = np.asarray(beta, dtype=np.float64).reshape(2, 2).copy()
        if rows is None:
            self.lib.or_qwgemm(ta.encode(), tb.encode(), m, n, k, _ptr(al), _ptr(a), lda, _ptr(b), ldb, _ptr(be),
                               _ptr(c), ldc, 0, None, None, None)
            return c
        rows = np.ascontiguousarray(rows, dtype=np.int64)
        cols = np.ascontiguousarray(cols, dtype=np.int64)
        out = np.zeros((len(rows), 2, 2))
        self.lib.or_qwgemm(ta.encode(), tb.encode(), m, n, k, _ptr(al), _ptr(a), lda, _ptr(b), ldb, _ptr(be),
                           _ptr(c), ldc, len(rows), _ptr(rows), _ptr(cols), _ptr(out))
        return out

    def qsyrk(self, uplo, trans, n, k, alpha, a, lda, beta, c, ldc):
        al = np.asarray(alpha, dtype=np.float64).reshape(2).copy()
        be = np.asarray(beta, dtype=np.float64).reshape(2).copy()
        self.lib.or_qsyrk(uplo.encode(), trans.encode(), n, k, _ptr(al), _ptr(a), lda, _ptr(be), _ptr(c), ldc)

    def qherk(self, uplo, trans, n, k, alpha, a, lda, beta, c, ldc):
        al = np.asarray(alpha, dtype=np.float64).reshape(2).copy()
        be = np.asarray(beta, dtype=np.float64).reshape(2).copy()
        self.lib.or_qherk(uplo.encode(), trans.encode(), n, k, _ptr(al), _ptr(a), lda, _ptr(be), _ptr(c), ldc)

    def qtrsm(self, side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb):
        al = np.asarray(alpha, dtype=np.float64).reshape(2).copy()
        self.lib.or_qtrsm(side.encode(), uplo.encode(), transa.encode(), diag.encode(), m, n, _ptr(al), _ptr(a),
                          lda, _ptr(b), ldb)

    def qgemv(self, trans, m, n, alpha, a, lda, x, incx, beta, y, incy):
        al = np.asarray(alpha, dtype=np.float64).reshape(2).copy()
        be = np.asarray(beta, dtype=np.float64).reshape(2).copy()
        self.lib.or_qgemv(trans.encode(), m, n, _ptr(al), _ptr(a), lda, _ptr(x), incx, _ptr(be), _ptr(y), incy)

    def qdot(self, n, x, incx, y, incy):
        out = np.zeros(2)
        self.lib.or_qdot(n, _ptr(x), incx, _ptr(y), incy, _ptr(out))
        return out

    def qaxpy(self, n, alpha, x, y):
        a = np.asarray(alpha, dtype=np.float64).reshape(2).copy()
        self.lib.or_qaxpy(n, _ptr(a), _ptr(x), _ptr(y))

    # CPU-baseline ports of the reference algorithms
    def port_mgemm(self, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, simd_order=0):
        al = np.asarray(alpha, dtype=np.float64).reshape(2).copy()
        be = np.asarray(beta, dtype=np.float64).reshape(2).copy()
        self.lib.or_port_mgemm(ta.encode(), tb.encode(), m, n, k, _ptr(al), _ptr(a), lda, _ptr(b), ldb, _ptr(be),
                               _ptr(c), ldc, simd_order)

    def port_mdot(self, n, x, y, team):
        out = np.zeros(2)
        self.lib.or_port_mdot(n, _ptr(x), _ptr(y), team, _ptr(out))
        return out

    def to_quad(self, x):
        """DD array (..., 2) -> raw binary128 buffer (uint8, 16 bytes per value)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        n = x.size // 2
        q = np.zeros(n * 16, dtype=np.uint8)
        self.lib.or_dd_to_q(_ptr(x), _ptr(q), n)
        return q

    def from_quad(self, q, shape):
        out = np.zeros(shape, dtype=np.float64)
        self.lib.or_q_to_dd(_ptr(q), _ptr(out), out.size // 2)
        return out

    def max_threads(self):
        return int(self.lib.or_max_threads())


# ---- error metric -------------------------------------------------------------------------

def dd_diff_abs(c, ref):
    """|c - ref| elementwise for DD arrays (..., 2), accurate to ~2^-106 relative."""
    c = np.asarray(c, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    return np.abs((c[..., 0] - ref[..., 0]) + (c[..., 1] - ref[..., 1]))


def dd_absmax(a):
    a = np.asarray(a, dtype=np.float64)
    return float(np.max(np.abs(a[..., 0]))) if a.size else 0.0


def dd_abs(x):
    x = np.asarray(x, dtype=np.float64).reshape(-1)
    return abs(x[0] + x[1]) if x.size == 2 else float(np.hypot(x[0] + x[1], x[2] + x[3]))


def normwise_error(c, ref, op_norm):
    """Reference fuzz metric: max|c - ref| / max(max|ref|, op_norm)."""
    num = float(np.max(dd_diff_abs(c, ref))) if np.size(c) else 0.0
    den = max(dd_absmax(ref), op_norm)
    if den == 0.0:
        return num
    return num / den


EPS_DD = 2.0 ** -104   # fuzz_util.fypp eps for real64x2
