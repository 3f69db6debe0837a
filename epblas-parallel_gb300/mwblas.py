"""ctypes binding of the mwblas C ABI (include/mwblas_gb300.h).

The binding is written against the Fortran-style symbols, so the same class
drives any library that exports them: libmwblas_gb300.so (the GB300 library),
or a build of the reference epblas-parallel mwblas. It is the binding a
Python caller of the reference would write.

Double-double arrays are numpy float64 arrays whose last axis holds the two
limbs (hi, lo). A column-major m x n matrix with leading dimension ld is a
C-ordered numpy array of shape (n, ld, 2) (element (i, j) at [j, i]); complex
matrices have shape (n, ld, 2, 2) ([..., 0, :] real part, [..., 1, :]
imaginary part). Arrays may also be passed as raw integer addresses (device
pointers from torch, for example).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_LIB = os.path.join(HERE, "libmwblas_gb300.so")


class Real64x2(C.Structure):
    _fields_ = [("limbs", C.c_double * 2)]

    def to_tuple(self):
        return (self.limbs[0], self.limbs[1])


class Complex64x2(C.Structure):
    _fields_ = [("re", Real64x2), ("im", Real64x2)]


_i64 = C.c_int64
_i32 = C.c_int
_p = C.c_void_p
_ch = C.c_char_p


def _ptr(a):
    """Address of a numpy array / torch tensor / integer / None."""
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    raise TypeError(f"cannot take the address of {type(a)}")


def real(x) -> Real64x2:
    """Real64x2 from a float, a (hi, lo) pair or a numpy array of two."""
    if isinstance(x, Real64x2):
        return x
    if np.ndim(x) == 0:
        return Real64x2((C.c_double * 2)(float(x), 0.0))
    a = np.asarray(x, dtype=np.float64).reshape(2)
    return Real64x2((C.c_double * 2)(a[0], a[1]))


def cplx(x) -> Complex64x2:
    """Complex64x2 from a python complex or an array of shape (2, 2)."""
    if isinstance(x, Complex64x2):
        return x
    if isinstance(x, complex) or np.ndim(x) == 0:
        z = complex(x)
        return Complex64x2(real(z.real), real(z.imag))
    a = np.asarray(x, dtype=np.float64).reshape(2, 2)
    return Complex64x2(real(a[0]), real(a[1]))


class MWBlas:
    """Binding of one library exporting the mwblas Fortran-style ABI."""

    def __init__(self, path: str = DEFAULT_LIB, extensions: bool = True):
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path} not found (build it first)")
        self.path = path
        self.lib = C.CDLL(path, mode=C.RTLD_GLOBAL)
        L = self.lib
        R, Cx = C.POINTER(Real64x2), C.POINTER(Complex64x2)
        for suf, I in (("_", _i32), ("_64_", _i64)):
            PI = C.POINTER(I)
            self._sig("mgemm" + suf, None, [_ch, _ch, PI, PI, PI, R, _p, PI, _p, PI, R, _p, PI])
            self._sig("wgemm" + suf, None, [_ch, _ch, PI, PI, PI, Cx, _p, PI, _p, PI, Cx, _p, PI])
            self._sig("msyrk" + suf, None, [_ch, _ch, PI, PI, R, _p, PI, R, _p, PI])
            self._sig("wherk" + suf, None, [_ch, _ch, PI, PI, R, _p, PI, R, _p, PI])
            self._sig("mtrsm" + suf, None, [_ch, _ch, _ch, _ch, PI, PI, R, _p, PI, _p, PI])
            self._sig("mgemmtr" + suf, None, [_ch, _ch, _ch, PI, PI, R, _p, PI, _p, PI, R, _p, PI])
            self._sig("wgemmtr" + suf, None, [_ch, _ch, _ch, PI, PI, Cx, _p, PI, _p, PI, Cx, _p, PI])
            self._sig("msymm" + suf, None, [_ch, _ch, PI, PI, R, _p, PI, _p, PI, R, _p, PI])
            self._sig("wsymm" + suf, None, [_ch, _ch, PI, PI, Cx, _p, PI, _p, PI, Cx, _p, PI])
            self._sig("whemm" + suf, None, [_ch, _ch, PI, PI, Cx, _p, PI, _p, PI, Cx, _p, PI])
            self._sig("msyr2k" + suf, None, [_ch, _ch, PI, PI, R, _p, PI, _p, PI, R, _p, PI])
            self._sig("wsyr2k" + suf, None, [_ch, _ch, PI, PI, Cx, _p, PI, _p, PI, Cx, _p, PI])
            self._sig("wher2k" + suf, None, [_ch, _ch, PI, PI, Cx, _p, PI, _p, PI, R, _p, PI])
            self._sig("wsyrk" + suf, None, [_ch, _ch, PI, PI, Cx, _p, PI, Cx, _p, PI])
            self._sig("mtrmm" + suf, None, [_ch, _ch, _ch, _ch, PI, PI, R, _p, PI, _p, PI])
            self._sig("wtrmm" + suf, None, [_ch, _ch, _ch, _ch, PI, PI, Cx, _p, PI, _p, PI])
            self._sig("wtrsm" + suf, None, [_ch, _ch, _ch, _ch, PI, PI, Cx, _p, PI, _p, PI])
            self._sig("wdotu" + suf, Complex64x2, [PI, _p, PI, _p, PI])
            self._sig("wdotc" + suf, Complex64x2, [PI, _p, PI, _p, PI])
            for nm in ("masum", "mwasum", "mnrm2", "mwnrm2"):
                self._sig(nm + suf, Real64x2, [PI, _p, PI])
            self._sig("waxpy" + suf, None, [PI, Cx, _p, PI, _p, PI])
            self._sig("mrot" + suf, None, [PI, _p, PI, _p, PI, R, R])
            self._sig("wmrot" + suf, None, [PI, _p, PI, _p, PI, R, R])
            self._sig("mrotm" + suf, None, [PI, _p, PI, _p, PI, _p])
            self._sig("mcabs1" + suf, Real64x2, [_p])
            self._sig("mrotg" + suf, None, [_p] * 4)
            self._sig("mrotmg" + suf, None, [_p] * 5)
            self._sig("wrotg" + suf, None, [_p] * 4)
            # level 2 beyond mgemv (all scalars and arrays passed as pointers)
            for nm, na in (("wgemv", 11), ("mgbmv", 13), ("wgbmv", 13), ("msymv", 10), ("whemv", 10),
                           ("msbmv", 11), ("whbmv", 11), ("mspmv", 9), ("whpmv", 9), ("mtrmv", 8), ("wtrmv", 8),
                           ("mtrsv", 8), ("wtrsv", 8), ("mtbmv", 9), ("wtbmv", 9), ("mtbsv", 9), ("wtbsv", 9),
                           ("mtpmv", 7), ("wtpmv", 7), ("mtpsv", 7), ("wtpsv", 7), ("mger", 9), ("wgeru", 9),
                           ("wgerc", 9), ("msyr", 7), ("wher", 7), ("mspr", 6), ("whpr", 6), ("msyr2", 9),
                           ("wher2", 9), ("mspr2", 8), ("whpr2", 8)):
                self._sig(nm + suf, None, [_p] * na)
            self._sig("mgemv" + suf, None, [_ch, PI, PI, R, _p, PI, _p, PI, R, _p, PI])
            self._sig("mdot" + suf, Real64x2, [PI, _p, PI, _p, PI])
            self._sig("maxpy" + suf, None, [PI, R, _p, PI, _p, PI])
            self._sig("mscal" + suf, None, [PI, R, _p, PI])
            self._sig("wscal" + suf, None, [PI, Cx, _p, PI])
            self._sig("wmscal" + suf, None, [PI, R, _p, PI])
            self._sig("mcopy" + suf, None, [PI, _p, PI, _p, PI])
            self._sig("wcopy" + suf, None, [PI, _p, PI, _p, PI])
            self._sig("mswap" + suf, None, [PI, _p, PI, _p, PI])
            self._sig("wswap" + suf, None, [PI, _p, PI, _p, PI])
            self._sig("imamax" + suf, I, [PI, _p, PI])
            self._sig("iwamax" + suf, I, [PI, _p, PI])
        self.has_ext = extensions and hasattr(L, "mwblas_version")
        if self.has_ext:
            PI = C.POINTER(_i64)
            self._sig("mgemm_plain_64_", None, [_ch, _ch, PI, PI, PI, R, _p, PI, _p, PI, R, _p, PI])
            self._sig("mgemm_ozaki_64_", None, [_ch, _ch, PI, PI, PI, R, _p, PI, _p, PI, R, _p, PI])
            self._sig("mgemm_fixed_64_", None, [_ch, _ch, PI, PI, PI, R, _p, PI, _p, PI, R, _p, PI])
            self._sig("mwblas_set_gemm_engine", _i32, [_i32])
            self._sig("mwblas_set_band_solve", _i32, [_i32])
            self._sig("mwblas_get_gemm_engine", _i32, [])
            self._sig("mwblas_set_ozaki_bits", _i32, [_i32])
            self._sig("mwblas_last_ozaki_moduli", _i32, [])
            self._sig("mwblas_last_ozaki_bits", _i32, [_i32])
            self._sig("mwblas_set_ozaki_mma", _i32, [_i32])
            self._sig("mwblas_set_kernel_timing", _i32, [_i32])
            self._sig("mwblas_last_phase_ms", C.c_float, [_i32])
            self._sig("mwblas_set_l1_partition", _i64, [_i64])
            self._sig("mwblas_set_stream", _i32, [_p])
            self._sig("mwblas_set_sync", _i32, [_i32])
            self._sig("mwblas_pageable_direct", _i32, [])
            self._sig("mwblas_last_error", _i32, [])
            self._sig("mwblas_last_error_message", _ch, [])
            self._sig("mwblas_last_error_routine", _ch, [])
            self._sig("mwblas_clear_error", None, [])
            self._sig("mwblas_debug_fail_alloc_after", None, [_i64])
            self._sig("mwblas_set_wait_limit_ns", C.c_uint64, [C.c_uint64])
            self._sig("mwblas_set_plain_tma", _i32, [_i32])
            self._sig("mwblas_set_residue_tc", _i32, [_i32])
            self._sig("mwblas_set_band_tile", _i32, [_i32])
            self._sig("mwblas_debug_lose_operand_loads", None, [_i32])
            self._sig("mwblas_launch_count", _i64, [])
            self._sig("mwblas_version", _ch, [])
            self._sig("mgemv_n_noalloc", _i32, [_i64, _i64, R, _p, _i64, _p, _i64, R, _p, _i64, _p])
            self._sig("mgemm_grouped", _i32, [_i64, _p, _p, _p, _p, _p, _p, _p, _p, _p, _p, _p, _p, _p])
            self._sig("mgemm_grouped_tune", _i32, [_i64, _p, _p, _p, _p, _p, _p, _p, _p, _p, _p, _p, _p, _p, _p])
            self._sig("mwblas_grouped_tuned_tile", _i32, [])
            self._sig("mwblas_set_grouped_tile", _i32, [_i32])
            self._sig("mwblas_set_grouped_tensor_min", _i32, [_i32])
            self._sig("mwblas_grouped_tuned_tensor_min", _i32, [])
            self._sig("mwblas_set_grouped_tensor_pack", _i32, [_i32])
            self._sig("mwblas_grouped_tuned_tensor_pack", _i32, [])
            self._sig("mtrsm_grouped", _i32, [_i64, C.c_char, C.c_char, C.c_char, C.c_char, _p, _p, _p, _p, _p,
                                              _p, _p])

    def _sig(self, name, res, args):
        f = getattr(self.lib, name, None)
        if f is None:
            return
        f.restype = res
        f.argtypes = args

    # ---- helpers -------------------------------------------------------------------------
    @staticmethod
    def _I(v, wide=True):
        return C.byref(_i64(v) if wide else _i32(v))

    def last_error(self):
        if not self.has_ext:
            return 0, ""
        return self.lib.mwblas_last_error(), self.lib.mwblas_last_error_message().decode()

    # ---- level 3 -----------------------------------------------------------------------
    def mgemm(self, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, wide=True, engine=None):
        I = lambda v: self._I(v, wide)
        if engine is None:
            f = self.lib.mgemm_64_ if wide else self.lib.mgemm_
        else:
            f = {"plain": self.lib.mgemm_plain_64_, "ozaki": self.lib.mgemm_ozaki_64_,
                 "fixed": self.lib.mgemm_fixed_64_}[engine]
            I = lambda v: self._I(v, True)
        f(ta.encode(), tb.encode(), I(m), I(n), I(k), C.byref(real(alpha)), _ptr(a), I(lda), _ptr(b), I(ldb),
          C.byref(real(beta)), _ptr(c), I(ldc))

    def wgemm(self, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, wide=True):
        I = lambda v: self._I(v, wide)
        f = self.lib.wgemm_64_ if wide else self.lib.wgemm_
        f(ta.encode(), tb.encode(), I(m), I(n), I(k), C.byref(cplx(alpha)), _ptr(a), I(lda), _ptr(b), I(ldb),
          C.byref(cplx(beta)), _ptr(c), I(ldc))

    def msyrk(self, uplo, trans, n, k, alpha, a, lda, beta, c, ldc, wide=True):
        I = lambda v: self._I(v, wide)
        f = self.lib.msyrk_64_ if wide else self.lib.msyrk_
        f(uplo.encode(), trans.encode(), I(n), I(k), C.byref(real(alpha)), _ptr(a), I(lda), C.byref(real(beta)),
          _ptr(c), I(ldc))

    def wherk(self, uplo, trans, n, k, alpha, a, lda, beta, c, ldc, wide=True):
        I = lambda v: self._I(v, wide)
        f = self.lib.wherk_64_ if wide else self.lib.wherk_
        f(uplo.encode(), trans.encode(), I(n), I(k), C.byref(real(alpha)), _ptr(a), I(lda), C.byref(real(beta)),
          _ptr(c), I(ldc))

    def mtrsm(self, side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb, wide=True):
        I = lambda v: self._I(v, wide)
        f = self.lib.mtrsm_64_ if wide else self.lib.mtrsm_
        f(side.encode(), uplo.encode(), transa.encode(), diag.encode(), I(m), I(n), C.byref(real(alpha)), _ptr(a),
          I(lda), _ptr(b), I(ldb))

    def _scal(self, cplx_, v):
        return C.byref(cplx(v)) if cplx_ else C.byref(real(v))

    def gemmtr(self, uplo, ta, tb, n, k, alpha, a, lda, b, ldb, beta, c, ldc, cplx_=False, wide=True):
        I = lambda v: self._I(v, wide)
        f = getattr(self.lib, ("wgemmtr" if cplx_ else "mgemmtr") + ("_64_" if wide else "_"))
        f(uplo.encode(), ta.encode(), tb.encode(), I(n), I(k), self._scal(cplx_, alpha), _ptr(a), I(lda), _ptr(b),
          I(ldb), self._scal(cplx_, beta), _ptr(c), I(ldc))

    def symm(self, name, side, uplo, m, n, alpha, a, lda, b, ldb, beta, c, ldc, wide=True):
        """name in msymm, wsymm, whemm."""
        I = lambda v: self._I(v, wide)
        cp = name != "msymm"
        getattr(self.lib, name + ("_64_" if wide else "_"))(
            side.encode(), uplo.encode(), I(m), I(n), self._scal(cp, alpha), _ptr(a), I(lda), _ptr(b), I(ldb),
            self._scal(cp, beta), _ptr(c), I(ldc))

    def syr2k(self, name, uplo, trans, n, k, alpha, a, lda, b, ldb, beta, c, ldc, wide=True):
        """name in msyr2k, wsyr2k, wher2k (real beta)."""
        I = lambda v: self._I(v, wide)
        cp = name != "msyr2k"
        getattr(self.lib, name + ("_64_" if wide else "_"))(
            uplo.encode(), trans.encode(), I(n), I(k), self._scal(cp, alpha), _ptr(a), I(lda), _ptr(b), I(ldb),
            self._scal(name == "wsyr2k", beta), _ptr(c), I(ldc))

    def wsyrk(self, uplo, trans, n, k, alpha, a, lda, beta, c, ldc, wide=True):
        I = lambda v: self._I(v, wide)
        f = self.lib.wsyrk_64_ if wide else self.lib.wsyrk_
        f(uplo.encode(), trans.encode(), I(n), I(k), C.byref(cplx(alpha)), _ptr(a), I(lda), C.byref(cplx(beta)),
          _ptr(c), I(ldc))

    def trxm(self, name, side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb, wide=True):
        """name in mtrmm, wtrmm, wtrsm."""
        I = lambda v: self._I(v, wide)
        getattr(self.lib, name + ("_64_" if wide else "_"))(
            side.encode(), uplo.encode(), transa.encode(), diag.encode(), I(m), I(n),
            self._scal(name != "mtrmm", alpha), _ptr(a), I(lda), _ptr(b), I(ldb))

    def cdot(self, name, n, x, incx, y, incy, wide=True):
        """wdotu / wdotc -> numpy (2, 2) [re, im] double-doubles."""
        I = lambda v: self._I(v, wide)
        r = getattr(self.lib, name + ("_64_" if wide else "_"))(I(n), _ptr(x), I(incx), _ptr(y), I(incy))
        return np.array([[r.re.limbs[0], r.re.limbs[1]], [r.im.limbs[0], r.im.limbs[1]]])

    def vnorm(self, name, n, x, incx, wide=True):
        """masum / mwasum / mnrm2 / mwnrm2 -> numpy (2,) double-double."""
        I = lambda v: self._I(v, wide)
        r = getattr(self.lib, name + ("_64_" if wide else "_"))(I(n), _ptr(x), I(incx))
        return np.array([r.limbs[0], r.limbs[1]])

    def waxpy(self, n, alpha, x, incx, y, incy, wide=True):
        I = lambda v: self._I(v, wide)
        f = self.lib.waxpy_64_ if wide else self.lib.waxpy_
        f(I(n), C.byref(cplx(alpha)), _ptr(x), I(incx), _ptr(y), I(incy))

    def rot(self, name, n, x, incx, y, incy, c, s, wide=True):
        """mrot / wmrot."""
        I = lambda v: self._I(v, wide)
        getattr(self.lib, name + ("_64_" if wide else "_"))(I(n), _ptr(x), I(incx), _ptr(y), I(incy),
                                                             C.byref(real(c)), C.byref(real(s)))

    def rotm(self, n, x, incx, y, incy, param, wide=True):
        I = lambda v: self._I(v, wide)
        p = np.ascontiguousarray(np.asarray(param, dtype=np.float64).reshape(5, 2))
        (self.lib.mrotm_64_ if wide else self.lib.mrotm_)(I(n), _ptr(x), I(incx), _ptr(y), I(incy), _ptr(p))

    def generator(self, name, *bufs, wide=True):
        """mcabs1 / mrotg / mrotmg / wrotg on float64 arrays, in the reference's
        argument order (modified in place); mcabs1 returns its (2,) value."""
        f = getattr(self.lib, name + ("_64_" if wide else "_"))
        r = f(*[_ptr(b) for b in bufs])
        return np.array([r.limbs[0], r.limbs[1]]) if name == "mcabs1" else None

    def l2(self, name, *args, wide=True):
        """Level-2 routines beyond mgemv: arguments in the Fortran order; str
        for flags, int for sizes/increments, numpy arrays or device pointers
        for arrays, array-likes for scalars (real (2,) or complex (2, 2))."""
        conv, keep = [], []
        IT = _i64 if wide else _i32
        for a in args:
            if isinstance(a, str):
                b = C.c_char_p(a.encode())
                keep.append(b)
                conv.append(C.cast(b, C.c_void_p))
            elif isinstance(a, (int, np.integer)):
                b = IT(int(a))
                keep.append(b)
                conv.append(C.cast(C.pointer(b), C.c_void_p))
            elif isinstance(a, tuple) and len(a) == 1:     # (device pointer,)
                conv.append(C.c_void_p(a[0]))
            else:
                arr = np.ascontiguousarray(np.asarray(a, dtype=np.float64)) if not isinstance(a, np.ndarray) else a
                keep.append(arr)
                conv.append(C.c_void_p(arr.ctypes.data))
        getattr(self.lib, name + ("_64_" if wide else "_"))(*conv)

    # ---- batched (extension) -----------------------------------------------------------
    @staticmethod
    def _grouped_arrays(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc):
        cnt = len(m)
        arr = lambda v: np.ascontiguousarray(np.asarray(v, dtype=np.int64))
        ptrs = lambda v: np.ascontiguousarray(np.asarray([_ptr(x) for x in v], dtype=np.uint64))
        scal = lambda v: np.ascontiguousarray(np.asarray(v, dtype=np.float64).reshape(cnt, 2))
        return [cnt, np.frombuffer("".join(ta).encode(), dtype=np.uint8).copy(),
                np.frombuffer("".join(tb).encode(), dtype=np.uint8).copy(), arr(m), arr(n), arr(k), scal(alpha),
                ptrs(a), arr(lda), ptrs(b), arr(ldb), scal(beta), ptrs(c), arr(ldc)]

    def mgemm_grouped(self, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc):
        """Lists of per-instance flags/sizes/scalars; a, b, c: device pointers."""
        args = self._grouped_arrays(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc)
        return int(self.lib.mgemm_grouped(args[0], *[x.ctypes.data for x in args[1:]]))

    def mgemm_grouped_tune(self, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc):
        args = self._grouped_arrays(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc)
        chosen = C.c_int(-1)
        rc = int(self.lib.mgemm_grouped_tune(args[0], *[x.ctypes.data for x in args[1:]], C.addressof(chosen)))
        return rc, chosen.value

    def mtrsm_grouped(self, side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb):
        cnt = len(m)
        arr = lambda v: np.ascontiguousarray(np.asarray(v, dtype=np.int64))
        ptrs = lambda v: np.ascontiguousarray(np.asarray([_ptr(x) for x in v], dtype=np.uint64))
        al = np.ascontiguousarray(np.asarray(alpha, dtype=np.float64).reshape(cnt, 2))
        keep = [arr(m), arr(n), al, ptrs(a), arr(lda), ptrs(b), arr(ldb)]
        return int(self.lib.mtrsm_grouped(cnt, side.encode(), uplo.encode(), transa.encode(), diag.encode(),
                                          *[x.ctypes.data for x in keep]))

    # ---- level 2 -----------------------------------------------------------------------
    def mgemv(self, trans, m, n, alpha, a, lda, x, incx, beta, y, incy, wide=True):
        I = lambda v: self._I(v, wide)
        f = self.lib.mgemv_64_ if wide else self.lib.mgemv_
        f(trans.encode(), I(m), I(n), C.byref(real(alpha)), _ptr(a), I(lda), _ptr(x), I(incx), C.byref(real(beta)),
          _ptr(y), I(incy))

    def mgemv_n_noalloc(self, m, n, alpha, a, lda, x, incx, beta, y, incy, stream=None):
        """y := alpha*A*x + beta*y on device arrays without any device allocation."""
        return int(self.lib.mgemv_n_noalloc(m, n, C.byref(real(alpha)), _ptr(a), lda, _ptr(x), incx,
                                            C.byref(real(beta)), _ptr(y), incy, stream))

    # ---- level 1 -----------------------------------------------------------------------
    def mdot(self, n, x, incx, y, incy, wide=True):
        I = lambda v: self._I(v, wide)
        f = self.lib.mdot_64_ if wide else self.lib.mdot_
        r = f(I(n), _ptr(x), I(incx), _ptr(y), I(incy))
        return r.to_tuple()

    def maxpy(self, n, alpha, x, incx, y, incy, wide=True):
        I = lambda v: self._I(v, wide)
        f = self.lib.maxpy_64_ if wide else self.lib.maxpy_
        f(I(n), C.byref(real(alpha)), _ptr(x), I(incx), _ptr(y), I(incy))

    def mscal(self, n, alpha, x, incx, wide=True):
        I = lambda v: self._I(v, wide)
        (self.lib.mscal_64_ if wide else self.lib.mscal_)(I(n), C.byref(real(alpha)), _ptr(x), I(incx))

    def wscal(self, n, alpha, x, incx, wide=True):
        I = lambda v: self._I(v, wide)
        (self.lib.wscal_64_ if wide else self.lib.wscal_)(I(n), C.byref(cplx(alpha)), _ptr(x), I(incx))

    def wmscal(self, n, alpha, x, incx, wide=True):
        I = lambda v: self._I(v, wide)
        (self.lib.wmscal_64_ if wide else self.lib.wmscal_)(I(n), C.byref(real(alpha)), _ptr(x), I(incx))

    def mcopy(self, n, x, incx, y, incy, wide=True, cplx_=False):
        I = lambda v: self._I(v, wide)
        name = ("wcopy" if cplx_ else "mcopy") + ("_64_" if wide else "_")
        getattr(self.lib, name)(I(n), _ptr(x), I(incx), _ptr(y), I(incy))

    def mswap(self, n, x, incx, y, incy, wide=True, cplx_=False):
        I = lambda v: self._I(v, wide)
        name = ("wswap" if cplx_ else "mswap") + ("_64_" if wide else "_")
        getattr(self.lib, name)(I(n), _ptr(x), I(incx), _ptr(y), I(incy))

    def imamax(self, n, x, incx, wide=True, cplx_=False):
        I = lambda v: self._I(v, wide)
        name = ("iwamax" if cplx_ else "imamax") + ("_64_" if wide else "_")
        return int(getattr(self.lib, name)(I(n), _ptr(x), I(incx)))


# ---- array helpers -----------------------------------------------------------------------

def dd_normalize(hi, lo):
    """Renormalises (hi, lo) pairs so that |lo| <= ulp(hi)/2 (fast two-sum)."""
    s = hi + lo
    e = lo - (s - hi)
    return s, e


def random_dd(rng, shape, scale=1.0):
    """hi ~ U[-1,1)*scale, lo = hi * 2^-53 * U[-1,1), renormalised."""
    hi = (rng.random(shape) * 2.0 - 1.0) * scale
    lo = hi * 2.0 ** -53 * (rng.random(shape) * 2.0 - 1.0)
    hi, lo = dd_normalize(hi, lo)
    return np.stack([hi, lo], axis=-1)


def random_cdd(rng, shape, scale=1.0):
    return np.stack([random_dd(rng, shape, scale), random_dd(rng, shape, scale)], axis=-2)


def dd_matrix(rng, m, n, ld=None, cplx_=False, fill=None):
    """Column-major DD matrix as (n, ld, 2) [or (n, ld, 2, 2)], padding rows = fill."""
    ld = max(1, m) if ld is None else ld
    shape = (n, ld)
    a = random_cdd(rng, shape) if cplx_ else random_dd(rng, shape)
    if fill is not None and ld > m:
        a[:, m:] = fill
    return np.ascontiguousarray(a)
