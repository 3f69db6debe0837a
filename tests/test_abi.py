"""C-ABI checks that need no GPU: symbols, argument validation, quick returns."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT, mwb


def header_functions():
    text = open(os.path.join(ROOT, "include", "mwblas_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b([a-z_][a-z0-9_]*)\s*\(", text)
    skip = {"typedef", "if", "sizeof", "defined", "void"}
    fns = []
    for nm in names:
        if nm in skip or nm.startswith("mwblas_error_hook"):
            continue
        fns.append(nm)
    # function-pointer typedef name appears as "(*mwblas_error_hook)"
    return sorted(set(fns))


def test_library_exports_every_declared_symbol(libpath):
    lib = C.CDLL(libpath)
    missing = [f for f in header_functions() if not hasattr(lib, f)]
    assert not missing, f"declared in include/mwblas_gb300.h but not exported: {missing}"


def test_lp64_and_ilp64_twins_exported(libpath):
    lib = C.CDLL(libpath)
    for r in ["mgemm", "wgemm", "msyrk", "wherk", "mtrsm", "mgemv", "mdot", "maxpy", "mscal", "mcopy", "mswap",
              "imamax", "wscal", "wmscal", "wcopy", "wswap", "iwamax"]:
        assert hasattr(lib, r + "_") and hasattr(lib, r + "_64_"), r


def test_reference_symbol_set_covered(libpath):
    """Every hot-path symbol of the reference's mwblas is exported (common/epblas_facade.h pairs)."""
    lib = C.CDLL(libpath)
    for s in ("mgemm_ mgemm_64_ wgemm_ wgemm_64_ msyrk_ msyrk_64_ wherk_ wherk_64_ mtrsm_ mtrsm_64_ mgemv_ "
              "mgemv_64_ mdot_ mdot_64_ maxpy_ maxpy_64_ mscal_ mscal_64_ mcopy_ mcopy_64_ mswap_ mswap_64_ "
              "imamax_ imamax_64_ wscal_ wcopy_ wswap_ iwamax_ wmscal_").split():
        assert hasattr(lib, s), s


def test_invalid_flags_are_reported_without_touching_outputs(lib):
    c = np.full((2, 2, 2), 7.0)
    a = np.zeros((2, 2, 2))
    lib.mgemm("X", "N", 2, 2, 2, 1.0, a, 2, a, 2, 0.0, c, 2)
    code, msg = lib.last_error()
    assert code == 1 and "transa" in msg
    assert np.all(c == 7.0)
    lib.mgemm("N", "Q", 2, 2, 2, 1.0, a, 2, a, 2, 0.0, c, 2)
    assert lib.last_error()[0] == 2
    lib.mgemm("N", "N", 2, 2, 2, 1.0, a, 1, a, 2, 0.0, c, 2)   # lda < m
    assert lib.last_error()[0] == 8
    lib.mgemm("N", "N", 2, 2, 2, 1.0, a, 2, a, 1, 0.0, c, 2)   # ldb < k
    assert lib.last_error()[0] == 10
    lib.mgemm("N", "N", 2, 2, 2, 1.0, a, 2, a, 2, 0.0, c, 1)   # ldc < m
    assert lib.last_error()[0] == 13
    assert np.all(c == 7.0)


def test_quick_returns_need_no_device(lib):
    """Sizes <= 0 and the reference's special scalars return before any GPU work."""
    c = np.full((3, 3, 2), 5.0)
    lib.mgemm("N", "N", 0, 3, 3, 1.0, c, 3, c, 3, 0.0, c, 3)
    assert lib.last_error()[0] == 0 and np.all(c == 5.0)
    x = np.full((4, 2), 3.0)
    lib.mscal(4, 1.0, x, 1)                 # alpha == 1: mscal.cpp:91
    lib.mscal(-1, 2.0, x, 1)
    lib.maxpy(4, 0.0, x, 1, x, 1)          # alpha == 0: maxpy.cpp:99
    assert lib.last_error()[0] == 0 and np.all(x == 3.0)
    assert lib.imamax(0, x, 1) == 0
    assert lib.imamax(4, x, 0) == 0         # incx <= 0: imamax.cpp:180
    assert lib.imamax(1, x, 1) == 1
    assert lib.mdot(0, x, 1, x, 1) == (0.0, 0.0)


def test_lowercase_and_conjugate_flags_accepted(lib):
    """'c' on a real routine folds to 'T' (blas_char.h:36): validation passes it."""
    a = np.zeros((2, 2, 2))
    c = np.zeros((2, 2, 2))
    lib.mgemm("c", "t", 0, 2, 2, 1.0, a, 2, a, 2, 0.0, c, 2)
    assert lib.last_error()[0] == 0


def test_error_hook_is_called(lib):
    seen = []
    HOOK = C.CFUNCTYPE(None, C.c_char_p, C.c_int, C.c_char_p)
    cb = HOOK(lambda r, i, m: seen.append((r.decode(), i)))
    lib.lib.mwblas_set_error_hook.restype = C.c_void_p
    lib.lib.mwblas_set_error_hook.argtypes = [HOOK]
    lib.lib.mwblas_set_error_hook(cb)
    try:
        a = np.zeros((2, 2, 2))
        lib.mgemm("N", "N", 2, 2, 2, 1.0, a, 1, a, 2, 0.0, a, 2)
    finally:
        lib.lib.mwblas_set_error_hook(HOOK())
    assert seen == [("mgemm", 8)]


def test_version_string(lib):
    assert b"sm_103a" in lib.lib.mwblas_version()
