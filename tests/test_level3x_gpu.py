"""GEMMTR, SYMM/HEMM, SYR2K/HER2K, complex SYRK, TRMM and complex TRSM on the
GPU, through the C ABI.

Expected values come from the binary128 oracle GEMMs (or_qgemm / or_qwgemm)
applied to dense forms of the structured operands, built here from the
reference's semantics:
  * SYMM/HEMM read A from its uplo triangle, mirror it (conjugated for HEMM)
    and take a Hermitian diagonal as real (msymm_parallel.cpp:37-102,
    whemm_serial.cpp:11-12);
  * TRMM/TRSM read the uplo triangle, with ones on the diagonal for diag='U'
    (mtrmm_parallel.cpp:37-106, wtrsm_parallel.cpp:39-105);
  * GEMMTR/SYR2K/HER2K/SYRK write only the uplo triangle; HER2K uses
    conj(alpha) on the second product, a real beta and a real diagonal
    (mgemmtr_parallel.cpp:35-80, msyr2k_parallel.cpp:38-83,
    wher2k_parallel.cpp:40-91).
Errors use the reference's normwise metric (fuzz_util_body.fypp:242-271)
with tolerance max(10, 4k) * 2^-104 for k-term products (2k for the rank-2k
updates); complex TRSM is checked by its residual in binary128. The other
triangle and the leading-dimension padding must come back untouched.
"""
import numpy as np
import pytest

from conftest import mwb, orc

pytestmark = pytest.mark.gpu

SENT = -7.37e18


def scal(rng, cplx_):
    return mwb.random_cdd(rng, ()) if cplx_ else mwb.random_dd(rng, ())


def mat(rng, m, n, ld, cplx_, fill=None):
    return mwb.dd_matrix(rng, m, n, ld, cplx_=cplx_, fill=fill)


def zero_like_scalar(cplx_):
    return np.zeros((2, 2)) if cplx_ else np.zeros(2)


def one_scalar(cplx_):
    return np.array([[1.0, 0.0], [0.0, 0.0]]) if cplx_ else np.array([1.0, 0.0])


def qgemm(oracle, cplx_, *args):
    return (oracle.qwgemm if cplx_ else oracle.qgemm)(*args)


def tri_mask(n, uplo):
    """mask[j, i] (array layout: column j, row i) of the stored uplo triangle."""
    i = np.arange(n)[None, :]
    j = np.arange(n)[:, None]
    return (i <= j) if uplo == "U" else (i >= j)


def expand_sym(A, na, uplo, cplx_, herm):
    """Dense na x na (array layout (col, row, ...)) from the uplo triangle."""
    M = A[:na, :na].copy()
    T = np.swapaxes(M, 0, 1).copy()          # T[j, i] = element (j, i)
    if herm:
        T[..., 1, :] = -T[..., 1, :]
    mask = tri_mask(na, uplo)
    shape = (na, na) + (1,) * (M.ndim - 2)
    F = np.where(mask.reshape(shape), M, T)
    if herm:
        d = np.arange(na)
        F[d, d, 1, :] = 0.0
    return np.ascontiguousarray(F)


def expand_tri(A, na, uplo, unit):
    M = A[:na, :na].copy()
    mask = tri_mask(na, uplo)
    shape = (na, na) + (1,) * (M.ndim - 2)
    F = np.where(mask.reshape(shape), M, 0.0)
    if unit:
        d = np.arange(na)
        F[d, d] = np.array([[1.0, 0.0], [0.0, 0.0]]) if M.ndim == 4 else np.array([1.0, 0.0])
    return np.ascontiguousarray(F)


def check_triangle(got, want, C0, n, uplo, tol, opn):
    mask = tri_mask(n, uplo)
    shape = (n, n) + (1,) * (got.ndim - 2)
    m3 = mask.reshape(shape)
    # the other triangle and the padding rows are untouched
    assert np.array_equal(np.where(m3, 0.0, got[:, :n]), np.where(m3, 0.0, C0[:, :n]))
    if got.shape[1] > n:
        assert np.all(got[:, n:] == SENT)
    g = np.where(m3, got[:, :n], 0.0)
    w = np.where(m3, want[:, :n], 0.0)
    err = orc.normwise_error(g, w, opn)
    assert err <= tol, err


@pytest.mark.parametrize("cplx_", [False, True])
@pytest.mark.parametrize("uplo", ["U", "L"])
@pytest.mark.parametrize("ta,tb", [("N", "T"), ("T", "N"), ("N", "N"), ("C", "T")])
def test_gemmtr(gpu, oracle, rng, cplx_, uplo, ta, tb):
    for n, k in [(1, 1), (37, 19), (130, 257)]:
        lda = (n if ta == "N" else k) + 1
        ldb = (k if tb == "N" else n) + 2
        ldc = n + 1
        A = mat(rng, n if ta == "N" else k, k if ta == "N" else n, lda, cplx_)
        B = mat(rng, k if tb == "N" else n, n if tb == "N" else k, ldb, cplx_)
        C0 = mat(rng, n, n, ldc, cplx_, fill=SENT)
        al, be = scal(rng, cplx_), scal(rng, cplx_)
        want = qgemm(oracle, cplx_, ta, tb, n, n, k, al, A, lda, B, ldb, be, C0.copy(), ldc)
        got = C0.copy()
        gpu.gemmtr(uplo, ta, tb, n, k, al, A, lda, B, ldb, be, got, ldc, cplx_=cplx_)
        assert gpu.last_error()[0] == 0, gpu.last_error()
        opn = orc.dd_abs(al) * k * orc.dd_absmax(A) * orc.dd_absmax(B) + orc.dd_abs(be) * orc.dd_absmax(C0[:, :n])
        check_triangle(got, want, C0, n, uplo, max(10, 4 * k) * orc.EPS_DD, opn)


@pytest.mark.parametrize("name", ["msymm", "wsymm", "whemm"])
@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("uplo", ["U", "L"])
def test_symm_hemm(gpu, oracle, rng, name, side, uplo):
    cplx_ = name != "msymm"
    for m, n in [(1, 3), (45, 31), (140, 200)]:
        na = m if side == "L" else n
        lda, ldb, ldc = na + 2, m + 1, m + 3
        A = mat(rng, na, na, lda, cplx_)
        B = mat(rng, m, n, ldb, cplx_)
        C0 = mat(rng, m, n, ldc, cplx_, fill=SENT)
        al, be = scal(rng, cplx_), scal(rng, cplx_)
        F = expand_sym(A, na, uplo, cplx_, name == "whemm")
        if side == "L":
            want = qgemm(oracle, cplx_, "N", "N", m, n, na, al, F, na, B, ldb, be, C0.copy(), ldc)
        else:
            want = qgemm(oracle, cplx_, "N", "N", m, n, na, al, B, ldb, F, na, be, C0.copy(), ldc)
        got = C0.copy()
        gpu.symm(name, side, uplo, m, n, al, A, lda, B, ldb, be, got, ldc)
        assert gpu.last_error()[0] == 0, gpu.last_error()
        assert np.all(got[:, m:] == SENT)
        opn = orc.dd_abs(al) * na * orc.dd_absmax(F) * orc.dd_absmax(B) + orc.dd_abs(be) * orc.dd_absmax(C0[:, :m])
        err = orc.normwise_error(got[:, :m], want[:, :m], opn)
        assert err <= max(10, 4 * na) * orc.EPS_DD, (m, n, err)


@pytest.mark.parametrize("name", ["msyr2k", "wsyr2k", "wher2k"])
@pytest.mark.parametrize("uplo", ["U", "L"])
@pytest.mark.parametrize("trans", ["N", "T"])
def test_syr2k_her2k(gpu, oracle, rng, name, uplo, trans):
    cplx_ = name != "msyr2k"
    herm = name == "wher2k"
    tr = ("C" if herm else "T") if trans == "T" else "N"
    for n, k in [(1, 1), (33, 20), (150, 130)]:
        nr = n if tr == "N" else k
        lda, ldb, ldc = nr + 1, nr + 2, n + 1
        A = mat(rng, nr, k if tr == "N" else n, lda, cplx_)
        B = mat(rng, nr, k if tr == "N" else n, ldb, cplx_)
        C0 = mat(rng, n, n, ldc, cplx_, fill=SENT)
        al = scal(rng, cplx_)
        be = mwb.random_dd(rng, ()) if herm else scal(rng, cplx_)
        be_c = np.stack([be, np.zeros(2)]) if herm else be
        t1 = "N" if tr == "N" else tr
        t2 = ("C" if herm else "T") if tr == "N" else "N"
        # C1 = alpha op(A) op(B)^T(H) + beta C0 ; C2 = alpha' op(B) op(A)^T(H) + C1
        C1 = qgemm(oracle, cplx_, t1, t2, n, n, k, al, A, lda, B, ldb, be_c, C0.copy(), ldc)
        al2 = al.copy()
        if herm:
            al2[1] = -al2[1]
        want = qgemm(oracle, cplx_, t1, t2, n, n, k, al2, B, ldb, A, lda, one_scalar(cplx_), C1, ldc)
        if herm:
            d = np.arange(n)
            want[d, d, 1, :] = 0.0
        got = C0.copy()
        gpu.syr2k(name, uplo, tr, n, k, al, A, lda, B, ldb, be, got, ldc)
        assert gpu.last_error()[0] == 0, gpu.last_error()
        opn = 2 * orc.dd_abs(al) * k * orc.dd_absmax(A) * orc.dd_absmax(B) + orc.dd_abs(be) * orc.dd_absmax(C0[:, :n])
        check_triangle(got, want, C0, n, uplo, max(10, 8 * k) * orc.EPS_DD, opn)
        if herm:
            d = np.arange(n)
            assert np.all(got[d, d, 1, :] == 0.0)


@pytest.mark.parametrize("uplo", ["U", "L"])
@pytest.mark.parametrize("trans", ["N", "T"])
def test_wsyrk_complex_symmetric(gpu, oracle, rng, uplo, trans):
    for n, k in [(1, 1), (40, 23), (129, 140)]:
        nr = n if trans == "N" else k
        lda, ldc = nr + 1, n + 2
        A = mat(rng, nr, k if trans == "N" else n, lda, True)
        C0 = mat(rng, n, n, ldc, True, fill=SENT)
        al, be = scal(rng, True), scal(rng, True)
        ta, tb = ("N", "T") if trans == "N" else ("T", "N")
        want = oracle.qwgemm(ta, tb, n, n, k, al, A, lda, A, lda, be, C0.copy(), ldc)
        got = C0.copy()
        gpu.wsyrk(uplo, trans, n, k, al, A, lda, be, got, ldc)
        assert gpu.last_error()[0] == 0, gpu.last_error()
        opn = orc.dd_abs(al) * k * orc.dd_absmax(A) ** 2 + orc.dd_abs(be) * orc.dd_absmax(C0[:, :n])
        check_triangle(got, want, C0, n, uplo, max(10, 4 * k) * orc.EPS_DD, opn)


@pytest.mark.parametrize("name", ["mtrmm", "wtrmm"])
@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("uplo", ["U", "L"])
@pytest.mark.parametrize("transa", ["N", "T", "C"])
@pytest.mark.parametrize("diag", ["N", "U"])
def test_trmm(gpu, oracle, rng, name, side, uplo, transa, diag):
    cplx_ = name == "wtrmm"
    if transa == "C" and not cplx_:
        pytest.skip("real 'C' folds to 'T'")
    for m, n in [(1, 2), (70, 45)]:
        na = m if side == "L" else n
        lda, ldb = na + 1, m + 2
        A = mat(rng, na, na, lda, cplx_)
        B0 = mat(rng, m, n, ldb, cplx_, fill=SENT)
        al = scal(rng, cplx_)
        F = expand_tri(A, na, uplo, diag == "U")
        zero = zero_like_scalar(cplx_)
        C = np.zeros_like(B0)
        if side == "L":
            want = qgemm(oracle, cplx_, transa, "N", m, n, na, al, F, na, B0, ldb, zero, C, ldb)
        else:
            want = qgemm(oracle, cplx_, "N", transa, m, n, na, al, B0, ldb, F, na, zero, C, ldb)
        got = B0.copy()
        gpu.trxm(name, side, uplo, transa, diag, m, n, al, A, lda, got, ldb)
        assert gpu.last_error()[0] == 0, gpu.last_error()
        assert np.all(got[:, m:] == SENT)
        opn = orc.dd_abs(al) * na * orc.dd_absmax(F) * orc.dd_absmax(B0[:, :m])
        err = orc.normwise_error(got[:, :m], want[:, :m], opn)
        assert err <= max(10, 4 * na) * orc.EPS_DD, (m, n, err)


@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("uplo", ["U", "L"])
@pytest.mark.parametrize("transa", ["N", "T", "C"])
@pytest.mark.parametrize("diag", ["N", "U"])
def test_wtrsm_residual(gpu, oracle, rng, side, uplo, transa, diag):
    """op(A) X = alpha B (or X op(A) = alpha B) on a diagonally dominant
    triangle (fuzz_mtrsm.fypp:67-117): the binary128 residual of the GPU
    solution stays within max(20, 8 na) * 2^-104 of |A||X| + |alpha B|."""
    for m, n in [(1, 1), (45, 20), (140, 100)]:
        na = m if side == "L" else n
        lda, ldb = na + 1, m + 1
        A = mat(rng, na, na, lda, True) / na        # off-diagonal |a_ij| < 1/na: well conditioned
        d = np.arange(na)
        A[d, d, 0, 0] = 1.0 + rng.random(na)        # |a_ii| in [1, 2)
        A[d, d, 0, 1] = 0.0
        B0 = mat(rng, m, n, ldb, True, fill=SENT)
        al = scal(rng, True)
        got = B0.copy()
        gpu.trxm("wtrsm", side, uplo, transa, diag, m, n, al, A, lda, got, ldb)
        assert gpu.last_error()[0] == 0, gpu.last_error()
        assert np.all(got[:, m:] == SENT)
        F = expand_tri(A, na, uplo, diag == "U")
        # R = op(A) X - alpha B (binary128 inside the oracle GEMM, one rounding)
        neg_al = -al
        zero = np.zeros((2, 2))
        AX = np.zeros_like(B0)
        if side == "L":
            AX = oracle.qwgemm(transa, "N", m, n, na, np.array([[1.0, 0], [0, 0]]), F, na, got, ldb, zero, AX, ldb)
        else:
            AX = oracle.qwgemm("N", transa, m, n, na, np.array([[1.0, 0], [0, 0]]), got, ldb, F, na, zero, AX, ldb)
        rhs = np.zeros_like(B0)
        ident = np.zeros((m, m, 2, 2))
        ident[np.arange(m), np.arange(m), 0, 0] = 1.0
        rhs = oracle.qwgemm("N", "N", m, n, m, al, ident, m, B0, ldb, zero, rhs, ldb)
        scale = na * orc.dd_absmax(F) * orc.dd_absmax(got[:, :m]) + orc.dd_abs(al) * orc.dd_absmax(B0[:, :m])
        err = orc.normwise_error(AX[:, :m], rhs[:, :m], scale)
        assert err <= max(20, 8 * na) * orc.EPS_DD, (m, n, err)


def test_quick_returns_and_errors(gpu, rng):
    """alpha == 0 scales (GEMMTR/SYR2K: triangle only, HER2K with beta == 1
    still zeroes Im(diag)); invalid flags leave outputs untouched."""
    n = 9
    C0 = mat(rng, n, n, n, True)
    got = C0.copy()
    gpu.syr2k("wher2k", "U", "N", n, 4, np.zeros((2, 2)), C0, n, C0, n, np.array([1.0, 0.0]), got, n)
    assert gpu.last_error()[0] == 0
    d = np.arange(n)
    assert np.all(got[d, d, 1, :] == 0.0)
    want = C0.copy()
    want[d, d, 1, :] = 0.0
    assert np.array_equal(got, want)
    Cr = mat(rng, n, n, n, False)
    got = Cr.copy()
    gpu.gemmtr("Q", "N", "N", n, 3, np.array([1.0, 0.0]), Cr, n, Cr, n, np.array([0.5, 0.0]), got, n)
    assert gpu.last_error()[0] != 0
    assert np.array_equal(got, Cr)
    got = Cr.copy()
    gpu.gemmtr("L", "N", "N", n, 0, np.array([1.0, 0.0]), Cr, n, Cr, n, np.array([0.5, 0.0]), got, n)
    assert gpu.last_error()[0] == 0
    mask = tri_mask(n, "L")[:, :, None]
    assert np.array_equal(np.where(mask, 0.0, got), np.where(mask, 0.0, Cr))
    assert np.allclose(np.where(mask, got, 0.0)[..., 0], np.where(mask, Cr * 0.5, 0.0)[..., 0])
