"""Level-2/3 parity on the GPU, through the C ABI.

Every result is compared with the binary128 oracle using the reference's
normwise error (fuzz_util_body.fypp:242-271) and its tolerances:
GEMM/SYRK/HERK max(10, 4k) * 2^-104, TRSM max(20, 8 na^2) * 2^-104 on a
diagonally dominant triangle (fuzz_mtrsm.fypp:67-117), GEMV max(10, 4 max(m,n))
* 2^-104 (fuzz_mgemv.fypp:65). Padding rows of leading dimensions and the
off-uplo triangle carry sentinels that must come back untouched
(fuzz_util_body.fypp:224-240). The reference's own outputs from the golden
fixtures are checked the same way.
"""
import numpy as np
import pytest

from conftest import mwb, orc

pytestmark = pytest.mark.gpu

SENT = -7.37e18
ENGINES = ["plain", "fixed"]


def alpha_beta(rng, cplx_=False):
    def scal():
        if cplx_:
            return mwb.random_cdd(rng, ())
        v = mwb.random_dd(rng, ())
        return v
    r = rng.random()
    beta = scal() if r < 0.6 else (np.zeros((2, 2)) if cplx_ else np.zeros(2)) if r < 0.8 else \
        (np.array([[1.0, 0], [0, 0]]) if cplx_ else np.array([1.0, 0.0]))
    return scal(), beta


def op_norm(alpha, k, A, B, beta, C0):
    return orc.dd_abs(alpha) * k * orc.dd_absmax(A) * orc.dd_absmax(B) + orc.dd_abs(beta) * orc.dd_absmax(C0)


def check_sentinel(C, m):
    if C.shape[1] > m:
        assert np.all(C[:, m:] == SENT), "leading-dimension padding was written"


@pytest.mark.parametrize("engine", ENGINES)
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("N", "T"), ("T", "N"), ("T", "T"), ("C", "N")])
def test_mgemm_random(gpu, oracle, rng, engine, ta, tb):
    for (m, n, k) in [(1, 1, 1), (7, 5, 3), (33, 17, 65), (64, 64, 64), (130, 70, 257), (257, 129, 100)]:
        pad = int(rng.integers(0, 3))
        lda = (m if ta == "N" else k) + pad
        ldb = (k if tb == "N" else n) + pad
        ldc = m + 1 + pad
        A = mwb.dd_matrix(rng, m if ta == "N" else k, k if ta == "N" else m, lda)
        B = mwb.dd_matrix(rng, k if tb == "N" else n, n if tb == "N" else k, ldb)
        C0 = mwb.dd_matrix(rng, m, n, ldc, fill=SENT)
        al, be = alpha_beta(rng)
        want = oracle.qgemm(ta, tb, m, n, k, al, A, lda, B, ldb, be, C0.copy(), ldc)
        got = C0.copy()
        gpu.mgemm(ta, tb, m, n, k, al, A, lda, B, ldb, be, got, ldc, engine=engine)
        assert gpu.last_error()[0] == 0, gpu.last_error()
        check_sentinel(got, m)
        err = orc.normwise_error(got[:, :m], want[:, :m], op_norm(al, k, A, B, be, C0[:, :m]))
        assert err <= max(10, 4 * k) * orc.EPS_DD, (m, n, k, err)


def test_fixed_engine_long_k_scaled_rows_and_nonfinite(gpu, oracle, rng):
    """The integer-pipe engine: K beyond one launch's 16384, rows/columns
    scaled by 2^+-300 (per-row/column scaling keeps them exact), and a
    non-finite entry turning its row of C into NaN."""
    m, n, k = 9, 7, 20000
    A = mwb.dd_matrix(rng, m, k)
    B = mwb.dd_matrix(rng, k, n)
    A *= (2.0 ** rng.integers(-300, 300, m))[None, :, None]
    B *= (2.0 ** rng.integers(-300, 300, n))[:, None, None]
    C0 = mwb.dd_matrix(rng, m, n)
    al, be = mwb.random_dd(rng, ()), mwb.random_dd(rng, ())
    want = oracle.qgemm("N", "N", m, n, k, al, A, m, B, k, be, C0.copy(), m)
    got = C0.copy()
    gpu.mgemm("N", "N", m, n, k, al, A, m, B, k, be, got, m, engine="fixed")
    assert gpu.last_error()[0] == 0, gpu.last_error()
    # each entry against its own row/column scale
    ra = np.max(np.abs(A[..., 0]), axis=0)          # per row of A
    cb = np.max(np.abs(B[..., 0]), axis=1)          # per column of B
    scale = orc.dd_abs(al) * k * np.outer(cb, ra) + orc.dd_abs(be) * np.abs(C0[..., 0])
    err = np.abs((got[..., 0] - want[..., 0]) + (got[..., 1] - want[..., 1]))
    assert np.all(err <= 4 * k * orc.EPS_DD * scale), np.max(err / scale)
    A2 = A[:, :, :].copy()
    A2[k // 2, 3] = (np.inf, 0.0)                   # row 3 of A
    got = C0.copy()
    gpu.mgemm("N", "N", m, n, k, al, A2, m, B, k, be, got, m, engine="fixed")
    assert np.all(np.isnan(got[:, 3, 0])), "row with an infinity must be NaN"
    rest = [i for i in range(m) if i != 3]
    assert np.all(np.isfinite(got[:, rest, 0]))


def test_mgemm_lp64_and_special_scalars(gpu, oracle, rng):
    m, n, k = 40, 30, 20
    A = mwb.dd_matrix(rng, m, k); B = mwb.dd_matrix(rng, k, n)
    C0 = mwb.dd_matrix(rng, m, n)
    # alpha = 0: only the beta pass (mgemm_parallel.cpp:68-78)
    got = C0.copy()
    gpu.mgemm("N", "N", m, n, k, 0.0, A, m, B, k, 2.0, got, m, wide=False)
    want = C0.copy(); oracle.qgemm("N", "N", m, n, k, np.zeros(2), A, m, B, k, np.array([2.0, 0.0]), want, m)
    assert orc.normwise_error(got, want, 2 * orc.dd_absmax(C0)) <= 4 * orc.EPS_DD
    # beta = 0 must not read C: NaN in C is overwritten
    got = np.full_like(C0, np.nan)
    gpu.mgemm("N", "N", m, n, k, 1.0, A, m, B, k, 0.0, got, m)
    assert np.all(np.isfinite(got))
    # k = 0 with beta = 1 leaves C bit-identical
    got = C0.copy()
    gpu.mgemm("N", "N", m, n, 0, 1.0, A, m, B, 1, 1.0, got, m)
    np.testing.assert_array_equal(got, C0)


def test_wgemm_random(gpu, oracle, rng):
    for ta, tb in [("N", "N"), ("N", "C"), ("C", "T"), ("T", "N"), ("C", "C")]:
        for (m, n, k) in [(5, 3, 2), (33, 31, 40), (70, 65, 129)]:
            lda = (m if ta == "N" else k) + 1
            ldb = (k if tb == "N" else n)
            ldc = m + 2
            A = mwb.dd_matrix(rng, m if ta == "N" else k, k if ta == "N" else m, lda, cplx_=True)
            B = mwb.dd_matrix(rng, k if tb == "N" else n, n if tb == "N" else k, ldb, cplx_=True)
            C0 = mwb.dd_matrix(rng, m, n, ldc, cplx_=True, fill=SENT)
            al, be = alpha_beta(rng, True)
            want = oracle.qwgemm(ta, tb, m, n, k, al, A, lda, B, ldb, be, C0.copy(), ldc)
            got = C0.copy()
            gpu.wgemm(ta, tb, m, n, k, al, A, lda, B, ldb, be, got, ldc)
            assert gpu.last_error()[0] == 0, gpu.last_error()
            check_sentinel(got, m)
            opn = op_norm(al, k, A, B, be, C0[:, :m]) * 2
            err = orc.normwise_error(got[:, :m], want[:, :m], opn)
            assert err <= max(10, 4 * k) * orc.EPS_DD, (ta, tb, m, n, k, err)


@pytest.mark.parametrize("uplo", ["U", "L"])
@pytest.mark.parametrize("trans", ["N", "T"])
def test_msyrk(gpu, oracle, rng, uplo, trans):
    for (n, k) in [(1, 1), (9, 4), (65, 33), (130, 70)]:
        lda = (n if trans == "N" else k) + 1
        ldc = n + 2
        A = mwb.dd_matrix(rng, n if trans == "N" else k, k if trans == "N" else n, lda)
        C0 = mwb.dd_matrix(rng, n, n, ldc, fill=SENT)
        off = np.triu_indices(n, 1) if uplo == "L" else np.tril_indices(n, -1)
        C0[off[1], off[0]] = SENT          # (j, i) storage: mark the other triangle
        al, be = alpha_beta(rng)
        want = C0.copy(); oracle.qsyrk(uplo, trans, n, k, al, A, lda, be, want, ldc)
        got = C0.copy()
        gpu.msyrk(uplo, trans, n, k, al, A, lda, be, got, ldc)
        assert gpu.last_error()[0] == 0, gpu.last_error()
        check_sentinel(got, n)
        assert np.all(got[off[1], off[0]] == SENT), "off-triangle written"
        tri = np.tril_indices(n) if uplo == "L" else np.triu_indices(n)
        g, w = got[tri[1], tri[0]], want[tri[1], tri[0]]
        err = orc.normwise_error(g, w, op_norm(al, k, A, A, be, C0[tri[1], tri[0]]))
        assert err <= max(10, 4 * k) * orc.EPS_DD, (n, k, err)


@pytest.mark.parametrize("uplo", ["U", "L"])
@pytest.mark.parametrize("trans", ["N", "C"])
def test_wherk(gpu, oracle, rng, uplo, trans):
    for (n, k) in [(1, 2), (9, 4), (40, 65)]:
        lda = (n if trans == "N" else k)
        ldc = n + 1
        A = mwb.dd_matrix(rng, n if trans == "N" else k, k if trans == "N" else n, lda, cplx_=True)
        C0 = mwb.dd_matrix(rng, n, n, ldc, cplx_=True, fill=SENT)
        al, be = alpha_beta(rng)
        want = C0.copy(); oracle.qherk(uplo, trans, n, k, al, A, lda, be, want, ldc)
        got = C0.copy()
        gpu.wherk(uplo, trans, n, k, al, A, lda, be, got, ldc)
        assert gpu.last_error()[0] == 0, gpu.last_error()
        check_sentinel(got, n)
        d = np.arange(n)
        assert np.all(got[d, d, 1] == 0.0), "HERK diagonal must be real"
        tri = np.tril_indices(n) if uplo == "L" else np.triu_indices(n)
        g, w = got[tri[1], tri[0]], want[tri[1], tri[0]]
        err = orc.normwise_error(g, w, 2 * op_norm(al, k, A, A, be, C0[tri[1], tri[0]]))
        assert err <= max(10, 4 * k) * orc.EPS_DD, (n, k, err)


def dominant_triangle(rng, na, lda):
    A = mwb.dd_matrix(rng, na, na, lda)
    A[..., 0] /= na
    A[..., 1] /= na
    for d in range(na):
        A[d, d] = (1.0 + rng.random(), 0.0)
    return A


@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("uplo", ["U", "L"])
@pytest.mark.parametrize("ta", ["N", "T"])
@pytest.mark.parametrize("diag", ["N", "U"])
def test_mtrsm(gpu, oracle, rng, side, uplo, ta, diag):
    # (150, 140) and (130, 300): at least 128 right-hand sides take the
    # block-inverse path (the last diagonal block is partial)
    for (m, n) in [(1, 1), (7, 5), (70, 33), (150, 20), (150, 140), (130, 300)]:
        if side == "R":
            m, n = n, m
        na = m if side == "L" else n
        lda, ldb = na + 1, m + 1
        A = dominant_triangle(rng, na, lda)
        B0 = mwb.dd_matrix(rng, m, n, ldb, fill=SENT)
        al = mwb.random_dd(rng, ())
        want = B0.copy(); oracle.qtrsm(side, uplo, ta, diag, m, n, al, A, lda, want, ldb)
        got = B0.copy()
        gpu.mtrsm(side, uplo, ta, diag, m, n, al, A, lda, got, ldb)
        assert gpu.last_error()[0] == 0, gpu.last_error()
        check_sentinel(got, m)
        err = orc.normwise_error(got[:, :m], want[:, :m], orc.dd_abs(al) * orc.dd_absmax(B0[:, :m]))
        assert err <= max(20, 8 * na * na) * orc.EPS_DD, (m, n, err)


@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("uplo", ["U", "L"])
@pytest.mark.parametrize("ta", ["N", "T"])
@pytest.mark.parametrize("diag", ["N", "U"])
def test_mtrsm_merged_inverse_leaves(gpu, oracle, rng, side, uplo, ta, diag):
    """order >= 1024 with >= 256 right-hand sides: 256 x 256 leaf inverses
    built by merging 64 x 64 ones (the last block partial); 4 sampled
    right-hand sides are checked against the oracle (they are independent)."""
    na, nr = 1100, 300
    m, n = (na, nr) if side == "L" else (nr, na)
    A = dominant_triangle(rng, na, na)
    B0 = mwb.dd_matrix(rng, m, n, m)
    al = mwb.random_dd(rng, ())
    got = B0.copy()
    gpu.mtrsm(side, uplo, ta, diag, m, n, al, A, na, got, m)
    assert gpu.last_error()[0] == 0, gpu.last_error()
    pick = np.sort(rng.choice(nr, 4, replace=False))
    if side == "L":
        sub = np.ascontiguousarray(B0[pick])                  # 4 columns, na x 4
        oracle.qtrsm("L", uplo, ta, diag, na, 4, al, A, na, sub, na)
        g = got[pick]
    else:
        sub = np.ascontiguousarray(B0[:, pick])               # 4 rows: (na, 4) -> 4 x na with ld 4
        oracle.qtrsm("R", uplo, ta, diag, 4, na, al, A, na, sub, 4)
        g = got[:, pick]
    err = orc.normwise_error(g, sub, orc.dd_abs(al) * orc.dd_absmax(B0))
    assert err <= max(20, 8 * na * na) * orc.EPS_DD, err
    assert err <= 1e-28, err   # well conditioned: far inside the reference's na^2 bound


@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("uplo", ["U", "L"])
@pytest.mark.parametrize("ta", ["N", "T"])
@pytest.mark.parametrize("diag", ["N", "U"])
def test_mtrsm_512_leaves(gpu, oracle, rng, side, uplo, ta, diag):
    """order >= 2048 with >= 512 right-hand sides: 512 x 512 leaf inverses,
    the merges of 128 and 256 blocks on the tensor cores (grouped residue
    GEMMs), the last leaf partial; 4 sampled right-hand sides against the
    oracle."""
    na, nr = 2100, 520
    m, n = (na, nr) if side == "L" else (nr, na)
    A = dominant_triangle(rng, na, na)
    B0 = mwb.dd_matrix(rng, m, n, m)
    al = mwb.random_dd(rng, ())
    got = B0.copy()
    gpu.mtrsm(side, uplo, ta, diag, m, n, al, A, na, got, m)
    assert gpu.last_error()[0] == 0, gpu.last_error()
    pick = np.sort(rng.choice(nr, 4, replace=False))
    if side == "L":
        sub = np.ascontiguousarray(B0[pick])
        oracle.qtrsm("L", uplo, ta, diag, na, 4, al, A, na, sub, na)
        g = got[pick]
    else:
        sub = np.ascontiguousarray(B0[:, pick])
        oracle.qtrsm("R", uplo, ta, diag, 4, na, al, A, na, sub, 4)
        g = got[:, pick]
    err = orc.normwise_error(g, sub, orc.dd_abs(al) * orc.dd_absmax(B0))
    assert err <= max(20, 8 * na * na) * orc.EPS_DD, err
    assert err <= 1e-28, err


@pytest.mark.parametrize("side,uplo,ta,diag", [("L", "L", "N", "N"), ("L", "U", "T", "U"), ("R", "U", "N", "N"),
                                               ("R", "L", "T", "N")])
def test_mtrsm_1024_leaves(gpu, oracle, rng, side, uplo, ta, diag):
    """order >= 4096 with >= 512 right-hand sides: 1024 x 1024 leaf inverses
    (five merge levels, the last three on the tensor cores), a partial last
    leaf; 4 sampled right-hand sides against the oracle."""
    na, nr = 4100, 512
    m, n = (na, nr) if side == "L" else (nr, na)
    A = dominant_triangle(rng, na, na)
    B0 = mwb.dd_matrix(rng, m, n, m)
    al = mwb.random_dd(rng, ())
    got = B0.copy()
    gpu.mtrsm(side, uplo, ta, diag, m, n, al, A, na, got, m)
    assert gpu.last_error()[0] == 0, gpu.last_error()
    pick = np.sort(rng.choice(nr, 4, replace=False))
    if side == "L":
        sub = np.ascontiguousarray(B0[pick])
        oracle.qtrsm("L", uplo, ta, diag, na, 4, al, A, na, sub, na)
        g = got[pick]
    else:
        sub = np.ascontiguousarray(B0[:, pick])
        oracle.qtrsm("R", uplo, ta, diag, 4, na, al, A, na, sub, 4)
        g = got[:, pick]
    err = orc.normwise_error(g, sub, orc.dd_abs(al) * orc.dd_absmax(B0))
    assert err <= 1e-28, err


@pytest.mark.parametrize("trans", ["N", "T"])
def test_mgemv(gpu, oracle, rng, trans):
    for (m, n, incx, incy) in [(1, 1, 1, 1), (17, 9, 1, 1), (300, 70, 2, -1), (70, 300, -3, 2), (1000, 4000, 1, 1)]:
        lda = m + 3
        A = mwb.dd_matrix(rng, m, n, lda, fill=SENT)
        lx, ly = (n, m) if trans == "N" else (m, n)
        x = mwb.random_dd(rng, (1 + (lx - 1) * abs(incx),))
        y0 = mwb.random_dd(rng, (1 + (ly - 1) * abs(incy),))
        al, be = alpha_beta(rng)
        want = y0.copy(); oracle.qgemv(trans, m, n, al, A, lda, x, incx, be, want, incy)
        got = y0.copy()
        gpu.mgemv(trans, m, n, al, A, lda, x, incx, be, got, incy)
        assert gpu.last_error()[0] == 0, gpu.last_error()
        opn = orc.dd_abs(al) * lx * orc.dd_absmax(A[:, :m]) * orc.dd_absmax(x) + orc.dd_abs(be) * orc.dd_absmax(y0)
        err = orc.normwise_error(got, want, opn)
        assert err <= max(10, 4 * max(m, n)) * orc.EPS_DD, (m, n, err)


@pytest.mark.parametrize("trans", ["N", "T"])
def test_mgemv_scaled_rows_componentwise(gpu, oracle, rng, trans):
    """Rows of A scaled by 2^e, e in [-200, 200]: each y(i) is accurate relative
    to its own |alpha| sum_j |A(i,j) x(j)| + |beta y(i)|, not only normwise."""
    m, n = 257, 1500
    A = mwb.dd_matrix(rng, m, n, m)
    A *= (2.0 ** rng.integers(-200, 200, m))[None, :, None]
    if trans == "T":
        A = np.ascontiguousarray(np.transpose(A, (1, 0, 2)))   # n x m, columns scaled
    rows, cols = (m, n) if trans == "N" else (n, m)
    lx, ly = (n, m) if trans == "N" else (n, m)
    x = mwb.random_dd(rng, (lx,))
    y0 = mwb.random_dd(rng, (ly,))
    y0 *= (2.0 ** rng.integers(-200, 200, ly))[:, None]
    al, be = alpha_beta(rng)
    want = y0.copy(); oracle.qgemv(trans, rows, cols, al, A, rows, x, 1, be, want, 1)
    got = y0.copy()
    gpu.mgemv(trans, rows, cols, al, A, rows, x, 1, be, got, 1)
    Ah = np.abs(A[..., 0])                       # (cols, rows)
    xs = np.abs(x[:, 0])
    absum = (Ah.T @ xs) if trans == "N" else (Ah @ xs)
    bound = orc.dd_abs(al) * absum + orc.dd_abs(be) * np.abs(y0[:, 0])
    err = np.abs((got[:, 0] - want[:, 0]) + (got[:, 1] - want[:, 1]))
    assert np.all(err <= 4 * lx * orc.EPS_DD * bound), np.max(err / bound)


def test_golden_reference_outputs(gpu, golden):
    """GPU results agree with the reference's own outputs within its tolerances."""
    z, meta = golden
    for c in meta["l3"]:
        k = c["key"]
        if c["kind"] == "gemm":
            got = z[k + "_C"].copy()
            gpu.mgemm(c["ta"], c["tb"], c["m"], c["n"], c["k"], z[k + "_alpha"], z[k + "_A"], c["lda"],
                      z[k + "_B"], c["ldb"], z[k + "_beta"], got, c["ldc"])
            opn = op_norm(z[k + "_alpha"], c["k"], z[k + "_A"], z[k + "_B"], z[k + "_beta"], z[k + "_C"])
            tol = max(10, 4 * c["k"]) * orc.EPS_DD
            m = c["m"]
            assert orc.normwise_error(got[:, :m], z[k + "_q"][:, :m], opn) <= tol, k
            assert orc.normwise_error(got[:, :m], z[k + "_ref"][:, :m], opn) <= 2 * tol, k
        elif c["kind"] == "trsm":
            got = z[k + "_B"].copy()
            gpu.mtrsm(c["side"], c["uplo"], c["ta"], c["diag"], c["m"], c["n"], z[k + "_alpha"], z[k + "_A"],
                      c["lda"], got, c["ldb"])
            na = c["m"] if c["side"] == "L" else c["n"]
            opn = orc.dd_abs(z[k + "_alpha"]) * orc.dd_absmax(z[k + "_B"][:, :c["m"]])
            tol = max(20, 8 * na * na) * orc.EPS_DD
            assert orc.normwise_error(got[:, :c["m"]], z[k + "_q"][:, :c["m"]], opn) <= tol, k


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("N", "T"), ("T", "N"), ("T", "T")])
def test_plain_engine_tma_staging_bit_identical(gpu, oracle, rng, ta, tb):
    """The FP64 engine's TMA-staged kernel (tensor copies into a ring of
    shared-memory stages, zero fill past the operand edges) gives the bits of
    the kernel that stages with plain loads: ragged m, n, k, padded leading
    dimensions, both tile sizes, short k (second extraction level)."""
    for (m, n, k) in [(1, 1, 1), (70, 33, 9), (130, 97, 64), (333, 301, 517), (1200, 700, 130)]:
        lda = (m if ta == "N" else k) + 3
        ldb = (k if tb == "N" else n) + 1
        A = mwb.dd_matrix(rng, m if ta == "N" else k, k if ta == "N" else m, lda)
        B = mwb.dd_matrix(rng, k if tb == "N" else n, n if tb == "N" else k, ldb)
        C0 = mwb.dd_matrix(rng, m, n, m + 2, fill=SENT)
        al, be = mwb.random_dd(rng, ()), mwb.random_dd(rng, ())
        outs = []
        for tma in (1, 0):
            prev = gpu.lib.mwblas_set_plain_tma(tma)
            try:
                c = C0.copy()
                gpu.mgemm(ta, tb, m, n, k, al, A, lda, B, ldb, be, c, m + 2, engine="plain")
                assert gpu.last_error()[0] == 0, gpu.last_error()
                outs.append(c)
            finally:
                gpu.lib.mwblas_set_plain_tma(prev)
        np.testing.assert_array_equal(outs[0], outs[1])
        check_sentinel(outs[0], m)
        want = oracle.qgemm(ta, tb, m, n, k, al, A, lda, B, ldb, be, C0.copy(), m + 2)
        err = orc.normwise_error(outs[0][:, :m], want[:, :m], op_norm(al, k, A, B, be, C0[:, :m]))
        assert err <= max(10, 4 * k) * orc.EPS_DD, (m, n, k, err)


@pytest.mark.parametrize("uplo", ["U", "L"])
def test_plain_engine_tma_syrk_bit_identical(gpu, rng, uplo):
    n, k = 400, 300
    A = mwb.dd_matrix(rng, n, k)
    C0 = mwb.dd_matrix(rng, n, n)
    al, be = mwb.random_dd(rng, ()), mwb.random_dd(rng, ())
    outs = []
    prev_e = gpu.lib.mwblas_set_gemm_engine(1)
    try:
        for tma in (1, 0):
            prev = gpu.lib.mwblas_set_plain_tma(tma)
            try:
                c = C0.copy()
                gpu.msyrk(uplo, "N", n, k, al, A, n, be, c, n)
                assert gpu.last_error()[0] == 0
                outs.append(c)
            finally:
                gpu.lib.mwblas_set_plain_tma(prev)
    finally:
        gpu.lib.mwblas_set_gemm_engine(prev_e)
    np.testing.assert_array_equal(outs[0], outs[1])
