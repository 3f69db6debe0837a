"""Level-2 routines beyond mgemv on the GPU, through the C ABI: complex GEMV,
GBMV, SYMV/HEMV/SBMV/HBMV/SPMV/HPMV, TRMV/TBMV/TPMV, TRSV/TBSV/TPSV,
GER/GERU/GERC, SYR/HER/SPR/HPR, SYR2/HER2/SPR2/HPR2.

The structured operand is expanded here into a dense matrix following the
BLAS storage conventions the reference uses (band: AB(ku+1+i-j, j);
packed upper AP(i + j(j-1)/2), lower AP(i + (j-1)(2n-j)/2), 1-based;
Hermitian diagonals real), and the expected result is the binary128 oracle
GEMM of the dense forms (or_qgemm / or_qwgemm), rounded once. Tolerance:
the reference's GEMV bound max(10, 4 max(m, n)) * 2^-104 (fuzz_mgemv.fypp:65)
for products and rank updates; the triangular solves are checked through
their binary128 residual with max(20, 8n) * 2^-104 (fuzz_mtrsm.fypp:113-114).
"""
import numpy as np
import pytest

from conftest import mwb, orc

pytestmark = pytest.mark.gpu

ONE = {False: np.array([1.0, 0.0]), True: np.array([[1.0, 0.0], [0.0, 0.0]])}
ZERO = {False: np.zeros(2), True: np.zeros((2, 2))}


def scal(rng, c):
    return mwb.random_cdd(rng, ()) if c else mwb.random_dd(rng, ())


def dense(rng, m, n, c, ld=None):
    return mwb.dd_matrix(rng, m, n, ld, cplx_=c)


def vecs(rng, n, inc, c):
    span = 1 + (n - 1) * abs(inc)
    return mwb.random_cdd(rng, (span,)) if c else mwb.random_dd(rng, (span,))


def gather(v, n, inc):
    idx = np.arange(n) * inc if inc >= 0 else (n - 1 - np.arange(n)) * (-inc)
    return np.ascontiguousarray(v[idx])


def qmm(oracle, c, *a):
    return (oracle.qwgemm if c else oracle.qgemm)(*a)


def matvec(oracle, c, trans, M, m_out, k, x, alpha, beta, y0):
    """alpha * op(M) * x + beta * y0 in binary128 (M dense, ld = rows)."""
    ld = M.shape[1]
    X = np.ascontiguousarray(x[None])
    Y = np.ascontiguousarray(y0[None])
    return qmm(oracle, c, trans, "N", m_out, 1, k, alpha, M, ld, X, k, beta, Y, m_out)[0]


def herm_fix(F, herm):
    if herm:
        d = np.arange(F.shape[0])
        F[d, d, 1, :] = 0.0
    return F


def sym_from_tri(A, n, uplo, herm):
    M = A[:n, :n].copy()
    T = np.swapaxes(M, 0, 1).copy()
    if herm:
        T[..., 1, :] = -T[..., 1, :]
    i = np.arange(n)[None, :]
    j = np.arange(n)[:, None]
    mask = (i <= j) if uplo == "U" else (i >= j)
    shape = (n, n) + (1,) * (M.ndim - 2)
    return herm_fix(np.where(mask.reshape(shape), M, T), herm)


def to_band(F, kl, ku):
    """Dense (array [col, row, ...]) -> band AB (array [col, band row, ...])."""
    n, m = F.shape[0], F.shape[1]
    AB = np.zeros((n, kl + ku + 1) + F.shape[2:])
    for j in range(n):
        for i in range(max(0, j - ku), min(m, j + kl + 1)):
            AB[j, ku + i - j] = F[j, i]
    return AB


def band_keep(F, kl, ku):
    G = np.zeros_like(F)
    n, m = F.shape[0], F.shape[1]
    for j in range(n):
        lo, hi = max(0, j - ku), min(m, j + kl + 1)
        G[j, lo:hi] = F[j, lo:hi]
    return G


def to_packed(F, n, uplo):
    out = []
    for j in range(n):
        rows = range(0, j + 1) if uplo == "U" else range(j, n)
        for i in rows:
            out.append(F[j, i])
    return np.ascontiguousarray(np.array(out))


def tri_dense(F, n, uplo, unit):
    G = F[:n, :n].copy()
    i = np.arange(n)[None, :]
    j = np.arange(n)[:, None]
    mask = (i <= j) if uplo == "U" else (i >= j)
    shape = (n, n) + (1,) * (G.ndim - 2)
    G = np.where(mask.reshape(shape), G, 0.0)
    if unit:
        d = np.arange(n)
        G[d, d] = ONE[G.ndim == 4]
    return np.ascontiguousarray(G)


def err_ok(got, want, scale, tol):
    d = float(np.max(orc.dd_diff_abs(got, want))) if got.size else 0.0
    return d / max(orc.dd_absmax(want), scale) <= tol


@pytest.mark.parametrize("c", [False, True])
@pytest.mark.parametrize("trans", ["N", "T", "C"])
@pytest.mark.parametrize("band", [False, True])
def test_gemv_gbmv(gpu, oracle, rng, c, trans, band):
    if not c and not band:
        pytest.skip("real dense GEMV is mgemv (test_level3_gpu)")
    for m, n, kl, ku in [(1, 1, 0, 0), (37, 29, 3, 5), (130, 170, 20, 0)]:
        F = dense(rng, m, n, c)
        if band:
            F = band_keep(F, kl, ku)
            AB = np.ascontiguousarray(to_band(F, kl, ku))
        lx, ly = (n, m) if trans == "N" else (m, n)
        ix, iy = 2, -3
        x, y = vecs(rng, lx, ix, c), vecs(rng, ly, iy, c)
        al, be = scal(rng, c), scal(rng, c)
        want = matvec(oracle, c, trans if c else ("T" if trans != "N" else "N"), F, ly, lx, gather(x, lx, ix), al,
                      be, gather(y, ly, iy))
        got = y.copy()
        if band:
            gpu.l2("wgbmv" if c else "mgbmv", trans, m, n, kl, ku, al, AB, kl + ku + 1, x, ix, be, got, iy)
        else:
            gpu.l2("wgemv", trans, m, n, al, F, m, x, ix, be, got, iy)
        assert gpu.last_error()[0] == 0, gpu.last_error()
        scale = orc.dd_abs(al) * lx * orc.dd_absmax(F) * orc.dd_absmax(x) + orc.dd_abs(be) * orc.dd_absmax(y)
        assert err_ok(gather(got, ly, iy), want, scale, max(10, 4 * max(m, n)) * orc.EPS_DD), (m, n)


@pytest.mark.parametrize("name", ["msymv", "whemv", "msbmv", "whbmv", "mspmv", "whpmv"])
@pytest.mark.parametrize("uplo", ["U", "L"])
def test_symv_family(gpu, oracle, rng, name, uplo):
    c = name[0] == "w"
    herm = c
    fmt = {"y": 0, "e": 0, "b": 1, "p": 2}[name[2]]
    for n, k in [(1, 0), (40, 5), (150, 0), (150, 149)]:
        A = dense(rng, n, n, c)
        S = sym_from_tri(A, n, uplo, herm)
        if fmt == 1:
            S = band_keep(S, k, k)
        ix, iy = -2, 3
        x, y = vecs(rng, n, ix, c), vecs(rng, n, iy, c)
        al, be = scal(rng, c), scal(rng, c)
        want = matvec(oracle, c, "N", np.ascontiguousarray(S), n, n, gather(x, n, ix), al, be, gather(y, n, iy))
        got = y.copy()
        if fmt == 0:
            gpu.l2(name, uplo, n, al, A, n, x, ix, be, got, iy)
        elif fmt == 1:
            kl, ku = (0, k) if uplo == "U" else (k, 0)
            AB = np.ascontiguousarray(to_band(S, kl, ku) if uplo == "U" else to_band(S, kl, ku))
            gpu.l2(name, uplo, n, k, al, AB, k + 1, x, ix, be, got, iy)
        else:
            gpu.l2(name, uplo, n, al, to_packed(S, n, uplo), x, ix, be, got, iy)
        assert gpu.last_error()[0] == 0, gpu.last_error()
        scale = orc.dd_abs(al) * n * orc.dd_absmax(S) * orc.dd_absmax(x) + orc.dd_abs(be) * orc.dd_absmax(y)
        assert err_ok(gather(got, n, iy), want, scale, max(10, 4 * n) * orc.EPS_DD), (n, k)


@pytest.mark.parametrize("kind", ["tr", "tb", "tp"])
@pytest.mark.parametrize("c", [False, True])
@pytest.mark.parametrize("uplo", ["U", "L"])
@pytest.mark.parametrize("trans", ["N", "T", "C"])
@pytest.mark.parametrize("diag", ["N", "U"])
def test_triangular_mv_and_solve(gpu, oracle, rng, kind, c, uplo, trans, diag):
    if trans == "C" and not c:
        pytest.skip("real 'C' folds to 'T'")
    p = "w" if c else "m"
    for n, k in [(1, 0), (60, 7), (200, 45), (150, 70), (300, 7), (1000, 31)]:   # k <= 31, n > 64: partitioned
        A = dense(rng, n, n, c) / n
        d = np.arange(n)
        A[d, d] = ONE[c] * 0 + (np.array([[1.5, 0.0], [0.0, 0.0]]) if c else np.array([1.5, 0.0]))
        T = tri_dense(A, n, uplo, diag == "U")
        if kind == "tb":
            kl, ku = (0, k) if uplo == "U" else (k, 0)
            T = band_keep(T, kl, ku)
            Tin = np.ascontiguousarray(to_band(np.where(np.ones_like(T, bool), band_keep(A[:n, :n], kl, ku), 0), kl,
                                               ku))
        elif kind == "tp":
            Tin = to_packed(A, n, uplo)
        else:
            Tin = A
        inc = -2
        x = vecs(rng, n, inc, c)
        # multiply
        want = matvec(oracle, c, trans if c else ("T" if trans != "N" else "N"), T, n, n, gather(x, n, inc), ONE[c],
                      ZERO[c], np.zeros_like(gather(x, n, inc)))
        got = x.copy()
        args = (uplo, trans, diag, n) + ((k,) if kind == "tb" else ()) + (Tin,) + \
            (() if kind == "tp" else ((k + 1) if kind == "tb" else n,)) + (got, inc)
        gpu.l2(p + kind + "mv", *args)
        assert gpu.last_error()[0] == 0, gpu.last_error()
        scale = n * orc.dd_absmax(T) * orc.dd_absmax(x)
        assert err_ok(gather(got, n, inc), want, scale, max(10, 4 * n) * orc.EPS_DD), (n, "mv")
        # solve: residual op(T) x - b in binary128
        b = vecs(rng, n, inc, c)
        # band solves both in place from the band (1) and through a dense copy (2)
        for mode in ((1, 2) if kind == "tb" else (0,)):
            prev = gpu.lib.mwblas_set_band_solve(mode)
            sol = b.copy()
            args = (uplo, trans, diag, n) + ((k,) if kind == "tb" else ()) + (Tin,) + \
                (() if kind == "tp" else ((k + 1) if kind == "tb" else n,)) + (sol, inc)
            gpu.l2(p + kind + "sv", *args)
            gpu.lib.mwblas_set_band_solve(prev)
            assert gpu.last_error()[0] == 0, gpu.last_error()
            xs = gather(sol, n, inc)
            r = matvec(oracle, c, trans if c else ("T" if trans != "N" else "N"), T, n, n, xs, ONE[c], ZERO[c],
                       np.zeros_like(xs))
            scale = n * orc.dd_absmax(T) * orc.dd_absmax(xs) + orc.dd_absmax(b)
            assert err_ok(r, gather(b, n, inc), scale, max(20, 8 * n) * orc.EPS_DD), (n, "sv", mode)


@pytest.mark.parametrize("name", ["mger", "wgeru", "wgerc"])
def test_ger(gpu, oracle, rng, name):
    c = name != "mger"
    for m, n in [(1, 1), (33, 47), (140, 90)]:
        A = dense(rng, m, n, c, m + 2)
        ix, iy = 3, -2
        x, y = vecs(rng, m, ix, c), vecs(rng, n, iy, c)
        al = scal(rng, c)
        X = np.ascontiguousarray(gather(x, m, ix)[None])
        Y = np.ascontiguousarray(gather(y, n, iy)[None])
        want = qmm(oracle, c, "N", "C" if name == "wgerc" else "T", m, n, 1, al, X, m, Y, n, ONE[c], A.copy(), m + 2)
        got = A.copy()
        gpu.l2(name, m, n, al, x, ix, y, iy, got, m + 2)
        assert gpu.last_error()[0] == 0, gpu.last_error()
        assert np.array_equal(got[:, m:], A[:, m:])
        scale = orc.dd_abs(al) * orc.dd_absmax(x) * orc.dd_absmax(y) + orc.dd_absmax(A)
        assert err_ok(got[:, :m], want[:, :m], scale, 10 * orc.EPS_DD), (m, n)


@pytest.mark.parametrize("name", ["msyr", "wher", "mspr", "whpr", "msyr2", "wher2", "mspr2", "whpr2"])
@pytest.mark.parametrize("uplo", ["U", "L"])
def test_symmetric_rank_updates(gpu, oracle, rng, name, uplo):
    c = name[0] == "w"
    herm = c
    packed = name[1] == "s" and name[2] == "p" or name[1:3] == "hp"
    two = name.endswith("2")
    for n in [1, 45, 130]:
        A = dense(rng, n, n, c)
        if herm:
            A = herm_fix(A.copy(), True)
        ix, iy = -3, 2
        x = vecs(rng, n, ix, c)
        y = vecs(rng, n, iy, c) if two else None
        al = mwb.random_dd(rng, ()) if (herm and not two) else scal(rng, c)
        al_c = np.array([al, [0.0, 0.0]]) if (herm and not two) else al
        X = np.ascontiguousarray(gather(x, n, ix)[None])
        tb = "C" if herm else "T"
        if two:
            Y = np.ascontiguousarray(gather(y, n, iy)[None])
            W = qmm(oracle, c, "N", tb, n, n, 1, al_c, X, n, Y, n, ONE[c], A.copy(), n)
            al2 = al_c.copy()
            if herm:
                al2[1] = -al2[1]
            W = qmm(oracle, c, "N", tb, n, n, 1, al2, Y, n, X, n, ONE[c], W, n)
        else:
            W = qmm(oracle, c, "N", tb, n, n, 1, al_c, X, n, X, n, ONE[c], A.copy(), n)
        W = herm_fix(W, herm)
        i = np.arange(n)[None, :]
        j = np.arange(n)[:, None]
        mask = (i <= j) if uplo == "U" else (i >= j)
        if packed:
            ap = to_packed(A, n, uplo)
            got = ap.copy()
            args = (uplo, n, al, x, ix) + ((y, iy) if two else ()) + (got,)
            gpu.l2(name, *args)
            want = to_packed(W, n, uplo)
        else:
            got = A.copy()
            args = (uplo, n, al, x, ix) + ((y, iy) if two else ()) + (got, n)
            gpu.l2(name, *args)
            shape = (n, n) + (1,) * (A.ndim - 2)
            assert np.array_equal(np.where(mask.reshape(shape), 0.0, got), np.where(mask.reshape(shape), 0.0, A))
            got = np.where(mask.reshape(shape), got, 0.0)
            want = np.where(mask.reshape(shape), W, 0.0)
        assert gpu.last_error()[0] == 0, gpu.last_error()
        scale = 2 * orc.dd_abs(al) * orc.dd_absmax(x) * orc.dd_absmax(y if two else x) + orc.dd_absmax(A)
        assert err_ok(got, want, scale, 10 * orc.EPS_DD), (n,)


def _padded(AB, ldab):
    """Band storage with ldab rows per column (the band in the first rows)."""
    out = np.zeros((AB.shape[0], ldab) + AB.shape[2:])
    out[:, :AB.shape[1]] = AB
    return np.ascontiguousarray(out)


@pytest.mark.parametrize("c", [False, True])
@pytest.mark.parametrize("uplo", ["U", "L"])
def test_band_rows_over_many_blocks(gpu, oracle, rng, c, uplo):
    """A symmetric (Hermitian) band product over many row blocks, read in
    place from band storage with a tight and with a padded leading dimension:
    both agree bit for bit and with the oracle."""
    name = "whbmv" if c else "msbmv"
    n, k = 1100, 7
    A = dense(rng, n, n, c)
    S = band_keep(sym_from_tri(A, n, uplo, c), k, k)
    kl, ku = (0, k) if uplo == "U" else (k, 0)
    AB = np.ascontiguousarray(to_band(S, kl, ku))
    ix, iy = 1, -2
    x, y = vecs(rng, n, ix, c), vecs(rng, n, iy, c)
    al, be = scal(rng, c), scal(rng, c)
    outs = []
    for ldab in (k + 1, k + 1 + 400):
        got = y.copy()
        gpu.l2(name, uplo, n, k, al, _padded(AB, ldab), ldab, x, ix, be, got, iy)
        assert gpu.last_error()[0] == 0, gpu.last_error()
        outs.append(got)
    np.testing.assert_array_equal(outs[0], outs[1])
    want = matvec(oracle, c, "N", np.ascontiguousarray(S), n, n, gather(x, n, ix), al, be, gather(y, n, iy))
    scale = orc.dd_abs(al) * n * orc.dd_absmax(S) * orc.dd_absmax(x) + orc.dd_abs(be) * orc.dd_absmax(y)
    assert err_ok(gather(outs[0], n, iy), want, scale, max(10, 4 * n) * orc.EPS_DD)


@pytest.mark.parametrize("trans", ["N", "T"])
def test_general_band_rows_over_many_blocks(gpu, oracle, rng, trans):
    """GBMV with op(A) = A and A^T over many row blocks, tight and padded
    leading dimension."""
    m, n, kl, ku = 700, 900, 3, 6
    F = band_keep(dense(rng, m, n, False), kl, ku)
    AB = np.ascontiguousarray(to_band(F, kl, ku))
    lx, ly = (n, m) if trans == "N" else (m, n)
    x, y = vecs(rng, lx, 1, False), vecs(rng, ly, 1, False)
    al, be = scal(rng, False), scal(rng, False)
    outs = []
    for ldab in (kl + ku + 1, kl + ku + 1 + 500):
        got = y.copy()
        gpu.l2("mgbmv", trans, m, n, kl, ku, al, _padded(AB, ldab), ldab, x, 1, be, got, 1)
        assert gpu.last_error()[0] == 0, gpu.last_error()
        outs.append(got)
    np.testing.assert_array_equal(outs[0], outs[1])
    want = matvec(oracle, False, trans, F, ly, lx, x, al, be, y)
    scale = orc.dd_abs(al) * lx * orc.dd_absmax(F) * orc.dd_absmax(x) + orc.dd_abs(be) * orc.dd_absmax(y)
    assert err_ok(outs[0], want, scale, max(10, 4 * max(m, n)) * orc.EPS_DD)


def _sbmv_both(gpu, *args, name="msbmv"):
    """msbmv (mspmv) through the shared-memory band tiles (the two coalesced
    halves of the packed kernels) and through a thread or warp per row
    reading the stored triangle in place."""
    outs = []
    prev = gpu.lib.mwblas_set_band_tile(1)
    try:
        for on in (1, 0):
            gpu.lib.mwblas_set_band_tile(on)
            got = args[-2].copy()
            gpu.l2(name, *args[:-2], got, args[-1])
            assert gpu.last_error()[0] == 0, gpu.last_error()
            outs.append(got)
    finally:
        gpu.lib.mwblas_set_band_tile(prev)
    return outs


@pytest.mark.parametrize("uplo", ["U", "L"])
def test_band_tile_matches_thread_per_row(gpu, oracle, rng, uplo):
    """Real symmetric band products from shared-memory tiles of 128 rows and
    from band storage read in place both agree with the oracle, over
    bandwidths 0..32 (33 takes the in-place kernels on both settings), orders
    around the tile size, padded leading dimensions, negative and strided
    increments and the three kinds of beta. Band-storage entries outside the
    matrix hold NaN, so reading one would show. (The two need not agree bit
    for bit: the tiles fix each row's block exponent before the products,
    the in-place kernels move it as larger terms arrive, and both keep the
    sum exact to about 2^-130 of its largest term before the one rounding.)"""
    cases = [(1, 0), (5, 3), (127, 1), (128, 16), (129, 31), (700, 32), (1100, 16), (300, 33)]
    for t, (n, k) in enumerate(cases):
        S = band_keep(sym_from_tri(dense(rng, n, n, False), n, uplo, False), k, k)
        kl, ku = (0, k) if uplo == "U" else (k, 0)
        AB = to_band(S, kl, ku)
        for j in range(n):
            for b in range(k + 1):
                i = j - k + b if uplo == "U" else j + b
                if i < 0 or i >= n:
                    AB[j, b] = np.nan
        ldab = k + 1 + (t % 3)
        ABp = _padded(AB, ldab)
        ix, iy = [(1, 1), (-2, 3), (3, -1)][t % 3]
        x, y = vecs(rng, n, ix, False), vecs(rng, n, iy, False)
        al = scal(rng, False)
        be = [ZERO[False], ONE[False], scal(rng, False)][t % 3]
        tile, rows = _sbmv_both(gpu, uplo, n, k, al, ABp, ldab, x, ix, be, y, iy)
        want = matvec(oracle, False, "N", np.ascontiguousarray(S), n, n, gather(x, n, ix), al, be,
                      gather(y, n, iy))
        scale = orc.dd_abs(al) * n * orc.dd_absmax(S) * orc.dd_absmax(x) + orc.dd_abs(be) * orc.dd_absmax(y)
        for got in (tile, rows):
            assert err_ok(gather(got, n, iy), want, scale, max(10, 4 * n) * orc.EPS_DD), (n, k)


@pytest.mark.parametrize("uplo", ["U", "L"])
def test_band_tile_non_finite_entry(gpu, rng, uplo):
    """An infinity stored at band entry (i0, j0) makes exactly rows i0 and j0
    of the result NaN (the reference's double-double product of an infinity
    is NaN), on both kernels, and leaves the other rows finite."""
    n, k, i0, j0 = 300, 16, 130, 140
    S = band_keep(sym_from_tri(dense(rng, n, n, False), n, uplo, False), k, k)
    kl, ku = (0, k) if uplo == "U" else (k, 0)
    AB = to_band(S, kl, ku)
    si, sj = (i0, j0) if uplo == "U" else (j0, i0)       # the stored triangle's entry
    AB[sj, (k + si - sj) if uplo == "U" else (si - sj)] = np.array([np.inf, 0.0])
    x, y = vecs(rng, n, 1, False), vecs(rng, n, 1, False)
    tile, rows = _sbmv_both(gpu, uplo, n, k, scal(rng, False), np.ascontiguousarray(AB), k + 1, x, 1,
                            scal(rng, False), y, 1)
    for got in (tile, rows):
        bad = np.flatnonzero(np.isnan(got[:, 0]))
        assert list(bad) == [i0, j0], bad
        assert np.isfinite(np.delete(got, bad, axis=0)).all()


@pytest.mark.parametrize("uplo", ["U", "L"])
def test_packed_halves_match_oracle(gpu, oracle, rng, uplo):
    """Real symmetric packed products from the two coalesced halves (row
    halves in 512-column chunks, column halves a warp per row) and from a
    warp per row in place both agree with the oracle, over orders around the
    chunk size, negative and strided increments, y overlapping x (through a
    copy) and the three kinds of beta."""
    for t, n in enumerate([1, 2, 33, 511, 512, 513, 1100, 2049]):
        S = sym_from_tri(dense(rng, n, n, False), n, uplo, False)
        AP = to_packed(S, n, uplo)
        ix, iy = [(1, 1), (-2, 3), (3, -1)][t % 3]
        x, y = vecs(rng, n, ix, False), vecs(rng, n, iy, False)
        al = scal(rng, False)
        be = [ZERO[False], ONE[False], scal(rng, False)][t % 3]
        packed, rows = _sbmv_both(gpu, uplo, n, al, AP, x, ix, be, y, iy, name="mspmv")
        want = matvec(oracle, False, "N", np.ascontiguousarray(S), n, n, gather(x, n, ix), al, be,
                      gather(y, n, iy))
        scale = orc.dd_abs(al) * n * orc.dd_absmax(S) * orc.dd_absmax(x) + orc.dd_abs(be) * orc.dd_absmax(y)
        for got in (packed, rows):
            assert err_ok(gather(got, n, iy), want, scale, max(10, 4 * n) * orc.EPS_DD), (n, uplo)


@pytest.mark.parametrize("uplo", ["U", "L"])
def test_packed_halves_non_finite_and_zero(gpu, rng, uplo):
    """An infinity at packed entry (i0, j0) makes exactly rows i0 and j0 NaN on
    both paths; zero entries and a zero x take the general decode and leave
    the other rows finite and in agreement."""
    n, i0, j0 = 700, 600, 650
    S = sym_from_tri(dense(rng, n, n, False), n, uplo, False)
    S[10:20, :] = 0.0
    S[:, 10:20] = 0.0
    si, sj = (i0, j0) if uplo == "U" else (j0, i0)
    S[sj, si] = np.array([np.inf, 0.0])           # column sj, row si of the stored triangle
    AP = to_packed(S, n, uplo)
    x, y = vecs(rng, n, 1, False), vecs(rng, n, 1, False)
    x[5] = 0.0
    al, be = scal(rng, False), scal(rng, False)
    packed, rows = _sbmv_both(gpu, uplo, n, al, AP, x, 1, be, y, 1, name="mspmv")
    for got in (packed, rows):
        bad = np.flatnonzero(np.isnan(got[:, 0]))
        assert list(bad) == [i0, j0], bad
    ok = np.setdiff1d(np.arange(n), [i0, j0])
    finite = np.where(np.isfinite(S), S, 0.0)
    scale = orc.dd_abs(al) * n * orc.dd_absmax(finite) * orc.dd_absmax(x) + orc.dd_abs(be) * orc.dd_absmax(y)
    d = float(np.max(orc.dd_diff_abs(packed[ok], rows[ok])))
    assert d <= 8 * n * orc.EPS_DD * scale, d
