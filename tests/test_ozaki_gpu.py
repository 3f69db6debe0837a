"""Ozaki-scheme (integer-exact tensor-core) GEMM parity on the GPU.

* normwise error against the binary128 oracle within the reference's GEMM
  tolerance max(10, 4k) * 2^-104, on the reference's value distribution and
  on an exponent-spread stress input (rows of A / columns of B scaled by 2^e,
  e uniform in [-30, 30]);
* the tcgen05 residue GEMM and the independent CUDA-core residue GEMM give
  bit-identical results (both are exact integer computations);
* non-finite entries of A or B make their output rows/columns NaN, as the FP64
  engine (and the reference's double-double products of an infinity) do.
"""
import numpy as np
import pytest

from conftest import mwb, orc

pytestmark = pytest.mark.gpu


def op_norm(alpha, k, A, B, beta, C0):
    return orc.dd_abs(alpha) * k * orc.dd_absmax(A) * orc.dd_absmax(B) + orc.dd_abs(beta) * orc.dd_absmax(C0)


SHAPES = [(1, 1, 1), (5, 3, 70), (128, 256, 64), (130, 300, 1500), (257, 129, 2100), (64, 600, 33)]


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("N", "T"), ("T", "N"), ("T", "T")])
def test_ozaki_matches_oracle(gpu, oracle, rng, ta, tb):
    for (m, n, k) in SHAPES:
        lda = (m if ta == "N" else k) + 1
        ldb = (k if tb == "N" else n) + 2
        ldc = m + 3
        A = mwb.dd_matrix(rng, m if ta == "N" else k, k if ta == "N" else m, lda)
        B = mwb.dd_matrix(rng, k if tb == "N" else n, n if tb == "N" else k, ldb)
        C0 = mwb.dd_matrix(rng, m, n, ldc, fill=-7.37e18)
        al, be = mwb.random_dd(rng, ()), mwb.random_dd(rng, ())
        want = oracle.qgemm(ta, tb, m, n, k, al, A, lda, B, ldb, be, C0.copy(), ldc)
        got = C0.copy()
        gpu.mgemm(ta, tb, m, n, k, al, A, lda, B, ldb, be, got, ldc, engine="ozaki")
        assert gpu.last_error()[0] == 0, gpu.last_error()
        assert gpu.lib.mwblas_last_ozaki_moduli() >= 10
        assert np.all(got[:, m:] == -7.37e18)
        err = orc.normwise_error(got[:, :m], want[:, :m], op_norm(al, k, A, B, be, C0[:, :m]))
        assert err <= max(10, 4 * k) * orc.EPS_DD, (ta, tb, m, n, k, err)


def test_tensor_core_and_cuda_core_paths_bit_identical(gpu, rng):
    m, n, k = 200, 300, 2500
    A = mwb.dd_matrix(rng, m, k)
    B = mwb.dd_matrix(rng, k, n)
    al, be = mwb.random_dd(rng, ()), np.zeros(2)
    outs = []
    for kind in (0, 1, 2, 3):   # per-tile tcgen05, CUDA cores, persistent tcgen05, CTA pairs
        prev = gpu.lib.mwblas_set_ozaki_mma(kind)
        try:
            c = np.zeros((n, m, 2))
            gpu.mgemm("N", "N", m, n, k, al, A, m, B, k, be, c, m, engine="ozaki")
            assert gpu.last_error()[0] == 0, gpu.last_error()
            outs.append(c)
        finally:
            gpu.lib.mwblas_set_ozaki_mma(prev)
    np.testing.assert_array_equal(outs[0], outs[1])
    np.testing.assert_array_equal(outs[0], outs[2])
    np.testing.assert_array_equal(outs[0], outs[3])


@pytest.mark.parametrize("k", [300, 512, 1024, 1500, 2600])
@pytest.mark.parametrize("uplo", [0, 1])
def test_persistent_tensor_core_kernel(gpu, rng, k, uplo):
    """The persistent residue-GEMM kernel (units taken two at a time, their K
    chunks interleaved) gives the per-tile kernel's bits for one, two and more
    K chunks (512 each), full and triangular outputs, and CTAs left with an
    odd unit at the end."""
    n = 700
    A = mwb.dd_matrix(rng, n, k)
    outs = []
    for kind in (0, 2, 3):
        prev = gpu.lib.mwblas_set_ozaki_mma(kind)
        try:
            c = np.zeros((n, n, 2))
            with engine(gpu, OZAKI):
                if uplo:
                    gpu.msyrk("U", "N", n, k, 1.0, A, n, 0.0, c, n)
                else:
                    gpu.mgemm("N", "T", n, n, k, 1.0, A, n, A, n, 0.0, c, n)
            assert gpu.last_error()[0] == 0, gpu.last_error()
            outs.append(c)
        finally:
            gpu.lib.mwblas_set_ozaki_mma(prev)
    np.testing.assert_array_equal(outs[0], outs[1])
    np.testing.assert_array_equal(outs[0], outs[2])


def test_exponent_spread_stress(gpu, oracle, rng):
    """Entries m_ij * 2^e with e uniform in [-30, 30] per row of A / column of B."""
    m, n, k = 192, 160, 777
    A = mwb.dd_matrix(rng, m, k)
    B = mwb.dd_matrix(rng, k, n)
    ea = rng.integers(-30, 31, size=m).astype(float)
    eb = rng.integers(-30, 31, size=n).astype(float)
    A *= (2.0 ** ea)[None, :, None]
    B *= (2.0 ** eb)[:, None, None]
    al, be = np.array([1.0, 0.0]), np.zeros(2)
    want = oracle.qgemm("N", "N", m, n, k, al, A, m, B, k, be, np.zeros((n, m, 2)), m)
    got = np.zeros((n, m, 2))
    gpu.mgemm("N", "N", m, n, k, al, A, m, B, k, be, got, m, engine="ozaki")
    assert gpu.last_error()[0] == 0
    err = orc.normwise_error(got, want, op_norm(al, k, A, B, be, got))
    assert err <= 4 * k * orc.EPS_DD, err
    # per-element relative accuracy follows the per-row/column scaling
    scale = (2.0 ** ea)[None, :] * (2.0 ** eb)[:, None] * k
    rel = orc.dd_diff_abs(got, want) / scale
    assert float(rel.max()) <= 4 * k * orc.EPS_DD * 4


def test_nonfinite_inputs_match_fp64_engine(gpu, rng):
    m, n, k = 40, 30, 50
    A = mwb.dd_matrix(rng, m, k)
    B = mwb.dd_matrix(rng, k, n)
    A[3, 5] = (np.inf, 0.0)
    c1 = np.zeros((n, m, 2)); c2 = np.zeros((n, m, 2))
    gpu.mgemm("N", "N", m, n, k, 1.0, A, m, B, k, 0.0, c1, m, engine="ozaki")
    gpu.mgemm("N", "N", m, n, k, 1.0, A, m, B, k, 0.0, c2, m, engine="plain")
    np.testing.assert_array_equal(np.isfinite(c1), np.isfinite(c2))
    assert np.all(np.isnan(c1[:, 5])) and np.all(np.isfinite(np.delete(c1, 5, axis=1)))
    # column 7 of B as well, through the complex-free SYRK-free path with beta != 0
    B[7, 2] = (np.nan, 0.0)
    c3 = np.ones((n, m, 2))
    gpu.mgemm("N", "N", m, n, k, 1.0, A, m, B, k, 0.5, c3, m, engine="ozaki")
    assert np.all(np.isnan(c3[7, :])) and np.all(np.isnan(c3[:, 5]))


def test_auto_engine_and_bits_control(gpu, oracle, rng):
    m = n = k = 300
    A = mwb.dd_matrix(rng, m, k); B = mwb.dd_matrix(rng, k, n)
    want = oracle.qgemm("N", "N", m, n, k, np.array([1.0, 0]), A, m, B, k, np.zeros(2), np.zeros((n, m, 2)), m)
    prev = gpu.lib.mwblas_set_ozaki_bits(60)
    try:
        got = np.zeros((n, m, 2))
        gpu.mgemm("N", "N", m, n, k, 1.0, A, m, B, k, 0.0, got, m, engine="ozaki")
        few = gpu.lib.mwblas_last_ozaki_moduli()
        err60 = orc.normwise_error(got, want, k * orc.dd_absmax(A) * orc.dd_absmax(B))
    finally:
        gpu.lib.mwblas_set_ozaki_bits(prev)
    got = np.zeros((n, m, 2))
    gpu.mgemm("N", "N", m, n, k, 1.0, A, m, B, k, 0.0, got, m, engine="ozaki")
    many = gpu.lib.mwblas_last_ozaki_moduli()
    err = orc.normwise_error(got, want, k * orc.dd_absmax(A) * orc.dd_absmax(B))
    assert few < many
    assert err < err60 and err60 < 2.0 ** -50 and err <= 4 * k * orc.EPS_DD


class engine:
    """Forces the GEMM engine for every routine built on it (wgemm_, msyrk_...)."""

    def __init__(self, lib, which):
        self.lib, self.which = lib, which

    def __enter__(self):
        self.prev = self.lib.lib.mwblas_set_gemm_engine(self.which)

    def __exit__(self, *a):
        self.lib.lib.mwblas_set_gemm_engine(self.prev)


OZAKI, PLAIN = 2, 1


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("N", "C"), ("C", "T"), ("T", "C")])
def test_ozaki_complex_matches_oracle(gpu, oracle, rng, ta, tb):
    for (m, n, k) in [(3, 2, 5), (130, 257, 1100), (64, 33, 40)]:
        lda = (m if ta == "N" else k) + 1
        ldb = (k if tb == "N" else n)
        ldc = m + 2
        A = mwb.dd_matrix(rng, m if ta == "N" else k, k if ta == "N" else m, lda, cplx_=True)
        B = mwb.dd_matrix(rng, k if tb == "N" else n, n if tb == "N" else k, ldb, cplx_=True)
        C0 = mwb.dd_matrix(rng, m, n, ldc, cplx_=True)
        al, be = mwb.random_cdd(rng, ()), mwb.random_cdd(rng, ())
        want = oracle.qwgemm(ta, tb, m, n, k, al, A, lda, B, ldb, be, C0.copy(), ldc)
        got = C0.copy()
        with engine(gpu, OZAKI):
            gpu.wgemm(ta, tb, m, n, k, al, A, lda, B, ldb, be, got, ldc)
        assert gpu.last_error()[0] == 0, gpu.last_error()
        opn = 2 * op_norm(al, k, A, B, be, C0[:, :m])
        err = orc.normwise_error(got[:, :m], want[:, :m], opn)
        assert err <= max(10, 4 * k) * orc.EPS_DD, (ta, tb, m, n, k, err)


def test_ozaki_complex_tc_equals_cuda_core(gpu, rng):
    m, n, k = 140, 270, 1300
    A = mwb.dd_matrix(rng, m, k, cplx_=True)
    B = mwb.dd_matrix(rng, k, n, cplx_=True)
    outs = []
    for kind in (0, 1, 2, 3):
        prev = gpu.lib.mwblas_set_ozaki_mma(kind)
        try:
            c = np.zeros((n, m, 2, 2))
            with engine(gpu, OZAKI):
                gpu.wgemm("N", "C", m, n, k, 1.0, A, m, B, n, 0.0, c, m)
            outs.append(c)
        finally:
            gpu.lib.mwblas_set_ozaki_mma(prev)
    np.testing.assert_array_equal(outs[0], outs[1])
    np.testing.assert_array_equal(outs[0], outs[2])
    np.testing.assert_array_equal(outs[0], outs[3])


@pytest.mark.parametrize("uplo", ["U", "L"])
@pytest.mark.parametrize("trans", ["N", "T"])
def test_ozaki_syrk(gpu, oracle, rng, uplo, trans):
    n, k = 300, 700
    lda = (n if trans == "N" else k)
    A = mwb.dd_matrix(rng, n if trans == "N" else k, k if trans == "N" else n, lda)
    C0 = mwb.dd_matrix(rng, n, n)
    off = np.triu_indices(n, 1) if uplo == "L" else np.tril_indices(n, -1)
    C0[off[1], off[0]] = -7.37e18
    al, be = mwb.random_dd(rng, ()), mwb.random_dd(rng, ())
    want = C0.copy(); oracle.qsyrk(uplo, trans, n, k, al, A, lda, be, want, n)
    got = C0.copy()
    with engine(gpu, OZAKI):
        gpu.msyrk(uplo, trans, n, k, al, A, lda, be, got, n)
    assert gpu.last_error()[0] == 0
    assert np.all(got[off[1], off[0]] == -7.37e18)
    tri = np.tril_indices(n) if uplo == "L" else np.triu_indices(n)
    err = orc.normwise_error(got[tri[1], tri[0]], want[tri[1], tri[0]], op_norm(al, k, A, A, be, C0[tri[1], tri[0]]))
    assert err <= 4 * k * orc.EPS_DD, err


@pytest.mark.parametrize("uplo", ["U", "L"])
@pytest.mark.parametrize("trans", ["N", "C"])
def test_ozaki_herk(gpu, oracle, rng, uplo, trans):
    n, k = 200, 300
    lda = (n if trans == "N" else k)
    A = mwb.dd_matrix(rng, n if trans == "N" else k, k if trans == "N" else n, lda, cplx_=True)
    C0 = mwb.dd_matrix(rng, n, n, cplx_=True)
    al, be = mwb.random_dd(rng, ()), mwb.random_dd(rng, ())
    want = C0.copy(); oracle.qherk(uplo, trans, n, k, al, A, lda, be, want, n)
    got = C0.copy()
    with engine(gpu, OZAKI):
        gpu.wherk(uplo, trans, n, k, al, A, lda, be, got, n)
    assert gpu.last_error()[0] == 0
    d = np.arange(n)
    assert np.all(got[d, d, 1] == 0.0)
    tri = np.tril_indices(n) if uplo == "L" else np.triu_indices(n)
    err = orc.normwise_error(got[tri[1], tri[0]], want[tri[1], tri[0]],
                             2 * op_norm(al, k, A, A, be, C0[tri[1], tri[0]]))
    assert err <= 4 * k * orc.EPS_DD, err


def test_ozaki_trsm_trailing_updates(gpu, oracle, rng):
    """Blocked TRSM whose trailing GEMMs run on the Ozaki engine."""
    m, n = 400, 96
    A = mwb.dd_matrix(rng, m, m)
    A[..., 0] /= m
    A[..., 1] /= m
    for d in range(m):
        A[d, d] = (1.0 + rng.random(), 0.0)
    B0 = mwb.dd_matrix(rng, m, n)
    al = mwb.random_dd(rng, ())
    for uplo in ("L", "U"):
        want = B0.copy(); oracle.qtrsm("L", uplo, "N", "N", m, n, al, A, m, want, m)
        got = B0.copy()
        with engine(gpu, OZAKI):
            gpu.mtrsm("L", uplo, "N", "N", m, n, al, A, m, got, m)
        assert gpu.last_error()[0] == 0
        err = orc.normwise_error(got, want, orc.dd_abs(al) * orc.dd_absmax(B0))
        assert err <= max(20, 8 * m * m) * orc.EPS_DD


@pytest.mark.parametrize("cplx_", [False, True])
def test_pair_kernel_large_device_product_bit_identical(gpu, rng, cplx_):
    """A device-resident product above 2048 x 2048 (a short last 256-column
    tile, beta != 0): the CTA-pair kernel gives the single-SM persistent
    kernel's bits."""
    import torch
    m, n, k = 2100, 2300, 300
    dev = torch.device("cuda", 0)
    A = torch.from_numpy(mwb.dd_matrix(rng, m, k, cplx_=cplx_)).to(dev)
    B = torch.from_numpy(mwb.dd_matrix(rng, k, n, cplx_=cplx_)).to(dev)
    C0 = torch.from_numpy(mwb.dd_matrix(rng, m, n, cplx_=cplx_)).to(dev)
    al = mwb.random_cdd(rng, ()) if cplx_ else mwb.random_dd(rng, ())
    be = mwb.random_cdd(rng, ()) if cplx_ else mwb.random_dd(rng, ())
    outs = []
    for kind in (3, 2):
        prev = gpu.lib.mwblas_set_ozaki_mma(kind)
        try:
            C = C0.clone()
            with engine(gpu, OZAKI):
                if cplx_:
                    gpu.wgemm("N", "N", m, n, k, al, A.data_ptr(), m, B.data_ptr(), k, be, C.data_ptr(), m)
                else:
                    gpu.mgemm("N", "N", m, n, k, al, A.data_ptr(), m, B.data_ptr(), k, be, C.data_ptr(), m)
            assert gpu.last_error()[0] == 0, gpu.last_error()
            outs.append(C.cpu().numpy())
        finally:
            gpu.lib.mwblas_set_ozaki_mma(prev)
    assert np.array_equal(outs[0].view(np.uint64), outs[1].view(np.uint64))


# ---- moduli count from the operands' significant width ---------------------------------------
# (measured for top-level products of at least 1024^3, so the shapes below are that large)

def _lo0(rng, rows, cols):
    """FP64 values (lo = 0), hi ~ U[-1, 1): the reference fuzz's real64x2(2u - 1)."""
    a = mwb.dd_matrix(rng, rows, cols)
    a[..., 1] = 0.0
    return a


def _dev(torch, a):
    return torch.from_numpy(a).cuda()


def _same_but_last_rounding(a, b):
    """Equal up to the final rounding to double-double: the CRT fraction is
    accurate to ~2^-145 of the moduli product, which differs between two
    moduli sets, so an exact value next to a rounding boundary may round
    either way (a few outputs in a million, one unit of the lo limb)."""
    fin = np.isfinite(b[..., 0])
    assert np.array_equal(np.isfinite(a[..., 0]), fin)
    diff = orc.dd_diff_abs(a, b)[fin]
    assert np.all(diff <= 2.0 ** -104 * np.abs(b[..., 0][fin])), float(np.max(diff))
    assert np.mean(np.all(a == b, axis=-1)) > 0.999


def _ozaki_dev(gpu, torch, ta, tb, m, n, k, al, dA, lda, dB, ldb, be, C0, bits=0):
    """One tensor-core GEMM on device arrays at a given bits setting; returns
    the output, the moduli count and the bits of op(A), op(B)."""
    dC = _dev(torch, C0)
    prev = gpu.lib.mwblas_set_ozaki_bits(bits)
    try:
        gpu.mgemm(ta, tb, m, n, k, al, dA.data_ptr(), lda, dB.data_ptr(), ldb, be, dC.data_ptr(), m,
                  engine="ozaki")
        assert gpu.last_error()[0] == 0, gpu.last_error()
    finally:
        gpu.lib.mwblas_set_ozaki_bits(prev)
    return (dC.cpu().numpy(), gpu.lib.mwblas_last_ozaki_moduli(),
            (gpu.lib.mwblas_last_ozaki_bits(0), gpu.lib.mwblas_last_ozaki_bits(1)))


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "T")])
def test_fp64_inputs_take_fewer_moduli_with_identical_results(gpu, oracle, rng, ta, tb):
    """lo = 0 operands are exact integers at about 60-70 bits after the row /
    column scaling, so the automatic width cuts the moduli count; the exact
    integer product is the same as at 106 bits, and so is the result up to
    its final rounding."""
    import torch
    m, n, k = 1024, 1040, 1024
    A = _lo0(rng, m if ta == "N" else k, k if ta == "N" else m)
    B = _lo0(rng, k if tb == "N" else n, n if tb == "N" else k)
    C0 = mwb.dd_matrix(rng, m, n)
    al, be = mwb.random_dd(rng, ()), mwb.random_dd(rng, ())
    lda, ldb = A.shape[1], B.shape[1]
    dA, dB = _dev(torch, A), _dev(torch, B)
    auto, md_auto, (ba, bb) = _ozaki_dev(gpu, torch, ta, tb, m, n, k, al, dA, lda, dB, ldb, be, C0, 0)
    full, md_full, bw_full = _ozaki_dev(gpu, torch, ta, tb, m, n, k, al, dA, lda, dB, ldb, be, C0, 106)
    assert bw_full == (106, 106)
    assert 50 <= ba < 106 and 50 <= bb < 106, (ba, bb)
    assert md_auto <= md_full - 7, (md_auto, md_full)
    _same_but_last_rounding(auto, full)
    rows, cols = rng.integers(0, m, 256), rng.integers(0, n, 256)
    want = oracle.qgemm(ta, tb, m, n, k, al, A, lda, B, ldb, be, C0, m, rows=rows, cols=cols)
    err = orc.normwise_error(auto[cols, rows], want, op_norm(al, k, A, B, be, C0))
    assert err <= max(10, 4 * k) * orc.EPS_DD, err


def test_width_is_full_for_double_double_inputs(gpu, rng):
    import torch
    m = n = k = 1024
    A, B = mwb.dd_matrix(rng, m, k), mwb.dd_matrix(rng, k, n)
    C0 = np.zeros((n, m, 2))
    dA, dB = _dev(torch, A), _dev(torch, B)
    _, _, bw = _ozaki_dev(gpu, torch, "N", "N", m, n, k, np.array([1.0, 0.0]), dA, m, dB, k, np.zeros(2), C0)
    assert bw == (106, 106)


def test_small_integer_inputs_use_few_moduli_and_are_exact(gpu, rng):
    """Entries in {-3..3}: a few bits per operand and a handful of moduli. The
    hi limbs are the exact integer products; the lo limbs hold at most the
    reconstruction's fraction error (~2^-136 relative here), far below the
    double-double unit."""
    import torch
    m, n, k = 1030, 1040, 1024
    A = np.zeros((k, m, 2)); A[..., 0] = rng.integers(-3, 4, (k, m))
    B = np.zeros((n, k, 2)); B[..., 0] = rng.integers(-3, 4, (n, k))
    dA, dB = _dev(torch, A), _dev(torch, B)
    dC = torch.zeros((n, m, 2), dtype=torch.float64, device="cuda")
    gpu.mgemm("N", "N", m, n, k, np.array([1.0, 0.0]), dA.data_ptr(), m, dB.data_ptr(), k, np.zeros(2),
              dC.data_ptr(), m, engine="ozaki")
    assert gpu.last_error()[0] == 0
    md = gpu.lib.mwblas_last_ozaki_moduli()
    assert gpu.lib.mwblas_last_ozaki_bits(0) <= 8 and md <= 5, md
    exact = (A[..., 0].T @ B[..., 0].T)          # m x n, exact in float64 here
    got = dC.cpu().numpy()
    np.testing.assert_array_equal(got[..., 0], exact.T)
    assert np.all(np.abs(got[..., 1]) <= 2.0 ** -104 * np.abs(got[..., 0]))


def test_width_ignores_nonfinite_and_zero_rows(gpu, rng):
    """A row of op(A) holding an Inf (its outputs become NaN) and an all-zero
    row do not widen the operand; the other outputs equal the full-width
    ones up to the final rounding. One entry far below the rest of its row does widen it (to the full
    106 bits, as exactness would need ~950)."""
    import torch
    m, n, k = 1024, 1024, 1024
    A = _lo0(rng, m, k)
    B = _lo0(rng, k, n)
    A[:, 5, 0] = 0.0                             # row 5 all zero
    A[17, 9, 0] = np.inf                         # row 9 holds an Inf
    C0 = np.zeros((n, m, 2))
    one, zero = np.array([1.0, 0.0]), np.zeros(2)
    dA, dB = _dev(torch, A), _dev(torch, B)
    auto, md_auto, (ba, _) = _ozaki_dev(gpu, torch, "N", "N", m, n, k, one, dA, m, dB, k, zero, C0, 0)
    full, md_full, _ = _ozaki_dev(gpu, torch, "N", "N", m, n, k, one, dA, m, dB, k, zero, C0, 106)
    assert ba < 106 and md_auto < md_full
    assert np.all(np.isnan(auto[:, 9, 0])) and np.all(np.isnan(full[:, 9, 0]))
    _same_but_last_rounding(np.delete(auto, 9, axis=1), np.delete(full, 9, axis=1))
    assert np.all(auto[:, 5] == 0)
    A[3, 11, 0] = 2.0 ** -900                    # row 11: one entry far below the others
    dA = _dev(torch, A)
    _, _, (ba, _) = _ozaki_dev(gpu, torch, "N", "N", m, n, k, one, dA, m, dB, k, zero, C0, 0)
    assert ba == 106


def test_fp64_inputs_complex_and_syrk(gpu, oracle, rng):
    """The width also sizes complex products (real and imaginary parts
    together) and SYRK, where one conversion serves both operands."""
    import torch
    n, k = 1040, 1024
    A = _lo0(rng, n, k)
    dA = _dev(torch, A)
    al, be = mwb.random_dd(rng, ()), mwb.random_dd(rng, ())
    C0 = mwb.dd_matrix(rng, n, n)
    got = []
    for bits in (0, 106):
        dC = _dev(torch, C0)
        prev = gpu.lib.mwblas_set_ozaki_bits(bits)
        prev_e = gpu.lib.mwblas_set_gemm_engine(2)
        try:
            gpu.msyrk("U", "N", n, k, al, dA.data_ptr(), n, be, dC.data_ptr(), n)
            assert gpu.last_error()[0] == 0
            got.append((dC.cpu().numpy(), gpu.lib.mwblas_last_ozaki_moduli()))
        finally:
            gpu.lib.mwblas_set_ozaki_bits(prev)
            gpu.lib.mwblas_set_gemm_engine(prev_e)
    assert got[0][1] < got[1][1]
    _same_but_last_rounding(got[0][0], got[1][0])
    # complex, conjugate-transposed B
    m, n, k = 1024, 1024, 1024
    Ac = mwb.dd_matrix(rng, m, k, cplx_=True); Ac[..., 1] = 0.0
    Bc = mwb.dd_matrix(rng, n, k, cplx_=True); Bc[..., 1] = 0.0
    cal, cbe = mwb.random_cdd(rng, ()), mwb.random_cdd(rng, ())
    Cc = mwb.dd_matrix(rng, m, n, cplx_=True)
    dAc, dBc = _dev(torch, Ac), _dev(torch, Bc)
    outs = []
    for bits in (0, 106):
        dC = _dev(torch, Cc)
        prev = gpu.lib.mwblas_set_ozaki_bits(bits)
        prev_e = gpu.lib.mwblas_set_gemm_engine(2)
        try:
            gpu.wgemm("N", "C", m, n, k, cal, dAc.data_ptr(), m, dBc.data_ptr(), n, cbe, dC.data_ptr(), m)
            assert gpu.last_error()[0] == 0
            outs.append((dC.cpu().numpy(), gpu.lib.mwblas_last_ozaki_moduli()))
        finally:
            gpu.lib.mwblas_set_ozaki_bits(prev)
            gpu.lib.mwblas_set_gemm_engine(prev_e)
    assert outs[0][1] < outs[1][1]
    _same_but_last_rounding(outs[0][0], outs[1][0])
    rows, cols = rng.integers(0, m, 256), rng.integers(0, n, 256)
    want = oracle.qwgemm("N", "C", m, n, k, cal, Ac, m, Bc, n, cbe, Cc, m, rows=rows, cols=cols)
    op = orc.dd_abs(cal) * k * orc.dd_absmax(Ac) * orc.dd_absmax(Bc) + orc.dd_abs(cbe) * orc.dd_absmax(Cc)
    assert orc.normwise_error(outs[0][0][cols, rows], want, op) <= max(10, 4 * k) * orc.EPS_DD


# ---- residue conversion on the tensor cores ----------------------------------------------------

class residue_path:
    """Selects the residue conversion of real operands: 1 tcgen05 MMAs, 0 FP32 FMAs."""

    def __init__(self, lib, on):
        self.lib, self.on = lib, on

    def __enter__(self):
        self.prev = self.lib.lib.mwblas_set_residue_tc(self.on)

    def __exit__(self, *a):
        self.lib.lib.mwblas_set_residue_tc(self.prev)


def _both_residue_paths(gpu, run):
    outs = []
    for on in (1, 0):
        with residue_path(gpu, on):
            outs.append(run())
            assert gpu.last_error()[0] == 0, gpu.last_error()
    assert np.array_equal(outs[0].view(np.uint64), outs[1].view(np.uint64))
    return outs[0]


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("N", "T"), ("T", "N"), ("T", "T")])
def test_residue_conversion_tensor_cores_bit_identical(gpu, oracle, rng, ta, tb):
    """The limb dot products as tcgen05 MMAs give the FMA path's residues,
    hence the same output bits: ragged m, n, k (rows past the operand and k
    past its end are zero residues), padded leading dimensions, one to many
    16 x 32 tiles per CTA."""
    for (m, n, k) in [(1, 1, 1), (5, 3, 70), (37, 300, 33), (130, 97, 1500), (257, 129, 2100), (700, 520, 130)]:
        lda = (m if ta == "N" else k) + 3
        ldb = (k if tb == "N" else n) + 1
        A = mwb.dd_matrix(rng, m if ta == "N" else k, k if ta == "N" else m, lda)
        B = mwb.dd_matrix(rng, k if tb == "N" else n, n if tb == "N" else k, ldb)
        C0 = mwb.dd_matrix(rng, m, n, m + 2, fill=-7.37e18)
        al, be = mwb.random_dd(rng, ()), mwb.random_dd(rng, ())

        def run():
            c = C0.copy()
            gpu.mgemm(ta, tb, m, n, k, al, A, lda, B, ldb, be, c, m + 2, engine="ozaki")
            return c
        got = _both_residue_paths(gpu, run)
        assert np.all(got[:, m:] == -7.37e18)
        want = oracle.qgemm(ta, tb, m, n, k, al, A, lda, B, ldb, be, C0.copy(), m + 2)
        err = orc.normwise_error(got[:, :m], want[:, :m], op_norm(al, k, A, B, be, C0[:, :m]))
        assert err <= max(10, 4 * k) * orc.EPS_DD, (ta, tb, m, n, k, err)


def test_residue_conversion_tensor_cores_special_operands(gpu, oracle, rng):
    """Exponent-spread rows and columns, zero rows, non-finite entries, a
    device-resident product over 2048 x 2048, the shared conversion of SYRK
    and 30 moduli (bits = 120): identical bits on both residue paths."""
    import torch
    m, n, k = 192, 160, 777
    A = mwb.dd_matrix(rng, m, k)
    B = mwb.dd_matrix(rng, k, n)
    A *= (2.0 ** rng.integers(-30, 31, size=m).astype(float))[None, :, None]
    B *= (2.0 ** rng.integers(-30, 31, size=n).astype(float))[:, None, None]
    A[:, 7] = 0.0
    B[11, :] = 0.0
    A[5, 20] = (np.inf, 0.0)
    al, be = mwb.random_dd(rng, ()), mwb.random_dd(rng, ())

    def run():
        c = np.zeros((n, m, 2))
        gpu.mgemm("N", "N", m, n, k, al, A, m, B, k, be, c, m, engine="ozaki")
        return c
    got = _both_residue_paths(gpu, run)
    assert np.all(np.isnan(got[:, 20, 0])) and np.isfinite(got[:, 19, 0]).all()

    m, n, k = 2100, 2300, 300
    dev = torch.device("cuda", 0)
    dA = torch.from_numpy(mwb.dd_matrix(rng, m, k)).to(dev)
    dB = torch.from_numpy(mwb.dd_matrix(rng, k, n)).to(dev)
    C0 = torch.from_numpy(mwb.dd_matrix(rng, m, n)).to(dev)

    def run_dev():
        C = C0.clone()
        gpu.mgemm("N", "N", m, n, k, al, dA.data_ptr(), m, dB.data_ptr(), k, be, C.data_ptr(), m, engine="ozaki")
        return C.cpu().numpy()
    _both_residue_paths(gpu, run_dev)

    n, k = 300, 700
    A = mwb.dd_matrix(rng, n, k)
    C0 = mwb.dd_matrix(rng, n, n)

    def run_syrk():
        c = C0.copy()
        with engine(gpu, OZAKI):
            gpu.msyrk("U", "N", n, k, al, A, n, be, c, n)
        return c
    _both_residue_paths(gpu, run_syrk)

    m, n, k = 100, 90, 1500
    A = mwb.dd_matrix(rng, m, k)
    B = mwb.dd_matrix(rng, k, n)
    prev = gpu.lib.mwblas_set_ozaki_bits(120)
    try:
        def run_bits():
            c = np.zeros((n, m, 2))
            gpu.mgemm("N", "N", m, n, k, al, A, m, B, k, be, c, m, engine="ozaki")
            return c
        _both_residue_paths(gpu, run_bits)
        assert 28 < gpu.lib.mwblas_last_ozaki_moduli() <= 32
    finally:
        gpu.lib.mwblas_set_ozaki_bits(prev)
