"""Parity at the benchmark configurations' own sizes, on the GPU.

Each workload of the benchmark suite is run at its stated size through the C
ABI and compared with the binary128 oracle, using the reference's normwise
error (fuzz_util_body.fypp:242-271) and its tolerances: GEMM/SYRK/HERK
max(10, 4k) 2^-104 (the fuzz_mgemm tolerance line), TRSM max(20, 8 n^2)
2^-104 (fuzz_mtrsm.fypp:113-114), GEMV max(10, 4 max(m, n)) 2^-104
(fuzz_mgemv.fypp:65), DOT max(10, 4n) 2^-104 (fuzz_mdot.fypp:44); AXPY is
bit-exact. Where a full binary128 product would take minutes, 256 entries
(or 64 whole columns for TRSM, 256 rows for GEMV) are sampled; the sampled
entries of a product are independent, so the sample is an exact check of
those entries.

Configurations (value distribution everywhere: hi ~ U[-1, 1), lo = hi 2^-53
U[-1, 1), renormalised):
  0: GEMM 512^3 NN, alpha = 1, beta = 0, full check (every engine and AUTO);
  1: GEMM 4096^3 on the FP64 error-free-transform and the tensor-core engines,
     all four transpose pairs, random alpha/beta of magnitude 0.5..2; one
     8192^3 call on the FP64 engine; complex 4096^3 on both engines;
  2: tensor-core GEMM at 8192^3 on that distribution and on the
     exponent-spread stress input (rows of A and columns of B scaled by 2^e,
     e uniform in [-30, 30]);
  4: SYRK upper n = 8192, k = 2048; HERK n = 4096, k = 1024; TRSM
     left-lower-notrans 4096 x 1024 (diagonal uniform in [n, 2n]); GEMV
     16384^2; DOT and AXPY at n = 2^28.
"""
import numpy as np
import pytest

from conftest import mwb, orc

pytestmark = pytest.mark.gpu

SAMPLES = 256
ENGINE = {"auto": 0, "plain": 1, "ozaki": 2, "fixed": 3}


def dev_dd(torch, gen, shape, cplx_=False):
    """Device DD array of the benchmark distribution, layout (..., 2)."""
    def one():
        hi = torch.rand(shape, generator=gen, device="cuda", dtype=torch.float64) * 2 - 1
        lo = hi * 2.0 ** -53 * (torch.rand(shape, generator=gen, device="cuda", dtype=torch.float64) * 2 - 1)
        s = hi + lo
        return torch.stack([s, lo - (s - hi)], -1)
    if cplx_:
        return torch.stack([one(), one()], -2).contiguous()
    return one().contiguous()


def scalar(rng, cplx_=False):
    """A random double-double of magnitude 0.5..2 (complex: both parts)."""
    def one():
        mag = 0.5 + 1.5 * rng.random()
        v = mag if rng.random() < 0.5 else -mag
        return np.array([v, v * 2.0 ** -53 * (2 * rng.random() - 1)])
    return np.stack([one(), one()]) if cplx_ else one()


def op_norm(alpha, k, A, B, beta, C0):
    return orc.dd_abs(alpha) * k * orc.dd_absmax(A) * orc.dd_absmax(B) + orc.dd_abs(beta) * orc.dd_absmax(C0)


@pytest.fixture
def tgen(rng):
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(int(rng.integers(1 << 31)))
    return g


def with_engine(gpu, name):
    return gpu.lib.mwblas_set_gemm_engine(ENGINE[name])


# ---- config 0 ------------------------------------------------------------------------------

@pytest.mark.parametrize("engine", ["auto", "plain", "fixed", "ozaki"])
def test_config0_gemm_512_full(gpu, oracle, rng, engine):
    m = n = k = 512
    A = mwb.dd_matrix(rng, m, k)
    B = mwb.dd_matrix(rng, k, n)
    al, be = np.array([1.0, 0.0]), np.zeros(2)
    C = np.full((n, m, 2), np.nan)           # beta = 0: C is never read
    want = oracle.qgemm("N", "N", m, n, k, al, A, m, B, k, be, np.zeros((n, m, 2)), m)
    prev = with_engine(gpu, engine)
    try:
        gpu.mgemm("N", "N", m, n, k, al, A, m, B, k, be, C, m)
        assert gpu.last_error()[0] == 0, gpu.last_error()
    finally:
        gpu.lib.mwblas_set_gemm_engine(prev)
    err = orc.normwise_error(C, want, k * orc.dd_absmax(A) * orc.dd_absmax(B))
    assert err <= max(10, 4 * k) * orc.EPS_DD, (engine, err)
    assert err <= 1e-30


# ---- config 1 / 2: sampled GEMMs -----------------------------------------------------------

def _sampled_gemm(gpu, oracle, rng, torch, ta, tb, n, A, B, C0, al, be, engine, cplx_=False):
    """C := al op(A) op(B) + be C on device arrays, n^3; sampled binary128 check."""
    C = C0.clone()
    prev = with_engine(gpu, engine)
    try:
        if cplx_:
            gpu.wgemm(ta, tb, n, n, n, al, A.data_ptr(), n, B.data_ptr(), n, be, C.data_ptr(), n)
        else:
            gpu.mgemm(ta, tb, n, n, n, al, A.data_ptr(), n, B.data_ptr(), n, be, C.data_ptr(), n)
        assert gpu.last_error()[0] == 0, gpu.last_error()
        moduli = int(gpu.lib.mwblas_last_ozaki_moduli())
    finally:
        gpu.lib.mwblas_set_gemm_engine(prev)
    rows, cols = rng.integers(0, n, SAMPLES), rng.integers(0, n, SAMPLES)
    hA, hB, hC0 = A.cpu().numpy(), B.cpu().numpy(), C0.cpu().numpy()
    got = C[torch.from_numpy(cols).cuda(), torch.from_numpy(rows).cuda()].cpu().numpy()
    q = oracle.qwgemm if cplx_ else oracle.qgemm
    want = q(ta, tb, n, n, n, al, hA, n, hB, n, be, hC0, n, rows=rows, cols=cols)
    err = orc.normwise_error(got, want, op_norm(al, n, hA, hB, be, hC0))
    return err, moduli


@pytest.fixture(scope="module")
def mats4096():
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(4096)
    return [dev_dd(torch, g, (4096, 4096)) for _ in range(3)]


@pytest.mark.parametrize("engine", ["plain", "ozaki"])
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("N", "T"), ("T", "N"), ("T", "T")])
def test_config1_gemm_4096(gpu, oracle, rng, mats4096, engine, ta, tb):
    import torch
    A, B, C0 = mats4096
    n = 4096
    err, moduli = _sampled_gemm(gpu, oracle, rng, torch, ta, tb, n, A, B, C0, scalar(rng), scalar(rng), engine)
    assert err <= max(10, 4 * n) * orc.EPS_DD, (engine, ta, tb, err)
    assert err <= 1e-30, err
    if engine == "ozaki":
        assert moduli > 0


@pytest.mark.parametrize("engine", ["plain", "ozaki"])
def test_config1_complex_gemm_4096(gpu, oracle, rng, tgen, engine):
    import torch
    n = 4096
    A, B, C0 = (dev_dd(torch, tgen, (n, n), cplx_=True) for _ in range(3))
    err, _ = _sampled_gemm(gpu, oracle, rng, torch, "N", "C", n, A, B, C0, scalar(rng, True), scalar(rng, True),
                           engine, cplx_=True)
    assert err <= max(10, 4 * n) * orc.EPS_DD, (engine, err)
    assert err <= 1e-30, err


@pytest.fixture(scope="module")
def mats8192():
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(8192)
    return [dev_dd(torch, g, (8192, 8192)) for _ in range(3)]


@pytest.mark.parametrize("engine", ["plain", "ozaki"])
def test_config1_2_gemm_8192(gpu, oracle, rng, mats8192, engine):
    import torch
    A, B, C0 = mats8192
    n = 8192
    err, moduli = _sampled_gemm(gpu, oracle, rng, torch, "N", "N", n, A, B, C0, scalar(rng), scalar(rng), engine)
    assert err <= max(10, 4 * n) * orc.EPS_DD, (engine, err)
    assert err <= 1e-30, err
    print(f"{engine} 8192^3: normwise error {err:.2e}, moduli {moduli}")


def test_config2_stress_8192(gpu, oracle, rng, tgen):
    import torch
    n = 8192

    def spread(row_scaled):
        u = torch.rand((n, n), generator=tgen, device="cuda", dtype=torch.float64) * 2 - 1
        mant = torch.where(u < 0, -1.0, 1.0) * (1 + u.abs())
        lo = mant * 2.0 ** -53 * (torch.rand((n, n), generator=tgen, device="cuda", dtype=torch.float64) * 2 - 1)
        hi = mant + lo
        lo = lo - (hi - mant)
        sc = torch.pow(2.0, torch.randint(-30, 31, (n,), generator=tgen, device="cuda").to(torch.float64))
        sc = sc[None, :] if row_scaled else sc[:, None]      # storage [column, row]
        return torch.stack([hi * sc, lo * sc], -1).contiguous()
    A, B = spread(True), spread(False)
    C0 = dev_dd(torch, tgen, (n, n))
    err, moduli = _sampled_gemm(gpu, oracle, rng, torch, "N", "N", n, A, B, C0, scalar(rng), scalar(rng), "ozaki")
    assert err <= max(10, 4 * n) * orc.EPS_DD, err
    assert err <= 1e-30, err
    assert moduli > 0
    print(f"stress 8192^3: normwise error {err:.2e}, moduli {moduli}")


# ---- config 4 ------------------------------------------------------------------------------

def test_config4_syrk_upper_8192_2048(gpu, oracle, rng, tgen):
    import torch
    n, k = 8192, 2048
    A = dev_dd(torch, tgen, (k, n))           # n x k, column-major
    C0 = dev_dd(torch, tgen, (n, n))
    C = C0.clone()
    al, be = scalar(rng), scalar(rng)
    gpu.msyrk("U", "N", n, k, al, A.data_ptr(), n, be, C.data_ptr(), n)
    assert gpu.last_error()[0] == 0, gpu.last_error()
    # the strictly lower triangle is untouched
    low = torch.tril(torch.ones((n, n), dtype=torch.bool, device="cuda"), -1).T    # [col, row]: row > col
    assert torch.equal(C[low], C0[low])
    i = rng.integers(0, n, SAMPLES)
    j = rng.integers(0, n, SAMPLES)
    rows, cols = np.minimum(i, j), np.maximum(i, j)       # upper entries
    hA, hC0 = A.cpu().numpy(), C0.cpu().numpy()
    want = oracle.qgemm("N", "T", n, n, k, al, hA, n, hA, n, be, hC0, n, rows=rows, cols=cols)
    got = C[torch.from_numpy(cols).cuda(), torch.from_numpy(rows).cuda()].cpu().numpy()
    err = orc.normwise_error(got, want, op_norm(al, k, hA, hA, be, hC0))
    assert err <= max(10, 4 * k) * orc.EPS_DD, err


def test_config4_herk_4096_1024(gpu, oracle, rng, tgen):
    import torch
    n, k = 4096, 1024
    A = dev_dd(torch, tgen, (k, n), cplx_=True)
    C0 = dev_dd(torch, tgen, (n, n), cplx_=True)
    C = C0.clone()
    al, be = scalar(rng), scalar(rng)
    gpu.wherk("U", "N", n, k, al, A.data_ptr(), n, be, C.data_ptr(), n)
    assert gpu.last_error()[0] == 0, gpu.last_error()
    d = torch.arange(n, device="cuda")
    assert torch.all(C[d, d, 1] == 0)                       # Im(diag) = 0
    low = torch.tril(torch.ones((n, n), dtype=torch.bool, device="cuda"), -1).T
    assert torch.equal(C[low], C0[low])
    i = rng.integers(0, n, SAMPLES)
    j = rng.integers(0, n, SAMPLES)
    rows, cols = np.minimum(i, j), np.maximum(i, j)
    hA, hC0 = A.cpu().numpy(), C0.cpu().numpy()
    hC0r = hC0.copy()
    hC0r[np.arange(n), np.arange(n), 1] = 0                 # HERK reads Re(c_ii) only
    cal, cbe = np.stack([al, np.zeros(2)]), np.stack([be, np.zeros(2)])
    want = oracle.qwgemm("N", "C", n, n, k, cal, hA, n, hA, n, cbe, hC0r, n, rows=rows, cols=cols)
    want[rows == cols, 1] = 0
    got = C[torch.from_numpy(cols).cuda(), torch.from_numpy(rows).cuda()].cpu().numpy()
    err = orc.normwise_error(got, want, op_norm(al, k, hA, hA, be, hC0))
    assert err <= max(10, 4 * k) * orc.EPS_DD, err


def test_config4_trsm_lln_4096_1024(gpu, oracle, rng, tgen):
    import torch
    m, n = 4096, 1024
    A = dev_dd(torch, tgen, (m, m))
    d = torch.arange(m, device="cuda")
    diag = m * (1 + torch.rand(m, generator=tgen, device="cuda", dtype=torch.float64))   # uniform [n, 2n]
    A[d, d, 0] = diag
    A[d, d, 1] = 0
    B0 = dev_dd(torch, tgen, (n, m))
    B = B0.clone()
    al = scalar(rng)
    gpu.mtrsm("L", "L", "N", "N", m, n, al, A.data_ptr(), m, B.data_ptr(), m)
    assert gpu.last_error()[0] == 0, gpu.last_error()
    pick = np.sort(rng.choice(n, 64, replace=False))
    hA = A.cpu().numpy()
    hB0 = B0.cpu().numpy()
    sub = np.ascontiguousarray(hB0[pick])                  # 64 whole columns
    oracle.qtrsm("L", "L", "N", "N", m, 64, al, hA, m, sub, m)
    got = B[torch.from_numpy(pick).cuda()].cpu().numpy()
    err = orc.normwise_error(got, sub, orc.dd_abs(al) * orc.dd_absmax(hB0))
    assert err <= max(20, 8 * m * m) * orc.EPS_DD, err
    assert err <= 1e-29, err     # strongly dominant: far inside the n^2 bound


def test_config4_gemv_16384(gpu, oracle, rng, tgen):
    import torch
    m = n = 16384
    A = dev_dd(torch, tgen, (n, m))
    x = dev_dd(torch, tgen, (n,))
    y0 = dev_dd(torch, tgen, (m,))
    y = y0.clone()
    al, be = scalar(rng), scalar(rng)
    gpu.mgemv("N", m, n, al, A.data_ptr(), m, x.data_ptr(), 1, be, y.data_ptr(), 1)
    assert gpu.last_error()[0] == 0, gpu.last_error()
    rows = rng.integers(0, m, SAMPLES)
    hA, hx, hy0 = A.cpu().numpy(), x.cpu().numpy(), y0.cpu().numpy()
    want = oracle.qgemm("N", "N", m, 1, n, al, hA, m, hx, n, be, hy0, m, rows=rows, cols=np.zeros_like(rows))
    got = y.cpu().numpy()[rows]
    err = orc.normwise_error(got, want, op_norm(al, n, hA, hx, be, hy0))
    assert err <= max(10, 4 * max(m, n)) * orc.EPS_DD, err


@pytest.fixture(scope="module")
def vecs_2p28():
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(28)
    n = 1 << 28
    return n, dev_dd(torch, g, (n,)), dev_dd(torch, g, (n,))


def test_config4_dot_2p28(gpu, oracle, vecs_2p28):
    n, x, y = vecs_2p28
    got = np.array(gpu.mdot(n, x.data_ptr(), 1, y.data_ptr(), 1))
    assert gpu.last_error()[0] == 0, gpu.last_error()
    hx, hy = x.cpu().numpy(), y.cpu().numpy()
    want = oracle.qdot(n, hx, 1, hy, 1)
    op = n * orc.dd_absmax(hx) * orc.dd_absmax(hy)
    err = orc.normwise_error(got[None], want[None], op)
    assert err <= max(10, 4 * n) * orc.EPS_DD, err


def test_config4_axpy_2p28_bitexact(gpu, oracle, rng, vecs_2p28):
    n, x, y = vecs_2p28
    y = y.clone()
    al = scalar(rng)
    team = 16
    prev = gpu.lib.mwblas_set_l1_partition(team)
    try:
        gpu.maxpy(n, al, x.data_ptr(), 1, y.data_ptr(), 1)
        assert gpu.last_error()[0] == 0, gpu.last_error()
    finally:
        gpu.lib.mwblas_set_l1_partition(prev)
    want = vecs_2p28[2].cpu().numpy()
    oracle.maxpy(n, al, x.cpu().numpy(), 1, want, 1, team=team)
    assert np.array_equal(y.cpu().numpy(), want)
