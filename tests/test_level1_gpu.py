"""Level-1 parity on the GPU, through the C ABI.

SCAL/AXPY (real and complex) and COPY/SWAP/I*AMAX are bit-exact to the
reference: the oracle's restatement (pinned to the reference's own outputs in
test_oracle_pin.py) is the expectation, for every OpenMP team size the
reference could have run with. DOT is a floating-point reduction: its
normwise error against the binary128 oracle must stay inside the reference's
fuzz tolerance max(10, 4n) * 2^-104 (fuzz_mdot.fypp).
"""
import numpy as np
import pytest

from conftest import mwb, orc

pytestmark = pytest.mark.gpu

NS = [1, 2, 3, 4, 5, 7, 8, 31, 1000, 2048, 2049, 4099, 100003]
INCS = [1, 2, -1, -3]


def vec(rng, n, inc, cplx_=False):
    span = 1 + (n - 1) * abs(inc) if n > 0 else 1
    return mwb.random_cdd(rng, (span,)) if cplx_ else mwb.random_dd(rng, (span,))


@pytest.mark.parametrize("team", [1, 3, 8, 72])
def test_mscal_wscal_wmscal_bitexact(gpu, oracle, rng, team):
    gpu.lib.mwblas_set_l1_partition(team)
    try:
        for n in NS:
            for inc in INCS:
                if inc != 1 and n > 5000:
                    continue
                t = team if (inc == 1 and n > 2048) else 1
                a = mwb.random_dd(rng, ())
                x = vec(rng, n, inc)
                want = x.copy(); oracle.mscal(n, a, want, inc, team=t)
                got = x.copy(); gpu.mscal(n, a, got, inc)
                assert gpu.last_error()[0] == 0
                np.testing.assert_array_equal(got, want, err_msg=f"mscal n={n} inc={inc} team={team}")
                ca = mwb.random_cdd(rng, ())
                cx = vec(rng, n, inc, True)
                want = cx.copy(); oracle.wscal(n, ca, want, inc, team=t)
                got = cx.copy(); gpu.wscal(n, ca, got, inc)
                np.testing.assert_array_equal(got, want, err_msg=f"wscal n={n} inc={inc} team={team}")
                want = cx.copy(); oracle.wmscal(n, a, want, inc, team=t)
                got = cx.copy(); gpu.wmscal(n, a, got, inc)
                np.testing.assert_array_equal(got, want, err_msg=f"wmscal n={n} inc={inc} team={team}")
    finally:
        gpu.lib.mwblas_set_l1_partition(0)


@pytest.mark.parametrize("team", [1, 8])
def test_maxpy_bitexact(gpu, oracle, rng, team):
    gpu.lib.mwblas_set_l1_partition(team)
    try:
        for n in NS:
            for incx, incy in [(1, 1), (2, 1), (1, -2), (-1, -1), (3, 2)]:
                if (incx, incy) != (1, 1) and n > 5000:
                    continue
                t = team if (incx == 1 and incy == 1 and n > 2048) else 1
                a = mwb.random_dd(rng, ())
                x = vec(rng, n, incx)
                y = vec(rng, n, incy)
                want = y.copy(); oracle.maxpy(n, a, x, incx, want, incy, team=t)
                got = y.copy(); gpu.maxpy(n, a, x, incx, got, incy)
                np.testing.assert_array_equal(got, want, err_msg=f"maxpy n={n} incs={incx},{incy}")
    finally:
        gpu.lib.mwblas_set_l1_partition(0)


def test_zero_increment_sequential_semantics(gpu, oracle, rng):
    """inc == 0 makes the reference loop sequential; the GPU repeats it exactly."""
    a = mwb.random_dd(rng, ())
    x = vec(rng, 1, 1)
    want = x.copy(); oracle.mscal(5, a, want, 0)
    got = x.copy(); gpu.mscal(5, a, got, 0)
    np.testing.assert_array_equal(got, want)
    xs = vec(rng, 6, 1)
    y = vec(rng, 1, 1)
    want = y.copy(); oracle.maxpy(6, a, xs, 1, want, 0)
    got = y.copy(); gpu.maxpy(6, a, xs, 1, got, 0)
    np.testing.assert_array_equal(got, want)
    # swap with a zero increment rotates through the sequence
    x1 = vec(rng, 1, 1); y1 = vec(rng, 4, 1)
    wx, wy = x1.copy(), y1.copy(); oracle.swap(4, wx, 0, wy, 1)
    gx, gy = x1.copy(), y1.copy(); gpu.mswap(4, gx, 0, gy, 1)
    np.testing.assert_array_equal(gx, wx); np.testing.assert_array_equal(gy, wy)


@pytest.mark.parametrize("cplx_", [False, True])
def test_copy_swap_bitexact(gpu, oracle, rng, cplx_):
    elem = 2 if cplx_ else 1
    for n in [1, 5, 33, 4099]:
        for incx, incy in [(1, 1), (2, -1), (-3, 2), (1, 0)]:
            x = vec(rng, n, incx, cplx_)
            y = vec(rng, n, incy, cplx_)
            wy = y.copy(); oracle.copy(n, x, incx, wy, incy, elem)
            gy = y.copy(); gpu.mcopy(n, x, incx, gy, incy, cplx_=cplx_)
            np.testing.assert_array_equal(gy, wy, err_msg=f"copy n={n} {incx},{incy}")
            if incy == 0:
                continue
            wx, wy = x.copy(), y.copy(); oracle.swap(n, wx, incx, wy, incy, elem)
            gx, gy = x.copy(), y.copy(); gpu.mswap(n, gx, incx, gy, incy, cplx_=cplx_)
            np.testing.assert_array_equal(gx, wx)
            np.testing.assert_array_equal(gy, wy)


def test_amax_exact_index(gpu, oracle, rng):
    for n in [3, 17, 256, 1000, 65537, 1 << 20]:
        for inc in (1, 2):
            x = vec(rng, n, inc)
            # plant exact ties and a lo-limb tie-break
            pos = np.sort(rng.choice(n, size=3, replace=False)) * inc
            x[pos[0]] = (3.0, 0.0)
            x[pos[1]] = (-3.0, 0.0)
            x[pos[2]] = (3.0, 0.0)
            assert gpu.imamax(n, x, inc) == oracle.imamax(n, x, inc) == pos[0] // inc + 1
            x[pos[2], 1] = 2.0 ** -55
            assert gpu.imamax(n, x, inc) == oracle.imamax(n, x, inc) == pos[2] // inc + 1
            cx = vec(rng, n, inc, True)
            assert gpu.imamax(n, cx, inc, cplx_=True) == oracle.iwamax(n, cx, inc)


def test_amax_special_values(gpu, oracle, rng):
    """Signed zeros tie, infinities and the lo limb order as FP64 '>' does, and
    a NaN never beats a number (the reference's -inf-seeded vector scan,
    imamax.cpp:88-131, used for unit stride and n >= 8)."""
    for n in [64, 4099, 100003]:
        x = vec(rng, n, 1)
        p = np.sort(rng.choice(n, size=6, replace=False))
        x[p[0]] = (7.0, -0.0)
        x[p[1]] = (-7.0, 0.0)          # magnitude (7, -0): ties with p[0]
        assert gpu.imamax(n, x, 1) == oracle.imamax(n, x, 1) == p[0] + 1
        x[p[2]] = (-7.0, -2.0 ** -60)  # magnitude (7, +2^-60) wins
        assert gpu.imamax(n, x, 1) == oracle.imamax(n, x, 1) == p[2] + 1
        x[p[3]] = (-np.inf, 0.0)
        x[p[4]] = (np.inf, 0.0)
        assert gpu.imamax(n, x, 1) == oracle.imamax(n, x, 1) == p[3] + 1
        y = vec(rng, n, 1)
        y[0] = (np.nan, 0.0)
        y[p[5]] = (np.nan, np.nan)
        clean = y.copy()
        clean[0] = clean[p[5]] = (0.0, 0.0)
        assert gpu.imamax(n, y, 1) == oracle.imamax(n, clean, 1)
        allnan = np.full((n, 2), np.nan)
        assert gpu.imamax(n, allnan, 1) == 1


def test_misaligned_device_operands_are_staged(gpu, oracle, rng):
    """A device array that is only 8-byte aligned is copied to an aligned
    buffer (and back when written) instead of being read with 16-byte loads."""
    import torch
    n = 3001
    x = mwb.random_dd(rng, (n,))
    y = mwb.random_dd(rng, (n,))
    a = mwb.random_dd(rng, ())
    buf = torch.zeros(4 * n + 8, dtype=torch.float64, device="cuda")
    xd = buf[1:1 + 2 * n]
    yd = buf[2 * n + 3:2 * n + 3 + 2 * n]
    assert xd.data_ptr() % 16 == 8 and yd.data_ptr() % 16 == 8
    xd.copy_(torch.from_numpy(x.reshape(-1)))
    yd.copy_(torch.from_numpy(y.reshape(-1)))
    want = y.copy(); oracle.maxpy(n, a, x, 1, want, 1, team=1)
    gpu.lib.mwblas_set_l1_partition(1)
    try:
        gpu.maxpy(n, a, xd.data_ptr(), 1, yd.data_ptr(), 1)
    finally:
        gpu.lib.mwblas_set_l1_partition(0)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(yd.cpu().numpy().reshape(n, 2), want)
    assert gpu.imamax(n, xd.data_ptr(), 1) == oracle.imamax(n, x, 1)
    m = k = 40
    A = mwb.random_dd(rng, (k, m))
    B = mwb.random_dd(rng, (k, m))
    Ad = torch.zeros(2 * m * k + 1, dtype=torch.float64, device="cuda")[1:]
    Ad.copy_(torch.from_numpy(A.reshape(-1)))
    C1 = np.zeros((m, m, 2)); C2 = np.zeros((m, m, 2))
    gpu.mgemm("N", "N", m, m, k, (1.0, 0.0), A, m, B, k, (0.0, 0.0), C1, m)
    gpu.mgemm("N", "N", m, m, k, (1.0, 0.0), Ad.data_ptr(), m, B, k, (0.0, 0.0), C2, m)
    np.testing.assert_array_equal(C1, C2)


def test_golden_amax_and_level1(gpu, golden):
    """The reference's own outputs from the golden fixtures, team 1."""
    z, meta = golden
    gpu.lib.mwblas_set_l1_partition(1)
    try:
        for ci, (n, inc) in enumerate(meta["l1_cases"]):
            x = z[f"l1_{ci}_x"].copy()
            gpu.mscal(n, z[f"l1_{ci}_alpha"], x, inc)
            np.testing.assert_array_equal(x, z[f"t1_mscal_{ci}"])
            y = z[f"l1_{ci}_y"].copy()
            gpu.maxpy(n, z[f"l1_{ci}_alpha"], z[f"l1_{ci}_x"], inc, y, inc)
            np.testing.assert_array_equal(y, z[f"t1_maxpy_{ci}"])
    finally:
        gpu.lib.mwblas_set_l1_partition(0)
    for c in meta["l3"]:
        if c["kind"] == "amax":
            k = c["key"]
            assert gpu.imamax(c["n"], z[k + "_x"], 1) == int(z[k + "_ref"][0])
            assert gpu.imamax(c["n"], z[k + "_cx"], 1, cplx_=True) == int(z[k + "_ref"][1])


def test_dot_within_tolerance(gpu, oracle, rng, golden):
    for n in [1, 2, 5, 100, 4097, 1 << 20]:
        for incx, incy in [(1, 1), (2, -1)]:
            x = vec(rng, n, incx)
            y = vec(rng, n, incy)
            got = np.array(gpu.mdot(n, x, incx, y, incy))
            want = oracle.qdot(n, x, incx, y, incy)
            op = n * orc.dd_absmax(x) * orc.dd_absmax(y)
            err = orc.normwise_error(got[None], want[None], op)
            assert err <= max(10, 4 * n) * orc.EPS_DD, (n, err)
    z, meta = golden
    for c in meta["l3"]:
        if c["kind"] == "dot":
            k = c["key"]
            got = np.array(gpu.mdot(c["n"], z[k + "_x"], 1, z[k + "_y"], 1))
            op = c["n"] * orc.dd_absmax(z[k + "_x"]) * orc.dd_absmax(z[k + "_y"])
            assert orc.normwise_error(got[None], z[k + "_q"][None], op) <= max(10, 4 * c["n"]) * orc.EPS_DD


def test_dot_exponent_range_cancellation_and_nonfinite(gpu, oracle, rng):
    """Products spanning 2^-600..2^600, exact cancellation, and non-finite inputs."""
    n = 3001
    x = vec(rng, n, 1)
    y = vec(rng, n, 1)
    sc = 2.0 ** rng.integers(-300, 300, n)
    x *= sc[:, None]
    y *= (2.0 ** rng.integers(-300, 300, n))[:, None]
    got = np.array(gpu.mdot(n, x, 1, y, 1))
    want = oracle.qdot(n, x, 1, y, 1)
    # normwise against n * max|x| * max|y|, and relative to the largest product
    op = n * orc.dd_absmax(x) * orc.dd_absmax(y)
    assert orc.normwise_error(got[None], want[None], op) <= max(10, 4 * n) * orc.EPS_DD
    pmax = np.max(np.abs(x[:, 0] * y[:, 0]))
    assert orc.normwise_error(got[None], want[None], pmax) <= 8 * orc.EPS_DD
    # x . [y, -y] over [x, x] cancels: what is left is far below the largest product
    xx = np.concatenate([x, x])
    yy = np.concatenate([y, -y])
    r = gpu.mdot(2 * n, xx, 1, yy, 1)
    assert abs(r[0]) <= orc.EPS_DD * pmax, (r, pmax)
    # a single non-finite element makes the result NaN
    for bad in (np.inf, -np.inf, np.nan):
        xb = x.copy()
        xb[n // 2] = (bad, 0.0)
        r = gpu.mdot(n, xb, 1, y, 1)
        assert np.isnan(r[0]), (bad, r)


def test_device_pointer_path_matches_host_path(gpu, oracle, rng):
    """Device-resident arrays are used in place (no staging) with the same bits."""
    import torch
    n = 50001
    a = mwb.random_dd(rng, ())
    x = mwb.random_dd(rng, (n,))
    y = mwb.random_dd(rng, (n,))
    gpu.lib.mwblas_set_l1_partition(1)
    try:
        want = y.copy(); oracle.maxpy(n, a, x, 1, want, 1, team=1)
        xd = torch.from_numpy(x).cuda()
        yd = torch.from_numpy(y).cuda()
        gpu.maxpy(n, a, xd.data_ptr(), 1, yd.data_ptr(), 1)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(yd.cpu().numpy(), want)
        assert gpu.imamax(n, xd.data_ptr(), 1) == oracle.imamax(n, x, 1)
    finally:
        gpu.lib.mwblas_set_l1_partition(0)


def test_injected_allocation_failure_is_reported(gpu, rng):
    """A failed device allocation surfaces as MWBLAS_ERR_ALLOC, outputs untouched."""
    x = mwb.random_dd(rng, (1000,))
    keep = x.copy()
    gpu.lib.mwblas_debug_fail_alloc_after(0)
    gpu.mscal(1000, 2.0, x, 1)
    code, msg = gpu.last_error()
    gpu.lib.mwblas_debug_fail_alloc_after(-1)
    assert code == -2 and "alloc" in msg
    np.testing.assert_array_equal(x, keep)
    gpu.mscal(1000, 2.0, x, 1)     # and the library keeps working
    assert gpu.last_error()[0] == 0
