"""Complex dots, sums of magnitudes, norms, complex AXPY and plane rotations
on the GPU, through the C ABI.

Expected values are binary128 products of the binary128 oracle GEMM
(or_qgemm / or_qwgemm): a dot is a 1 x 1 product over n, a rotation or an
AXPY an n x 1 product over the two stacked vectors. Tolerances and the error
metric are the reference's (fuzz_wdotc.fypp:44 and fuzz_waxpy.fypp:52:
max(10, 4n) * 2^-104; fuzz_masum.fypp:41, fuzz_mnrm2.fypp:41 and
fuzz_mrot.fypp:51: max(20, 8n) * 2^-104, relative to the largest reference
value). Quick returns follow masum.cpp:119, mnrm2.cpp:182-183,
waxpy.cpp:101 and mrotm.cpp:200.
"""
from decimal import Decimal, getcontext

import numpy as np
import pytest

from conftest import mwb, orc

pytestmark = pytest.mark.gpu

NS = [1, 2, 7, 100, 4099, 100003]
INCS = [1, 3, -2]
ONE_C = np.array([[1.0, 0.0], [0.0, 0.0]])
ZERO_C = np.zeros((2, 2))


def vec(rng, n, inc, cplx_):
    span = 1 + (n - 1) * abs(inc) if n > 0 else 1
    return mwb.random_cdd(rng, (span,)) if cplx_ else mwb.random_dd(rng, (span,))


def gather(v, n, inc):
    """The n logical elements in BLAS order (negative inc walks backwards)."""
    idx = np.arange(n) * inc if inc >= 0 else (n - 1 - np.arange(n)) * (-inc)
    return np.ascontiguousarray(v[idx])


def dd_mag(x):
    """|x| of double-double values (sign of the hi limb flips both limbs)."""
    s = np.where(x[..., :1] < 0, -1.0, 1.0)
    return np.ascontiguousarray(x * s)


def rel_err(got, want):
    d = float(np.max(orc.dd_diff_abs(got, want)))
    m = orc.dd_absmax(want)
    return d / m if m > 0 else d


@pytest.mark.parametrize("name", ["wdotu", "wdotc"])
def test_complex_dots(gpu, oracle, rng, name):
    for n in NS:
        for ix, iy in [(1, 1), (2, -3)]:
            x, y = vec(rng, n, ix, True), vec(rng, n, iy, True)
            gx, gy = gather(x, n, ix), gather(y, n, iy)
            want = oracle.qwgemm("C" if name == "wdotc" else "T", "N", 1, 1, n, ONE_C, gx, n, gy, n, ZERO_C,
                                 np.zeros((1, 1, 2, 2)), 1)[0, 0]
            got = gpu.cdot(name, n, x, ix, y, iy)
            assert gpu.last_error()[0] == 0, gpu.last_error()
            scale = n * orc.dd_absmax(gx) * orc.dd_absmax(gy)
            err = float(np.max(orc.dd_diff_abs(got, want))) / max(orc.dd_absmax(want), scale)
            assert err <= max(10, 4 * n) * orc.EPS_DD, (n, ix, iy, err)
    assert np.array_equal(gpu.cdot(name, 0, x, 1, y, 1), np.zeros((2, 2)))


@pytest.mark.parametrize("name", ["masum", "mwasum"])
def test_sums_of_magnitudes(gpu, oracle, rng, name):
    cplx_ = name == "mwasum"
    for n in NS:
        for inc in [1, 3]:
            x = vec(rng, n, inc, cplx_)
            gx = dd_mag(gather(x, n, inc)).reshape(-1, 2)      # complex: re and im as 2n reals
            m = gx.shape[0]
            ones = np.tile(np.array([1.0, 0.0]), (m, 1))
            want = oracle.qgemm("T", "N", 1, 1, m, np.array([1.0, 0.0]), gx[None], m, ones[None], m,
                                np.zeros(2), np.zeros((1, 1, 2)), 1)[0, 0]
            got = gpu.vnorm(name, n, x, inc)
            assert gpu.last_error()[0] == 0, gpu.last_error()
            assert rel_err(got[None], want[None]) <= max(20, 8 * n) * orc.EPS_DD, (n, inc)
    x = vec(rng, 5, 1, cplx_)
    assert np.array_equal(gpu.vnorm(name, 5, x, -1), np.zeros(2))   # incx < 1 returns 0
    assert np.array_equal(gpu.vnorm(name, 0, x, 1), np.zeros(2))


def dd_sqrt(v):
    """sqrt of a double-double to ~34 digits (decimal), back to double-double."""
    getcontext().prec = 60
    s = (Decimal(float(v[0])) + Decimal(float(v[1]))).sqrt()
    hi = float(s)
    lo = float(s - Decimal(hi))
    return np.array([hi, lo])


@pytest.mark.parametrize("name", ["mnrm2", "mwnrm2"])
@pytest.mark.parametrize("scale_exp", [0, 700, -700])
def test_norms(gpu, oracle, rng, name, scale_exp):
    """Including magnitudes whose squares leave the double range."""
    cplx_ = name == "mwnrm2"
    for n in [1, 2, 100, 4099, 100003]:
        x = vec(rng, n, 2, cplx_) * 2.0 ** scale_exp
        gx = gather(x, n, 2).reshape(-1, 2) * 2.0 ** -scale_exp      # square in range, scale back after
        m = gx.shape[0]
        ss = oracle.qgemm("T", "N", 1, 1, m, np.array([1.0, 0.0]), gx[None], m, gx[None], m, np.zeros(2),
                          np.zeros((1, 1, 2)), 1)[0, 0]
        want = dd_sqrt(ss) * 2.0 ** scale_exp
        got = gpu.vnorm(name, n, x, 2)
        assert gpu.last_error()[0] == 0, gpu.last_error()
        assert rel_err(got[None], want[None]) <= max(20, 8 * n) * orc.EPS_DD, (n, scale_exp, got, want)
    x = mwb.random_dd(rng, (1,))
    x[0] = -np.abs(x[0])
    assert np.array_equal(gpu.vnorm("mnrm2", 1, x, 1), -x[0])          # mnrm2.cpp:183: |x(1)| exactly


def test_waxpy(gpu, oracle, rng):
    for n in NS:
        for ix, iy in [(1, 1), (3, -2)]:
            x, y = vec(rng, n, ix, True), vec(rng, n, iy, True)
            al = mwb.random_cdd(rng, ())
            gx, gy = gather(x, n, ix), gather(y, n, iy)
            XY = np.ascontiguousarray(np.stack([gx, gy]))          # n x 2, columns x, y
            coef = np.ascontiguousarray(np.stack([al, ONE_C])[:, None])   # 2 x 1
            want = oracle.qwgemm("N", "N", n, 1, 2, ONE_C, XY, n, coef, 2, ZERO_C, np.zeros((1, n, 2, 2)), n)[0]
            got = y.copy()
            gpu.waxpy(n, al, x, ix, got, iy)
            assert gpu.last_error()[0] == 0, gpu.last_error()
            assert rel_err(gather(got, n, iy), want) <= max(10, 4 * n) * orc.EPS_DD, (n, ix, iy)
    y = vec(rng, 5, 1, True)
    got = y.copy()
    gpu.waxpy(5, ZERO_C, y, 1, got, 1)                               # waxpy.cpp:101: alpha == 0
    assert np.array_equal(got, y)


@pytest.mark.parametrize("name", ["mrot", "wmrot", "mrotm"])
def test_rotations(gpu, oracle, rng, name):
    cplx_ = name == "wmrot"
    for n in NS[:5]:
        for ix, iy in [(1, 1), (2, -3)]:
            x, y = vec(rng, n, ix, cplx_), vec(rng, n, iy, cplx_)
            gx = gather(x, n, ix).reshape(n, -1, 2)
            gy = gather(y, n, iy).reshape(n, -1, 2)
            if name == "mrotm":
                flag = float(rng.choice([-1.0, 0.0, 1.0]))
                h = mwb.random_dd(rng, (4,))                          # h11, h21, h12, h22
                param = np.concatenate([[[flag, 0.0]], h])
                h11, h21, h12, h22 = h
                if flag == 0.0:
                    h11 = h22 = np.array([1.0, 0.0])
                elif flag == 1.0:
                    h12, h21 = np.array([1.0, 0.0]), np.array([-1.0, 0.0])
            else:
                c, s = mwb.random_dd(rng, ()), mwb.random_dd(rng, ())
                h11, h12, h21, h22 = c, s, -s, c
            wx = np.empty_like(gx)
            wy = np.empty_like(gy)
            for comp in range(gx.shape[1]):
                XY = np.ascontiguousarray(np.stack([gx[:, comp], gy[:, comp]]))   # n x 2
                for out, (a, b) in ((wx, (h11, h12)), (wy, (h21, h22))):
                    coef = np.ascontiguousarray(np.stack([a, b])[:, None])
                    out[:, comp] = oracle.qgemm("N", "N", n, 1, 2, np.array([1.0, 0.0]), XY, n, coef, 2,
                                                np.zeros(2), np.zeros((1, n, 2)), n)[0]
            gotx, goty = x.copy(), y.copy()
            if name == "mrotm":
                gpu.rotm(n, gotx, ix, goty, iy, param)
            else:
                gpu.rot(name, n, gotx, ix, goty, iy, c, s)
            assert gpu.last_error()[0] == 0, gpu.last_error()
            tol = max(20, 8 * n) * orc.EPS_DD
            assert rel_err(gather(gotx, n, ix).reshape(n, -1, 2), wx) <= tol, (n, ix, iy)
            assert rel_err(gather(goty, n, iy).reshape(n, -1, 2), wy) <= tol, (n, ix, iy)
    if name == "mrotm":
        x, y = vec(rng, 9, 1, False), vec(rng, 9, 1, False)
        gx, gy = x.copy(), y.copy()
        gpu.rotm(9, gx, 1, gy, 1, np.concatenate([[[-2.0, 0.0]], mwb.random_dd(rng, (4,))]))   # identity
        assert np.array_equal(gx, x) and np.array_equal(gy, y)


def _generator_fixtures():
    import importlib.util
    import os
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "make_generators.py")
    spec = importlib.util.spec_from_file_location("make_generators", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod, np.load(path.replace("make_generators.py", "ref_generators.npz"))


@pytest.mark.parametrize("wide", [False, True])
@pytest.mark.parametrize("name", ["mcabs1", "mrotg", "mrotmg", "wrotg"])
def test_generators_bitexact(gpu, name, wide):
    """mcabs1 / mrotg / mrotmg / wrotg on the device reproduce the reference's
    own outputs (tests/golden/ref_generators.npz) bit for bit, including the
    outputs each branch leaves untouched (sentinel values)."""
    mg, z = _generator_fixtures()
    got = mg.run(lambda n: getattr(gpu.lib, n + ("_64_" if wide else "_")), name, z[name + "_in"])
    assert gpu.last_error()[0] == 0, gpu.last_error()
    want = z[name + "_out"]
    bad = np.nonzero((got.view(np.uint64) != want.view(np.uint64)).reshape(len(got), -1).any(axis=1))[0]
    assert bad.size == 0, (bad[:8], got[bad[:2]], want[bad[:2]])
