"""CPU check of the CRT reconstruction's integer extended-float arithmetic.

epblas-parallel_gb300/csrc/xfloat.cuh is __host__ __device__; this test
compiles it for the host (tests/xfloat_harness.cpp) and compares conversions,
products, sums and the alpha*x + beta*c update with exact rational arithmetic.
"""
import ctypes as C
import os
import subprocess
import tempfile
from fractions import Fraction

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def xf():
    d = tempfile.mkdtemp()
    so = os.path.join(d, "libxf.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", os.path.join(HERE, "xfloat_harness.cpp"),
                    "-o", so], check=True)
    lib = C.CDLL(so)
    D = C.c_double
    P = C.POINTER(D)
    lib.xf_roundtrip.argtypes = [D, D, P, P]
    lib.xf_mul_dd.argtypes = [D, D, D, D, P, P]
    lib.xf_add_dd.argtypes = [D, D, D, D, P, P]
    lib.xf_axpby.argtypes = [D] * 8 + [P, P]
    lib.xw_roundtrip.argtypes = [D, D, P, P]
    lib.xw_mul_dd.argtypes = [D, D, D, D, P, P]
    lib.xw_add_dd.argtypes = [D, D, D, D, P, P]
    lib.xw_axpby.argtypes = [D] * 8 + [P, P]
    return lib


IMPLS = ["xf", "xw"]   # __int128 forms (xfloat.cuh) and 32-bit words (xword.cuh)


def call(f, *args):
    h, l = C.c_double(), C.c_double()
    f(*args, C.byref(h), C.byref(l))
    return h.value, l.value


def dd(rng, scale_exp):
    hi = (rng.random() * 2 - 1) * 2.0 ** scale_exp
    lo = hi * 2.0 ** -53 * (rng.random() * 2 - 1)
    s = hi + lo
    return s, lo - (s - hi)


def exact(h, l):
    return Fraction(h) + Fraction(l)


def normalized(h, l):
    return h + l == h


@pytest.mark.parametrize("impl", IMPLS)
def test_roundtrip_is_exact(xf, impl):
    rng = np.random.default_rng(1)
    cases = [(0.0, 0.0), (1.0, 0.0), (-1.0, 2.0 ** -60), (2.0 ** -1000, 2.0 ** -1060), (3.0, -2.0 ** -52)]
    cases += [dd(rng, int(e)) for e in rng.integers(-300, 300, 500)]
    for h, l in cases:
        oh, ol = call(getattr(xf, impl + "_roundtrip"), h, l)
        assert exact(oh, ol) == exact(h, l) or abs(exact(oh, ol) - exact(h, l)) <= abs(exact(h, l)) * Fraction(2) ** -126
        assert normalized(oh, ol)


@pytest.mark.parametrize("impl", IMPLS)
def test_products(xf, impl):
    rng = np.random.default_rng(2)
    for _ in range(1000):
        a = dd(rng, int(rng.integers(-100, 100)))
        b = dd(rng, int(rng.integers(-100, 100)))
        oh, ol = call(getattr(xf, impl + "_mul_dd"), *a, *b)
        ex = exact(*a) * exact(*b)
        assert abs(exact(oh, ol) - ex) <= abs(ex) * Fraction(2) ** -105, (a, b)
        assert normalized(oh, ol)


@pytest.mark.parametrize("impl", IMPLS)
def test_sums_including_cancellation(xf, impl):
    rng = np.random.default_rng(3)
    for t in range(1000):
        a = dd(rng, int(rng.integers(-60, 60)))
        if t % 3 == 0:
            b = (-a[0], -a[1] * 0.5)            # heavy cancellation
        else:
            b = dd(rng, int(rng.integers(-60, 60)))
        oh, ol = call(getattr(xf, impl + "_add_dd"), *a, *b)
        ex = exact(*a) + exact(*b)
        scale = max(abs(exact(*a)), abs(exact(*b)))
        assert abs(exact(oh, ol) - ex) <= scale * Fraction(2) ** -105 + abs(ex) * Fraction(2) ** -105
        assert normalized(oh, ol)


@pytest.mark.parametrize("impl", IMPLS)
def test_alpha_x_plus_beta_c(xf, impl):
    rng = np.random.default_rng(4)
    for _ in range(500):
        al, x, be, c = (dd(rng, int(rng.integers(-40, 40))) for _ in range(4))
        oh, ol = call(getattr(xf, impl + "_axpby"), *al, *x, *be, *c)
        ex = exact(*al) * exact(*x) + exact(*be) * exact(*c)
        scale = abs(exact(*al) * exact(*x)) + abs(exact(*be) * exact(*c))
        assert abs(exact(oh, ol) - ex) <= scale * Fraction(2) ** -104


def _moduli(need_bits):
    """Greedy pairwise-coprime moduli from 361 downwards (as the engine picks them)."""
    from math import gcd, log2
    ps, have = [], 0.0
    for c in range(361, 2, -1):
        if have >= need_bits:
            break
        if all(gcd(c, q) == 1 for q in ps):
            ps.append(c)
            have += log2(c)
    return ps


@pytest.mark.parametrize("impl", ["crt_frac", "crt_frac_xw"])
@pytest.mark.parametrize("nmod_bits", [120, 180, 237, 300])
def test_crt_fraction_reconstruction(xf, nmod_bits, impl):
    """X from its residues: within M * 2^-140 absolute and 2^-104 relative.

    |X| <= M / 64, the headroom the engine keeps (it asks for 4 bits beyond
    the product bound plus the sign bit)."""
    fn = getattr(xf, impl)
    fn.argtypes = [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int,
                   C.POINTER(C.c_double), C.POINTER(C.c_double)]
    ps = _moduli(nmod_bits)
    M = 1
    for q in ps:
        M *= q
    rng = np.random.default_rng(nmod_bits)
    P = (C.c_int * len(ps))(*ps)
    xs = [0, 1, -1, M // 64, -(M // 64), 2 ** 106 - 1]
    for _ in range(300):
        bits = int(rng.integers(1, M.bit_length() - 7))
        x = int.from_bytes(rng.bytes(48), "little") % (1 << bits)
        xs.append(x if rng.random() < 0.5 else -x)
    for x in xs:
        cs = (C.c_int * len(ps))(*[x % q for q in ps])
        S2 = int(rng.integers(-50, 300))
        h, l = C.c_double(), C.c_double()
        fn(len(ps), P, cs, S2, C.byref(h), C.byref(l))
        got = exact(h.value, l.value)
        want = Fraction(x) / Fraction(2) ** S2
        tol = (abs(Fraction(x)) * Fraction(2) ** -104 + Fraction(M) * Fraction(2) ** -140) / Fraction(2) ** S2
        assert abs(got - want) <= tol, (x, S2, float(got), float(want))


def test_word_and_int128_forms_agree(xf):
    """The 32-bit-word forms (xword.cuh) against the __int128 forms
    (xfloat.cuh) across the exponent range, subnormal results, exact
    cancellation and power-of-two hi limbs with a negative lo."""
    rng = np.random.default_rng(7)
    cases = [((1.0, -2.0 ** -60), (3.0, 0.0)), ((2.0 ** -1070, 0.0), (2.0 ** -3, 0.0)),
             ((2.0 ** 1000, 2.0 ** 940), (2.0 ** 20, -2.0 ** -40)), ((5.0, 2.0 ** -52), (-5.0, -2.0 ** -52))]
    for _ in range(2000):
        a = dd(rng, int(rng.integers(-1000, 1000)))
        b = dd(rng, int(rng.integers(-1000, 1000)) if rng.random() < 0.3 else int(rng.integers(-30, 30)))
        cases.append((a, b))
    for a, b in cases:
        for op in ("mul_dd", "add_dd"):
            ex = exact(*a) * exact(*b) if op == "mul_dd" else exact(*a) + exact(*b)
            if op == "mul_dd" and not (Fraction(2) ** -1000 < abs(ex) < Fraction(2) ** 1000) and ex != 0:
                continue   # outside the range both forms round through FP64 scaling
            r1 = call(getattr(xf, "xf_" + op), *a, *b)
            r2 = call(getattr(xf, "xw_" + op), *a, *b)
            scale = abs(exact(*a) * exact(*b)) if op == "mul_dd" else max(abs(exact(*a)), abs(exact(*b)))
            assert abs(exact(*r1) - exact(*r2)) <= scale * Fraction(2) ** -104, (op, a, b, r1, r2)
            assert normalized(*r2)
        r = call(xf.xw_roundtrip, *a)
        assert r == a or abs(exact(*r) - exact(*a)) <= abs(exact(*a)) * Fraction(2) ** -126
