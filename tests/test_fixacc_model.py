"""CPU model of the fixed-point product path of csrc/fixacc.cuh (no GPU):
the straight-line decode, the alignment shift and the digit products, with
Python integers in place of the 32-bit words, checked against exact rational
arithmetic. It pins the facts the kernels rely on:

* decode_is_fast accepts hi normal and finite with lo zero or 33..64 binades
  below hi, and decode_fast then gives |hi + lo| = W * 2^e exactly, W < 2^118;
* an alignment shift of 118 or more leaves nothing of W (mul_fast clamps the
  shift at 127 instead of testing it);
* the 19 digit products of weight >= 2^72 miss the exact product X' * Y by
  less than 2^98, i.e. below 2^-130 of a block whose products reach 2^232.
"""
import math
import random
import struct
from fractions import Fraction

M32 = 0xFFFFFFFF


def bits(d):
    return struct.unpack("<Q", struct.pack("<d", d))[0]


def decode_is_fast(hi, lo):
    hh, lb = bits(hi) >> 32, bits(lo)
    lh, ll = lb >> 32, lb & M32
    eh, el = (hh >> 20) & 0x7FF, (lh >> 20) & 0x7FF
    lo_zero = ((lh << 1) & M32 | ll) == 0
    gap = (eh - el) & M32
    return ((eh - 1) & M32) < 0x7FE and (lo_zero or (((el - 1) & M32) < 0x7FE and ((gap - 33) & M32) <= 31))


def decode_fast(hi, lo):
    """(W, e, negative) as decode_fast forms them."""
    hb, lb = bits(hi), bits(lo)
    hh, hl, lh, ll = hb >> 32, hb & M32, lb >> 32, lb & M32
    eh, el = (hh >> 20) & 0x7FF, (lh >> 20) & 0x7FF
    lo_zero = ((lh << 1) & M32 | ll) == 0
    gap = (eh - el) & M32
    mh = ((hh & 0xFFFFF) | 0x100000) << 32 | hl            # hi's 53-bit mantissa
    ml = 0 if lo_zero else ((lh & 0xFFFFF) | 0x100000) << 32 | ll
    s = (64 - gap) & 31
    t = (ml << s) & ((1 << 96) - 1)                        # three words t2:t1:t0
    W = mh << 64
    W = W - t if (hh ^ lh) >> 31 else W + t
    return W, eh - 1075 - 64, bool(hh >> 31)


def random_dd(rng, lo_kind):
    hi = rng.uniform(-1, 1) * 2.0 ** rng.randint(-300, 300)
    if lo_kind == "zero":
        return hi, 0.0
    gap = {"normal": rng.randint(53, 60), "edge": rng.choice([33, 64])}[lo_kind]
    lo = math.copysign(rng.uniform(1, 2), rng.choice([-1, 1])) * 2.0 ** (math.frexp(hi)[1] - 1 - gap)
    return hi, lo


def test_fast_decode_is_exact_and_below_2_118():
    rng = random.Random(7)
    for kind in ("zero", "normal", "edge"):
        for _ in range(2000):
            hi, lo = random_dd(rng, kind)
            assert decode_is_fast(hi, lo), (hi, lo)
            W, e, neg = decode_fast(hi, lo)
            assert 0 < W < 1 << 118
            assert Fraction(W) * Fraction(2) ** e == abs(Fraction(hi) + Fraction(lo))
            assert neg == (hi < 0)


def test_fast_decode_rejects_the_general_cases():
    assert not decode_is_fast(0.0, 0.0)                    # zero
    assert not decode_is_fast(float("inf"), 0.0)
    assert not decode_is_fast(1.0, float("nan"))
    assert not decode_is_fast(5e-324, 0.0)                 # subnormal hi
    assert not decode_is_fast(1.0, 2.0 ** -70)             # lo 70 binades below: general path
    assert not decode_is_fast(1.0, 2.0 ** -20)             # lo too close (not normalised)
    assert decode_is_fast(1.0, 2.0 ** -33) and decode_is_fast(1.0, 2.0 ** -64)


def digits24(x):
    return [(x >> (24 * q)) & 0xFFFFFF for q in range(5)]


def test_shift_clamp_and_dropped_digit_products():
    rng = random.Random(11)
    for _ in range(3000):
        X = rng.getrandbits(118)
        Y = rng.getrandbits(118)
        for sh in (118, 120, 127):
            assert X >> sh == 0
        sh = rng.randint(2, 117)
        a, b = digits24(X >> sh), digits24(Y)
        kept = sum(a[s] * b[t] << (24 * (s + t)) for s in range(5) for t in range(5) if s + t >= 3)
        assert sum(1 for s in range(5) for t in range(5) if s + t >= 3) == 19
        exact = (X >> sh) * Y
        assert 0 <= exact - kept < 1 << 98
