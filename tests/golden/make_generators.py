"""Generates tests/golden/ref_generators.npz from the reference itself.

Runs in the development container only (it needs the reference sources):
`make -C oracle ref` compiles the reference's mcabs1.cpp, mrotg.cpp,
mrotmg.cpp and wrotg.cpp (src/epblas-parallel/multifloats/) against the
clean-room shim into oracle/_ref/libmwblas_ref.so. Seeded inputs go through
their C ABI; inputs and outputs are saved. Output buffers start filled with a
sentinel so the fixtures also record which outputs each branch leaves alone.

Input distributions: the reference's consistency fuzzers
(test/epblas-parallel/consistency/target_multifloats/fuzz_mrotg.fypp,
fuzz_mrotmg.fypp, fuzz_wrotg.fypp, fuzz_mcabs1.fypp: uniform [-1, 1) and, for
d1/d2 of ROTMG, [0.5, 1.5)) with both limbs random, plus the branch edges
(zero arguments, negative d1 or d2, y1 = 0, scales that drive the ROTMG
rescaling loops).

Usage: python tests/golden/make_generators.py
"""
from __future__ import annotations

import ctypes as C
import importlib.util
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "ref_generators.npz")
REF_MW = os.path.join(ROOT, "oracle", "_ref", "libmwblas_ref.so")
SEED = 20240618
SENTINEL = 7.0


def _load(name, path):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


orc = _load("oracle", os.path.join(ROOT, "oracle", "oracle.py"))


def dd(rng, shape, lo_scale=1.0, low=-1.0, high=1.0):
    hi = rng.uniform(low, high, shape)
    lo = hi * 2.0 ** -53 * rng.uniform(-1.0, 1.0, shape) * lo_scale
    s = hi + lo
    return np.stack([s, lo - (s - hi)], axis=-1)


def inputs(rng):
    n = 200
    z = lambda: np.zeros(2)
    one = np.array([1.0, 0.0])
    cases = {}
    # mrotg: (a, b)
    ab = dd(rng, (n, 2))
    ab[:20, :, 1] = 0.0                                  # the fuzzers' plain doubles
    ab[20] = [z(), one]                                  # a == 0
    ab[21] = [one, z()]                                  # b == 0
    ab[22] = [z(), z()]
    ab[23] = [[-0.75, 0.0], [0.75, 0.0]]                 # |a| == |b|
    ab[24:40] *= 2.0 ** rng.integers(-300, 300, (16, 1, 1))
    cases["mrotg"] = ab
    # mrotmg: (d1, d2, x1, y1)
    r = np.concatenate([dd(rng, (n, 2), low=0.5, high=1.5), dd(rng, (n, 2))], axis=1)
    r[:20, :, 1] = 0.0
    r[20, 0] = [-1.0, 0.0]                               # d1 < 0
    r[21, 3] = z()                                       # y1 == 0: flag -2
    r[22, 1] = z()                                       # d2 == 0
    r[23:35, 1] *= -1.0                                  # d2 < 0 (q2 < 0 or u <= 0)
    r[35:60, 0] *= 2.0 ** rng.integers(-90, 90, (25, 1))  # rescale d1
    r[60:85, 1] *= 2.0 ** rng.integers(-90, 90, (25, 1))  # rescale d2
    r[85:100, 2] *= 2.0 ** rng.integers(-30, 30, (15, 1))
    cases["mrotmg"] = r
    # wrotg: (a, b) complex
    w = dd(rng, (n, 2, 2))
    w[20, 1] = 0.0                                       # b == 0
    w[21, 0] = 0.0                                       # a == 0
    w[22] = 0.0
    w[23:40] *= 2.0 ** rng.integers(-200, 200, (17, 1, 1, 1))
    cases["wrotg"] = w
    # mcabs1: z
    c = dd(rng, (n, 2))
    c[20] = 0.0
    c[21, 0] = 0.0
    cases["mcabs1"] = c
    return cases


def run(fn_of, name, inp):
    """Runs one generator over every case; returns the output buffers."""
    f = fn_of(name)
    p = lambda a: a.ctypes.data
    outs = []
    for x in inp:
        x = np.ascontiguousarray(x, dtype=np.float64)
        if name == "mcabs1":
            r = f(p(x))
            outs.append(np.frombuffer(bytes(r), dtype=np.float64).reshape(1, 2).copy())
        elif name == "mrotg":
            a, b = x[0].copy(), x[1].copy()
            c, s = np.full(2, SENTINEL), np.full(2, SENTINEL)
            f(p(a), p(b), p(c), p(s))
            outs.append(np.stack([a, b, c, s]))
        elif name == "mrotmg":
            d1, d2, x1, y1 = (x[i].copy() for i in range(4))
            par = np.full((5, 2), SENTINEL)
            f(p(d1), p(d2), p(x1), p(y1), p(par))
            outs.append(np.concatenate([np.stack([d1, d2, x1]), par]))
        else:
            a, b = x[0].copy(), x[1].copy()
            c, s = np.full(2, SENTINEL), np.full((2, 2), SENTINEL)
            f(p(a), p(b), p(c), p(s))
            outs.append(np.concatenate([a, c[None], s]))
    return np.stack(outs)


def main():
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True, stdout=subprocess.DEVNULL)
    lib = C.CDLL(REF_MW)

    def fn_of(name):
        f = getattr(lib, name + "_")
        f.restype = orc.DD2 if name == "mcabs1" else None
        return f

    cases = inputs(np.random.default_rng(SEED))
    data = {}
    for name, inp in cases.items():
        data[name + "_in"] = inp
        data[name + "_out"] = run(fn_of, name, inp)
    np.savez_compressed(OUT, **data)
    print("wrote", OUT, {k: v.shape for k, v in data.items()})


if __name__ == "__main__":
    main()
