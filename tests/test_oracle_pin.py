"""Pins the CPU oracle against the reference's own outputs (no GPU).

The golden fixtures hold outputs of the reference's double-double sources and
of its kind16 binary128 routines on seeded inputs (tests/golden/make_golden.py).
The oracle's bit-exact restatements must reproduce the former bit for bit; its
binary128 routines must agree with the latter to binary128 rounding level.
"""
import json
import os

import numpy as np
import pytest

from conftest import ROOT, orc, ref_library


def l1_case(z, meta, ci):
    return tuple(meta["l1_cases"][ci])


@pytest.mark.parametrize("team", [1, 3, 8])
def test_bitexact_level1_matches_reference(oracle, golden, team):
    z, meta = golden
    for ci, (n, inc) in enumerate(meta["l1_cases"]):
        t = team if inc == 1 else 1
        alpha, calpha = z[f"l1_{ci}_alpha"], z[f"l1_{ci}_calpha"]
        x = z[f"l1_{ci}_x"].copy()
        oracle.mscal(n, alpha, x, inc, team=t if n > 2048 else 1)
        np.testing.assert_array_equal(x, z[f"t{team}_mscal_{ci}"], err_msg=f"mscal n={n} inc={inc}")
        cx = z[f"l1_{ci}_cx"].copy()
        oracle.wscal(n, calpha, cx, inc, team=t if n > 2048 else 1)
        np.testing.assert_array_equal(cx, z[f"t{team}_wscal_{ci}"], err_msg=f"wscal n={n} inc={inc}")
        cx = z[f"l1_{ci}_cx"].copy()
        oracle.wmscal(n, alpha, cx, inc, team=t if n > 2048 else 1)
        np.testing.assert_array_equal(cx, z[f"t{team}_wmscal_{ci}"], err_msg=f"wmscal n={n} inc={inc}")
        y = z[f"l1_{ci}_y"].copy()
        oracle.maxpy(n, alpha, z[f"l1_{ci}_x"], inc, y, inc, team=t if n > 2048 else 1)
        np.testing.assert_array_equal(y, z[f"t{team}_maxpy_{ci}"], err_msg=f"maxpy n={n} inc={inc}")


def test_dot_port_matches_reference(oracle, golden):
    """The port of mdot (per-slice Bailey accumulator, tid-order merge) is bit-exact."""
    z, meta = golden
    for team in meta["teams"]:
        for ci, (n, inc) in enumerate(meta["l1_cases"]):
            key = f"t{team}_mdot_{ci}"
            if key not in z.files:
                continue
            t = team if n > 8192 else 1   # MDOT_OMP_MIN
            got = oracle.port_mdot(n, z[f"l1_{ci}_x"], z[f"l1_{ci}_y"], t)
            np.testing.assert_array_equal(got, z[key], err_msg=f"mdot n={n} team={team}")


def test_amax_matches_reference(oracle, golden):
    z, meta = golden
    for c in meta["l3"]:
        if c["kind"] != "amax":
            continue
        k, n = c["key"], c["n"]
        assert oracle.imamax(n, z[k + "_x"], 1) == int(z[k + "_ref"][0])
        assert oracle.iwamax(n, z[k + "_cx"], 1) == int(z[k + "_ref"][1])


def _qclose(a, b, rel=2.0 ** -100):
    a = np.asarray(a); b = np.asarray(b)
    scale = max(float(np.max(np.abs(b[..., 0]))), 1e-300)
    assert float(np.max(orc.dd_diff_abs(a, b))) <= rel * scale


def test_binary128_oracle_matches_kind16(oracle, golden):
    z, meta = golden
    for c in meta["l3"]:
        k = c["key"]
        if c["kind"] == "gemm":
            out = oracle.qgemm(c["ta"], c["tb"], c["m"], c["n"], c["k"], z[k + "_alpha"], z[k + "_A"], c["lda"],
                               z[k + "_B"], c["ldb"], z[k + "_beta"], z[k + "_C"].copy(), c["ldc"])
            _qclose(out[:, :c["m"]], z[k + "_q"][:, :c["m"]])
        elif c["kind"] == "wgemm":
            out = oracle.qwgemm(c["ta"], c["tb"], c["m"], c["n"], c["k"], z[k + "_alpha"], z[k + "_A"], c["lda"],
                                z[k + "_B"], c["ldb"], z[k + "_beta"], z[k + "_C"].copy(), c["ldc"])
            _qclose(out[:, :c["m"]], z[k + "_q"][:, :c["m"]])
        elif c["kind"] == "syrk":
            out = z[k + "_C"].copy()
            oracle.qsyrk(c["uplo"], c["trans"], c["n"], c["k"], z[k + "_alpha"], z[k + "_A"], c["lda"],
                         z[k + "_beta"], out, c["ldc"])
            _qclose(out, z[k + "_q"])
        elif c["kind"] == "herk":
            out = z[k + "_C"].copy()
            oracle.qherk(c["uplo"], c["trans"], c["n"], c["k"], z[k + "_alpha"], z[k + "_A"], c["lda"],
                         z[k + "_beta"], out, c["ldc"])
            _qclose(out, z[k + "_q"])
        elif c["kind"] == "trsm":
            out = z[k + "_B"].copy()
            oracle.qtrsm(c["side"], c["uplo"], c["ta"], c["diag"], c["m"], c["n"], z[k + "_alpha"], z[k + "_A"],
                         c["lda"], out, c["ldb"])
            _qclose(out, z[k + "_q"], rel=2.0 ** -96)
        elif c["kind"] == "gemv":
            out = z[k + "_y"].copy()
            oracle.qgemv(c["trans"], c["m"], c["n"], z[k + "_alpha"], z[k + "_A"], c["lda"], z[k + "_x"],
                         c["incx"], z[k + "_beta"], out, c["incy"])
            _qclose(out, z[k + "_q"])
        elif c["kind"] == "dot":
            out = oracle.qdot(c["n"], z[k + "_x"], 1, z[k + "_y"], 1)
            _qclose(out, z[k + "_q"])


def test_reference_outputs_within_their_own_tolerance(golden):
    """The reference's DD results sit inside the fuzz tolerance of the quad result."""
    z, meta = golden
    for c in meta["l3"]:
        k = c["key"]
        if c["kind"] in ("gemm", "wgemm"):
            A, B, C0 = z[k + "_A"], z[k + "_B"], z[k + "_C"]
            op = orc.dd_abs(z[k + "_alpha"]) * c["k"] * orc.dd_absmax(A) * orc.dd_absmax(B) \
                + orc.dd_abs(z[k + "_beta"]) * orc.dd_absmax(C0)
            err = orc.normwise_error(z[k + "_ref"][:, :c["m"]], z[k + "_q"][:, :c["m"]], op)
            assert err <= max(10, 4 * c["k"]) * orc.EPS_DD, (k, err)


def test_gemm_port_is_bitexact_to_reference_simd_path(oracle, golden):
    """or_port_mgemm(simd_order=1) reproduces the reference's AVX2 GEMM bit for bit."""
    z, meta = golden
    for c in meta["l3"]:
        if c["kind"] != "gemm":
            continue
        k = c["key"]
        out = z[k + "_C"].copy()
        oracle.port_mgemm(c["ta"], c["tb"], c["m"], c["n"], c["k"], z[k + "_alpha"], z[k + "_A"], c["lda"],
                          z[k + "_B"], c["ldb"], z[k + "_beta"], out, c["ldc"], simd_order=1)
        np.testing.assert_array_equal(out[:, :c["m"]], z[k + "_ref"][:, :c["m"]], err_msg=k)


def test_gemm_port_is_bitexact_to_reference_scalar_path(oracle):
    """or_port_mgemm(simd_order=0) -- the CPU baseline timed on aarch64 hosts --
    reproduces the reference's GEMM built without its SIMD block (the scalar
    micro-kernel, mgemm_serial.cpp:355-407) bit for bit, across the MC/KC/NC
    block edges and every transpose pair (tests/golden/make_gemm_scalar.py)."""
    z = np.load(os.path.join(ROOT, "tests", "golden", "ref_gemm_scalar.npz"))
    meta = json.loads(bytes(z["meta_json"]).decode())
    assert len(meta) >= 7
    for c in meta:
        k = c["key"]
        out = z[k + "_C"].copy()
        oracle.port_mgemm(c["ta"], c["tb"], c["m"], c["n"], c["k"], z[k + "_alpha"], z[k + "_A"], c["lda"],
                          z[k + "_B"], c["ldb"], z[k + "_beta"], out, c["ldc"], simd_order=0)
        np.testing.assert_array_equal(out[:, :c["m"]], z[k + "_ref"][:, :c["m"]], err_msg=k)
        np.testing.assert_array_equal(out[:, c["m"]:], z[k + "_C"][:, c["m"]:], err_msg=k)   # padding untouched


@pytest.mark.skipif(ref_library() is None, reason="reference build not present (needs the reference sources)")
def test_live_reference_bitexact_random(oracle):
    """Fresh random inputs through the live reference build and the oracle."""
    import os
    ref = ref_library()
    rng = np.random.default_rng(7)
    for n in (1, 2, 7, 100, 1025):
        x = orc  # noqa: F841
        import mwblas as mwb
        xv = mwb.random_dd(rng, (n,))
        a = mwb.random_dd(rng, ())
        r1 = xv.copy()
        ref.mscal(n, a, r1, 1)
        r2 = xv.copy()
        oracle.mscal(n, a, r2, 1, team=1)
        np.testing.assert_array_equal(r1, r2)
        assert ref.imamax(n, xv, 1) == oracle.imamax(n, xv, 1)


# ---- scalar generators (mcabs1, mrotg, mrotmg, wrotg) ------------------------------------

def _generators():
    import importlib.util
    import os
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "make_generators.py")
    spec = importlib.util.spec_from_file_location("make_generators", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod, np.load(path.replace("make_generators.py", "ref_generators.npz"))


@pytest.mark.parametrize("name", ["mcabs1", "mrotg", "mrotmg", "wrotg"])
def test_generators_match_reference(oracle, name):
    """The oracle's restatements reproduce the reference's generators bit for
    bit, including which outputs each branch leaves untouched."""
    mg, z = _generators()
    got = mg.run(lambda n: getattr(oracle.lib, "or_" + n), name, z[name + "_in"])
    np.testing.assert_array_equal(got.view(np.uint64), z[name + "_out"].view(np.uint64))


def _exact_generator(name, x):
    """The same algorithms in 80-digit decimal arithmetic (an output the branch
    does not write keeps its input value)."""
    from decimal import Decimal, getcontext
    getcontext().prec = 80
    D = lambda v: Decimal(float(v[0])) + Decimal(float(v[1]))
    if name == "mcabs1":
        return [abs(D(x[0])) + abs(D(x[1]))]
    if name == "mrotg":
        a, b = D(x[0]), D(x[1])
        if b == 0:
            return [a, Decimal(0), Decimal(1), Decimal(0)]
        if a == 0:
            return [b, Decimal(1), Decimal(0), Decimal(1)]
        r = (a * a + b * b).sqrt()
        r = -r if a < 0 else r
        c, s = a / r, b / r
        return [r, s if abs(a) > abs(b) else 1 / c, c, s]
    if name == "wrotg":
        ar, ai, br, bi = D(x[0, 0]), D(x[0, 1]), D(x[1, 0]), D(x[1, 1])
        g2 = br * br + bi * bi
        if g2 == 0:
            return [ar, ai, Decimal(1), Decimal(0), Decimal(0)]
        f2 = ar * ar + ai * ai
        if f2 == 0:
            d = g2.sqrt()
            return [d, Decimal(0), Decimal(0), br / d, -bi / d]
        h2 = f2 + g2
        c = (f2 / h2).sqrt()
        d = (f2 * h2).sqrt()
        return [ar / c, ai / c, c, (br * ar + bi * ai) / d, (br * ai - bi * ar) / d]
    raise ValueError(name)


@pytest.mark.parametrize("name", ["mcabs1", "mrotg", "wrotg"])
def test_generators_accuracy(oracle, name):
    """Against the exact formulas: relative error within the reference's
    consistency tolerance (100 eps, fuzz_mrotg.fypp:34, fuzz_wrotg.fypp:39;
    10 eps for mcabs1, fuzz_mcabs1.fypp:34), so the unpinned division and
    square root are accurate ones."""
    from decimal import Decimal
    mg, z = _generators()
    got = mg.run(lambda n: getattr(oracle.lib, "or_" + n), name, z[name + "_in"])
    tol = (10 if name == "mcabs1" else 100) * orc.EPS_DD
    for x, g in zip(z[name + "_in"], got):
        want = _exact_generator(name, x)
        for w, gv in zip(want, g):
            d = abs(Decimal(float(gv[0])) + Decimal(float(gv[1])) - w)
            scale = abs(w) if w != 0 else Decimal(1)
            assert float(d / scale) <= tol, (name, x, gv, w)
