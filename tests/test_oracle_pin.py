"""Pins the CPU oracle against the reference's own outputs (no GPU).

The golden fixtures hold outputs of the reference's double-double sources and
of its kind16 binary128 routines on seeded inputs (tests/golden/make_golden.py).
The oracle's bit-exact restatements must reproduce the former bit for bit; its
binary128 routines must agree with the latter to binary128 rounding level.
"""
import numpy as np
import pytest

from conftest import orc, ref_library


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
