"""The dual-link harness (tests/dual/): several implementations in one binary.

As in the reference's dual-link benchmark (benchmark/dual/BENCH_PROTOCOL.md:
32-38), each static archive's exported names get a per-leg prefix with
objcopy, so this library (gb_*), the reference's own objects where a checkout
was built (ref_*) and the C port of its algorithms (or_*) link together and
are timed back to back on the same buffers in one process.

CPU: the renamed archive exports only prefixed ABI names and the driver
links. GPU: the driver runs; GEMM and DOT agree with the port within the
double-double tolerance, AXPY and SCAL bit for bit (same OpenMP team split).
"""
import os
import subprocess
import sys

import pytest

from conftest import ROOT

sys.path.insert(0, os.path.join(ROOT, "tests", "dual"))
import run_dual  # noqa: E402


def test_archive_namespaced_and_driver_links(libpath):
    exe, have_ref = run_dual.build()
    assert os.path.exists(exe)
    names = run_dual.exported_names(os.path.join(run_dual.BUILD, "lib_gb_ns.a"))
    assert "gb_mgemm_64_" in names and "gb_mdot_" in names and "gb_mwblas_set_l1_partition" in names
    assert not [n for n in names if not n.startswith("gb_")], "an exported name kept its plain form"
    syms = subprocess.run(["nm", exe], capture_output=True, text=True).stdout.split()
    assert "gb_mgemm_64_" in syms and "or_port_mgemm" in syms
    assert "mgemm_64_" not in syms
    if have_ref:
        assert "ref_mgemm_64_" in syms


@pytest.mark.gpu
def test_dual_link_legs_agree(gpu):
    rows = {r["routine"]: r for r in run_dual.run(reps=2, gemm_n=256, vec_n=1 << 16)}
    assert set(rows) == {"mgemm", "mdot", "maxpy", "mscal"}
    eps = 2.0 ** -104
    assert rows["mgemm"]["max_rel_diff_vs_port"] <= 4 * 256 * eps * 256
    assert rows["mdot"]["max_rel_diff_vs_port"] <= 4 * (1 << 16) * eps
    assert rows["maxpy"]["max_rel_diff_vs_port"] == 0.0
    assert rows["mscal"]["max_rel_diff_vs_port"] == 0.0
    for r in rows.values():
        assert r["ns_per_call"]["gb300"] > 0 and r["ns_per_call"]["port"] > 0
