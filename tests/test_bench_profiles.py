"""bench.py reads the DRAM traffic of its roofline lines from the ncu
summaries under profiles/ (no GPU needed)."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_traffic_lines_present_and_sane():
    # residue GEMM at 8192^3: above the 11.3 GB of operand and product bytes
    assert bench.tc_traffic_from_profile() > 11.3e9
    # band kernel: at least the band (1.14 GB) and the vectors
    assert 1.2e9 < bench.traffic_from_profile("k_sbmv_tile_n4M_k16_ncu.txt") < 1.6e9
    # packed halves: the triangle (2.15 GB) read once by each half
    assert 4.2e9 < bench.traffic_from_profile("mspmv_16384_launches.txt") < 4.5e9
    assert bench.traffic_from_profile("no_such_profile.txt") is None
