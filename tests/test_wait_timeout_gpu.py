"""The bounded-wait failure path of the tensor-core residue GEMM, on the GPU.

Every mbarrier wait of the tcgen05 kernels gives up after a limit; the kernel
then drains its own copies and MMAs, frees its tensor memory and returns, and
the routine reports MWBLAS_ERR_TIMEOUT when it synchronises. The test makes a
wait run out without a GPU fault: the library's injection hook makes the next
CTA-pair launch issue no operand loads, so the MMA issuer's first wait for a
landed stage has nothing to wait for (nothing is in flight anywhere). The
limit is shortened so that this takes milliseconds. Afterwards the limit is
restored and the next call must be correct against the binary128 oracle.
"""
import numpy as np
import pytest

from conftest import mwb, orc

pytestmark = pytest.mark.gpu

MWBLAS_ERR_TIMEOUT = -4


def _case(rng, m, n, k):
    A = mwb.dd_matrix(rng, m, k)
    B = mwb.dd_matrix(rng, k, n)
    C0 = mwb.dd_matrix(rng, m, n)
    return A, B, C0, mwb.random_dd(rng, ()), mwb.random_dd(rng, ())


def test_lost_operand_loads_report_timeout_and_next_call_is_correct(gpu, oracle, rng):
    import torch
    m, n, k = 256, 512, 1024
    A, B, C0, al, be = _case(rng, m, n, k)
    dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    dC = torch.from_numpy(C0).cuda()
    prev_kind = gpu.lib.mwblas_set_ozaki_mma(3)   # the CTA-pair kernel (the default)
    prev_limit = gpu.lib.mwblas_set_wait_limit_ns(20_000_000)   # 20 ms
    try:
        assert prev_limit == 2_000_000_000
        gpu.lib.mwblas_debug_lose_operand_loads(1)
        gpu.mgemm("N", "N", m, n, k, al, dA.data_ptr(), m, dB.data_ptr(), k, be, dC.data_ptr(), m, engine="ozaki")
        code, msg = gpu.last_error()
        assert code == MWBLAS_ERR_TIMEOUT, (code, msg)
        assert "gave up" in msg
    finally:
        gpu.lib.mwblas_debug_lose_operand_loads(0)
        assert gpu.lib.mwblas_set_wait_limit_ns(0) == 20_000_000
        gpu.lib.mwblas_set_ozaki_mma(prev_kind)
    # the context is still usable and the status word was cleared: the same
    # call again, checked against the oracle
    dC.copy_(torch.from_numpy(C0))
    torch.cuda.synchronize()
    gpu.mgemm("N", "N", m, n, k, al, dA.data_ptr(), m, dB.data_ptr(), k, be, dC.data_ptr(), m, engine="ozaki")
    assert gpu.last_error()[0] == 0, gpu.last_error()
    got = dC.cpu().numpy()
    want = oracle.qgemm("N", "N", m, n, k, al, A, m, B, k, be, C0.copy(), m)
    op = orc.dd_abs(al) * k * orc.dd_absmax(A) * orc.dd_absmax(B) + orc.dd_abs(be) * orc.dd_absmax(C0)
    assert orc.normwise_error(got, want, op) <= max(10, 4 * k) * orc.EPS_DD


def test_wait_limit_is_clamped_and_restored(gpu):
    prev = gpu.lib.mwblas_set_wait_limit_ns(5)          # raised to 1 ms
    try:
        assert gpu.lib.mwblas_set_wait_limit_ns(0) == 1_000_000
    finally:
        gpu.lib.mwblas_set_wait_limit_ns(0)
    assert prev == 2_000_000_000


def test_injection_applies_to_one_launch_only(gpu, oracle, rng):
    """Two injected launches fail, the third call (no injection left) succeeds."""
    m, n, k = 256, 256, 512
    A, B, C0, al, be = _case(rng, m, n, k)
    prev_kind = gpu.lib.mwblas_set_ozaki_mma(3)
    gpu.lib.mwblas_set_wait_limit_ns(20_000_000)
    try:
        gpu.lib.mwblas_debug_lose_operand_loads(2)
        for _ in range(2):
            c = C0.copy()
            gpu.mgemm("N", "N", m, n, k, al, A, m, B, k, be, c, m, engine="ozaki")
            assert gpu.last_error()[0] == MWBLAS_ERR_TIMEOUT
        c = C0.copy()
        gpu.mgemm("N", "N", m, n, k, al, A, m, B, k, be, c, m, engine="ozaki")
        assert gpu.last_error()[0] == 0, gpu.last_error()
    finally:
        gpu.lib.mwblas_debug_lose_operand_loads(0)
        gpu.lib.mwblas_set_wait_limit_ns(0)
        gpu.lib.mwblas_set_ozaki_mma(prev_kind)
    want = oracle.qgemm("N", "N", m, n, k, al, A, m, B, k, be, C0.copy(), m)
    op = orc.dd_abs(al) * k * orc.dd_absmax(A) * orc.dd_absmax(B) + orc.dd_abs(be) * orc.dd_absmax(C0)
    assert orc.normwise_error(c, want, op) <= max(10, 4 * k) * orc.EPS_DD
