"""mgemv_n_noalloc: the GEMV entry point that allocates no device memory.

Some callers cannot allocate device memory while they call into the library:
a framework whose own allocator owns the GPU's memory under a fixed budget,
or code that cannot take the driver allocator's locks or cudaFree's
device-wide synchronisation in the middle of its work. For them the
no-transpose GEMV keeps its partial sums in a fixed 1 MiB array inside the
library instead of allocating scratch per call. This test calls it through the
C ABI twice in a row on device arrays, with the library's allocation hook set
to fail the next device allocation (so any allocation on its path would turn
into an error), and checks each result against mgemv_'s within the GEMV
tolerance the other tests use. It lives in its own file, collected last.
"""
import numpy as np
import pytest

from conftest import mwb, orc

pytestmark = pytest.mark.gpu


def test_noalloc_gemv_matches_mgemv_on_two_calls(gpu, rng):
    import torch
    m, n, lda = 3000, 5000, 3003
    A = mwb.dd_matrix(rng, m, n, lda)
    x = mwb.random_dd(rng, (n,))
    y0 = mwb.random_dd(rng, (m,))
    alpha, beta = mwb.random_dd(rng, ()), mwb.random_dd(rng, ())
    want = y0.copy()
    gpu.mgemv("N", m, n, alpha, A, lda, x, 1, beta, want, 1)
    assert gpu.last_error()[0] == 0
    dA = torch.from_numpy(A).cuda()
    dx = torch.from_numpy(x).cuda()
    dy = torch.from_numpy(y0).cuda()
    torch.cuda.synchronize()
    opn = orc.dd_abs(alpha) * n * orc.dd_absmax(A[:, :m]) * orc.dd_absmax(x) + orc.dd_abs(beta) * orc.dd_absmax(y0)
    tol = max(10, 4 * max(m, n)) * orc.EPS_DD
    gpu.lib.mwblas_debug_fail_alloc_after(0)     # any device allocation would now fail
    try:
        for _ in range(2):
            dy.copy_(torch.from_numpy(y0))
            torch.cuda.synchronize()
            rc = gpu.mgemv_n_noalloc(m, n, alpha, dA.data_ptr(), lda, dx.data_ptr(), 1, beta, dy.data_ptr(), 1)
            torch.cuda.synchronize()
            assert rc == 0, gpu.last_error()
            got = dy.cpu().numpy()
            assert orc.normwise_error(got, want, opn) <= tol
    finally:
        gpu.lib.mwblas_debug_fail_alloc_after(-1)


def test_noalloc_gemv_rejects_rows_beyond_its_scratch(gpu):
    import torch
    m = 65537
    dA = torch.zeros((1, m, 2), dtype=torch.float64, device="cuda")
    dx = torch.zeros((1, 2), dtype=torch.float64, device="cuda")
    dy = torch.zeros((m, 2), dtype=torch.float64, device="cuda")
    rc = gpu.mgemv_n_noalloc(m, 1, 1.0, dA.data_ptr(), m, dx.data_ptr(), 1, 0.0, dy.data_ptr(), 1)
    assert rc == 1 and "65536" in gpu.last_error()[1]
