"""mgemv_n_noalloc: the GEMV entry point that allocates no device memory.

Some callers cannot allocate device memory while they call into the library:
a framework whose own allocator owns the GPU's memory under a fixed budget,
or code that cannot take the driver allocator's locks or cudaFree's
device-wide synchronisation in the middle of its work. For them the
no-transpose GEMV keeps its partial sums in a fixed 1 MiB array inside the
library instead of allocating scratch per call. These tests call it through
the C ABI twice in a row on device arrays, with the library's allocation hook
set to fail the next device allocation (so any allocation on its path would
turn into an error), and check each result against mgemv_'s and against the
binary128 oracle, within the GEMV tolerance max(10, 4 max(m, n)) 2^-104 the
other tests use. The cases cover negative increments, beta = 0 with a y full
of NaN (y must not be read), alpha = 0 (y is only scaled) and m = 65536, where
the scratch array holds one column chunk. The file is collected last.
"""
import numpy as np
import pytest

from conftest import mwb, orc

pytestmark = pytest.mark.gpu


def _vec(rng, n, inc):
    return mwb.random_dd(rng, (1 + (n - 1) * abs(inc),))


CASES = [
    # m, n, lda, incx, incy, alpha kind, beta kind
    (3000, 5000, 3003, 1, 1, "rand", "rand"),
    (3000, 700, 3000, -2, 1, "rand", "rand"),
    (1500, 900, 1501, 1, -2, "rand", "rand"),
    (1500, 900, 1501, -2, -2, "rand", "one"),
    (2000, 600, 2000, 1, 1, "rand", "zero_nan"),
    (2000, 600, 2000, -2, 1, "zero", "rand"),
    (65536, 3, 65536, 1, 1, "rand", "rand"),
]


@pytest.mark.parametrize("m,n,lda,incx,incy,akind,bkind", CASES)
def test_noalloc_gemv_matches_mgemv_and_oracle_on_two_calls(gpu, oracle, rng, m, n, lda, incx, incy, akind, bkind):
    import torch
    A = mwb.dd_matrix(rng, m, n, lda)
    x = _vec(rng, n, incx)
    y0 = _vec(rng, m, incy)
    alpha = np.zeros(2) if akind == "zero" else mwb.random_dd(rng, ())
    beta = {"rand": lambda: mwb.random_dd(rng, ()), "one": lambda: np.array([1.0, 0.0]),
            "zero_nan": lambda: np.zeros(2)}[bkind]()
    if bkind == "zero_nan":
        y0[:] = np.nan                       # beta = 0: y is written, never read
    want = y0.copy()
    gpu.mgemv("N", m, n, alpha, A, lda, x, incx, beta, want, incy)
    assert gpu.last_error()[0] == 0, gpu.last_error()
    q = np.zeros_like(y0) if bkind == "zero_nan" else y0.copy()
    oracle.qgemv("N", m, n, alpha, A, lda, x, incx, beta, q, incy)
    dA = torch.from_numpy(A).cuda()
    dx = torch.from_numpy(x).cuda()
    dy = torch.from_numpy(y0).cuda()
    torch.cuda.synchronize()
    y_fin = np.nan_to_num(y0, nan=0.0)
    opn = orc.dd_abs(alpha) * n * orc.dd_absmax(A[:, :m]) * orc.dd_absmax(x) + orc.dd_abs(beta) * orc.dd_absmax(y_fin)
    tol = max(10, 4 * max(m, n)) * orc.EPS_DD
    gpu.lib.mwblas_debug_fail_alloc_after(0)     # any device allocation would now fail
    try:
        for _ in range(2):
            dy.copy_(torch.from_numpy(y0))
            torch.cuda.synchronize()
            rc = gpu.mgemv_n_noalloc(m, n, alpha, dA.data_ptr(), lda, dx.data_ptr(), incx, beta, dy.data_ptr(), incy)
            torch.cuda.synchronize()
            assert rc == 0, gpu.last_error()
            got = dy.cpu().numpy()
            assert not np.isnan(got).any()
            assert orc.normwise_error(got, want, opn) <= tol
            assert orc.normwise_error(got, q, opn) <= tol
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
