"""GEMMs on host arrays large enough (>= 64 MB of operands) for the pipelined
path of the tensor-core engine: the uploads run on a copy stream that the
kernels wait on operand by operand, and C comes back in column chunks behind
the reconstruction. The result must be bit-identical to the same call on
device-resident operands (same kernels, same order of every sum), for
pageable and pinned host memory, real and complex, beta zero or not, and with
a column count that leaves a short last chunk; sampled entries are checked
against binary128 at the reference's tolerance (max(10, 4k) * 2^-104).
"""
import numpy as np
import pytest
import torch

from conftest import mwb, orc

pytestmark = pytest.mark.gpu


def _host(x, pinned):
    if not pinned:
        return x, x.ctypes.data
    t = torch.from_numpy(x).pin_memory()
    return t, t.data_ptr()


@pytest.mark.parametrize("pinned", [False, True])
@pytest.mark.parametrize("ta,tb,beta0", [("N", "N", False), ("T", "N", True), ("N", "T", False)])
@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("shape", ["blocks", "one_column_block", "one_row_block"])
def test_host_pipeline_matches_device(gpu, oracle, rng, cplx, ta, tb, beta0, pinned, shape):
    """op(B) and C above 512 columns arrive in column blocks of 512 (short
    last blocks included); at most 512 columns come as one block. A is
    uploaded whole."""
    m, n, k = {"blocks": ((1031, 997, 900), (1531, 1283, 1100)),
               "one_column_block": ((1500, 300, 1200), (2000, 400, 1800)),
               "one_row_block": ((300, 1500, 1200), (400, 1800, 2000))}[shape][0 if cplx else 1]
    rnd = mwb.random_cdd if cplx else mwb.random_dd
    A = rnd(rng, (k, m) if ta == "N" else (m, k))        # storage [column][row]: lda = rows of A
    B = rnd(rng, (n, k) if tb == "N" else (k, n))
    C0 = rnd(rng, (n, m))
    lda, ldb = (m if ta == "N" else k), (k if tb == "N" else n)
    if cplx:
        al, be = mwb.random_cdd(rng, ()), (np.zeros((2, 2)) if beta0 else mwb.random_cdd(rng, ()))
    else:
        al, be = mwb.random_dd(rng, ()), (np.zeros(2) if beta0 else mwb.random_dd(rng, ()))

    def call(pa, pb, pc):
        if cplx:
            gpu.wgemm(ta, tb, m, n, k, al, pa, lda, pb, ldb, be, pc, m)
        else:
            gpu.mgemm(ta, tb, m, n, k, al, pa, lda, pb, ldb, be, pc, m, engine="ozaki")
        assert gpu.last_error()[0] == 0, gpu.last_error()

    dev = torch.device("cuda", 0)
    dA, dB = torch.from_numpy(A).to(dev), torch.from_numpy(B).to(dev)
    dC = torch.from_numpy(C0).to(dev)
    call(dA.data_ptr(), dB.data_ptr(), dC.data_ptr())
    want_dev = dC.cpu().numpy()

    hA, pa = _host(A, pinned)
    hB, pb = _host(B, pinned)
    hC, pc = _host(C0.copy(), pinned)
    call(pa, pb, pc)
    got = hC.numpy() if pinned else hC
    assert np.array_equal(got.view(np.uint64), want_dev.view(np.uint64))

    rows, cols = rng.integers(0, m, 48), rng.integers(0, n, 48)
    if cplx:
        want = oracle.qwgemm(ta, tb, m, n, k, al, A, lda, B, ldb, be, C0, m, rows=rows, cols=cols)
    else:
        want = oracle.qgemm(ta, tb, m, n, k, al, A, lda, B, ldb, be, C0, m, rows=rows, cols=cols)
    scale = orc.dd_abs(al) * k * orc.dd_absmax(A) * orc.dd_absmax(B) + orc.dd_abs(be) * orc.dd_absmax(C0)
    err = float(np.max(orc.dd_diff_abs(got[cols, rows], want))) / scale
    assert err <= max(10, 4 * k) * orc.EPS_DD, err


@pytest.mark.parametrize("fail_at", [0, 1, 2, 3, 4])
def test_host_pipeline_allocation_failure(gpu, rng, fail_at):
    """A device allocation that fails at any point of the pipelined host path
    (the staged operands, the engine's scratch) is reported as an error, no
    copy is left writing into freed memory, and the next call succeeds with
    the right result."""
    m, n, k = 1531, 1283, 1100
    A = mwb.random_dd(rng, (k, m))
    B = mwb.random_dd(rng, (n, k))
    C0 = mwb.random_dd(rng, (n, m))
    al, be = mwb.random_dd(rng, ()), mwb.random_dd(rng, ())
    dev = torch.device("cuda", 0)
    dA, dB, dC = (torch.from_numpy(x).to(dev) for x in (A, B, C0))   # kept alive through the call
    gpu.mgemm("N", "N", m, n, k, al, dA.data_ptr(), m, dB.data_ptr(), k, be, dC.data_ptr(), m, engine="ozaki")
    want = dC.cpu().numpy()
    C = C0.copy()
    gpu.lib.mwblas_debug_fail_alloc_after(fail_at)
    try:
        gpu.mgemm("N", "N", m, n, k, al, A, m, B, k, be, C, m, engine="ozaki")
        err = gpu.last_error()[0]
    finally:
        gpu.lib.mwblas_debug_fail_alloc_after(-1)
    assert err != 0
    C = C0.copy()
    gpu.mgemm("N", "N", m, n, k, al, A, m, B, k, be, C, m, engine="ozaki")
    assert gpu.last_error()[0] == 0, gpu.last_error()
    assert np.array_equal(C.view(np.uint64), want.view(np.uint64))


def test_pageable_arrays_read_in_place(gpu, rng):
    """Where the device reads pageable host memory through the system page
    tables, the pipelined GEMM uploads ordinary numpy arrays with copy
    kernels (one per operand block, counted among the library's launches)
    rather than with copies that would stall the host; pinned arrays keep the
    copy engines. The results are the same bits either way."""
    m, n, k = 1531, 1283, 1100
    A = mwb.random_dd(rng, (k, m))
    B = mwb.random_dd(rng, (n, k))
    C0 = mwb.random_dd(rng, (n, m))
    al, be = mwb.random_dd(rng, ()), mwb.random_dd(rng, ())
    outs, launches = [], []
    for pinned in (True, False):
        hA, pa = _host(A, pinned)
        hB, pb = _host(B, pinned)
        hC, pc = _host(C0.copy(), pinned)
        l0 = gpu.lib.mwblas_launch_count()
        gpu.mgemm("N", "N", m, n, k, al, pa, m, pb, k, be, pc, m, engine="ozaki")
        assert gpu.last_error()[0] == 0, gpu.last_error()
        launches.append(gpu.lib.mwblas_launch_count() - l0)
        outs.append((hC.numpy() if pinned else hC).copy())
    assert np.array_equal(outs[0].view(np.uint64), outs[1].view(np.uint64))
    if gpu.lib.mwblas_pageable_direct():
        # A whole, B and C in three column blocks each: at least 5 copy kernels
        assert launches[1] >= launches[0] + 5, launches
    else:
        assert launches[1] == launches[0], launches
