"""Batched uneven GEMM / TRSM (extensions without a reference counterpart).

Each instance is checked against the binary128 oracle with the same
tolerances as the single-instance routines; graph replays must reproduce the
first call bit for bit; the split-K autotuner must leave C untouched and its
choice must give correct results.
"""
import numpy as np
import pytest

from conftest import mwb, orc

pytestmark = pytest.mark.gpu


class DeviceArena:
    """Places numpy DD arrays in one device buffer and hands out pointers."""

    def __init__(self, arrays):
        import torch
        self.offsets, tot = [], 0
        for a in arrays:
            self.offsets.append(tot)
            tot += a.size
        host = np.zeros(max(tot, 2))
        for a, o in zip(arrays, self.offsets):
            host[o:o + a.size] = a.reshape(-1)
        self.buf = torch.from_numpy(host).cuda()
        self.shapes = [a.shape for a in arrays]

    def ptr(self, i):
        return self.buf.data_ptr() + 8 * self.offsets[i]

    def get(self, i):
        o = self.offsets[i]
        n = int(np.prod(self.shapes[i]))
        return self.buf[o:o + n].cpu().numpy().reshape(self.shapes[i])


def make_batch(rng, count, maxdim=200, big_k=None):
    inst = []
    for t in range(count):
        m, n, k = (int(x) for x in np.exp(rng.uniform(np.log(1), np.log(maxdim), 3)).round())
        if t == 3:
            m = 0
        if t == 5:
            k = 0
        if big_k and t % 7 == 0:
            # split instances with different split counts share the partial buffer
            m, n, k = 12, 20, big_k // (1 + (t // 7) % 3)
        ta, tb = rng.choice(["N", "T", "C"]), rng.choice(["N", "T"])
        lda = (m if ta == "N" else k) + int(rng.integers(0, 3))
        ldb = (k if tb == "N" else n) + int(rng.integers(0, 3))
        ldc = m + int(rng.integers(0, 3))
        A = mwb.dd_matrix(rng, m if ta == "N" else k, k if ta == "N" else m, max(lda, 1))
        B = mwb.dd_matrix(rng, k if tb == "N" else n, n if tb == "N" else k, max(ldb, 1))
        Cm = mwb.dd_matrix(rng, m, n, max(ldc, 1))
        al = mwb.random_dd(rng, ()) if t != 9 else np.zeros(2)
        be = mwb.random_dd(rng, ()) if t % 3 else np.zeros(2)
        inst.append(dict(m=m, n=n, k=k, ta=str(ta), tb=str(tb), lda=max(lda, 1), ldb=max(ldb, 1), ldc=max(ldc, 1),
                         A=A, B=B, C=Cm, alpha=al, beta=be))
    return inst


def run_grouped(gpu, inst, tune=False):
    arena = DeviceArena([x for d in inst for x in (d["A"], d["B"], d["C"])])
    args = dict(ta=[d["ta"] for d in inst], tb=[d["tb"] for d in inst], m=[d["m"] for d in inst],
                n=[d["n"] for d in inst], k=[d["k"] for d in inst], alpha=[d["alpha"] for d in inst],
                a=[arena.ptr(3 * i) for i in range(len(inst))], lda=[d["lda"] for d in inst],
                b=[arena.ptr(3 * i + 1) for i in range(len(inst))], ldb=[d["ldb"] for d in inst],
                beta=[d["beta"] for d in inst], c=[arena.ptr(3 * i + 2) for i in range(len(inst))],
                ldc=[d["ldc"] for d in inst])
    chosen = None
    if tune:
        rc, chosen = gpu.mgemm_grouped_tune(**args)
        assert rc == 0, gpu.last_error()
        for i, d in enumerate(inst):     # tuning must not touch C
            np.testing.assert_array_equal(arena.get(3 * i + 2), d["C"])
    rc = gpu.mgemm_grouped(**args)
    assert rc == 0, gpu.last_error()
    return arena, args, chosen


def check(oracle, inst, arena):
    for i, d in enumerate(inst):
        got = arena.get(3 * i + 2)
        m, n, k = d["m"], d["n"], d["k"]
        if m == 0 or n == 0:
            continue
        want = oracle.qgemm(d["ta"], d["tb"], m, n, k, d["alpha"], d["A"], d["lda"], d["B"], d["ldb"], d["beta"],
                            d["C"].copy(), d["ldc"])
        opn = orc.dd_abs(d["alpha"]) * max(k, 1) * orc.dd_absmax(d["A"]) * orc.dd_absmax(d["B"]) \
            + orc.dd_abs(d["beta"]) * orc.dd_absmax(d["C"])
        err = orc.normwise_error(got[:, :m], want[:, :m], opn)
        assert err <= max(10, 4 * k) * orc.EPS_DD, (i, m, n, k, err)
        if d["ldc"] > m:
            np.testing.assert_array_equal(got[:, m:], d["C"][:, m:])


def test_grouped_gemm_matches_oracle_and_replays(gpu, oracle, rng):
    inst = make_batch(rng, 60)
    arena, args, _ = run_grouped(gpu, inst)
    check(oracle, inst, arena)
    first = [arena.get(3 * i + 2) for i in range(len(inst))]
    # replay the cached graph on reset inputs: bit-identical
    for i, d in enumerate(inst):
        o = arena.offsets[3 * i + 2]
        import torch
        arena.buf[o:o + d["C"].size] = torch.from_numpy(d["C"].reshape(-1)).cuda()
    assert gpu.mgemm_grouped(**args) == 0
    for i in range(len(inst)):
        np.testing.assert_array_equal(arena.get(3 * i + 2), first[i])


def test_grouped_gemm_split_k_and_tuner(gpu, oracle, rng):
    inst = make_batch(rng, 30, maxdim=120, big_k=3000)
    arena, args, chosen = run_grouped(gpu, inst, tune=True)
    assert chosen in (0, 2048, 1024, 512, 256, 128)
    assert gpu.lib.mwblas_grouped_tuned_tile() in (16, 32, 64)
    check(oracle, inst, arena)


@pytest.mark.parametrize("tile", [16, 32, 64])
def test_grouped_gemm_every_tile_shape(gpu, oracle, rng, tile):
    """Each tile edge the tuner can choose: ragged instances (tiles cut by m, n),
    split-K instances (partial tiles of tile^2 extended floats), and a graph
    replay that gives the same bits."""
    inst = make_batch(rng, 40, maxdim=150, big_k=2500)
    prev = gpu.lib.mwblas_set_grouped_tile(tile)
    try:
        arena, args, _ = run_grouped(gpu, inst)
        check(oracle, inst, arena)
        first = [arena.get(3 * i + 2) for i in range(len(inst))]
        import torch
        for i, d in enumerate(inst):
            o = arena.offsets[3 * i + 2]
            arena.buf[o:o + d["C"].size] = torch.from_numpy(d["C"].reshape(-1)).cuda()
        assert gpu.mgemm_grouped(**args) == 0
        for i in range(len(inst)):
            np.testing.assert_array_equal(arena.get(3 * i + 2), first[i])
    finally:
        gpu.lib.mwblas_set_grouped_tile(prev)


@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("uplo,trans", [("L", "N"), ("U", "N"), ("L", "T"), ("U", "T")])
@pytest.mark.parametrize("diag", ["N", "U"])
def test_grouped_trsm(gpu, oracle, rng, side, uplo, trans, diag):
    import torch
    inst = []
    for t in range(12):
        na = int(np.exp(rng.uniform(np.log(2), np.log(120))))
        nrhs = int(rng.integers(1, 70))
        m, n = (na, nrhs) if side == "L" else (nrhs, na)
        lda, ldb = na + int(rng.integers(0, 2)), m + int(rng.integers(0, 2))
        A = mwb.dd_matrix(rng, na, na, lda)
        A[..., 0] /= na
        A[..., 1] /= na
        for d in range(na):
            A[d, d] = (1.0 + rng.random(), 0.0)
        B = mwb.dd_matrix(rng, m, n, ldb)
        inst.append(dict(m=m, n=n, na=na, lda=lda, ldb=ldb, A=A, B=B, alpha=mwb.random_dd(rng, ())))
    arena = DeviceArena([x for d in inst for x in (d["A"], d["B"])])
    rc = gpu.mtrsm_grouped(side, uplo, trans, diag, [d["m"] for d in inst], [d["n"] for d in inst],
                           [d["alpha"] for d in inst], [arena.ptr(2 * i) for i in range(len(inst))],
                           [d["lda"] for d in inst], [arena.ptr(2 * i + 1) for i in range(len(inst))],
                           [d["ldb"] for d in inst])
    assert rc == 0, gpu.last_error()
    for i, d in enumerate(inst):
        want = d["B"].copy()
        oracle.qtrsm(side, uplo, trans, diag, d["m"], d["n"], d["alpha"], d["A"], d["lda"], want, d["ldb"])
        got = arena.get(2 * i + 1)
        err = orc.normwise_error(got[:, :d["m"]], want[:, :d["m"]], orc.dd_abs(d["alpha"]) * orc.dd_absmax(d["B"]))
        assert err <= max(20, 8 * d["na"] ** 2) * orc.EPS_DD, (i, err)


def test_grouped_gemm_long_k_scaled_and_nonfinite(gpu, oracle, rng):
    """K beyond one split's 16384 multiply-adds, rows scaled by 2^+-200, and an
    instance whose A holds an infinity (its rows become NaN, the others are
    unaffected)."""
    inst = make_batch(rng, 6, maxdim=40)
    inst[0].update(m=5, n=3, k=20000, ta="N", tb="N", lda=5, ldb=20000, ldc=5)
    inst[0]["A"] = mwb.dd_matrix(rng, 5, 20000, 5) * (2.0 ** rng.integers(-200, 200, 5))[None, :, None]
    inst[0]["B"] = mwb.dd_matrix(rng, 20000, 3, 20000)
    inst[0]["C"] = mwb.dd_matrix(rng, 5, 3, 5)
    bad = inst[1]
    bad.update(ta="N")
    bad["lda"] = max(bad["m"], 1)
    bad["A"] = mwb.dd_matrix(rng, bad["m"], bad["k"], bad["lda"])
    if bad["m"] > 0 and bad["k"] > 0 and bad["n"] > 0:
        bad["A"][0, 0] = (np.inf, 0.0)
    arena, args, _ = run_grouped(gpu, inst)
    # instance 0: entrywise against its own row scale
    d = inst[0]
    got = arena.get(2)
    want = oracle.qgemm("N", "N", 5, 3, 20000, d["alpha"], d["A"], 5, d["B"], 20000, d["beta"], d["C"].copy(), 5)
    ra = np.max(np.abs(d["A"][..., 0]), axis=0)
    scale = orc.dd_abs(d["alpha"]) * 20000 * np.outer(np.max(np.abs(d["B"][..., 0]), axis=1), ra) \
        + orc.dd_abs(d["beta"]) * np.abs(d["C"][..., 0])
    err = np.abs((got[..., 0] - want[..., 0]) + (got[..., 1] - want[..., 1]))
    assert np.all(err <= 4 * 20000 * orc.EPS_DD * scale), np.max(err / scale)
    if bad["m"] > 0 and bad["k"] > 0 and bad["n"] > 0:
        gb = arena.get(5)
        assert np.all(np.isnan(gb[:, 0, 0])), "row with an infinity must be NaN"
    for i in range(2, len(inst)):
        check(oracle, [inst[i]], _Shift(arena, 3 * i))


class _Shift:
    """View of a DeviceArena whose indices start at instance `base`."""

    def __init__(self, arena, base):
        self.arena, self.base = arena, base

    def get(self, i):
        return self.arena.get(self.base + i)


def _trsm_batch(rng, count, side, max_na=120):
    inst = []
    for t in range(count):
        na = int(np.exp(rng.uniform(np.log(2), np.log(max_na))))
        nrhs = int(rng.integers(1, 70))
        m, n = (na, nrhs) if side == "L" else (nrhs, na)
        lda, ldb = na + int(rng.integers(0, 2)), m + int(rng.integers(0, 2))
        A = mwb.dd_matrix(rng, na, na, lda)
        A[..., 0] /= na
        A[..., 1] /= na
        for d in range(na):
            A[d, d] = (1.0 + rng.random(), 0.0)
        B = mwb.dd_matrix(rng, m, n, ldb)
        inst.append(dict(m=m, n=n, na=na, lda=lda, ldb=ldb, A=A, B=B, alpha=mwb.random_dd(rng, ())))
    return inst


def _trsm_call(gpu, side, inst, arena):
    return gpu.mtrsm_grouped(side, "L", "N", "N", [d["m"] for d in inst], [d["n"] for d in inst],
                             [d["alpha"] for d in inst], [arena.ptr(2 * i) for i in range(len(inst))],
                             [d["lda"] for d in inst], [arena.ptr(2 * i + 1) for i in range(len(inst))],
                             [d["ldb"] for d in inst])


def test_grouped_trsm_graph_replay(gpu, oracle, rng):
    """The persistent grouped TRSM is captured in a graph per batch layout: a
    second call on the same layout replays it (same bits), new right-hand
    sides in the same arrays are solved correctly by the replay, and a
    different layout is captured anew."""
    inst = _trsm_batch(rng, 40, "L")
    arena = DeviceArena([x for d in inst for x in (d["A"], d["B"])])
    b0 = arena.buf.clone()
    outs = []
    for _ in range(2):
        arena.buf.copy_(b0)
        assert _trsm_call(gpu, "L", inst, arena) == 0, gpu.last_error()
        outs.append([arena.get(2 * i + 1) for i in range(len(inst))])
    for a, b in zip(*outs):
        np.testing.assert_array_equal(a, b)
    # new data, same layout (graph replay)
    for i, d in enumerate(inst):
        d["B"] = mwb.dd_matrix(rng, d["m"], d["n"], d["ldb"])
    arena2 = DeviceArena([x for d in inst for x in (d["A"], d["B"])])
    arena.buf.copy_(arena2.buf)
    assert _trsm_call(gpu, "L", inst, arena) == 0, gpu.last_error()
    for i, d in enumerate(inst):
        want = d["B"].copy()
        oracle.qtrsm("L", "L", "N", "N", d["m"], d["n"], d["alpha"], d["A"], d["lda"], want, d["ldb"])
        err = orc.normwise_error(arena.get(2 * i + 1)[:, :d["m"]], want[:, :d["m"]],
                                 orc.dd_abs(d["alpha"]) * orc.dd_absmax(d["B"]))
        assert err <= max(20, 8 * d["na"] ** 2) * orc.EPS_DD, (i, err)
    # a different layout: fewer instances, longer triangles
    inst3 = _trsm_batch(rng, 7, "L", max_na=250)
    arena3 = DeviceArena([x for d in inst3 for x in (d["A"], d["B"])])
    assert _trsm_call(gpu, "L", inst3, arena3) == 0, gpu.last_error()
    for i, d in enumerate(inst3):
        want = d["B"].copy()
        oracle.qtrsm("L", "L", "N", "N", d["m"], d["n"], d["alpha"], d["A"], d["lda"], want, d["ldb"])
        err = orc.normwise_error(arena3.get(2 * i + 1)[:, :d["m"]], want[:, :d["m"]],
                                 orc.dd_abs(d["alpha"]) * orc.dd_absmax(d["B"]))
        assert err <= max(20, 8 * d["na"] ** 2) * orc.EPS_DD, (i, err)


def _mixed_batch(rng, count, fill=None):
    """Large instances (m, n >= 128, k >= 64: the tensor-core path) mixed with
    small ones, every transpose pair, padded leading dimensions, beta = 0 / 1 /
    random, and an Inf in one large instance."""
    inst = []
    for t in range(count):
        big = t % 2 == 0
        if big:
            m, n = (int(x) for x in rng.integers(128, 530, 2))
            k = int(rng.integers(64, 600))
        else:
            m, n, k = (int(x) for x in rng.integers(1, 100, 3))
        ta, tb = str(rng.choice(["N", "T", "C"])), str(rng.choice(["N", "T"]))
        lda = (m if ta == "N" else k) + int(rng.integers(0, 3))
        ldb = (k if tb == "N" else n) + int(rng.integers(0, 3))
        ldc = m + int(rng.integers(0, 3))
        A = mwb.dd_matrix(rng, m if ta == "N" else k, k if ta == "N" else m, lda)
        B = mwb.dd_matrix(rng, k if tb == "N" else n, n if tb == "N" else k, ldb)
        Cm = mwb.dd_matrix(rng, m, n, ldc, fill=fill)
        be = [mwb.random_dd(rng, ()), np.zeros(2), np.array([1.0, 0.0])][t % 3]
        if t == 4:
            A[0, 0] = (np.inf, 0.0)     # row 0 of op(A) (or column 0) holds an Inf
        inst.append(dict(m=m, n=n, k=k, ta=ta, tb=tb, lda=lda, ldb=ldb, ldc=ldc, A=A, B=B, C=Cm,
                         alpha=mwb.random_dd(rng, ()), beta=be))
    return inst


def test_grouped_gemm_tensor_core_path(gpu, oracle, rng):
    """Instances with m, n >= 128 and k >= 64 run on the tensor cores (padding
    classes, one residue GEMM per class, batched conversion and
    reconstruction), the rest on the integer pipes, in one graph; results
    within the GEMM tolerance, non-finite rows/columns NaN, padding rows of C
    untouched, and a replay that gives the same bits."""
    import torch
    inst = _mixed_batch(rng, 24, fill=-7.37e18)
    prev = gpu.lib.mwblas_set_grouped_tensor_min(128)
    try:
        arena, args, _ = run_grouped(gpu, inst)
        first = [arena.get(3 * i + 2) for i in range(len(inst))]
        for i, d in enumerate(inst):
            o = arena.offsets[3 * i + 2]
            arena.buf[o:o + d["C"].size] = torch.from_numpy(d["C"].reshape(-1)).cuda()
        assert gpu.mgemm_grouped(**args) == 0, gpu.last_error()
        for i in range(len(inst)):
            np.testing.assert_array_equal(arena.get(3 * i + 2), first[i])
    finally:
        gpu.lib.mwblas_set_grouped_tensor_min(prev)
    for i, d in enumerate(inst):
        got = first[i]
        m, n, k = d["m"], d["n"], d["k"]
        want = oracle.qgemm(d["ta"], d["tb"], m, n, k, d["alpha"], d["A"], d["lda"], d["B"], d["ldb"], d["beta"],
                            d["C"].copy(), d["ldc"])
        if d["ldc"] > m:
            assert np.all(got[:, m:] == -7.37e18), i
        if i == 4:
            bad = ~np.isfinite(want[:, :m, 0])
            assert bad.any() and np.all(np.isnan(got[:, :m, 0][bad])), i
            continue
        opn = orc.dd_abs(d["alpha"]) * max(k, 1) * orc.dd_absmax(d["A"]) * orc.dd_absmax(d["B"]) \
            + orc.dd_abs(d["beta"]) * orc.dd_absmax(d["C"][:, :m])
        err = orc.normwise_error(got[:, :m], want[:, :m], opn)
        assert err <= max(10, 4 * k) * orc.EPS_DD, (i, m, n, k, err)


def test_grouped_gemm_tuner_chooses_tensor_threshold(gpu, oracle, rng):
    inst = _mixed_batch(rng, 16)
    inst[4]["A"][0, 0] = (0.5, 0.0)
    arena, args, chosen = run_grouped(gpu, inst, tune=True)
    assert gpu.lib.mwblas_grouped_tuned_tensor_min() in (0, 64, 128, 256)
    check(oracle, inst, arena)


def _small_batch(rng, count, skinny=()):
    """Small instances (m, n <= 200) with k from 4 to 300: those with k >= the
    packing depth share 256 x 256 tensor-core slots, the rest stay on the
    integer pipes; odd m and n (a row pair straddles two instances of a slot),
    every transpose pair, padded ldc, an Inf in one instance. `skinny` appends
    instances of the given (m, n, k), shared as pieces of at most 256 x 256."""
    inst = []
    for t in range(count + len(skinny)):
        m, n = (int(x) for x in rng.integers(1, 201, 2))
        k = int(rng.integers(4, 301))
        if t % 5 == 0:
            m, n = 2 * int(rng.integers(1, 30)) + 1, 2 * int(rng.integers(1, 30)) + 1
        if t >= count:
            m, n, k = skinny[t - count]
        ta, tb = str(rng.choice(["N", "T", "C"])), str(rng.choice(["N", "T"]))
        lda = (m if ta == "N" else k) + int(rng.integers(0, 3))
        ldb = (k if tb == "N" else n) + int(rng.integers(0, 3))
        ldc = m + int(rng.integers(0, 3))
        A = mwb.dd_matrix(rng, m if ta == "N" else k, k if ta == "N" else m, lda)
        B = mwb.dd_matrix(rng, k if tb == "N" else n, n if tb == "N" else k, ldb)
        Cm = mwb.dd_matrix(rng, m, n, ldc, fill=-7.37e18)
        be = [mwb.random_dd(rng, ()), np.zeros(2), np.array([1.0, 0.0])][t % 3]
        inst.append(dict(m=m, n=n, k=k, ta=ta, tb=tb, lda=lda, ldb=ldb, ldc=ldc, A=A, B=B, C=Cm,
                         alpha=mwb.random_dd(rng, ()), beta=be))
    inst[7]["A"][0, 0] = (np.inf, 0.0)
    return inst


def _check_small(oracle, inst, outs):
    for i, d in enumerate(inst):
        got, m, n, k = outs[i], d["m"], d["n"], d["k"]
        want = oracle.qgemm(d["ta"], d["tb"], m, n, k, d["alpha"], d["A"], d["lda"], d["B"], d["ldb"], d["beta"],
                            d["C"].copy(), d["ldc"])
        if d["ldc"] > m:
            assert np.all(got[:, m:] == -7.37e18), i
        if i == 7:
            bad = ~np.isfinite(want[:, :m, 0])
            assert bad.any() and np.all(np.isnan(got[:, :m, 0][bad])), i
            continue
        opn = orc.dd_abs(d["alpha"]) * max(k, 1) * orc.dd_absmax(d["A"]) * orc.dd_absmax(d["B"]) \
            + orc.dd_abs(d["beta"]) * orc.dd_absmax(d["C"][:, :m])
        err = orc.normwise_error(got[:, :m], want[:, :m], opn)
        assert err <= max(10, 4 * k) * orc.EPS_DD, (i, m, n, k, err)


@pytest.mark.parametrize("oz_min,pack_k", [(0, 16), (128, 32)])
def test_grouped_gemm_shared_tensor_slots(gpu, oracle, rng, oz_min, pack_k):
    """Small instances packed several to a tensor-core slot (block-diagonal:
    own rows and output columns, K from 0), alone or beside instances with
    slots of their own, and skinny instances (m or n above 256) split into
    pieces of at most 256 x 256; within the GEMM tolerance, and a graph replay
    gives the same bits."""
    import torch
    inst = _small_batch(rng, 60, skinny=[(600, 37, 100), (20, 530, 290), (513, 300, 40), (257, 1, 64)])
    prev_oz = gpu.lib.mwblas_set_grouped_tensor_min(oz_min)
    prev_pk = gpu.lib.mwblas_set_grouped_tensor_pack(pack_k)
    try:
        arena, args, _ = run_grouped(gpu, inst)
        first = [arena.get(3 * i + 2) for i in range(len(inst))]
        for i, d in enumerate(inst):
            o = arena.offsets[3 * i + 2]
            arena.buf[o:o + d["C"].size] = torch.from_numpy(d["C"].reshape(-1)).cuda()
        assert gpu.mgemm_grouped(**args) == 0, gpu.last_error()
        for i in range(len(inst)):
            np.testing.assert_array_equal(arena.get(3 * i + 2), first[i])
    finally:
        gpu.lib.mwblas_set_grouped_tensor_min(prev_oz)
        gpu.lib.mwblas_set_grouped_tensor_pack(prev_pk)
    _check_small(oracle, inst, first)
