"""Index arithmetic of the band-tile and packed-halves kernels, checked on the
CPU (no GPU): every product a row forms reads the stored entry it means,
every shared-memory and global index stays inside its buffer, and each row's
entries are covered exactly once.

The formulas are those of csrc/level2x.cu (k_sbmv_tile, k_spmv_rows,
k_spmv_cols, k_spmv_final); LAPACK band storage AB(k + i - j, j) (upper) /
AB(i - j, j) (lower) and packed storage AP[i + j(j+1)/2] (upper) /
AP[i + j(2n-j-1)/2] (lower), 0-based.
"""
import pytest

R = 128          # kSbRows
SP_CHUNK = 512   # kSpChunk


def band_pos(n, k, upper, i, j):
    """(column, band row) of the stored entry (i, j) of a symmetric band."""
    if upper:
        assert i <= j and j - i <= k
        return j, k + i - j
    assert i >= j and i - j <= k
    return j, i - j


@pytest.mark.parametrize("upper", [True, False])
@pytest.mark.parametrize("n,k", [(1, 0), (5, 3), (5, 30), (127, 1), (128, 16), (129, 31), (300, 32), (700, 32)])
def test_sbmv_tile_indices(n, k, upper):
    kp = k + 1
    sp = kp | 1
    m = ((1 << 20) + kp - 1) // kp
    for r0 in range(0, n, R):
        cb = r0 if upper else max(r0 - k, 0)
        ce = min(r0 + R + k if upper else r0 + R, n)
        xb, xe = max(r0 - k, 0), min(r0 + R + k, n)
        # the copy: idx -> (col, b) by the multiply-shift, every slot once
        total = (ce - cb) * kp
        assert total * m < 1 << 32
        seen = set()
        for idx in range(total):
            col = (idx * m) >> 20
            b = idx - col * kp
            assert (col, b) == divmod(idx, kp)
            seen.add(col * sp + b)
        assert len(seen) == total and max(seen) < (R + k) * sp
        assert xe - xb <= R + 2 * k
        for t in range(R):
            r = r0 + t
            if r >= n:
                break
            lo, hi = min(r, k), min(n - 1 - r, k)
            cofs, xofs = r0 - cb, r0 - xb + t
            cols = []
            for d in range(-lo, hi + 1):
                ad = abs(d)
                lj = t + cofs + ((d if d > 0 else 0) if upper else (d if d < 0 else 0))
                b = k - ad if upper else ad
                c = r + d
                i, j = (min(r, c), max(r, c)) if upper else (max(r, c), min(r, c))
                assert (cb + lj, b) == band_pos(n, k, upper, i, j)
                assert 0 <= lj < ce - cb and 0 <= b <= k
                assert 0 <= xofs + d < xe - xb and xb + xofs + d == c
                cols.append(c)
            assert cols == list(range(max(0, r - k), min(n - 1, r + k) + 1))


def packed_addr(n, upper, i, j):
    if upper:
        assert i <= j
        return i + j * (j + 1) // 2
    assert i >= j
    return i + j * (2 * n - j - 1) // 2


@pytest.mark.parametrize("upper", [True, False])
@pytest.mark.parametrize("n", [1, 2, 33, 511, 512, 513, 1100])
def test_spmv_halves_indices(n, upper):
    nch = (n + SP_CHUNK - 1) // SP_CHUNK
    step = (lambda c: c + 1) if upper else (lambda c: n - c - 1)
    stored = n * (n + 1) // 2
    cover = {}
    chunks_with_rows = {r: [] for r in range(n)}
    # row halves: thread r, chunk q
    for q in range(nch):
        c0, c1 = q * SP_CHUNK, min(n, (q + 1) * SP_CHUNK)
        for r in range(n):
            cb = max(c0, r) if upper else c0
            ce = c1 if upper else min(c1, r + 1)
            if cb >= ce:
                continue
            chunks_with_rows[r].append(q)
            at = cb * (cb + 1) // 2 + r if upper else r + cb * (2 * n - cb - 1) // 2
            for c in range(cb, ce):
                i, j = (r, c) if upper else (r, c)
                assert at == packed_addr(n, upper, i, j) and 0 <= at < stored
                cover[(r, c)] = cover.get((r, c), 0) + 1
                at += step(c)
    # column halves: warp per row r over the contiguous column r
    for r in range(n):
        cb, ce = (0, r) if upper else (r + 1, n)
        base = (r * (r + 1) // 2 if upper else r * (2 * n - r - 1) // 2 + r + 1) - cb
        for c in range(cb, ce):
            a = base + c
            assert a == packed_addr(n, upper, c, r) and 0 <= a < stored
            cover[(r, c)] = cover.get((r, c), 0) + 1
    # every entry of every row exactly once
    assert len(cover) == n * n and set(cover.values()) == {1}
    # the final sums read exactly the chunks the row halves wrote
    for r in range(n):
        q0, q1 = (r // SP_CHUNK, nch) if upper else (0, r // SP_CHUNK + 1)
        assert list(range(q0, q1)) == chunks_with_rows[r]
