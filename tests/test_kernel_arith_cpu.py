"""Index arithmetic of the kernels, emulated on the CPU.

The data-tiled form's row slices partition the rows exactly (test at the end).

bay_div_dim (csrc/device/bay_batch.cuh) finds the walker of a tile element, e / dim, from a
float reciprocal instead of an integer division: q = trunc(fl(e) * rcp_rn(dim)), then one
step of correction.  The claim is that the corrected q equals the exact quotient for every
e < 2^24 (the kernels' elements per tile stay below 256 x 4096 = 2^20) and every dim in
[1, 4096].  numpy's float32 multiply and divide round to nearest like __fmul_rn and
__frcp_rn, and astype(uint32) truncates like __float2uint_rz.
"""
import numpy as np


def _div_dim(e, dim):
    inv = np.float32(1.0) / np.float32(dim)
    q = (e.astype(np.float32) * inv).astype(np.uint32)
    hi = q * np.uint32(dim) > e
    q = np.where(hi, q - 1, q)
    lo = (~hi) & ((q + 1) * np.uint32(dim) <= e)
    return np.where(lo, q + 1, q).astype(np.uint32)


def test_div_dim_exact_near_every_multiple():
    """Every dim in [1, 4096]; e at every multiple of dim and one either side, up to
    2^20 (the largest tile), plus random e below 2^24."""
    rng = np.random.default_rng(0)
    for dim in range(1, 4097):
        k = np.arange(0, (1 << 20) // dim + 2, dtype=np.int64)
        e = np.concatenate([k * dim, k * dim + 1, np.maximum(k * dim - 1, 0),
                            rng.integers(0, 1 << 24, 256)]).astype(np.uint32)
        e = e[e < (1 << 24)]
        q = _div_dim(e, dim)
        np.testing.assert_array_equal(q, e // np.uint32(dim), err_msg="dim %d" % dim)


def test_div_dim_exhaustive_small_tiles():
    """Exhaustively for the common dimensions (2..257) over a whole 256-walker tile."""
    for dim in range(2, 258):
        e = np.arange(0, 256 * dim, dtype=np.uint32)
        np.testing.assert_array_equal(_div_dim(e, dim), e // np.uint32(dim))


def _slices(n, ns):
    """The data-tiled form's row slices (bay_stretch_tiled): slice sl of ns covers rows
    [rb, rb + rn)."""
    rps = (((n + ns - 1) // ns + 3) & ~3) if ns > 1 else n
    out = []
    for sl in range(ns):
        rb = min(sl * rps, n)
        out.append((rb, min(n - rb, rps)))
    return rps, out


def test_tile_slices_cover_every_row_once():
    """Every row count up to 5,000 (and some large ones) and every slice count 1..16: the
    slices are disjoint, cover [0, n) in order, start on a multiple of 4 rows (16-byte TMA
    starts for any row length), and none is longer than the host's shared-memory plan
    (min(rps, n) rows)."""
    ns_all = range(1, 17)
    for n in list(range(0, 5001)) + [10000, 30001, 1000000, 2 ** 24 + 3]:
        for ns in ns_all:
            rps, sl = _slices(n, ns)
            pos = 0
            for rb, rn in sl:
                assert rb % 4 == 0 or rn == 0, (n, ns, rb)
                if rn:
                    assert rb == pos, (n, ns, rb, pos)
                    pos = rb + rn
                assert rn <= min(rps, n)
            assert pos == n, (n, ns, pos)
