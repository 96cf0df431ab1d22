"""Batched transform / quant (xin_gpu_tq_batch) against the oracle's per-block TU
path (orc_tq_block): mixed sizes 4..64, DCT2 / skip / DST7 / DCT8 MTS pairs,
implicit MTS, QP 0..63, RDOQ and intra-picture rounding, 8- and 10-bit; every
tile choice (fixed, autotuned, each group size) bit-exact."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def make_batch(n, bd, seed, kernel_bench_mix=False):
    """Seeded block list.  kernel_bench_mix: sizes from {4..64}^2 with a geometric
    tail biased to 8 and 16, residuals 11-bit Laplacian (scale 12), DCT2 70 % /
    DST7-DCT8 MTS pairs 30 % restricted to sides <= 32, QP uniform in [22, 42]."""
    from xin26x_gb300 import _lib
    rng = np.random.default_rng(seed)
    blocks = (_lib.xin_gpu_tq_block * n)()
    off = 0
    lg_p = np.array([0.12, 0.34, 0.30, 0.16, 0.08])
    for i in range(n):
        lw, lh = (int(rng.choice(5, p=lg_p)) + 2, int(rng.choice(5, p=lg_p)) + 2)
        if kernel_bench_mix:
            mts = 0 if rng.random() < 0.7 or lw > 5 or lh > 5 else int(rng.integers(2, 6))
            qp = int(rng.integers(22, 43))
            flags = 0
        else:
            mts = int(rng.integers(0, 6))
            if mts >= 1 and (lw > 5 or lh > 5):
                mts = 0
            qp = int(rng.integers(0, 64))
            flags = int(rng.integers(0, 32))
        blocks[i].offset, blocks[i].log2w, blocks[i].log2h = off, lw, lh
        blocks[i].mts, blocks[i].flags, blocks[i].qp = mts, flags, qp
        off += 1 << (lw + lh)
    lim = 1023 if kernel_bench_mix else (1 << bd) - 1
    scale = 12 if kernel_bench_mix else 60
    resid = np.clip(np.rint(rng.laplace(0, scale, size=off)), -lim, lim)
    return blocks, resid.astype(np.int16 if bd == 8 else np.int32)


def oracle_batch(o, blocks, resid):
    n = len(blocks)
    q, r, ro = np.zeros_like(resid), np.zeros_like(resid), np.zeros_like(resid)
    nz = np.zeros(n, np.uint64)
    for i in range(n):
        b = blocks[i]
        w, h, off = 1 << b.log2w, 1 << b.log2h, b.offset
        f = b.flags
        o.tq_block(O.ptr(resid, off), w, w, h, 1 if f & 2 else 0, b.mts, b.qp, 1 if f & 4 else 0, 1 if f & 8 else 0,
                   1 if f & 1 else 0, 1 if f & 16 else 0, O.ptr(q, off), O.ptr(r, off), O.ptr(ro, off), w, O.ptr(nz, i))
    return q, r, ro, nz


@pytest.mark.parametrize("bd", (8, 10))
def test_tq_batch_matches_oracle_every_tile(bd):
    from xin26x_gb300 import _lib
    g = _lib.load(bd)
    assert g.xin_gpu_init(0) == 0
    o = O.oracle(bd)
    blocks, resid = make_batch(600, bd, seed=bd)
    want = oracle_batch(o, blocks, resid)
    for tile in (0, -1, 32, 64, 128, 256, -1):
        q, r, ro = np.zeros_like(resid), np.zeros_like(resid), np.zeros_like(resid)
        nz = np.zeros(len(blocks), np.uint64)
        st = g.xin_gpu_tq_batch(blocks, len(blocks), resid.ctypes.data, q.ctypes.data, r.ctypes.data, ro.ctypes.data,
                                nz.ctypes.data, resid.size, tile)
        assert st == 0, g.xin_gpu_last_error()
        for name, a, b in zip(("q", "r", "resid_out", "nz"), (q, r, ro, nz), want):
            bad = np.nonzero(a != b)[0]
            assert bad.size == 0, (bd, tile, name, bad[:5])


def test_tq_batch_kernel_bench_mix_and_errors():
    from xin26x_gb300 import _lib
    g = _lib.load(10)
    o = O.oracle(10)
    blocks, resid = make_batch(2000, 10, seed=7, kernel_bench_mix=True)
    want = oracle_batch(o, blocks, resid)
    q, r, ro = np.zeros_like(resid), np.zeros_like(resid), np.zeros_like(resid)
    nz = np.zeros(len(blocks), np.uint64)
    assert g.xin_gpu_tq_batch(blocks, len(blocks), resid.ctypes.data, q.ctypes.data, r.ctypes.data, ro.ctypes.data,
                              nz.ctypes.data, resid.size, -1) == 0
    for a, b in zip((q, r, ro, nz), want):
        assert np.array_equal(a, b)
    # a block reaching past the arrays, and a 64-point skip or DST7, are refused before any launch
    bad = (_lib.xin_gpu_tq_block * 1)()
    bad[0].offset, bad[0].log2w, bad[0].log2h, bad[0].mts = resid.size - 8, 3, 3, 0
    assert g.xin_gpu_tq_batch(bad, 1, resid.ctypes.data, q.ctypes.data, r.ctypes.data, ro.ctypes.data, nz.ctypes.data,
                              resid.size, 0) == -2
    for mts in (1, 2):
        bad[0].offset, bad[0].log2w, bad[0].log2h, bad[0].mts = 0, 6, 4, mts
        assert g.xin_gpu_tq_batch(bad, 1, resid.ctypes.data, q.ctypes.data, r.ctypes.data, ro.ctypes.data,
                                  nz.ctypes.data, resid.size, 0) == -2
