"""Batched transform / quant (xin_gpu_tq_batch) against the oracle's per-block TU
path (orc_tq_block): mixed sizes 4..64, DCT2 / skip / DST7 / DCT8 MTS pairs,
implicit MTS, QP 0..63, RDOQ and intra-picture rounding, 8- and 10-bit; every
tile choice (fixed, autotuned, each group size) bit-exact.  The 65,536-block
kernel-bench mix is checked on a 2,000-block draw and at full size through the
device entry point (autotuned and fixed tiles give identical outputs)."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def make_batch(n, bd, seed, kernel_bench_mix=False):
    from xin26x_gb300 import synth
    return synth.tq_blocks(n, seed, bitdepth=bd, kernel_bench_mix=kernel_bench_mix)


def oracle_batch(o, blocks, resid):
    n = len(blocks)
    q, r, ro = np.zeros_like(resid), np.zeros_like(resid), np.zeros_like(resid)
    nz = np.zeros(n, np.uint64)
    for i in range(n):
        lw, lh, off, f = int(blocks["log2w"][i]), int(blocks["log2h"][i]), int(blocks["offset"][i]), int(blocks["flags"][i])
        w, h = 1 << lw, 1 << lh
        o.tq_block(O.ptr(resid, off), w, w, h, 1 if f & 2 else 0, int(blocks["mts"][i]), int(blocks["qp"][i]),
                   1 if f & 4 else 0, 1 if f & 8 else 0, 1 if f & 1 else 0, 1 if f & 16 else 0,
                   O.ptr(q, off), O.ptr(r, off), O.ptr(ro, off), w, O.ptr(nz, i))
    return q, r, ro, nz


@pytest.mark.parametrize("bd", (8, 10))
def test_tq_batch_matches_oracle_every_tile(bd):
    from xin26x_gb300 import _lib
    g = _lib.load(bd)
    assert g.xin_gpu_init(0) == 0
    o = O.oracle(bd)
    blocks, resid = make_batch(600, bd, seed=bd)
    want = oracle_batch(o, blocks, resid)
    for tile in (0, -1, 32, 64, 128, 256, -1, -2):
        q, r, ro = np.zeros_like(resid), np.zeros_like(resid), np.zeros_like(resid)
        nz = np.zeros(len(blocks), np.uint64)
        st = g.xin_gpu_tq_batch(blocks.ctypes.data, len(blocks), resid.ctypes.data, q.ctypes.data, r.ctypes.data, ro.ctypes.data,
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
    assert g.xin_gpu_tq_batch(blocks.ctypes.data, len(blocks), resid.ctypes.data, q.ctypes.data, r.ctypes.data, ro.ctypes.data,
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


def test_tq_batch_full_kernel_bench_autotuned_equals_fixed():
    """65,536 blocks on device arrays: autotuned tiles, fixed tiles and the tensor-core
    form bit-identical, and a seeded sample of 300 blocks bit-exact against the oracle."""
    import torch
    from xin26x_gb300 import _lib
    g = _lib.load(10)
    o = O.oracle(10)
    blocks, resid = make_batch(65536, 10, seed=65536, kernel_bench_mix=True)
    d_res = torch.from_numpy(resid).cuda()
    outs = []
    stream = torch.cuda.current_stream().cuda_stream
    for tile in (-1, 0, -2):
        q, r, ro = torch.zeros_like(d_res), torch.zeros_like(d_res), torch.zeros_like(d_res)
        nz = torch.zeros(len(blocks), dtype=torch.int64, device="cuda")
        used = (C.c_int32 * 49)()
        if tile != -1:
            st = g.xin_gpu_tq_batch_device(blocks.ctypes.data, len(blocks), d_res.data_ptr(), q.data_ptr(), r.data_ptr(),
                                           ro.data_ptr(), nz.data_ptr(), resid.size, tile, stream, used)
            assert st == 0, g.xin_gpu_last_error()
        else:   # the plan form: tune on the first run, then two asynchronous runs over the same outputs
            plan = C.c_void_p()
            assert g.xin_gpu_tq_plan_create(blocks.ctypes.data, len(blocks), resid.size, tile, C.byref(plan)) == 0
            for _ in range(3):
                assert g.xin_gpu_tq_plan_run(plan, d_res.data_ptr(), q.data_ptr(), r.data_ptr(), ro.data_ptr(),
                                             nz.data_ptr(), stream) == 0, g.xin_gpu_last_error()
            assert g.xin_gpu_tq_plan_tiles(plan, used) == 0
            g.xin_gpu_tq_plan_destroy(plan)
            torch.cuda.synchronize()
            assert all(u in (32, 64, 128, 256) for u, n in zip(used, np.bincount(
                blocks["log2w"].astype(int) * 7 + blocks["log2h"], minlength=49)) if n)
        assert all(u in (0, 32, 64, 128, 256) for u in used)
        outs.append([t.cpu().numpy() for t in (q, r, ro, nz)])
    for other in outs[1:]:             # fixed tiles and the tensor-core form agree with the autotuned run
        for a, b in zip(outs[0], other):
            assert np.array_equal(a, b)
    pick = np.random.default_rng(5).choice(len(blocks), 300, replace=False)
    q, r, ro, nz = outs[0]
    for i in pick:
        off, n = int(blocks["offset"][i]), 1 << (int(blocks["log2w"][i]) + int(blocks["log2h"][i]))
        sub = blocks[i:i + 1].copy()
        sub["offset"] = 0
        wq, wr, wro, wnz = oracle_batch(o, sub, resid[off:off + n].copy())
        assert np.array_equal(q[off:off + n], wq) and np.array_equal(r[off:off + n], wr)
        assert np.array_equal(ro[off:off + n], wro) and int(nz[i]) == int(wnz[0].astype(np.int64))


def test_tq_tensor_form_with_unaligned_offsets():
    """Blocks at offsets that are not multiples of 8 samples (which the tensor-core
    kernel's vector loads cannot take) go to the CUDA cores; the batch stays bit-exact."""
    from xin26x_gb300 import _lib
    g = _lib.load(10)
    o = O.oracle(10)
    blocks, packed = make_batch(300, 10, seed=77)
    resid = np.zeros(packed.size + 3 * len(blocks), packed.dtype)
    off = 0
    for i in range(len(blocks)):
        n = 1 << (int(blocks["log2w"][i]) + int(blocks["log2h"][i]))
        src = int(blocks["offset"][i])
        off += 3 * (i % 2)                      # every other block starts 3 samples later
        resid[off:off + n] = packed[src:src + n]
        blocks["offset"][i] = off
        off += n
    want = oracle_batch(o, blocks, resid)
    q, r, ro = np.zeros_like(resid), np.zeros_like(resid), np.zeros_like(resid)
    nz = np.zeros(len(blocks), np.uint64)
    assert g.xin_gpu_tq_batch(blocks.ctypes.data, len(blocks), resid.ctypes.data, q.ctypes.data, r.ctypes.data,
                              ro.ctypes.data, nz.ctypes.data, resid.size, -2) == 0, g.xin_gpu_last_error()
    for name, a, b in zip(("q", "r", "resid_out", "nz"), (q, r, ro, nz), want):
        assert np.array_equal(a, b), name


def test_tq_tensor_wait_timeout_is_reported_and_recovers():
    """The tensor-core engine's bounded MMA wait, made to give up at once (0 polls):
    the plan's status reports XIN_GPU_ERR_TIMEOUT without a hang, the flag is
    cleared by that report, and the same plan with the default limit then gives
    the oracle's outputs (the context stayed usable)."""
    import torch
    from xin26x_gb300 import _lib
    g = _lib.load(10)
    assert g.xin_gpu_init(0) == 0
    o = O.oracle(10)
    blocks, resid = make_batch(400, 10, seed=99, kernel_bench_mix=True)
    want = oracle_batch(o, blocks, resid)
    plan = C.c_void_p()
    assert g.xin_gpu_tq_plan_create(blocks.ctypes.data, len(blocks), resid.size, -2, C.byref(plan)) == 0
    try:
        d_res = torch.from_numpy(resid).cuda()
        outs = [torch.zeros_like(d_res) for _ in range(3)]
        d_nz = torch.zeros(len(blocks), dtype=torch.int64, device="cuda")

        def run():
            return g.xin_gpu_tq_plan_run(plan, d_res.data_ptr(), outs[0].data_ptr(), outs[1].data_ptr(),
                                         outs[2].data_ptr(), d_nz.data_ptr(), None)

        assert g.xin_gpu_tq_plan_set_wait_tries(plan, 0) == 0
        assert run() == 0
        assert g.xin_gpu_tq_plan_status(plan) == -5
        assert g.xin_gpu_tq_plan_status(plan) == 0          # reported once
        assert g.xin_gpu_tq_plan_set_wait_tries(plan, -1) == -2
        assert g.xin_gpu_tq_plan_set_wait_tries(plan, 1 << 26) == 0
        for t in outs:
            t.zero_()
        assert run() == 0
        assert g.xin_gpu_tq_plan_status(plan) == 0, g.xin_gpu_last_error()
        got = [t.cpu().numpy() for t in outs] + [d_nz.cpu().numpy().view(np.uint64)]
        for name, a, b in zip(("q", "r", "resid_out", "nz"), got, want):
            assert np.array_equal(a, b), name
    finally:
        g.xin_gpu_tq_plan_destroy(plan)
