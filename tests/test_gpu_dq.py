"""Dependent quantisation on the GPU (xin_gpu_dep_quant_* / xin_gpu_dq_plan_* /
XinGpuDepQuant) against the oracle restatement of Xin266DepQuant
(h266_encoder/source/h266_dep_quant.c:1789), itself pinned to the reference's C
(test_oracle_vs_ref.py, test_oracle_golden.py).  Bit-exact q, r and non-zero
map for every block size 4..64, QP 0..51, Y / Cb / Cr, root cbf on and off,
several context sets, strided layouts, all-below-threshold blocks, saturated
coefficients, the 65,536-block kernel-bench mix, and the per-call form on the
reference's structure layout."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _oracle_blocks(o, blocks, t, sets, full=True):
    """Expected q, r, nz: zeros over each whole block, oracle output over its low 32x32."""
    q, r = np.zeros_like(t), np.zeros_like(t)
    nz = np.zeros(len(blocks), np.uint64)
    for i, b in enumerate(blocks):
        w, h, st, off = 1 << int(b["log2_w"]), 1 << int(b["log2_h"]), int(b["stride"]), int(b["offset"])
        ctx = np.ascontiguousarray(sets[int(b["ctx_set"])])
        o.dep_quant(O.ptr(t, off), st, w, h, int(b["qp"]), int(b["comp"]), ctx.ctypes.data, int(b["root_cbf"]),
                    O.ptr(q, off), O.ptr(r, off), O.ptr(nz, i))
    return q, r, nz


def _mixed(bd, seed, n_per_size=6, n_sets=3):
    """Every size twice over, strided rows, QP 0..51, varied magnitudes."""
    from xin26x_gb300 import synth as S
    rng = np.random.default_rng(seed)
    sizes = [(lw, lh) for lw in range(2, 7) for lh in range(2, 7)]
    rows = []
    off = 0
    for i in range(n_per_size * len(sizes)):
        lw, lh = sizes[i % len(sizes)]
        w, h = 1 << lw, 1 << lh
        stride = w + int(rng.choice([0, 0, 8, 24]))
        rows.append((off, stride, lw, lh, int(rng.integers(0, 52)), int(rng.integers(0, 3)), int(rng.integers(0, 2)),
                     int(rng.integers(0, n_sets))))
        off += h * stride
    blocks = np.zeros(len(rows), S.DQ_BLOCK_DTYPE)
    for i, (o_, st, lw, lh, qp, comp, root, cs) in enumerate(rows):
        blocks[i] = (o_, st, lw, lh, qp, comp, root if comp == 0 else 0, 0, cs)
    t = np.zeros(off, np.int16 if bd == 8 else np.int32)
    for i, b in enumerate(blocks):
        w, h, st, o_ = 1 << int(b["log2_w"]), 1 << int(b["log2_h"]), int(b["stride"]), int(b["offset"])
        view = t[o_:o_ + h * st].reshape(h, st)
        if i % 29 == 0:
            view[:, :w] = 0                                           # nothing above the threshold
        elif i % 31 == 0:
            view[:, :w] = np.where(rng.random((h, w)) < 0.5, 32767, -32768)
        else:
            view[:, :w] = S.coefficients(rng, w, h, bd, scale=0.4 if i % 7 == 0 else None)
    return blocks, t, S.contexts(rng, n_sets)


def _diff(name, a, b):
    bad = np.nonzero(a != b)[0]
    assert bad.size == 0, (name, bad[:8], a[bad[:8]], b[bad[:8]])


@pytest.mark.parametrize("bd", (8, 10))
def test_dep_quant_batch_matches_oracle(bd):
    from xin26x_gb300 import _lib
    g = _lib.load(bd)
    assert g.xin_gpu_init(0) == 0
    o = O.oracle(bd)
    blocks, t, sets = _mixed(bd, seed=30 + bd)
    want = _oracle_blocks(o, blocks, t, sets)
    q, r = np.full_like(t, 9), np.full_like(t, 9)
    nz = np.zeros(len(blocks), np.uint64)
    st = g.xin_gpu_dep_quant_batch(blocks.ctypes.data, len(blocks), t.ctypes.data, q.ctypes.data, r.ctypes.data,
                                   nz.ctypes.data, t.size, sets.ctypes.data, sets.shape[0])
    assert st == 0, g.xin_gpu_last_error()
    _diff("q", q, want[0])
    _diff("r", r, want[1])
    _diff("nz", nz, want[2])


@pytest.mark.parametrize("bd", (8, 10))
def test_dep_quant_plan_kernel_bench_mix(bd):
    """65,536 blocks of the kernel-bench shapes on device arrays through a plan:
    a 600-block sample equals the oracle, and a second run is identical."""
    import torch
    from xin26x_gb300 import _lib, synth as S
    g = _lib.load(bd)
    assert g.xin_gpu_init(0) == 0
    o = O.oracle(bd)
    blocks, t, sets = S.dq_blocks(65536, seed=11, bitdepth=bd, n_sets=4)
    dt = torch.from_numpy(t).cuda()
    dq, dr = torch.zeros_like(dt), torch.zeros_like(dt)
    dnz = torch.zeros(len(blocks), dtype=torch.int64, device="cuda")
    dsets = torch.from_numpy(sets.view(np.uint8).reshape(-1)).cuda()
    plan = C.c_void_p()
    assert g.xin_gpu_dq_plan_create(blocks.ctypes.data, len(blocks), t.size, sets.shape[0], C.byref(plan)) == 0, \
        g.xin_gpu_last_error()
    outs = []
    for _ in range(2):
        dq.fill_(7); dr.fill_(7)
        st = g.xin_gpu_dq_plan_run(plan, dt.data_ptr(), dq.data_ptr(), dr.data_ptr(), dnz.data_ptr(), dsets.data_ptr(),
                                   C.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert st == 0, g.xin_gpu_last_error()
        torch.cuda.synchronize()
        outs.append((dq.cpu().numpy(), dr.cpu().numpy(), dnz.cpu().numpy().view(np.uint64)))
    g.xin_gpu_dq_plan_destroy(plan)
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(a, b)
    q, r, nz = outs[0]
    rng = np.random.default_rng(5)
    idx = rng.choice(len(blocks), 600, replace=False)
    sub = blocks[idx]
    wq, wr, wnz = _oracle_blocks(o, sub, t, sets)
    for j, i in enumerate(idx):
        b = blocks[i]
        off, n = int(b["offset"]), (1 << int(b["log2_w"])) * (1 << int(b["log2_h"]))
        assert np.array_equal(q[off:off + n], wq[off:off + n]), i
        assert np.array_equal(r[off:off + n], wr[off:off + n]), i
        assert nz[i] == wnz[j], i
    # the workload is not degenerate: most blocks keep some level
    assert np.count_nonzero(nz) > len(blocks) // 2


@pytest.mark.parametrize("bd", (8, 10))
def test_dep_quant_per_call_on_reference_structs(bd):
    """XinGpuDepQuant with the XinDepQuant signature, fed structures laid out like
    the reference's xin_dep_quant / xin_fast_md_buf / xin_full_md_buf; writes only
    the low 32x32 of the block (the rest of the caller's array is untouched)."""
    from xin26x_gb300 import _lib, synth as S
    g = _lib.load(bd)
    assert g.xin_gpu_init(0) == 0
    o = O.oracle(bd)
    rng = np.random.default_rng(90 + bd)
    sets = S.contexts(rng, 1)
    ctx = np.ascontiguousarray(sets[0])
    dq_struct = (C.c_uint8 * 64)()
    C.c_void_p.from_address(C.addressof(dq_struct) + 8).value = ctx.ctypes.data
    full = (C.c_uint8 * 4096)()
    fast = (C.c_uint8 * 888)()
    C.c_void_p.from_address(C.addressof(fast) + 0).value = C.addressof(full)
    for i, (w, h) in enumerate([(4, 4), (8, 4), (16, 16), (32, 8), (64, 64), (32, 64), (8, 32), (16, 64)]):
        for comp in (0, 1, 2):
            for mode, tunum in ((3, 1), (0, 1), (0, 2)):
                C.c_uint32.from_address(C.addressof(fast) + 880).value = mode
                C.c_uint32.from_address(C.addressof(full) + 2184).value = tunum
                stride = w + 8
                qp = int(rng.integers(0, 52))
                t = np.zeros((h, stride), np.int16 if bd == 8 else np.int32)
                t[:, :w] = S.coefficients(rng, w, h, bd)
                q, r = np.full_like(t, 3), np.full_like(t, 3)
                nz = np.zeros(1, np.uint64)
                g.XinGpuDepQuant(C.addressof(dq_struct), C.addressof(fast), None, t.ctypes.data, r.ctypes.data,
                                 q.ctypes.data, stride, qp, w, h, nz.ctypes.data, comp)
                assert g.xin_gpu_last_status() == 0, g.xin_gpu_last_error()
                wq, wr, wnz = np.full_like(t, 3), np.full_like(t, 3), np.zeros(1, np.uint64)
                root = int(comp == 0 and mode != 3 and tunum == 1)
                o.dep_quant(O.ptr(t), stride, w, h, qp, comp, ctx.ctypes.data, root, O.ptr(wq), O.ptr(wr), wnz.ctypes.data)
                assert np.array_equal(q, wq) and np.array_equal(r, wr) and nz[0] == wnz[0], (w, h, comp, mode, tunum, qp)


def test_dep_quant_errors():
    from xin26x_gb300 import _lib, synth as S
    g = _lib.load(8)
    assert g.xin_gpu_init(0) == 0
    blocks = np.zeros(1, S.DQ_BLOCK_DTYPE)
    blocks[0] = (0, 8, 3, 3, 30, 0, 0, 0, 0)
    t = np.zeros(64, np.int16)
    q, r = np.zeros_like(t), np.zeros_like(t)
    nz = np.zeros(1, np.uint64)
    sets = S.contexts(np.random.default_rng(0), 1)

    def run(b, n=64, nsets=1):
        return g.xin_gpu_dep_quant_batch(b.ctypes.data, len(b), t.ctypes.data, q.ctypes.data, r.ctypes.data,
                                         nz.ctypes.data, n, sets.ctypes.data, nsets)
    assert run(blocks) == 0
    for field, val in (("qp", 52), ("log2_w", 7), ("log2_h", 1), ("comp", 3), ("ctx_set", 1), ("stride", 4)):
        b = blocks.copy()
        b[0][field] = val
        assert run(b) == -2, field
    assert run(blocks, n=63) == -2                  # block reaches past the array
    assert run(blocks, nsets=0) == -2
    q16 = np.zeros(16, np.int16)
    g.XinGpuDepQuant(None, None, None, q16.ctypes.data, q16.ctypes.data, q16.ctypes.data, 4, 30, 4, 4, nz.ctypes.data, 0)
    assert g.xin_gpu_last_status() == -2
