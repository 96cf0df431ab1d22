"""The allocation-free forward 2-D DCT2 (xin_gpu_fdct2_wxh_noalloc) through the C ABI.

It is meant for callers that cannot call cudaMalloc -- a real-time host thread
that must not risk a device synchronisation, code recording a CUDA graph, a
fixed memory budget -- so the test hands it device buffers it allocated itself
(the entry point allocates nothing) and checks its output against the
allocating per-call form XinGpuFDct2WxH, bit for bit, on two calls in a row:
the second call reuses the shared scratch array that still holds the first
call's intermediate.  The two calls run on a host thread of their own that
has made no other library call, and the device's free memory is the same
before and after them: nothing was allocated on their behalf.  Also checks
that an oversized block is refused.

This file sorts last so that a run stopping at the first failure has run every
other test before it; it also passes alone in a fresh process.
"""
import ctypes as C
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("bd", (8, 10))
def test_noalloc_fdct2_matches_allocating_form(bd):
    import torch

    from xin26x_gb300 import _lib
    g = _lib.load(bd)
    assert g.xin_gpu_init(0) == 0, g.xin_gpu_last_error()
    torch.cuda.set_device(0)
    coef = np.int16 if bd == 8 else np.int32
    tcoef = torch.int16 if bd == 8 else torch.int32
    lim = (1 << bd) - 1
    rng = np.random.default_rng(42 + bd)
    stream = torch.cuda.current_stream().cuda_stream
    # two calls in a row, the second with a different shape and data; the expected
    # outputs come from the allocating form first, on this thread
    cases = []
    for (w, h) in [(64, 64), (16, 32)]:
        lw, lh = w.bit_length() - 1, h.bit_length() - 1
        s1, s2 = lw + bd + 6 - 15, lh + 6
        x = rng.integers(-lim, lim + 1, size=(h, w + 3)).astype(coef)
        want = np.zeros((h, w + 1), coef)
        g.XinGpuFDct2WxH(x.ctypes.data, w + 3, want.ctypes.data, w + 1, w, h, None, s1, s2)
        _lib.check(g, "XinGpuFDct2WxH")
        d_in = torch.from_numpy(x).cuda()
        d_out = torch.zeros((h, w + 1), dtype=tcoef, device="cuda")
        cases.append((w, h, s1, s2, want, d_in, d_out))
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    status = []

    def caller():
        for (w, h, s1, s2, _, d_in, d_out) in cases:
            status.append((g.xin_gpu_fdct2_wxh_noalloc(d_in.data_ptr(), w + 3, d_out.data_ptr(), w + 1, w, h, s1, s2,
                                                       stream), g.xin_gpu_last_error()))

    t = threading.Thread(target=caller)
    t.start()
    t.join()
    torch.cuda.synchronize()
    assert [st for st, _ in status] == [0, 0], status
    assert torch.cuda.mem_get_info()[0] == free0
    for (w, h, _, _, want, _, d_out) in cases:
        got = d_out.cpu().numpy()
        assert np.array_equal(got[:, :w], want[:, :w]), (bd, w, h)
        assert np.all(got[:, w:] == 0)      # nothing written outside the block

    d_in = torch.zeros((128, 128), dtype=tcoef, device="cuda")
    d_out = torch.zeros((128, 128), dtype=tcoef, device="cuda")
    st = g.xin_gpu_fdct2_wxh_noalloc(d_in.data_ptr(), 128, d_out.data_ptr(), 128, 128, 64, 7, 12, stream)
    assert st == -2 and b"exceeds" in g.xin_gpu_last_error()
