"""Batched frame form (xin_gpu_stream_* through the C ABI, host buffers) against
the oracle's per-CU hot path: every CU of every level -- integer search,
sub-pel search, costs, non-zero maps, SSDs, coefficient planes and
reconstructed planes -- bit-exact on seeded synthetic pictures."""
import numpy as np
import pytest

from xin26x_gb300 import synth
from xin26x_gb300.frame import FrameStream
from tests import oracle_frame

pytestmark = pytest.mark.gpu


def _compare(out, ref, levels, label):
    recs, q, rec = ref
    cu = out["cu"]
    for name in ("mvx", "mvy", "int_cost", "cost"):
        bad = np.nonzero(cu[name] != recs[name])[0]
        assert bad.size == 0, (label, name, bad[:5], cu[bad[:5]], recs[bad[:5]])
    for name in ("nz", "ssd"):
        bad = np.nonzero(np.any(cu[name] != recs[name], axis=1))[0]
        assert bad.size == 0, (label, name, bad.size, bad[:5], cu[bad[:3]], recs[bad[:3]])
    for p in range(3):
        for li, (size, first, cx, cy) in enumerate(levels):
            s = size if p == 0 else size // 2
            hh, ww = cy * s, cx * s          # the area the level's CUs cover
            assert np.array_equal(out["q"][p][li, :hh, :ww], q[p][li, :hh, :ww]), (label, "q", p, size)
            assert np.array_equal(out["rec"][p][li, :hh, :ww], rec[p][li, :hh, :ww]), (label, "rec", p, size)


@pytest.mark.parametrize("bd", (8, 10))
# search ranges that are not multiples of 8 put the band's first column off the
# 8-sample grid the staging loads from; R = 3 wraps the 32 lanes of a pass over
# several candidate rows; widths that are not multiples of 64 leave partial tiles
@pytest.mark.parametrize("w,h,R,ctu", [(192, 128, 16, 64), (208, 120, 24, 64), (256, 136, 8, 128),
                                       (200, 104, 13, 64), (136, 72, 3, 64), (176, 96, 37, 128),
                                       (202, 100, 11, 64)])
def test_frame_pipeline_matches_oracle(bd, w, h, R, ctu):
    seq = synth.sequence(w, h, 3, seed=w + h + R, bitdepth=bd, objects=1)
    fs = FrameStream(w, h, ctu=ctu, search_range=R, out_q=True, out_rec=True, bitdepth=bd)
    try:
        fs.submit(*seq[0], qp=32, uv_qp=32, sad_lambda=70)
        fs.wait()
        for k in (1, 2):
            qp = 27 + 5 * k
            fs.submit(*seq[k], qp=qp, uv_qp=qp + 1, sad_lambda=40 + 30 * k)
            out = fs.wait()
            ref = oracle_frame.run(seq[k], seq[k - 1], fs.levels, ctu=ctu, search_range=R, qp=qp, uv_qp=qp + 1,
                                   sad_lambda=40 + 30 * k, bitdepth=bd)
            _compare(out, ref, fs.levels, (bd, w, h, R, k))
    finally:
        fs.close()


def test_frame_graph_and_direct_paths_agree():
    w, h = 192, 128
    seq = synth.sequence(w, h, 4, seed=3, objects=2)
    outs = []
    for graph in (True, False):
        fs = FrameStream(w, h, search_range=32, out_q=True, out_rec=True, use_graph=graph)
        res = []
        for k in range(4):
            fs.submit(*seq[k], qp=30 + k, uv_qp=31, sad_lambda=55)
            r = fs.wait()
            if k:
                res.append(r)
        fs.close()
        outs.append(res)
    for a, b in zip(*outs):
        assert np.array_equal(a["cu"], b["cu"])
        for p in range(3):
            assert np.array_equal(a["q"][p], b["q"][p]) and np.array_equal(a["rec"][p], b["rec"][p])


def test_frame_full_search_range_64():
    """The benchmark's search range on a 416x240 picture (every level), checked on a CU sample."""
    w, h, R = 416, 240, 64
    seq = synth.sequence(w, h, 2, seed=11)
    fs = FrameStream(w, h, search_range=R, out_q=True, out_rec=True)
    fs.submit(*seq[0], qp=32, uv_qp=32, sad_lambda=64)
    fs.wait()
    fs.submit(*seq[1], qp=32, uv_qp=32, sad_lambda=64)
    out = fs.wait()
    rng = np.random.default_rng(0)
    sample = []
    for (size, first, cx, cy) in fs.levels:
        n = cx * cy
        sample += list(first + rng.choice(n, size=min(n, 12), replace=False))
    recs, q, rec = oracle_frame.run(seq[1], seq[0], fs.levels, search_range=R, qp=32, uv_qp=32, sad_lambda=64, cus=sample)
    fs.close()
    for i in sample:
        for name in ("mvx", "mvy", "int_cost", "cost"):
            assert out["cu"][name][i] == recs[name][i], (i, name)
        assert np.array_equal(out["cu"]["nz"][i], recs["nz"][i]) and np.array_equal(out["cu"]["ssd"][i], recs["ssd"][i])


@pytest.mark.parametrize("bd,R", [(10, 64), (8, 256), (10, 256)])
def test_frame_wide_search_sampled(bd, R):
    """Search ranges up to the reference maximum (+-256, clamped by the picture window)
    at both bit depths, checked on a CU sample of every level."""
    w, h = 384, 256
    seq = synth.sequence(w, h, 2, seed=R + bd, bitdepth=bd, objects=2)
    fs = FrameStream(w, h, search_range=R, out_q=True, out_rec=True, bitdepth=bd)
    fs.submit(*seq[0], qp=32, uv_qp=32, sad_lambda=64)
    fs.wait()
    fs.submit(*seq[1], qp=37, uv_qp=37, sad_lambda=91)
    out = fs.wait()
    rng = np.random.default_rng(R)
    sample = []
    for (size, first, cx, cy), n_pick in zip(fs.levels, (2, 3, 6, 12)):
        n = cx * cy
        sample += list(first + rng.choice(n, size=min(n, n_pick), replace=False))
    recs, q, rec = oracle_frame.run(seq[1], seq[0], fs.levels, search_range=R, qp=37, uv_qp=37, sad_lambda=91,
                                    bitdepth=bd, cus=sample)
    fs.close()
    for i in sample:
        for name in ("mvx", "mvy", "int_cost", "cost"):
            assert out["cu"][name][i] == recs[name][i], (bd, R, i, name)
        assert np.array_equal(out["cu"]["nz"][i], recs["nz"][i]) and np.array_equal(out["cu"]["ssd"][i], recs["ssd"][i])


@pytest.mark.parametrize("dpb,refs,tu_mode,graph", [(0, 1, 0, True), (3, 1, 0, True), (3, 1, 0, False), (3, 1, 1, True),
                                                    (4, 2, 0, True)])
def test_frame_two_in_flight_equals_one_at_a_time(dpb, refs, tu_mode, graph):
    """Two pictures in flight (submit k + 1 before collecting k) give the same results
    as submit / wait one picture at a time; a third submit and an empty wait are refused.
    With a slot more than the references need (dpb 3 for one reference, 4 for two),
    picture k + 1 starts once picture k's planes are written, beside k's tails."""
    w, h = 256, 192
    seq = synth.sequence(w, h, 6, seed=5, objects=2)
    kw = {"dpb": dpb, "refs": refs, "tu_mode": tu_mode, "use_graph": graph}
    ref = []
    fs = FrameStream(w, h, search_range=24, out_q=True, out_rec=True, **kw)
    for k in range(6):
        fs.submit(*seq[k], qp=27 + k, uv_qp=28 + k, sad_lambda=50 + k)
        r = fs.wait()
        if k:
            ref.append(r)
    fs.close()
    fs = FrameStream(w, h, search_range=24, out_q=True, out_rec=True, **kw)
    got = []
    fs.submit(*seq[0], qp=27, uv_qp=28, sad_lambda=50)
    fs.submit(*seq[1], qp=28, uv_qp=29, sad_lambda=51)
    with pytest.raises(RuntimeError, match=r"\(-6\)"):
        fs.submit(*seq[2], qp=29, uv_qp=30, sad_lambda=52)
    fs.wait()                                   # picture 0: the reference only
    for k in range(2, 6):
        fs.submit(*seq[k], qp=27 + k, uv_qp=28 + k, sad_lambda=50 + k)
        got.append(fs.wait())
    got.append(fs.wait())
    with pytest.raises(RuntimeError, match=r"\(-6\)"):
        fs.wait()
    fs.close()
    for a, b in zip(ref, got):
        assert np.array_equal(a["cu"], b["cu"])
        for p in range(3):
            assert np.array_equal(a["q"][p], b["q"][p]) and np.array_equal(a["rec"][p], b["rec"][p])


@pytest.mark.parametrize("w,h,R,ctu", [(192, 128, 16, 64), (416, 240, 64, 64), (256, 136, 24, 128),
                                       (200, 104, 13, 64)])
def test_frame_8bit_input_in_10bit_build(w, h, R, ctu):
    """8-bit pictures into the 10-bit library (input_bitdepth 8: samples << 2, the
    integer search on the 8-bit samples with SADs x 4) give exactly the results
    of the same pictures shifted to 10 bits and fed as 10-bit samples (search on
    10-bit words), and of the 10-bit oracle on those samples -- every CU, level,
    coefficient plane and reconstructed plane; with and without graph capture."""
    seq = synth.sequence(w, h, 3, seed=w + R, objects=2)
    up = [tuple((p.astype(np.uint16) << 2) for p in f) for f in seq]
    runs = []
    for inb, frames, graph in ((8, seq, True), (0, up, True), (8, seq, False)):
        fs = FrameStream(w, h, ctu=ctu, search_range=R, out_q=True, out_rec=True, bitdepth=10, input_bitdepth=inb,
                         use_graph=graph)
        res = []
        try:
            fs.submit(*frames[0], qp=32, uv_qp=32, sad_lambda=256)
            fs.wait()
            for k in (1, 2):
                qp = 27 + 5 * k
                fs.submit(*frames[k], qp=qp, uv_qp=qp + 1, sad_lambda=160 + 120 * k)
                res.append(fs.wait())
        finally:
            fs.close()
        runs.append(res)
    for a, b in zip(runs[0], runs[1]):
        assert np.array_equal(a["cu"], b["cu"])
        for p in range(3):
            assert np.array_equal(a["q"][p], b["q"][p]) and np.array_equal(a["rec"][p], b["rec"][p])
    for a, b in zip(runs[0], runs[2]):
        assert np.array_equal(a["cu"], b["cu"])
    if R <= 24:
        levels = FrameStream(w, h, ctu=ctu, search_range=R, bitdepth=10).levels
        ref = oracle_frame.run(up[2], up[1], levels, ctu=ctu, search_range=R, qp=37, uv_qp=38, sad_lambda=400, bitdepth=10)
        _compare(runs[0][1], ref, levels, ("8-bit input", w, h, R))


@pytest.mark.parametrize("w,h", [(200, 104), (202, 100)])
@pytest.mark.parametrize("bd,inb", [(8, 0), (10, 0), (10, 8)])
def test_device_io_matches_host(bd, inb, w, h):
    """device_io streams (pictures already in GPU memory, results left there) fill
    their slots from the caller's device planes -- 8-bit samples << 2 in the
    10-bit library with input_bitdepth 8 -- and give the CU records of a
    host-buffer stream on the same pictures (an odd search range, a partial tile,
    a width that is not a multiple of 8)."""
    torch = pytest.importorskip("torch")
    import ctypes as C
    from xin26x_gb300 import _lib
    from xin26x_gb300.frame import CU_DTYPE

    R = 13
    seq = synth.sequence(w, h, 3, seed=11, bitdepth=inb or bd, objects=1)
    lam = [70, 40, 90]
    fs = FrameStream(w, h, search_range=R, out_q=False, out_rec=False, bitdepth=bd, input_bitdepth=inb)
    host = []
    try:
        for k in range(3):
            fs.submit(*seq[k], qp=30 + k, uv_qp=31 + k, sad_lambda=lam[k])
            out = fs.wait()
            if k:
                host.append(out["cu"].copy())
    finally:
        fs.close()

    class _Dev:      # a device byte range as a CUDA array for torch
        def __init__(self, ptr, n):
            self.__cuda_array_interface__ = {"shape": (n,), "typestr": "|u1", "data": (ptr, False), "version": 3}

    lib = _lib.load(bd)
    cfg = _lib.xin_gpu_stream_cfg(w, h, 64, R, 120, 0, 1, 1, inb)
    hs = C.c_void_p()
    assert lib.xin_gpu_stream_open(C.byref(cfg), C.byref(hs)) == 0, lib.xin_gpu_last_error()
    try:
        ncus = lib.xin_gpu_stream_num_cus(hs)
        dev = [[torch.from_numpy(np.ascontiguousarray(p)).cuda() for p in f] for f in seq]
        for k in range(3):
            pic = _lib.xin_gpu_picture()
            for i, t in enumerate(dev[k]):
                pic.plane[i] = t.data_ptr()
                pic.stride[i] = t.shape[1]
            pic.qp, pic.uv_qp, pic.sad_lambda = 30 + k, 31 + k, lam[k]
            assert lib.xin_gpu_frame_submit(hs, C.byref(pic)) == 0, lib.xin_gpu_last_error()
            res = _lib.xin_gpu_results()
            assert lib.xin_gpu_frame_wait(hs, C.byref(res), 60000) == 0, lib.xin_gpu_last_error()
            if k:
                cu, q, r = C.c_void_p(), (C.c_void_p * 3)(), (C.c_void_p * 3)()
                assert lib.xin_gpu_stream_device_results(hs, C.byref(cu), q, r) == 0
                raw = torch.as_tensor(_Dev(cu.value, ncus * CU_DTYPE.itemsize), device="cuda").cpu().numpy()
                got = raw.view(CU_DTYPE)
                assert np.array_equal(got, host[k - 1]), (bd, inb, k)
    finally:
        lib.xin_gpu_stream_close(hs)


def test_frame_1080p_benchmark_configuration():
    """The benchmark's own workload compared in full, as its end-to-end leg runs it:
    the first four pictures of bench.py's 1920x1080 stream (8-bit 4:2:0 into the
    10-bit library, input_bitdepth 8), +-64 exhaustive search, CU levels
    64/32/16/8, QPs 32, 37 and 27 with their lambdas; three picture slots, both
    autotuners run after picture 1, pictures 2 and 3 in flight together (picture
    3 starting beside picture 2's tails).  Every CU record and every coefficient
    and reconstructed plane of every level against the oracle's 10-bit build on
    all host cores."""
    import ctypes as C
    import bench
    frames = bench.make_frames(4)
    fs = FrameStream(bench.W, bench.H, search_range=bench.SEARCH, levels=bench.LEVELS, out_q=True, out_rec=True,
                     bitdepth=bench.BD, input_bitdepth=bench.IN_BD, dpb=3)
    qps = {1: 32, 2: 37, 3: 27}

    def check(k, out):
        cur, ref = [tuple(p.astype(np.uint16) << (bench.BD - bench.IN_BD) for p in f) for f in (frames[k], frames[k - 1])]
        want = oracle_frame.run(cur, ref, fs.levels, search_range=bench.SEARCH, qp=qps[k], uv_qp=qps[k],
                                sad_lambda=bench.LAMBDA_BD[qps[k]], bitdepth=bench.BD, threads=0)
        _compare(out, want, fs.levels, ("1080p", k))

    try:
        assert sum(cx * cy for (_, _, cx, cy) in fs.levels) == fs.ncus
        fs.submit(*frames[0], qp=32, uv_qp=32, sad_lambda=bench.LAMBDA_BD[32])
        fs.wait()
        fs.submit(*frames[1], qp=32, uv_qp=32, sad_lambda=bench.LAMBDA_BD[32])
        check(1, fs.wait())
        assert fs.lib.xin_gpu_stream_tune_search(fs.h, None, None) == 0, fs.lib.xin_gpu_last_error()
        cpb = (C.c_int32 * 2)()
        assert fs.lib.xin_gpu_stream_tune_tails(fs.h, cpb, None) == 0, fs.lib.xin_gpu_last_error()
        for k in (2, 3):
            fs.submit(*frames[k], qp=qps[k], uv_qp=qps[k], sad_lambda=bench.LAMBDA_BD[qps[k]])
        outs = {k: fs.wait() for k in (2, 3)}
        for k in (2, 3):
            check(k, outs[k])
    finally:
        fs.close()


def test_frame_wait_timeout_then_collect():
    """xin_gpu_frame_wait with a 0 ms limit right after a 1080p submit returns
    XIN_GPU_ERR_TIMEOUT (the picture takes about a millisecond); the picture is
    then collected normally and equals the same picture through a stream that
    never timed out."""
    import ctypes as C
    from xin26x_gb300 import _lib
    w, h = 1920, 1080
    seq = synth.sequence(w, h, 2, seed=5, objects=2)
    outs = []
    for probe in (True, False):
        fs = FrameStream(w, h, search_range=64, out_q=True, out_rec=False)
        try:
            fs.submit(*seq[0], qp=32, uv_qp=32, sad_lambda=64)
            fs.wait()
            fs.submit(*seq[1], qp=32, uv_qp=32, sad_lambda=64)
            if probe:
                res = _lib.xin_gpu_results()
                assert fs.lib.xin_gpu_frame_wait(fs.h, C.byref(res), 0) == -5
                assert fs.lib.xin_gpu_last_status() == -5
            outs.append(fs.wait())
        finally:
            fs.close()
    assert np.array_equal(outs[0]["cu"], outs[1]["cu"])
    for p in range(3):
        assert np.array_equal(outs[0]["q"][p], outs[1]["q"][p])


@pytest.mark.parametrize("bd,mode", [(8, 0), (10, 1)])
def test_frame_tma_wait_bound_is_reported_and_recovers(bd, mode):
    """The TMA loads of the quarter-pel planes' tiles are waited for with a
    bounded poll.  With the bound set to 0 polls every wait gives up at once:
    frame_wait reports XIN_GPU_ERR_TIMEOUT for that picture (the kernel then
    stages its tiles with plain loads once the copies have landed), and after
    the default bound is restored the next picture equals the same picture
    through a stream that never gave up."""
    w, h = 192, 128
    seq = synth.sequence(w, h, 3, seed=77, bitdepth=bd, objects=2)
    outs = []
    for probe in (True, False):
        fs = FrameStream(w, h, search_range=16, out_q=True, out_rec=True, bitdepth=bd, search_mode=mode)
        try:
            fs.submit(*seq[0], qp=32, uv_qp=32, sad_lambda=64)
            fs.wait()
            if probe:
                assert fs.lib.xin_gpu_stream_set_wait_tries(fs.h, 0) == 0
            fs.submit(*seq[1], qp=32, uv_qp=32, sad_lambda=64)
            if probe:
                with pytest.raises(RuntimeError, match=r"\(-5\).*bound"):
                    fs.wait()
                assert fs.lib.xin_gpu_stream_set_wait_tries(fs.h, -1) == 0
                assert fs.lib.xin_gpu_stream_set_wait_tries(fs.h, -2) == -2
            else:
                fs.wait()
            fs.submit(*seq[2], qp=32, uv_qp=32, sad_lambda=64)
            outs.append(fs.wait())
        finally:
            fs.close()
    for k in ("cu",):
        assert np.array_equal(outs[0][k], outs[1][k])
    for p in range(3):
        assert np.array_equal(outs[0]["q"][p], outs[1]["q"][p])
        assert np.array_equal(outs[0]["rec"][p], outs[1]["rec"][p])


@pytest.mark.parametrize("bd,inb", [(8, 0), (10, 0), (10, 8)])
@pytest.mark.parametrize("w,h,R,ctu", [(192, 128, 16, 64), (208, 120, 64, 64), (200, 104, 37, 128), (384, 256, 256, 128)])
def test_frame_hier_search_matches_oracle(bd, inb, w, h, R, ctu):
    """search_mode 1 (search by resolution levels): every CU of every level, the
    coefficient and reconstructed planes, against the oracle's per-CU hot path
    with orc_me_hier on the oracle's own 1/2 and 1/4 planes; search ranges up to
    the reference maximum +-256, 8-bit pictures into the 10-bit library."""
    seq = synth.sequence(w, h, 3, seed=w + R, bitdepth=8 if inb == 8 else bd, objects=2)
    fs = FrameStream(w, h, ctu=ctu, search_range=R, out_q=True, out_rec=True, bitdepth=bd, input_bitdepth=inb,
                     search_mode=1)
    try:
        fs.submit(*seq[0], qp=32, uv_qp=32, sad_lambda=64)
        fs.wait()
        for k in (1, 2):
            qp = 27 + 5 * k
            lam = (40 + 30 * k) << (2 if inb == 8 else 0)
            fs.submit(*seq[k], qp=qp, uv_qp=qp, sad_lambda=lam)
            out = fs.wait()
            cur, ref = seq[k], seq[k - 1]
            if inb == 8:
                cur, ref = [tuple(p.astype(np.uint16) << 2 for p in f) for f in (cur, ref)]
            want = oracle_frame.run(cur, ref, fs.levels, ctu=ctu, search_range=R, qp=qp, uv_qp=qp, sad_lambda=lam,
                                    bitdepth=bd, threads=0, search_mode=1)
            _compare(out, want, fs.levels, ("hier", bd, inb, w, h, R, k))
    finally:
        fs.close()


@pytest.mark.parametrize("bd,inb,search_mode", [(8, 0, 0), (10, 0, 1), (10, 8, 0), (8, 0, 1)])
@pytest.mark.parametrize("w,h,R", [(192, 128, 16), (200, 104, 24)])
def test_frame_bi_matches_oracle(bd, inb, search_mode, w, h, R):
    """refs 2 (two references and the bi search): picture 1 (lists 0 and 1 both
    picture 0), pictures 2 and 3 (list 0 the previous picture, list 1 the one
    before) and picture 8 (a graph captured for picture 2 run again): every CU's
    list-0 and list-1 searches, bi pair, bi cost and choice, and the coded
    prediction's coefficient and reconstructed planes, against the oracle's
    restatement of Xin266InterBiSearch and of the bi motion compensation (pinned
    to the reference's C)."""
    from xin26x_gb300.frame import BI_DTYPE
    seq = synth.sequence(w, h, 9, seed=w + h + R, bitdepth=8 if inb == 8 else bd, objects=3)
    fs = FrameStream(w, h, search_range=R, out_q=True, out_rec=True, bitdepth=bd, input_bitdepth=inb,
                     search_mode=search_mode, refs=2)
    dirs = np.zeros(4, np.int64)
    try:
        fs.submit(*seq[0], qp=32, uv_qp=32, sad_lambda=64)
        fs.wait()
        for k in range(1, 9):
            qp = 27 + (k % 3) * 5
            lam = (40 + 10 * k) << (2 if inb == 8 else 0)
            fs.submit(*seq[k], qp=qp, uv_qp=qp, sad_lambda=lam)
            out = fs.wait()
            if k not in (1, 2, 3, 8):
                continue
            cur, r0, r1 = seq[k], seq[k - 1], seq[max(k - 2, 0)]
            if inb == 8:
                cur, r0, r1 = [tuple(p.astype(np.uint16) << 2 for p in f) for f in (cur, r0, r1)]
            want = oracle_frame.run(cur, r0, fs.levels, search_range=R, qp=qp, uv_qp=qp, sad_lambda=lam, bitdepth=bd,
                                    threads=0, search_mode=search_mode, ref1=r1)
            label = ("bi", bd, inb, search_mode, w, h, R, k)
            _compare(out, want[:3], fs.levels, label)
            got, exp = out["bi"], want[3]
            for name in BI_DTYPE.names:
                bad = np.nonzero(np.any((got[name] != exp[name]).reshape(len(got), -1), axis=1))[0]
                assert bad.size == 0, (label, name, bad[:5], got[bad[:5]], exp[bad[:5]])
            dirs += np.bincount(got["inter_dir"].astype(np.int64), minlength=4)[:4]
    finally:
        fs.close()
    assert dirs[0] == 0 and dirs[3] > 0 and dirs[1] + dirs[2] > 0, dirs   # both kinds of choice occur


@pytest.mark.parametrize("bd,inb,search_mode,tu_mode", [(8, 0, 0, 0), (10, 8, 1, 1)])
def test_frame_random_access_gop_matches_oracle(bd, inb, search_mode, tu_mode):
    """Two GOPs of 8 in random-access coding order (synth.ra_gop) with the
    references named per picture (xin_gpu_frame_submit_refs; dpb 12, the least
    that two GOPs of 8 need -- picture 12, POC 9, reaches back to picture 1, POC 8): key pictures from the previous key
    picture, B pictures from their past and future references.  Selected
    pictures of both GOPs against the oracle with those references; references
    out of reach are refused."""
    from xin26x_gb300 import synth as S
    from xin26x_gb300.frame import BI_DTYPE
    w, h, R = 192, 128, 16
    ctx = S.contexts(np.random.default_rng(5), 1)[0] if tu_mode else None
    seq = synth.sequence(w, h, 17, seed=w + 17 + bd, bitdepth=8 if inb == 8 else bd, objects=3)
    order = S.ra_gop(8, 2)
    fs = FrameStream(w, h, search_range=R, out_q=True, out_rec=True, bitdepth=bd, input_bitdepth=inb,
                     search_mode=search_mode, tu_mode=tu_mode, contexts=ctx, refs=2, dpb=12)
    num = {0: 0}                     # POC -> picture number (submit order)
    try:
        fs.submit(*seq[0], qp=27, uv_qp=27, sad_lambda=64)
        fs.wait()
        for n, (poc, r0, r1) in enumerate(order, start=1):
            qp, lam = (27, 32, 37)[n % 3], (40 + 5 * n) << (2 if inb == 8 else 0)
            fs.submit(*seq[poc], qp=qp, uv_qp=qp, sad_lambda=lam, ref0=num[r0], ref1=num[r1])
            num[poc] = n
            out = fs.wait()
            if poc not in (8, 2, 5, 16, 12, 15):
                continue
            cur, p0, p1 = seq[poc], seq[r0], seq[r1]
            if inb == 8:
                cur, p0, p1 = [tuple(p.astype(np.uint16) << 2 for p in f) for f in (cur, p0, p1)]
            want = oracle_frame.run(cur, p0, fs.levels, search_range=R, qp=qp, uv_qp=qp, sad_lambda=lam, bitdepth=bd,
                                    threads=0, search_mode=search_mode, tu_mode=tu_mode, contexts=ctx, ref1=p1)
            label = ("ra", bd, inb, search_mode, tu_mode, poc)
            _compare(out, want[:3], fs.levels, label)
            if tu_mode:
                for name in ("satd_cost", "ncand", "nz", "ssd"):
                    bad = np.nonzero(np.any((out["mts"][name] != want[3][name]).reshape(len(out["mts"]), -1), axis=1))[0]
                    assert bad.size == 0, (label, name, bad[:5])
            for name in BI_DTYPE.names:
                bad = np.nonzero(np.any((out["bi"][name] != want[-1][name]).reshape(len(out["bi"]), -1), axis=1))[0]
                assert bad.size == 0, (label, name, bad[:5], out["bi"][bad[:5]], want[-1][bad[:5]])
        # 17 pictures submitted: picture 17 may reach back to picture 6 (dpb 12), not further
        for r0, r1 in ((5, 16), (16, 17), (16, 5)):
            with pytest.raises(RuntimeError, match="out of reach"):
                fs.submit(*seq[1], qp=32, uv_qp=32, sad_lambda=64, ref0=r0, ref1=r1)
    finally:
        fs.close()


@pytest.mark.parametrize("bd,inb,R", [(8, 0, 64), (10, 8, 24)])
def test_frame_search_tuning_keeps_results(bd, inb, R):
    """xin_gpu_stream_tune_search: the geometry it picks (timed on the last
    picture) changes no result -- pictures after the tuning equal those of an
    untuned stream on the same input, every record and plane."""
    import ctypes as C
    w, h = 416, 240
    seq = synth.sequence(w, h, 5, seed=99 + bd, bitdepth=8 if inb == 8 else bd, objects=2)
    outs = []
    for tune in (False, True):
        fs = FrameStream(w, h, search_range=R, out_q=True, out_rec=True, bitdepth=bd, input_bitdepth=inb)
        try:
            got = []
            for k in range(5):
                fs.submit(*seq[k], qp=32, uv_qp=32, sad_lambda=64 << (2 if inb == 8 else 0))
                got.append(fs.wait())
                if tune and k == 1:
                    bands, ms = C.c_int32(), (C.c_float * 2)()
                    assert fs.lib.xin_gpu_stream_tune_search(fs.h, C.byref(bands), ms) == 0, fs.lib.xin_gpu_last_error()
                    assert bands.value >= 1 and ms[0] > 0 and 0 < ms[1] <= ms[0]
            outs.append(got)
        finally:
            fs.close()
    for k in range(2, 5):
        a, b = outs[0][k], outs[1][k]
        assert np.array_equal(a["cu"], b["cu"]), k
        for p in range(3):
            assert np.array_equal(a["q"][p], b["q"][p]) and np.array_equal(a["rec"][p], b["rec"][p]), (k, p)


def test_frame_tail_tuning_keeps_results():
    """xin_gpu_stream_tune_tails: the CUs per CTA it picks for the 16 x 16 and
    8 x 8 tails (timed on the last picture) change no result -- pictures after
    the tuning equal those of an untuned stream, every record and plane; a
    stream with two references is refused."""
    import ctypes as C
    w, h = 416, 240
    seq = synth.sequence(w, h, 5, seed=77, bitdepth=8, objects=2)
    outs, picked = [], None
    for tune in (False, True):
        fs = FrameStream(w, h, search_range=16, out_q=True, out_rec=True)
        try:
            got = []
            for k in range(5):
                fs.submit(*seq[k], qp=32, uv_qp=32, sad_lambda=64)
                got.append(fs.wait())
                if tune and k == 1:
                    cpb, ms = (C.c_int32 * 2)(), (C.c_float * 6)()
                    assert fs.lib.xin_gpu_stream_tune_tails(fs.h, cpb, ms) == 0, fs.lib.xin_gpu_last_error()
                    picked = list(cpb)
                    assert all(c in (2, 4, 8) for c in picked) and all(ms[i] > 0 for i in range(6))
            outs.append(got)
        finally:
            fs.close()
    for k in range(2, 5):
        a, b = outs[0][k], outs[1][k]
        assert np.array_equal(a["cu"], b["cu"]), (k, picked)
        for p in range(3):
            assert np.array_equal(a["q"][p], b["q"][p]) and np.array_equal(a["rec"][p], b["rec"][p]), (k, p, picked)
    fs = FrameStream(w, h, search_range=16, out_q=False, out_rec=False, refs=2)
    try:
        for k in range(2):
            fs.submit(*seq[k], qp=32, uv_qp=32, sad_lambda=64)
            fs.wait()
        assert fs.lib.xin_gpu_stream_tune_tails(fs.h, None, None) == -6
    finally:
        fs.close()


def test_frame_bi_needs_levels_up_to_64():
    """refs 2 is refused with the 128 x 128 level, and more than two references."""
    for kw in ({"ctu": 128, "search_mode": 1, "levels": (128, 64), "refs": 2}, {"refs": 3}):
        with pytest.raises(RuntimeError, match="two references need CU levels up to 64"):
            FrameStream(256, 256, search_range=16, **kw)


@pytest.mark.parametrize("bd,inb,search_mode", [(8, 0, 0), (10, 0, 1), (10, 8, 1)])
@pytest.mark.parametrize("w,h,R", [(192, 128, 16), (200, 104, 24)])
def test_frame_preset4_tu_matches_oracle(bd, inb, search_mode, w, h, R):
    """tu_mode 1 (the preset-4 TU work): for every CU of every level, every transform
    candidate (luma DCT2 and MTS 2..5 up to 32, chroma DCT2) through dependent
    quantisation, inverse transform and reconstruction -- each candidate's
    non-zero map and SSD, the DCT2 candidate's coefficient and reconstructed
    planes, the SATD cost -- against the oracle's restatement of
    Xin266Transform's DepQuant branch (pinned to the reference's C) on seeded
    context sets and QPs 12 .. 37."""
    from xin26x_gb300 import synth as S
    rng = np.random.default_rng(w + R + bd)
    ctx = S.contexts(rng, 1)[0]
    seq = synth.sequence(w, h, 3, seed=w + h, bitdepth=8 if inb == 8 else bd, objects=2)
    fs = FrameStream(w, h, search_range=R, out_q=True, out_rec=True, bitdepth=bd, input_bitdepth=inb,
                     search_mode=search_mode, tu_mode=1, contexts=ctx)
    try:
        fs.submit(*seq[0], qp=22, uv_qp=22, sad_lambda=64)
        fs.wait()
        for k, qp in ((1, 12), (2, 27 if bd == 10 else 37)):
            lam = 50 << (2 if inb == 8 else 0)
            fs.submit(*seq[k], qp=qp, uv_qp=qp + 1, sad_lambda=lam)
            out = fs.wait()
            cur, ref = seq[k], seq[k - 1]
            if inb == 8:
                cur, ref = [tuple(p.astype(np.uint16) << 2 for p in f) for f in (cur, ref)]
            recs, q, rec, mts = oracle_frame.run(cur, ref, fs.levels, search_range=R, qp=qp, uv_qp=qp + 1, sad_lambda=lam,
                                                 bitdepth=bd, threads=0, search_mode=search_mode, tu_mode=1,
                                                 contexts=ctx)
            _compare(out, (recs, q, rec), fs.levels, ("tu", bd, inb, w, h, R, k))
            for name in ("satd_cost", "ncand", "nz", "ssd"):
                bad = np.nonzero(np.any((out["mts"][name] != mts[name]).reshape(len(mts), -1), axis=1))[0]
                assert bad.size == 0, (name, bad[:5], out["mts"][bad[:3]], mts[bad[:3]])
    finally:
        fs.close()


@pytest.mark.parametrize("bd,inb,search_mode", [(8, 0, 0), (10, 8, 1)])
def test_frame_preset4_bi_matches_oracle(bd, inb, search_mode):
    """tu_mode 1 with two references: the bi search with SATD as the decision's
    distortion (the uni lists' final-prediction SATD costs and the averaged
    prediction's SATD), the coded prediction (list 0, list 1 or the pair) through
    every transform candidate and dependent quantisation, and the SATD cost with
    the coded MVs' bits, against the oracle for pictures 1 .. 3."""
    from xin26x_gb300 import synth as S
    from xin26x_gb300.frame import BI_DTYPE
    w, h, R = 192, 128, 16
    rng = np.random.default_rng(77 + bd)
    ctx = S.contexts(rng, 1)[0]
    seq = synth.sequence(w, h, 4, seed=w + bd, bitdepth=8 if inb == 8 else bd, objects=3)
    fs = FrameStream(w, h, search_range=R, out_q=True, out_rec=True, bitdepth=bd, input_bitdepth=inb,
                     search_mode=search_mode, tu_mode=1, contexts=ctx, refs=2)
    dirs = np.zeros(4, np.int64)
    try:
        fs.submit(*seq[0], qp=22, uv_qp=22, sad_lambda=64)
        fs.wait()
        for k in (1, 2, 3):
            qp, lam = 22 + 5 * k, (40 + 10 * k) << (2 if inb == 8 else 0)
            fs.submit(*seq[k], qp=qp, uv_qp=qp, sad_lambda=lam)
            out = fs.wait()
            cur, r0, r1 = seq[k], seq[k - 1], seq[max(k - 2, 0)]
            if inb == 8:
                cur, r0, r1 = [tuple(p.astype(np.uint16) << 2 for p in f) for f in (cur, r0, r1)]
            recs, q, rec, mts, bis = oracle_frame.run(cur, r0, fs.levels, search_range=R, qp=qp, uv_qp=qp, sad_lambda=lam,
                                                      bitdepth=bd, threads=0, search_mode=search_mode, tu_mode=1,
                                                      contexts=ctx, ref1=r1)
            label = ("p4bi", bd, inb, search_mode, k)
            _compare(out, (recs, q, rec), fs.levels, label)
            for name in ("satd_cost", "ncand", "nz", "ssd"):
                bad = np.nonzero(np.any((out["mts"][name] != mts[name]).reshape(len(mts), -1), axis=1))[0]
                assert bad.size == 0, (label, name, bad[:5], out["mts"][bad[:3]], mts[bad[:3]])
            for name in BI_DTYPE.names:
                bad = np.nonzero(np.any((out["bi"][name] != bis[name]).reshape(len(bis), -1), axis=1))[0]
                assert bad.size == 0, (label, name, bad[:5], out["bi"][bad[:5]], bis[bad[:5]])
            dirs += np.bincount(out["bi"]["inter_dir"].astype(np.int64), minlength=4)[:4]
    finally:
        fs.close()
    assert dirs[3] > 0 and dirs[1] + dirs[2] > 0, dirs


@pytest.mark.parametrize("bd,inb", [(8, 0), (10, 8)])
@pytest.mark.parametrize("w,h,R", [(384, 256, 64), (392, 264, 37)])
def test_frame_level_128_matches_oracle(bd, inb, w, h, R):
    """The 128 x 128 CU level (CTU 128, search by resolution levels) beside levels
    64 .. 8: every CU record, coefficient and reconstructed plane against the
    oracle, whose 128 x 128 CUs are coded as four 64 x 64 luma and four 32 x 32
    chroma TUs per plane; pictures whose sizes are not multiples of 128."""
    seq = synth.sequence(w, h, 3, seed=w + h + R, bitdepth=8 if inb == 8 else bd, objects=2)
    fs = FrameStream(w, h, ctu=128, search_range=R, levels=(128, 64, 32, 16, 8), out_q=True, out_rec=True, bitdepth=bd,
                     input_bitdepth=inb, search_mode=1)
    try:
        assert [lv[0] for lv in fs.levels] == [64, 32, 16, 8, 128]
        fs.submit(*seq[0], qp=32, uv_qp=32, sad_lambda=64)
        fs.wait()
        for k, qp in ((1, 22), (2, 37)):
            lam = 50 << (2 if inb == 8 else 0)
            fs.submit(*seq[k], qp=qp, uv_qp=qp, sad_lambda=lam)
            out = fs.wait()
            cur, ref = seq[k], seq[k - 1]
            if inb == 8:
                cur, ref = [tuple(p.astype(np.uint16) << 2 for p in f) for f in (cur, ref)]
            want = oracle_frame.run(cur, ref, fs.levels, ctu=128, search_range=R, qp=qp, uv_qp=qp, sad_lambda=lam,
                                    bitdepth=bd, threads=0, search_mode=1)
            _compare(out, want, fs.levels, ("128", bd, inb, w, h, R, k))
    finally:
        fs.close()


def test_frame_level_128_needs_ctu_128_and_search_by_levels():
    """The 128 x 128 level is refused with CTU 64, with the exhaustive search and
    with the preset-4 TU stage."""
    for kw in ({"ctu": 64, "search_mode": 1}, {"ctu": 128, "search_mode": 0}, {"ctu": 128, "search_mode": 1, "tu_mode": 1}):
        with pytest.raises(RuntimeError, match="128 x 128 level"):
            FrameStream(256, 256, search_range=16, levels=(128, 64), **kw)


def test_frame_preset4_1080p_two_in_flight():
    """The bench's preset-4 workload compared in full: bench.py's 1920x1080 pictures
    (8-bit into the 10-bit library), search by resolution levels, every transform
    candidate through the trellis with the bench's seeded context set, QPs 32 and
    37.  Pictures 1 and 2 are in flight together on a stream of three slots, as in
    the bench: picture 2 starts once picture 1's planes are written, beside its
    tails and TU stage, each on its own picture set and search keys.  Every CU
    record, transform-candidate record and plane of both against the oracle on
    all host cores."""
    import bench
    from xin26x_gb300 import synth as S
    frames = bench.make_frames(3)
    ctx = np.ascontiguousarray(S.contexts(np.random.default_rng(4), 1)[0])
    fs = FrameStream(bench.W, bench.H, search_range=bench.SEARCH, levels=bench.LEVELS, out_q=True, out_rec=True,
                     bitdepth=bench.BD, input_bitdepth=bench.IN_BD, search_mode=1, tu_mode=1, contexts=ctx, dpb=3)
    try:
        fs.submit(*frames[0], qp=32, uv_qp=32, sad_lambda=bench.LAMBDA_BD[32])
        fs.wait()
        qps = {1: 32, 2: 37}
        for k in (1, 2):
            fs.submit(*frames[k], qp=qps[k], uv_qp=qps[k], sad_lambda=bench.LAMBDA_BD[qps[k]])
        outs = {k: fs.wait() for k in (1, 2)}
        for k in (1, 2):
            cur, ref = [tuple(p.astype(np.uint16) << (bench.BD - bench.IN_BD) for p in f) for f in (frames[k], frames[k - 1])]
            recs, q, rec, mts = oracle_frame.run(cur, ref, fs.levels, search_range=bench.SEARCH, qp=qps[k], uv_qp=qps[k],
                                                 sad_lambda=bench.LAMBDA_BD[qps[k]], bitdepth=bench.BD, threads=0,
                                                 search_mode=1, tu_mode=1, contexts=ctx)
            _compare(outs[k], (recs, q, rec), fs.levels, ("1080p preset 4", k))
            for name in ("satd_cost", "ncand", "nz", "ssd"):
                bad = np.nonzero(np.any((outs[k]["mts"][name] != mts[name]).reshape(len(mts), -1), axis=1))[0]
                assert bad.size == 0, (name, k, bad[:5])
    finally:
        fs.close()


def test_frame_preset4_random_access_1080p():
    """The bench's random-access preset-4 workload (preset4_ra_1080p) compared in
    full at 1920x1080: the first pictures of the GOP 16 coding order -- POC 16
    (both lists POC 0) and POC 8 (list 0 POC 0, list 1 POC 16) -- through the
    stream the bench opens (8-bit into the 10-bit library, search by resolution
    levels, two references named per picture, dpb 32, the bi search with SATD,
    every transform candidate through the trellis), both pictures in flight
    together; every CU, bi and transform-candidate record and every plane
    against the oracle on all host cores."""
    import bench
    from xin26x_gb300 import synth as S
    from xin26x_gb300.frame import BI_DTYPE
    frames = bench.make_frames(17)
    ctx = np.ascontiguousarray(S.contexts(np.random.default_rng(4), 1)[0])
    fs = FrameStream(bench.W, bench.H, search_range=bench.SEARCH, levels=bench.LEVELS, out_q=True, out_rec=True,
                     bitdepth=bench.BD, input_bitdepth=bench.IN_BD, search_mode=1, tu_mode=1, contexts=ctx, refs=2, dpb=32)
    order = S.ra_gop(16, 1)[:2]                 # (16, 0, 0), (8, 0, 16)
    num = {0: 0}
    try:
        fs.submit(*frames[0], qp=32, uv_qp=32, sad_lambda=bench.LAMBDA_BD[32])
        fs.wait()
        qps = {16: 32, 8: 37}
        for k, (poc, r0, r1) in enumerate(order, start=1):
            fs.submit(*frames[poc], qp=qps[poc], uv_qp=qps[poc], sad_lambda=bench.LAMBDA_BD[qps[poc]], ref0=num[r0],
                      ref1=num[r1])
            num[poc] = k
        outs = {poc: fs.wait() for poc, _, _ in order}
        for poc, r0, r1 in order:
            cur, p0, p1 = [tuple(p.astype(np.uint16) << (bench.BD - bench.IN_BD) for p in f)
                           for f in (frames[poc], frames[r0], frames[r1])]
            recs, q, rec, mts, bis = oracle_frame.run(cur, p0, fs.levels, search_range=bench.SEARCH, qp=qps[poc],
                                                      uv_qp=qps[poc], sad_lambda=bench.LAMBDA_BD[qps[poc]],
                                                      bitdepth=bench.BD, threads=0, search_mode=1, tu_mode=1,
                                                      contexts=ctx, ref1=p1)
            _compare(outs[poc], (recs, q, rec), fs.levels, ("1080p random access", poc))
            for name in ("satd_cost", "ncand", "nz", "ssd"):
                bad = np.nonzero(np.any((outs[poc]["mts"][name] != mts[name]).reshape(len(mts), -1), axis=1))[0]
                assert bad.size == 0, (name, poc, bad[:5])
            for name in BI_DTYPE.names:
                bad = np.nonzero(np.any((outs[poc]["bi"][name] != bis[name]).reshape(len(bis), -1), axis=1))[0]
                assert bad.size == 0, (name, poc, bad[:5], outs[poc]["bi"][bad[:3]], bis[bad[:3]])
    finally:
        fs.close()


def test_frame_preset4_tu_qp_limit():
    """The trellis's parameters stop at QP 51: at 10 bits (QP + 12) a slice QP above
    39 is refused before any launch."""
    fs = FrameStream(64, 64, search_range=8, bitdepth=10, tu_mode=1)
    try:
        seq = synth.sequence(64, 64, 2, seed=1, bitdepth=10)
        fs.submit(*seq[0], qp=39, uv_qp=39, sad_lambda=64)
        fs.wait()
        with pytest.raises(RuntimeError, match="QP above 39"):
            fs.submit(*seq[1], qp=40, uv_qp=40, sad_lambda=64)
    finally:
        fs.close()
