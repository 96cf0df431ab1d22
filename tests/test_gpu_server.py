"""Serving layer (xin_gpu_server_*): a stream's CU results through the server are
bit-identical to the same stream run alone through xin_gpu_frame_* (itself
checked against the oracle in test_gpu_frame.py), whether it shares the GPU with
other streams or not; admission by device footprint and by promised Mpixel/s;
join / leave while other streams run; argument and queue errors."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

R = 16


def _frames(w, h, n, seed):
    from xin26x_gb300 import synth
    return synth.sequence(w, h, n, seed=seed, objects=2)


def _alone(w, h, frames, **kw):
    from xin26x_gb300.frame import FrameStream
    fs = FrameStream(w, h, search_range=R, out_q=False, out_rec=False, **kw)
    out = []
    for k, f in enumerate(frames):
        fs.submit(*f, qp=27 + 5 * (k % 3), uv_qp=27 + 5 * (k % 3), sad_lambda=64)
        r = fs.wait()
        if k:
            out.append(r["cu"].copy())
    fs.close()
    return out


def _serve(streams, max_inflight=4, leave_after=None, kws=None):
    """streams: list of (w, h, frames).  Pictures are submitted round-robin;
    leave_after = (stream number, pictures) makes that stream leave early;
    kws: per stream extra stream options."""
    from xin26x_gb300.server import Server
    got = {}
    kws = kws or [{}] * len(streams)
    with Server(max_inflight=max_inflight, max_queue=2) as srv:
        sids = [srv.join(w, h, fps=30, search_range=R, **kw) for (w, h, _), kw in zip(streams, kws)]
        nxt = [0] * len(streams)
        limit = [len(f) for (_, _, f) in streams]
        if leave_after:
            limit[leave_after[0]] = leave_after[1]
        outstanding = 0
        left = False
        while any(nxt[i] < limit[i] for i in range(len(streams))) or outstanding:
            for i, (w, h, fr) in enumerate(streams):
                if nxt[i] >= limit[i]:
                    continue
                k = nxt[i]
                st = srv.submit(sids[i], *fr[k], qp=27 + 5 * (k % 3), sad_lambda=64, tag=i * 1000 + k)
                if st == 0:
                    nxt[i] += 1
                    outstanding += 1
                else:
                    assert st == -6          # queue full: collect and retry
            if leave_after and not left and nxt[leave_after[0]] >= leave_after[1]:
                assert srv.leave(sids[leave_after[0]], 30000) == 0
                left = True
            for d, cu in srv.poll(timeout_ms=20):
                outstanding -= 1
                assert d.status == 0
                assert d.user_tag == sids.index(d.stream_id) * 1000 + d.frame_index
                assert d.has_results == (d.frame_index > 0)
                assert d.latency_ms >= d.queue_ms >= 0
                if d.has_results:
                    got[(sids.index(d.stream_id), d.frame_index)] = cu
        st = srv.stats()
        assert st["running"] == 0 and st["queued"] == 0
    return got


def test_server_results_equal_alone_and_mixed():
    x = (416, 240, _frames(416, 240, 6, seed=11))
    others = [(640, 360, _frames(640, 360, 5, seed=12)), (256, 128, _frames(256, 128, 7, seed=13)),
              (416, 240, _frames(416, 240, 5, seed=14))]
    want = _alone(*x)
    alone = _serve([x], max_inflight=1)
    mixed = _serve([x] + others, max_inflight=3)
    for k in range(1, len(x[2])):
        assert np.array_equal(alone[(0, k)], want[k - 1]), k
        assert np.array_equal(mixed[(0, k)], want[k - 1]), k
    # every other stream equals its own solo run too
    for i, o in enumerate(others, 1):
        w = _alone(*o)
        for k in range(1, len(o[2])):
            assert np.array_equal(mixed[(i, k)], w[k - 1]), (i, k)


def test_server_preset4_streams_alone_and_mixed():
    """Streams in the preset-4 form (search by resolution levels, every transform
    candidate through the trellis) served beside plain streams: each one's CU
    records (whose non-zero maps and SSDs come from the trellis stage) equal the
    same stream run alone, with several pictures of different streams in flight."""
    p4 = {"search_mode": 1, "tu_mode": 1}
    a = (192, 128, _frames(192, 128, 5, seed=31))
    b = (256, 128, _frames(256, 128, 4, seed=32))
    c = (416, 240, _frames(416, 240, 4, seed=33))
    want_a, want_b = _alone(*a, **p4), _alone(*b, **p4)
    want_c = _alone(*c)
    mixed = _serve([a, b, c], max_inflight=3, kws=[p4, p4, {}])
    for i, (x, want) in enumerate(((a, want_a), (b, want_b), (c, want_c))):
        for k in range(1, len(x[2])):
            assert np.array_equal(mixed[(i, k)], want[k - 1]), (i, k)


def test_server_leave_while_others_run():
    x = (416, 240, _frames(416, 240, 6, seed=21))
    y = (640, 360, _frames(640, 360, 6, seed=22))
    want = _alone(*x)
    got = _serve([x, y], max_inflight=2, leave_after=(1, 3))
    for k in range(1, 6):
        assert np.array_equal(got[(0, k)], want[k - 1])
    assert (1, 2) in got and (1, 3) not in got


def test_server_admission_by_footprint_and_throughput():
    from xin26x_gb300.server import Admission, Server
    probe = Server(hbm_budget=1)
    fp, _ = probe.footprint(416, 240, search_range=R)
    with pytest.raises(Admission):
        probe.join(416, 240, search_range=R)
    probe.close()
    with Server(hbm_budget=2 * fp + fp // 2) as srv:
        a = srv.join(416, 240, search_range=R)
        srv.join(416, 240, search_range=R)
        with pytest.raises(Admission):
            srv.join(416, 240, search_range=R)
        assert srv.stats()["hbm_used"] == 2 * fp
        assert srv.leave(a, 10000) == 0
        srv.join(416, 240, search_range=R)
    with Server(mpix_budget=10.0) as srv:       # 416x240 at 30 fps = 3.0 Mpixel/s each
        for _ in range(3):
            srv.join(416, 240, fps=30, search_range=R)
        with pytest.raises(Admission):
            srv.join(416, 240, fps=30, search_range=R)
        srv.join(416, 240, fps=5, search_range=R)


def test_server_argument_and_queue_errors():
    import ctypes as C
    from xin26x_gb300 import _lib
    from xin26x_gb300.server import Server
    fr = _frames(1920, 1080, 2, seed=31)
    with Server(max_queue=1, max_inflight=1) as srv:
        sid = srv.join(1920, 1080, search_range=64)
        assert srv.submit(sid + 100, *fr[0]) == -2                 # no such stream
        assert srv.submit(sid, *fr[0], qp=64) == -2                # QP out of range
        assert srv.submit(sid, *fr[0], sad_lambda=(1 << 20) + 1) == -2   # lambda the search cannot pack
        assert srv.submit(sid, *fr[0]) == 0
        pic = _lib.xin_gpu_picture()
        planes = [np.ascontiguousarray(p) for p in fr[1]]
        for i, p in enumerate(planes):
            pic.plane[i] = p.ctypes.data
            pic.stride[i] = p.shape[1]
        pic.qp = pic.uv_qp = 32
        assert srv.lib.xin_gpu_server_submit(srv.h, sid, C.byref(pic), None, 0) == -2    # no cu_out after picture 0
        full = 0
        accepted = 1
        for k in range(40):
            st = srv.submit(sid, *fr[k % 2])
            if st == -6:
                full += 1
            else:
                assert st == 0
                accepted += 1
        assert full > 0
        seen = 0
        while seen < accepted:
            for d, _ in srv.poll(timeout_ms=1000):
                assert d.status == 0
                seen += 1


def test_server_planes_equal_alone():
    """xin_gpu_server_submit_planes: a served stream joined with XIN_GPU_OUT_Q
    returns each picture's coefficient planes straight into caller buffers
    (pinned host memory), equal to the same stream run alone; a stream beside
    it without planes is unaffected; planes are refused for a stream joined
    without XIN_GPU_OUT_Q."""
    import torch
    from xin26x_gb300.frame import FrameStream
    from xin26x_gb300.server import Server
    w, h = 256, 128
    a = _frames(w, h, 4, seed=41)
    b = _frames(192, 128, 4, seed=42)
    fs = FrameStream(w, h, search_range=R, out_q=True, out_rec=False)
    want = []
    for k, f in enumerate(a):
        fs.submit(*f, qp=27 + 5 * (k % 3), uv_qp=27 + 5 * (k % 3), sad_lambda=64)
        r = fs.wait()
        want.append((r["cu"].copy(), [q.copy() for q in r["q"]]) if k else None)
    nlev, coef = len(fs.levels), fs.coef
    fs.close()
    want_b = _alone(192, 128, b)
    with Server(max_inflight=3, max_queue=2) as srv:
        sa = srv.join(w, h, fps=30, search_range=R, out_q=True)
        sb = srv.join(192, 128, fps=30, search_range=R)
        tdt = torch.int16 if coef == np.int16 else torch.int32
        bufs = {k: [torch.empty((nlev, hh, ww), dtype=tdt, pin_memory=True).numpy()
                    for hh, ww in ((h, w), (h // 2, w // 2), (h // 2, w // 2))] for k in range(4)}
        got, got_b = {}, {}
        for k in range(4):
            assert srv.submit(sa, *a[k], qp=27 + 5 * (k % 3), sad_lambda=64, tag=k, q_out=bufs[k]) == 0
            assert srv.submit(sb, *b[k], qp=27 + 5 * (k % 3), sad_lambda=64, tag=100 + k) == 0
            while len(got) + len(got_b) < 2 * (k + 1):
                for d, cu in srv.poll(timeout_ms=1000):
                    assert d.status == 0
                    (got if d.user_tag < 100 else got_b)[d.user_tag % 100] = cu
        with pytest.raises(RuntimeError):
            st = srv.submit(sb, *b[0], qp=32, sad_lambda=64, tag=999, q_out=bufs[0])
            if st:
                raise RuntimeError(st)
    for k in range(1, 4):
        assert np.array_equal(got[k], want[k][0]), k
        for p in range(3):
            assert np.array_equal(bufs[k][p], want[k][1][p]), (k, p)
        assert np.array_equal(got_b[k], want_b[k - 1]), k


def test_server_cross_stream_batches_equal_alone():
    """Cross-stream batches (xg_batch.cuh): three plain streams of one shape, two
    of them returning coefficient planes, share one launch per stage (the
    window holds the oldest picture until the three have arrived); a stream of
    another shape runs beside them.  Every stream's CU records and planes equal
    the same stream run alone, and the server counts the batches.  128 x 64
    pictures at +-16: a picture's integer search is 2 tiles x 33 bands = 66
    CTAs, so four fit the two waves of SMs a batch may fill."""
    import torch
    from xin26x_gb300.frame import FrameStream
    from xin26x_gb300.server import Server
    w, h, n = 128, 64, 5
    seqs = [_frames(w, h, n, seed=51 + i) for i in range(3)]
    other = _frames(256, 128, n, seed=54)
    qp = [27 + 5 * (k % 3) for k in range(n)]
    want = []
    for fr in seqs:
        fs = FrameStream(w, h, search_range=R, out_q=True, out_rec=False)
        ww = []
        for k, f in enumerate(fr):
            fs.submit(*f, qp=qp[k], uv_qp=qp[k], sad_lambda=64)
            r = fs.wait()
            ww.append((r["cu"].copy(), [q.copy() for q in r["q"]]) if k else None)
        nlev, coef = len(fs.levels), fs.coef
        fs.close()
        want.append(ww)
    want_o = _alone(256, 128, other)
    tdt = torch.int16 if coef == np.int16 else torch.int32
    bufs = {(i, k): [torch.empty((nlev, hh, ww_), dtype=tdt, pin_memory=True).numpy()
                     for hh, ww_ in ((h, w), (h // 2, w // 2), (h // 2, w // 2))] for i in range(2) for k in range(n)}
    got = {}
    with Server(max_inflight=8, max_queue=2, batch_max=3, batch_window_us=200000) as srv:
        sids = [srv.join(w, h, fps=30, search_range=R, out_q=i < 2) for i in range(3)]
        so = srv.join(256, 128, fps=30, search_range=R)
        for k in range(n):
            for i in range(3):
                assert srv.submit(sids[i], *seqs[i][k], qp=qp[k], sad_lambda=64, tag=100 * i + k,
                                  q_out=bufs[(i, k)] if i < 2 else None) == 0
            assert srv.submit(so, *other[k], qp=qp[k], sad_lambda=64, tag=300 + k) == 0
            while len(got) < 4 * (k + 1):
                for d, cu in srv.poll(timeout_ms=2000):
                    assert d.status == 0
                    got[d.user_tag] = cu
        st = srv.stats()
    assert st["batches"] == n - 1 and st["batched_pictures"] == 3 * (n - 1), st
    for k in range(1, n):
        for i in range(3):
            assert np.array_equal(got[100 * i + k], want[i][k][0]), (i, k)
            if i < 2:
                for p in range(3):
                    assert np.array_equal(bufs[(i, k)][p], want[i][k][1][p]), (i, k, p)
        assert np.array_equal(got[300 + k], want_o[k - 1]), k
