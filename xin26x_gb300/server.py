"""Host-side API of the serving layer (xin_gpu_server_*): many live picture
streams on one GPU with admission by device-memory footprint and promised
throughput, per-stream ordering and continuous batching across streams.

    srv = Server(mpix_budget=800)
    sid = srv.join(1920, 1080, fps=30)          # raises Admission when refused
    srv.submit(sid, y, u, v, qp=32, sad_lambda=64, tag=7)
    for done, cu in srv.poll(timeout_ms=100): ...
    srv.leave(sid); srv.close()
"""
from __future__ import annotations

import ctypes as C
import threading

import numpy as np

from . import _lib
from .frame import CU_DTYPE

ERR_ADMIT = -7


class Admission(RuntimeError):
    """join refused: the stream's footprint or throughput does not fit."""


class Server:
    def __init__(self, hbm_budget: int = 0, mpix_budget: float = 0.0, max_inflight: int = 8, max_streams: int = 256,
                 max_queue: int = 4, bitdepth: int = 8, device: int = 0, batch_max: int = 0, batch_window_us: int = 0):
        """batch_max: pictures of different plain streams of one shape a launch
        may carry (0 = the library's default, 1 = no cross-stream batches);
        batch_window_us: how long the oldest waiting picture may be held for
        others to join its batch."""
        self.lib = _lib.load(bitdepth)
        self.pix = np.uint8 if bitdepth == 8 else np.uint16
        if self.lib.xin_gpu_init(device) != 0:
            raise RuntimeError("xin_gpu_init: " + self.lib.xin_gpu_last_error().decode())
        cfg = _lib.xin_gpu_server_cfg(hbm_budget, mpix_budget, max_inflight, max_streams, max_queue, batch_max,
                                      batch_window_us, 0)
        h = C.c_void_p()
        if self.lib.xin_gpu_server_open(C.byref(cfg), C.byref(h)) != 0:
            raise RuntimeError("xin_gpu_server_open: " + self.lib.xin_gpu_last_error().decode())
        self.h = h
        self._ncus = {}
        self._pending = {}          # (stream, frame index) -> cu array kept alive until polled
        self._next = {}
        self._mu = threading.Lock()

    @staticmethod
    def stream_cfg(width, height, ctu=64, search_range=64, levels=(64, 32, 16, 8), input_bitdepth=0, search_mode=0,
                   tu_mode=0, out_q=False):
        """search_mode 1: search by resolution levels; tu_mode 1: the preset-4 TU
        stage (every transform candidate through the trellis, the stream's
        default context set); out_q: coefficient planes returned (submit(q_out=))."""
        mask = 0
        for s in levels:
            mask |= int(s)
        return _lib.xin_gpu_stream_cfg(width, height, ctu, search_range, mask, 1 if out_q else 0, 1, 0, input_bitdepth,
                                       search_mode, tu_mode)

    def footprint(self, width, height, **kw):
        d, hbytes = C.c_uint64(), C.c_uint64()
        st = self.lib.xin_gpu_stream_footprint(C.byref(self.stream_cfg(width, height, **kw)), C.byref(d), C.byref(hbytes))
        if st:
            raise ValueError(self.lib.xin_gpu_last_error().decode())
        return d.value, hbytes.value

    def join(self, width, height, fps=30.0, **kw) -> int:
        cfg = self.stream_cfg(width, height, **kw)
        sid = C.c_int32()
        st = self.lib.xin_gpu_server_join(self.h, C.byref(cfg), float(fps), C.byref(sid))
        if st == ERR_ADMIT:
            raise Admission(self.lib.xin_gpu_last_error().decode())
        if st:
            raise RuntimeError(f"xin_gpu_server_join ({st}): " + self.lib.xin_gpu_last_error().decode())
        n = 0
        for s in kw.get("levels", (64, 32, 16, 8)):
            n += (width // s) * (height // s)
        with self._mu:
            self._ncus[sid.value] = n
            self._next[sid.value] = 0
        return sid.value

    def submit(self, sid, y, u, v, qp=32, uv_qp=None, sad_lambda=64, tag=0, q_out=None) -> int:
        """Queue a picture; returns the status (0, or -6 when the stream's queue is full).
        One thread submits to a given stream.  q_out: three arrays [levels, h, w]
        (pinned host memory keeps the copies asynchronous) that receive the
        picture's coefficient planes (a stream joined with out_q); they must stay
        alive and untouched until the picture is polled."""
        pic = _lib.xin_gpu_picture()
        planes = [np.ascontiguousarray(p, dtype=self.pix) for p in (y, u, v)]
        for i, p in enumerate(planes):
            pic.plane[i] = p.ctypes.data
            pic.stride[i] = p.shape[1]
        pic.qp, pic.uv_qp, pic.sad_lambda = qp, qp if uv_qp is None else uv_qp, sad_lambda
        with self._mu:      # registered before the call: the picture may complete before it returns
            if sid not in self._next:
                return self.lib.xin_gpu_server_submit(self.h, sid, C.byref(pic), None, tag)   # the library's error
            idx = self._next[sid]
            cu = np.zeros(self._ncus[sid], CU_DTYPE) if idx > 0 else None
            self._pending[(sid, idx)] = cu
        if q_out is None:
            st = self.lib.xin_gpu_server_submit(self.h, sid, C.byref(pic), cu.ctypes.data if cu is not None else None, tag)
        else:
            qp3 = (C.c_void_p * 3)(*[q.ctypes.data for q in q_out])
            st = self.lib.xin_gpu_server_submit_planes(self.h, sid, C.byref(pic), cu.ctypes.data if cu is not None else None,
                                                       qp3, tag)
        with self._mu:
            if st == 0:
                self._next[sid] = idx + 1
            else:
                self._pending.pop((sid, idx), None)
        return st

    def poll(self, max_n=64, timeout_ms=100):
        """Completed pictures: list of (xin_gpu_server_done, cu array or None)."""
        arr = (_lib.xin_gpu_server_done * max_n)()
        n = C.c_int32()
        self.lib.xin_gpu_server_poll(self.h, arr, max_n, timeout_ms, C.byref(n))
        out = []
        with self._mu:
            for i in range(n.value):
                d = arr[i]
                cu = self._pending.pop((d.stream_id, d.frame_index), None)
                out.append((_lib.xin_gpu_server_done.from_buffer_copy(d), cu))
        return out

    def leave(self, sid, timeout_ms=-1) -> int:
        return self.lib.xin_gpu_server_leave(self.h, sid, timeout_ms)

    def stats(self):
        s = _lib.xin_gpu_server_stats()
        self.lib.xin_gpu_server_get_stats(self.h, C.byref(s))
        return {k: getattr(s, k) for k, _ in s._fields_ if k != "reserved"}

    def close(self):
        if self.h:
            self.lib.xin_gpu_server_close(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
