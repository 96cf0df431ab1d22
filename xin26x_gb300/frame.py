"""Host-side API of the batched frame form (xin_gpu_stream_* / xin_gpu_frame_*).

A FrameStream owns one device stream of pictures: reference picture, padded
planes, quarter-pel planes and outputs stay resident on the GPU; each submitted
picture runs the whole hot path (integer + sub-pel search, motion compensation,
transform / quant / dequant / inverse transform / reconstruction) for every CU
of every enabled quadtree level as one captured CUDA graph.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

CU_DTYPE = np.dtype([("mvx", "<i4"), ("mvy", "<i4"), ("cost", "<u4"), ("int_cost", "<u4"),
                     ("nz", "<u8", (3,)), ("ssd", "<u8", (3,))])
OUT_Q, OUT_REC = 1, 2
# xin_gpu_cu_mts: the transform candidates of a CU (tu_mode 1)
MTS_DTYPE = np.dtype([("satd_cost", "<u4"), ("ncand", "<u4"), ("nz", "<u8", (5,)), ("ssd", "<u8", (5,))])
# xin_gpu_cu_bi: list 1's search, the bi pair and the choice of a CU (refs 2)
BI_DTYPE = np.dtype([("mvx1", "<i4"), ("mvy1", "<i4"), ("cost1", "<u4"), ("int_cost1", "<u4"), ("bmv", "<i4", (4,)),
                     ("bi_cost", "<u4"), ("inter_dir", "<u4")])


class FrameStream:
    def __init__(self, width: int, height: int, ctu: int = 64, search_range: int = 64,
                 levels=(64, 32, 16, 8), out_q: bool = True, out_rec: bool = False, use_graph: bool = True,
                 bitdepth: int = 8, device: int = 0, input_bitdepth: int = 0, search_mode: int = 0,
                 tu_mode: int = 0, contexts=None, refs: int = 1, dpb: int = 0):
        """bitdepth: the library (8 or 10, the reference's ENABLE_10BIT_ENCODER);
        input_bitdepth 8 with bitdepth 10: 8-bit pictures coded at 10 bits;
        search_mode 0 exhaustive integer search, 1 by resolution levels;
        tu_mode 1 the preset-4 TU work (transform candidates with dependent
        quantisation), contexts its CABAC context set (synth.PROB_DTYPE records);
        refs 2: two references (by default the previous two pictures) with the bi
        search; dpb: pictures kept as references (0 = refs + 1, up to 32)."""
        self.lib = _lib.load(bitdepth)
        self.bitdepth = bitdepth
        self.in_pix = np.uint8 if (bitdepth == 8 or input_bitdepth == 8) else np.uint16
        self.pix = np.uint8 if bitdepth == 8 else np.uint16
        self.coef = np.int16 if bitdepth == 8 else np.int32
        if self.lib.xin_gpu_init(device) != 0:
            raise RuntimeError("xin_gpu_init: " + self.lib.xin_gpu_last_error().decode())
        mask = 0
        for s in levels:
            mask |= int(s)
        self.cfg = _lib.xin_gpu_stream_cfg(width, height, ctu, search_range, mask,
                                           (OUT_Q if out_q else 0) | (OUT_REC if out_rec else 0), 1 if use_graph else 0,
                                           0, input_bitdepth, search_mode, tu_mode, refs, dpb)
        h = C.c_void_p()
        st = self.lib.xin_gpu_stream_open(C.byref(self.cfg), C.byref(h))
        if st != 0:
            raise RuntimeError(f"xin_gpu_stream_open ({st}): " + self.lib.xin_gpu_last_error().decode())
        self.h = h
        self.width, self.height = width, height
        self.ncus = self.lib.xin_gpu_stream_num_cus(h)
        self.levels = []
        for i in range(self.lib.xin_gpu_stream_num_levels(h)):
            a, b, c, d = i32(), i32(), i32(), i32()
            self.lib.xin_gpu_stream_level_info(h, i, C.byref(a), C.byref(b), C.byref(c), C.byref(d))
            self.levels.append((a.value, b.value, c.value, d.value))
        self.out_q, self.out_rec = out_q, out_rec
        self.tu_mode = tu_mode
        self.refs = refs
        if tu_mode and contexts is not None:
            ctx = np.ascontiguousarray(contexts)
            if self.lib.xin_gpu_stream_set_contexts(h, ctx.ctypes.data) != 0:
                raise RuntimeError("xin_gpu_stream_set_contexts: " + self.lib.xin_gpu_last_error().decode())

    def submit(self, y, u, v, qp: int = 32, uv_qp: int = 32, sad_lambda: int = 64, ref0: int = -1, ref1: int = -1) -> None:
        """ref0 / ref1: picture numbers of the references (-1: the previous picture,
        the one before)."""
        planes = [np.ascontiguousarray(p, dtype=self.in_pix) for p in (y, u, v)]
        pic = _lib.xin_gpu_picture()
        for i, p in enumerate(planes):
            pic.plane[i] = p.ctypes.data
            pic.stride[i] = p.shape[1]
        pic.qp, pic.uv_qp, pic.sad_lambda = qp, uv_qp, sad_lambda
        st = self.lib.xin_gpu_frame_submit_refs(self.h, C.byref(pic), ref0, ref1)
        if st != 0:
            raise RuntimeError(f"xin_gpu_frame_submit ({st}): " + self.lib.xin_gpu_last_error().decode())

    def wait(self, timeout_ms: int = 60000, copy: bool = True):
        """Results of the oldest picture in flight (at most two are): dict with 'cu'
        (structured array), 'q' / 'rec' (lists of per-plane arrays [levels, h, w])
        and 'gpu_ms'.  copy=False leaves the views of the stream's pinned buffers
        unread (valid until the second submit after this call)."""
        res = _lib.xin_gpu_results()
        bufs = {}
        if copy:
            bufs["cu"] = np.zeros(self.ncus, CU_DTYPE)
            res.cu = bufs["cu"].ctypes.data
            if self.tu_mode:
                bufs["mts"] = np.zeros(self.ncus, MTS_DTYPE)
                res.mts = bufs["mts"].ctypes.data
            if self.refs == 2:
                bufs["bi"] = np.zeros(self.ncus, BI_DTYPE)
                res.bi = bufs["bi"].ctypes.data
            nl = len(self.levels)
            for p in range(3):
                hh, ww = (self.height, self.width) if p == 0 else (self.height // 2, self.width // 2)
                if self.out_q:
                    bufs[("q", p)] = np.zeros((nl, hh, ww), self.coef)
                    res.q[p] = bufs[("q", p)].ctypes.data
                if self.out_rec:
                    bufs[("rec", p)] = np.zeros((nl, hh, ww), self.pix)
                    res.rec[p] = bufs[("rec", p)].ctypes.data
        st = self.lib.xin_gpu_frame_wait(self.h, C.byref(res), timeout_ms)
        if st != 0:
            raise RuntimeError(f"xin_gpu_frame_wait ({st}): " + self.lib.xin_gpu_last_error().decode())
        if not copy:
            return res
        out = {"cu": bufs["cu"], "gpu_ms": res.gpu_ms}
        if self.tu_mode:
            out["mts"] = bufs["mts"]
        if self.refs == 2:
            out["bi"] = bufs["bi"]
        if self.out_q:
            out["q"] = [bufs[("q", p)] for p in range(3)]
        if self.out_rec:
            out["rec"] = [bufs[("rec", p)] for p in range(3)]
        return out

    def close(self) -> None:
        if self.h:
            self.lib.xin_gpu_stream_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


i32 = C.c_int32
