"""Run the batched frame form on resident pictures and print per-stage device
times -- the program for profiling (ncu) and quick timing of the kernels.

    python -m xin26x_gb300.profile_frame [--frames 6] [--width 1920] [--height 1080]
                                         [--search 64] [--bitdepth 8] [--ctu 64]
                                         [--objects 4] [--octaves 1] [--input-bitdepth 0]
                                         [--search-mode 0] [--tu-mode 0] [--refs 1]

--bitdepth 10 --input-bitdepth 8: 8-bit pictures coded by the 10-bit library.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json

import numpy as np

from . import _lib, synth


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--frames", type=int, default=6)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--search", type=int, default=64)
    ap.add_argument("--bitdepth", type=int, default=8)
    ap.add_argument("--levels", default="64,32,16,8")
    ap.add_argument("--ctu", type=int, default=64)
    ap.add_argument("--objects", type=int, default=4)
    ap.add_argument("--octaves", type=int, default=1)
    ap.add_argument("--input-bitdepth", type=int, default=0)
    ap.add_argument("--search-mode", type=int, default=0, help="0 exhaustive, 1 by resolution levels")
    ap.add_argument("--tu-mode", type=int, default=0, help="1: the preset-4 TU work (transform candidates, trellis)")
    ap.add_argument("--refs", type=int, default=1, help="2: two references (the previous two pictures), bi search")
    ap.add_argument("--qp", type=int, default=32)
    a = ap.parse_args()
    import torch
    lib = _lib.load(a.bitdepth)
    assert lib.xin_gpu_init(0) == 0
    seq = synth.sequence(a.width, a.height, min(a.frames, 8), seed=1080, bitdepth=a.input_bitdepth or a.bitdepth,
                         objects=a.objects, octaves=a.octaves)
    dev = [tuple(torch.from_numpy(np.ascontiguousarray(p)).cuda() for p in f) for f in seq]
    mask = sum(int(s) for s in a.levels.split(","))
    cfg = _lib.xin_gpu_stream_cfg(a.width, a.height, a.ctu, a.search, mask, 0, 1, 1, a.input_bitdepth, a.search_mode,
                                  a.tu_mode, a.refs)
    h = C.c_void_p()
    if lib.xin_gpu_stream_open(C.byref(cfg), C.byref(h)) != 0:
        raise RuntimeError(lib.xin_gpu_last_error().decode())
    res = _lib.xin_gpu_results()
    stages = []
    for k in range(a.frames):
        pic = _lib.xin_gpu_picture()
        for i, t in enumerate(dev[k % len(dev)]):
            pic.plane[i] = t.data_ptr()
            pic.stride[i] = t.shape[1]
        pic.qp = pic.uv_qp = a.qp
        pic.sad_lambda = 64 if a.bitdepth == 8 else 256
        assert lib.xin_gpu_frame_submit(h, C.byref(pic)) == 0, lib.xin_gpu_last_error()
        assert lib.xin_gpu_frame_wait(h, C.byref(res), -1) == 0, lib.xin_gpu_last_error()
        if k:
            st = (C.c_float * 4)()
            lib.xin_gpu_stream_stage_ms(h, st)
            stages.append(list(st) + [res.gpu_ms])
    lib.xin_gpu_stream_close(h)
    s = np.array(stages)
    print(json.dumps({"frames": a.frames, "size": [a.width, a.height], "search": a.search, "search_mode": a.search_mode,
                      "tu_mode": a.tu_mode, "refs": a.refs, "qp": a.qp,
                      "bitdepth": a.bitdepth,
                      "input_bitdepth": a.input_bitdepth or a.bitdepth,
                      "ctu": a.ctu, "mpix_s": a.width * a.height / float(np.median(s[:, 4])) / 1e3,
                      "ms": {"prep": float(np.median(s[:, 0])), "integer_search": float(np.median(s[:, 1])),
                             "subpel_mc_tq": float(np.median(s[:, 2])), "copies": float(np.median(s[:, 3])),
                             "total": float(np.median(s[:, 4]))},
                      "launches": int(lib.xin_gpu_kernel_launches())}))


if __name__ == "__main__":
    main()
