"""Batched transform / quant driver for profilers: builds the seeded block list
(xin26x_gb300.synth.tq_blocks), runs a plan `--runs` times on device arrays and
prints the CUDA-event time per run as one JSON line.

  python -m xin26x_gb300.profile_tq [--blocks 65536] [--bitdepth 10] [--tile -1] [--runs 5]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json

import numpy as np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--blocks", type=int, default=65536)
    ap.add_argument("--bitdepth", type=int, default=10)
    ap.add_argument("--tile", type=int, default=-1)
    ap.add_argument("--runs", type=int, default=5)
    ap.add_argument("--seed", type=int, default=65536)
    a = ap.parse_args()
    import torch
    from xin26x_gb300 import _lib, synth
    g = _lib.load(a.bitdepth)
    assert g.xin_gpu_init(0) == 0
    blocks, resid = synth.tq_blocks(a.blocks, a.seed, bitdepth=a.bitdepth, kernel_bench_mix=True)
    d = torch.from_numpy(resid).cuda()
    q, r, ro = torch.empty_like(d), torch.empty_like(d), torch.empty_like(d)
    nz = torch.empty(a.blocks, dtype=torch.int64, device="cuda")
    s = torch.cuda.current_stream()
    plan = C.c_void_p()
    assert g.xin_gpu_tq_plan_create(blocks.ctypes.data, a.blocks, resid.size, a.tile, C.byref(plan)) == 0, \
        g.xin_gpu_last_error()
    ms = []
    for _ in range(a.runs):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        assert g.xin_gpu_tq_plan_run(plan, d.data_ptr(), q.data_ptr(), r.data_ptr(), ro.data_ptr(), nz.data_ptr(),
                                     s.cuda_stream) == 0, g.xin_gpu_last_error()
        e1.record(s)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    g.xin_gpu_tq_plan_destroy(plan)
    print(json.dumps({"blocks": a.blocks, "coefficients": int(resid.size), "ms": ms, "best_ms": float(np.min(ms[1:] or ms))}))


if __name__ == "__main__":
    main()
