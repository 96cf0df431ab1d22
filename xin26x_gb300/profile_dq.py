"""Dependent-quantisation driver for profilers: builds the seeded block list
(xin26x_gb300.synth.dq_blocks: the 65,536-block kernel-bench shapes, coefficient
spectra of an 11-bit Laplacian residual, one to several CABAC context sets),
runs a plan `--runs` times on device arrays and prints the CUDA-event time per
run with the trellis work (coefficient steps) as one JSON line.

  python -m xin26x_gb300.profile_dq [--blocks 65536] [--bitdepth 10] [--sets 4] [--runs 5]
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
    ap.add_argument("--sets", type=int, default=4)
    ap.add_argument("--runs", type=int, default=5)
    ap.add_argument("--seed", type=int, default=11)
    a = ap.parse_args()
    import torch
    from xin26x_gb300 import _lib, synth
    g = _lib.load(a.bitdepth)
    assert g.xin_gpu_init(0) == 0
    blocks, t, sets = synth.dq_blocks(a.blocks, a.seed, bitdepth=a.bitdepth, n_sets=a.sets)
    steps = int(synth.dq_steps(blocks, t, a.bitdepth).sum())
    dt = torch.from_numpy(t).cuda()
    dq, dr = torch.empty_like(dt), torch.empty_like(dt)
    nz = torch.empty(a.blocks, dtype=torch.int64, device="cuda")
    dsets = torch.from_numpy(sets.view(np.uint8).reshape(-1)).cuda()
    s = torch.cuda.current_stream()
    plan = C.c_void_p()
    assert g.xin_gpu_dq_plan_create(blocks.ctypes.data, a.blocks, t.size, a.sets, C.byref(plan)) == 0, g.xin_gpu_last_error()
    ms = []
    for _ in range(a.runs):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        assert g.xin_gpu_dq_plan_run(plan, dt.data_ptr(), dq.data_ptr(), dr.data_ptr(), nz.data_ptr(), dsets.data_ptr(),
                                     s.cuda_stream) == 0, g.xin_gpu_last_error()
        e1.record(s)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    g.xin_gpu_dq_plan_destroy(plan)
    best = float(np.min(ms[1:] or ms))
    print(json.dumps({"blocks": a.blocks, "coefficients": int(t.size), "trellis_steps": steps, "ms": ms, "best_ms": best,
                      "Gsteps_per_s": steps / best / 1e6}))


if __name__ == "__main__":
    main()
