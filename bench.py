"""Benchmark: 1080p VVC hot path (ME + TQ) on one GB300, batched frame form.

A step is one picture of the 1920x1080 8-bit 4:2:0 single-stream workload
through the whole hot path: exhaustive +-64 integer search for every CU of the
64/32/16/8 quadtree levels, full sub-pel search, luma + chroma motion
compensation, DCT2 / quant / dequant / inverse DCT2 / reconstruction of every
CU (the reference previous picture resident on the GPU, low-delay P).

  value   Mpixel/s with the pictures already in HBM (device-resident stream),
          device time of K steps measured with CUDA events, L2 flushed between
          steps (a 512 MB write outside the timed events)
  e2e     the same through the public C ABI with host buffers: picture H2D and
          CU results + coefficient planes D2H inside the timed region
  roofline  of the dominant kernel (integer search): absolute differences per
          second against this GPU's measured vabsdiff4+dp4a throughput
  cpu_baseline  the oracle (C restatement of the reference path) on a sample of
          CTUs on the host cores

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W, H = 1920, 1080
SEARCH = 64
LEVELS = (64, 32, 16, 8)
QPS = (27, 32, 37)
LAMBDA = {27: 45, 32: 64, 37: 91}      # sad lambda per QP at 8-bit SAD scale (fixed table for the synthetic run)
BD, IN_BD = 10, 8                      # the reference's 10-bit build on 8-bit pictures
LAMBDA_BD = {k: v << (BD - IN_BD) for k, v in LAMBDA.items()}   # x4: the SAD scales with the samples
NFRAMES = 30
SEED = 1080
ME_DRAM_BYTES = 9.84e6         # ncu: DRAM bytes of one k_me_tiles<8> launch of the 10-bit build at this workload
ME_ALGO_BYTES = 2 * 1920 * 1080 * 2   # current + reference luma, 16-bit samples


def workload_config():
    return {"workload": "1080p single stream, 8-bit 4:2:0 pictures coded at 10 bits (the reference's 10-bit build), "
                        "low-delay P with the previous picture as reference, "
                        "exhaustive +-64 integer search + full sub-pel search, CU levels 64/32/16/8, DCT2 TU=CU, "
                        "QP 27/32/37 cycling, 30 synthetic pictures (seeded texture + 4 moving rectangles)",
            "width": W, "height": H, "input_bitdepth": IN_BD, "internal_bitdepth": BD, "search_range": SEARCH,
            "levels": list(LEVELS), "frames": NFRAMES, "sad_lambda": LAMBDA_BD,
            "l2": "flushed between steps (512 MB write outside the timed events)",
            "preset4_random_access": "measured beside the headline as preset4_ra_1080p: GOP 16 coding order, two "
                                     "references per picture with the bi search, search by resolution levels, MTS "
                                     "candidates through dependent quantisation, SATD"}


def make_frames(n=NFRAMES):
    from xin26x_gb300 import synth
    return synth.sequence(W, H, n, seed=SEED, objects=4)


# ---------------------------------------------------------------- clocks
class ClockSampler:
    def __init__(self):
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "20", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.time()
            while not self.lines and time.time() - t0 < 3.0:    # sampling runs before the timed region starts
                time.sleep(0.01)
            self.lines.clear()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for name, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------- CPU legs
def cpu_sample(frames, seconds_target=15.0, threads=1):
    """Time the oracle's per-CU hot path on a sample of CTUs (all four levels of each
    CTU) and return Mpixel/s of luma, extrapolated per CTU area."""
    from oracle import oracle as O
    from tests import oracle_frame
    from xin26x_gb300.frame import CU_DTYPE  # noqa: F401

    cur, ref = [tuple(p.astype(np.uint16) << (BD - IN_BD) for p in f) for f in (frames[1], frames[0])]
    o = O.oracle(BD)
    ctus = [(x, y) for y in range(0, H - 63, 64) for x in range(0, W - 63, 64)]
    rng = np.random.default_rng(5)
    order = rng.permutation(len(ctus))
    levels = []
    first = 0
    for s in LEVELS:
        levels.append((s, first, W // s, H // s))
        first += (W // s) * (H // s)

    def cus_of_ctu(cx, cy):
        out = []
        for (s, f, nx, ny) in levels:
            for yy in range(cy, cy + 64, s):
                for xx in range(cx, cx + 64, s):
                    out.append(f + (yy // s) * nx + xx // s)
        return out

    done = 0
    t0 = time.perf_counter()
    lock = threading.Lock()
    idx = [0]

    def worker():
        nonlocal done
        while True:
            with lock:
                if time.perf_counter() - t0 > seconds_target or idx[0] >= len(order):
                    return
                k = order[idx[0]]
                idx[0] += 1
            cx, cy = ctus[k]
            oracle_frame.run(cur, ref, levels, search_range=SEARCH, qp=32, uv_qp=32, sad_lambda=LAMBDA_BD[32],
                             bitdepth=BD, cus=cus_of_ctu(cx, cy))
            with lock:
                done += 1

    ths = [threading.Thread(target=worker) for _ in range(threads)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    el = time.perf_counter() - t0
    mpx = done * 64 * 64 / el / 1e6
    del o
    return mpx, done, el


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    frames = make_frames(2)
    cores = os.cpu_count() or 1
    vals = []
    for i in range(args.warmup + args.steps):
        v, n, el = cpu_sample(frames, seconds_target=4.0 if i >= args.warmup else 1.0, threads=cores)
        if i >= args.warmup:
            vals.append(v)
    value = float(np.mean(vals))
    line = {"metric": "1080p VVC ME+TQ Mpixel/s", "value": value, "unit": "Mpixel/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u16", "data": "synthetic", "config": workload_config(),
            "cpu_baseline": {"value": value, "unit": "Mpixel/s", "cores": cores, "kind": "port",
                             "sample": "each step: as many 64x64 CTUs (all four CU levels, +-64 exhaustive search) as "
                                       "finish in ~4 s on all host threads, oracle C restatement (10-bit build)"},
            "e2e": {"value": value, "unit": "Mpixel/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------- replicas
def max_over_ranks(x, dist=None, device="cpu"):
    """The largest x over all ranks (the slowest replica's time); x itself without
    a process group."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, world, seconds):
    """Replicas only: every rank processes units_per_rank, the job takes the
    slowest rank's seconds; the rate counts the units of all ranks."""
    return units_per_rank * world / seconds


# ---------------------------------------------------------------- GPU legs
def run_gpu(args):
    import torch  # device memory for the resident pictures and the L2 flush buffer
    from xin26x_gb300 import _lib
    from xin26x_gb300.frame import FrameStream

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    lib = _lib.load(BD)
    assert lib.xin_gpu_init(local) == 0
    frames = make_frames()
    npix = W * H

    # resident pictures for the device-timed leg
    dev = []
    for (y, u, v) in frames:
        dev.append(tuple(torch.from_numpy(np.ascontiguousarray(p)).cuda() for p in (y, u, v)))
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")

    cfg = _lib.xin_gpu_stream_cfg(W, H, 64, SEARCH, sum(LEVELS), 0, 1, 1, IN_BD)
    h = C.c_void_p()
    assert lib.xin_gpu_stream_open(C.byref(cfg), C.byref(h)) == 0, lib.xin_gpu_last_error()

    def submit_dev(k):
        pic = _lib.xin_gpu_picture()
        y, u, v = dev[k % len(dev)]
        for i, t in enumerate((y, u, v)):
            pic.plane[i] = t.data_ptr()
            pic.stride[i] = t.shape[1]
        qp = QPS[k % 3]
        pic.qp, pic.uv_qp, pic.sad_lambda = qp, qp, LAMBDA_BD[qp]
        assert lib.xin_gpu_frame_submit(h, C.byref(pic)) == 0, lib.xin_gpu_last_error()

    res = _lib.xin_gpu_results()
    submit_dev(0)
    lib.xin_gpu_frame_wait(h, C.byref(res), -1)
    for k in range(1, args.warmup + 1):
        submit_dev(k)
        lib.xin_gpu_frame_wait(h, C.byref(res), -1)
    # the search's geometry (band count per tile) chosen by the library's autotuner
    # on the last warm-up picture; two more warm-up pictures capture the graphs again
    tune_bands, tune_ms = C.c_int32(), (C.c_float * 2)()
    assert lib.xin_gpu_stream_tune_search(h, C.byref(tune_bands), tune_ms) == 0, lib.xin_gpu_last_error()
    tn, tb, tm = C.c_int32(), (C.c_int32 * 6)(), (C.c_float * 6)()
    lib.xin_gpu_stream_tune_table(h, C.byref(tn), tb, tm)
    search_tuning = {"bands": tune_bands.value, "search_ms_default_geometry": tune_ms[0],
                     "timed": {str(tb[i]): round(float(tm[i]), 4) for i in range(tn.value)},
                     "search_ms_chosen": tune_ms[1], "candidates": "default band count and x1/2, x2, x3, x4, x6 of it",
                     "note": "xin_gpu_stream_tune_search: CUDA-event time of the search of the last warm-up picture "
                             "per geometry (one warm-up, three timed launches each); results do not depend on it"}
    # the CUs per CTA of the 16 x 16 and 8 x 8 tails, also autotuned on the last picture
    tcpb, tms = (C.c_int32 * 2)(), (C.c_float * 6)()
    assert lib.xin_gpu_stream_tune_tails(h, tcpb, tms) == 0, lib.xin_gpu_last_error()
    search_tuning["tails_cus_per_cta"] = {"16x16": tcpb[0], "8x8": tcpb[1],
                                          "timed_ms": {f"{s}x{s}": {str(c): round(float(tms[3 * j + o]), 4)
                                                                    for o, c in enumerate((2, 4, 8))}
                                                       for j, s in enumerate((16, 8))},
                                          "note": "xin_gpu_stream_tune_tails: CUDA-event time of the last warm-up "
                                                  "picture's tails per choice; results do not depend on it"}
    for k in range(args.warmup + 1, args.warmup + 3):
        submit_dev(k)
        lib.xin_gpu_frame_wait(h, C.byref(res), -1)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = ClockSampler()
    clocks.start()
    launches0 = lib.xin_gpu_kernel_launches()
    step_ms, stage = [], np.zeros(4)
    torch.cuda.synchronize()
    for k in range(args.steps):
        flush.fill_(k & 255)                       # evict L2 (outside the timed events)
        torch.cuda.synchronize()
        submit_dev(args.warmup + 1 + k)
        assert lib.xin_gpu_frame_wait(h, C.byref(res), -1) == 0
        step_ms.append(res.gpu_ms)
        st = (C.c_float * 4)()
        lib.xin_gpu_stream_stage_ms(h, st)
        stage += np.array(list(st))
    torch.cuda.synchronize()
    launches = lib.xin_gpu_kernel_launches() - launches0
    clk = clocks.stop()
    total_ms = max_over_ranks(float(np.sum(step_ms)), dist, "cuda")
    value = whole_job_rate(npix * args.steps, world, total_ms * 1e-3) / 1e6
    stage /= args.steps

    # roofline of the integer search kernel: on 8-bit pictures it runs the packed
    # 8-bit SAD (vabsdiff4.add), whose peak the 8-bit library's probe measures
    lib8 = _lib.load(8)
    assert lib8.xin_gpu_init(local) == 0
    peak = C.c_double()
    lib8.xin_gpu_measure_sad_peak(C.byref(peak))
    algo = (W // 8) * (H // 8) * (2 * SEARCH + 1) ** 2 * 64      # abs differences per launch (8x8 SADs)
    me_ms = stage[1]
    achieved = algo / (me_ms * 1e-3)
    lib.xin_gpu_stream_close(h)

    # e2e through the public API with host buffers
    # three picture slots: picture k + 1 (its own slot) starts beside picture k's tails
    e2e_fs = FrameStream(W, H, search_range=SEARCH, levels=LEVELS, out_q=True, out_rec=False, use_graph=True,
                         bitdepth=BD, input_bitdepth=IN_BD, dpb=3)
    cu_bytes = e2e_fs.ncus * 64
    q_bytes = sum((W * H if p == 0 else W * H // 4) * len(LEVELS) * 4 for p in range(3))
    e2e_fs.submit(*frames[0], qp=32, uv_qp=32, sad_lambda=LAMBDA_BD[32])
    e2e_fs.wait()
    # two pictures in flight: picture k + 1 is submitted before picture k is collected, so
    # one picture's copies and host work overlap the other's kernels
    lat, pending = [], []

    def e2e_submit(k):
        qp = QPS[k % 3]
        pending.append(time.perf_counter())
        e2e_fs.submit(*frames[k % len(frames)], qp=qp, uv_qp=qp, sad_lambda=LAMBDA_BD[qp])

    e2e_submit(1)
    e2e_fs.wait(copy=False)
    pending.pop(0)
    assert e2e_fs.lib.xin_gpu_stream_tune_search(e2e_fs.h, None, None) == 0, e2e_fs.lib.xin_gpu_last_error()
    assert e2e_fs.lib.xin_gpu_stream_tune_tails(e2e_fs.h, None, None) == 0, e2e_fs.lib.xin_gpu_last_error()
    e2e_submit(2)
    for k in range(args.warmup):
        e2e_submit(k + 3)
        e2e_fs.wait(copy=False)
        pending.pop(0)
    t0 = time.perf_counter()
    for k in range(args.steps):
        e2e_submit(args.warmup + k + 3)
        e2e_fs.wait(copy=False)
        lat.append((time.perf_counter() - pending.pop(0)) * 1e3)
    e2e_s = time.perf_counter() - t0
    e2e_fs.wait(copy=False)
    e2e_fs.close()
    e2e_s = max_over_ranks(e2e_s, dist, "cuda")
    e2e_val = whole_job_rate(npix * args.steps, world, e2e_s) / 1e6

    # plain per-call form on a sample of CUs (one synchronous launch per reference call)
    percall = percall_sample(lib, frames, bd=BD)
    kbatch = kernel_batch_bench(torch, flush, max(5, min(args.steps, 20)), args.warmup) if rank == 0 else None
    dq = dep_quant_bench(torch, flush, max(5, min(args.steps, 20)), args.warmup, cpu=(world == 1)) if rank == 0 else None
    p4 = preset4_bench(torch, flush, frames, max(5, min(args.steps, 20)), args.warmup) if rank == 0 else None
    p4ra = preset4_ra_bench(torch, flush, frames, 16) if rank == 0 else None
    wide = wide_search_bench(torch, flush) if rank == 0 else None
    if wide is not None:
        wide["by_resolution_levels"] = wide_search_bench(torch, flush, pictures=4, search_mode=1)
    variants = None
    if rank == 0:
        nvar = max(5, min(args.steps, 20))
        variants = {"eight_bit_build": pipeline_variant_bench(torch, flush, frames, nvar, args.warmup, 8, 0),
                    "ten_bit_samples": pipeline_variant_bench(torch, flush, frames, nvar, args.warmup, 10, 0),
                    "search_by_resolution_levels": pipeline_variant_bench(torch, flush, frames, nvar, args.warmup,
                                                                          BD, IN_BD, search_mode=1)}
    serving = serving_planes = None
    if rank == 0 and world == 1:
        # each serving run in a process of its own, as a server would be
        serving = serve_process(max_inflight=6)
        # the plane copies hold a picture's in-flight slot longer: more slots
        serving_planes = serve_process(max_inflight=16, planes=True)

    out = None
    if rank == 0:
        cpu = None
        if world == 1:
            v, n, el = cpu_sample(frames[:2], seconds_target=12.0, threads=1)
            cpu = {"value": v, "unit": "Mpixel/s", "cores": 1, "kind": "port",
                   "sample": f"{n} random 64x64 CTUs (all four CU levels, +-64 exhaustive search), oracle C restatement "
                             f"(10-bit build, pictures << 2), 1 thread, {el:.1f} s"}
        out = {"metric": "1080p VVC ME+TQ Mpixel/s", "value": value, "unit": "Mpixel/s", "n_gpus": world,
               "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u16",
               "data": "synthetic (seeded texture + 4 moving rectangles, 1920x1080 4:2:0)",
               "config": workload_config(),
               "stage_ms": {"prep": stage[0], "integer_search": stage[1], "subpel_mc_tq": stage[2], "copies": stage[3]},
               "search_tuning": search_tuning,
               "roofline": {"bound": "int", "kernel": "k_me_tiles<8> (8-bit samples, SADs x 4)", "achieved": achieved / 1e12,
                            "peak": peak.value / 1e12,
                            "unit": "Tabsdiff/s", "frac": achieved / peak.value, "traffic": ME_DRAM_BYTES,
                            "traffic_source": "dram__bytes.sum.per_second x duration of one k_me_tiles<8> launch "
                                              "(ncu, 1080p, +-64, 10-bit build, cold cache); algorithmic bytes "
                                              f"(current + reference luma, 16-bit samples) {ME_ALGO_BYTES:.3g}",
                            "peak_source": "xin_gpu_measure_sad_peak (8-bit library): the faster of vabsdiff4+dp4a and "
                                           "vabsdiff4.add register loops on this GPU, this run",
                            "algorithmic": f"(W/8)(H/8)(2R+1)^2*64 = {algo:.4g} abs differences per launch"},
               "e2e": {"value": e2e_val, "unit": "Mpixel/s", "h2d_bytes_per_step": W * H * 3 // 2,
                       "d2h_bytes_per_step": cu_bytes + q_bytes, "pictures_in_flight": 2, "picture_slots": 3,
                       "l2": "not flushed: every picture arrives from pinned host memory inside the timed region",
                       "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))}},
               "percall": percall,
               "kernel_batch": kbatch,
               "dep_quant": dq,
               "preset4_1080p": p4,
               "preset4_ra_1080p": p4ra,
               "wide_search_4k_10bit": wide,
               "pipeline_variants_1080p": variants,
               "serving": serving,
               "serving_with_planes": serving_planes,
               "gpu_launches": int(launches),
               "clocks": clk,
               "cpu_baseline": cpu}
        print(json.dumps(out), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def serve_process(max_inflight, planes=False, seconds=3.0, mpix_budget=1650.0):
    """serve_bench.py's 48-stream run in a fresh process (its last output line)."""
    cmd = [sys.executable, "-m", "xin26x_gb300.serve_bench", "--seconds", str(seconds), "--mpix-budget",
           str(mpix_budget), "--max-inflight", str(max_inflight)] + (["--planes"] if planes else [])
    clocks = ClockSampler()
    clocks.start()
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    clk = clocks.stop()
    if r.returncode != 0:
        raise RuntimeError(f"serve_bench failed ({r.returncode}): {r.stderr[-2000:]}")
    out = json.loads(r.stdout.strip().splitlines()[-1])
    out["clocks"] = clk
    return out


def kernel_batch_bench(torch, flush, steps, warmup, nblocks=65536, seed=65536):
    """Batched transform / quant on a 10-bit block list: 65,536 blocks of sides
    4..64 (biased to 8 and 16), 11-bit Laplacian residuals (scale 12), DCT2 70 %
    / DST7-DCT8 pairs 30 % (sides <= 32), QP uniform in [22, 42].  The plan form
    (block list resident on the device) timed with CUDA events per run, L2
    flushed between runs: the tensor-core form (tcgen05) and the CUDA-core form
    with autotuned and with fixed group sizes."""
    from xin26x_gb300 import _lib, synth
    g = _lib.load(10)
    assert g.xin_gpu_init(torch.cuda.current_device()) == 0
    blocks, resid = synth.tq_blocks(nblocks, seed, bitdepth=10, kernel_bench_mix=True)
    d_res = torch.from_numpy(resid).cuda()
    stream = torch.cuda.current_stream()
    out = {"workload": f"{nblocks} blocks, 10-bit, sides 4..64, 11-bit Laplacian residuals (scale 12), DCT2 70 % / "
                       "DST7-DCT8 pairs 30 % on sides <= 32, QP U[22,42]; forward transform + quant + dequant + "
                       "inverse transform per block",
           "coefficients": int(resid.size), "l2": "flushed between runs"}
    algo = resid.size * 4 * 4 + nblocks * (8 + 12 + 4)      # resid in, q/r/resid_out out, nz, job + list entry

    def time_plan(blocks, resid, d_res, tile):
        """mean CUDA-event ms of one plan run (L2 flushed before each) and the plan's tiles"""
        q, r, ro = torch.empty_like(d_res), torch.empty_like(d_res), torch.empty_like(d_res)
        nz = torch.empty(len(blocks), dtype=torch.int64, device="cuda")
        plan = C.c_void_p()
        assert g.xin_gpu_tq_plan_create(blocks.ctypes.data, len(blocks), resid.size, tile, C.byref(plan)) == 0, \
            g.xin_gpu_last_error()
        run = lambda: g.xin_gpu_tq_plan_run(plan, d_res.data_ptr(), q.data_ptr(), r.data_ptr(), ro.data_ptr(),
                                            nz.data_ptr(), stream.cuda_stream)
        for _ in range(max(3, warmup)):
            assert run() == 0, g.xin_gpu_last_error()
        times = []
        for _ in range(steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            assert run() == 0
            b.record(stream)
            b.synchronize()
            times.append(a.elapsed_time(b))
        tiles = (C.c_int32 * 49)()
        g.xin_gpu_tq_plan_tiles(plan, tiles)
        g.xin_gpu_tq_plan_destroy(plan)
        return float(np.mean(times)), tiles

    for name, tile in (("tensor_cores", -2), ("autotuned", -1), ("fixed", 0)):
        ms, tiles = time_plan(blocks, resid, d_res, tile)
        out[name] = {"ms": ms, "Mblocks_per_s": nblocks / ms / 1e3, "Gcoeff_per_s": resid.size / ms / 1e6,
                     "tiles": {f"{1 << (c // 7)}x{1 << (c % 7)}": int(tiles[c]) for c in range(49) if tiles[c]}}
    # the largest transforms alone (the frame form's 32 x 32 and 64 x 64 TUs): DCT2
    # blocks of one side, 4.2 M coefficients each, on either engine
    rng = np.random.default_rng(seed + 1)
    large = {}
    for lg, nb in ((5, 4096), (6, 1024)):
        bl = np.zeros(nb, synth.TQ_BLOCK_DTYPE)
        bl["offset"] = np.arange(nb, dtype=np.int64) << (2 * lg)
        bl["log2w"], bl["log2h"], bl["qp"] = lg, lg, rng.integers(22, 43, size=nb)
        rs = np.clip(np.rint(rng.laplace(0, 12, size=nb << (2 * lg))), -1023, 1023).astype(np.int32)
        d_rs = torch.from_numpy(rs).cuda()
        t_ms, _ = time_plan(bl, rs, d_rs, -2)
        c_ms, _ = time_plan(bl, rs, d_rs, -1)
        large[f"{1 << lg}x{1 << lg}"] = {"blocks": nb, "tensor_cores_ms": t_ms, "cuda_cores_autotuned_ms": c_ms,
                                         "tensor_speedup": c_ms / t_ms}
        del d_rs
    out["dct2_one_side"] = large
    peaks = _measured_peaks()
    hbm = peaks.get("hbm_gbs") if peaks else None
    achieved = algo / (out["tensor_cores"]["ms"] * 1e-3) / 1e9
    out["speedup_autotuned_vs_fixed"] = out["fixed"]["ms"] / out["autotuned"]["ms"]
    out["speedup_tensor_vs_autotuned"] = out["autotuned"]["ms"] / out["tensor_cores"]["ms"]
    out["roofline"] = {"bound": "hbm", "kernel": "k_tq_tc", "achieved": achieved, "peak": hbm or 6800.0, "unit": "GB/s",
                       "frac": achieved / (hbm or 6800.0), "algorithmic_bytes": int(algo),
                       "peak_source": "of measured (MEASURED_PEAKS.json hbm_gbs)" if hbm else "of fallback 6.8 TB/s"}
    return out


def dep_quant_bench(torch, flush, steps, warmup, nblocks=65536, seed=11, cpu=True):
    """Dependent quantisation (the reference's trellis quantiser, used from
    preset 4 up in place of plain quantisation) on the kernel-bench shapes:
    65,536 10-bit blocks of sides 4..64, coefficient spectra of an 11-bit
    Laplacian residual, QP U[22,39] (+12 internally at 10-bit), luma 2/3 and
    chroma 1/3, four CABAC context sets.  Plan form timed with CUDA events,
    L2 flushed between runs.  The work unit is a trellis step: one coefficient
    position walked by one block (from its last significant position to DC)."""
    from xin26x_gb300 import _lib, synth
    g = _lib.load(10)
    assert g.xin_gpu_init(torch.cuda.current_device()) == 0
    nsets = 4
    blocks, t, sets = synth.dq_blocks(nblocks, seed, bitdepth=10, n_sets=nsets)
    wsteps = synth.dq_steps(blocks, t, 10)
    nsteps = int(wsteps.sum())
    d_t = torch.from_numpy(t).cuda()
    q, r = torch.empty_like(d_t), torch.empty_like(d_t)
    nz = torch.empty(nblocks, dtype=torch.int64, device="cuda")
    d_sets = torch.from_numpy(sets.view(np.uint8).reshape(-1)).cuda()
    stream = torch.cuda.current_stream()
    plan = C.c_void_p()
    assert g.xin_gpu_dq_plan_create(blocks.ctypes.data, nblocks, t.size, nsets, C.byref(plan)) == 0, g.xin_gpu_last_error()
    run = lambda: g.xin_gpu_dq_plan_run(plan, d_t.data_ptr(), q.data_ptr(), r.data_ptr(), nz.data_ptr(), d_sets.data_ptr(),
                                        stream.cuda_stream)
    for _ in range(max(3, warmup)):
        assert run() == 0, g.xin_gpu_last_error()
    times = []
    for _ in range(steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        assert run() == 0
        b.record(stream)
        b.synchronize()
        times.append(a.elapsed_time(b))
    g.xin_gpu_dq_plan_destroy(plan)
    ms = float(np.mean(times))
    algo = t.size * 4 * 3 + nblocks * (16 + 8)             # t in, q / r out, block record, nz
    peaks = _measured_peaks()
    hbm = (peaks.get("hbm_gbs") if peaks else None) or 6800.0
    achieved = algo / (ms * 1e-3) / 1e9
    out = {"workload": f"{nblocks} blocks, 10-bit, sides 4..64 (kernel-bench shapes), coefficient spectra of an 11-bit "
                       "Laplacian(12) residual, QP U[22,39] (+12), luma 2/3 / Cb 1/6 / Cr 1/6, root cbf on half of "
                       f"the luma blocks, {nsets} CABAC context sets",
           "coefficients": int(t.size), "trellis_steps": nsteps, "blocks_with_trellis": int((wsteps > 0).sum()),
           "longest_trellis": int(wsteps.max()), "l2": "flushed between runs",
           "ms": ms, "Mblocks_per_s": nblocks / ms / 1e3, "Gsteps_per_s": nsteps / ms / 1e6,
           "roofline": {"bound": "latency", "kernel": "k_dq", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                        "frac": achieved / hbm, "algorithmic_bytes": int(algo),
                        "note": "HBM is not the limit: each block's trellis is a serial chain of coefficient steps "
                                "(four states on four lanes); the floor is the step latency times the longest "
                                "trellis of the batch",
                        "peak_source": "of measured (MEASURED_PEAKS.json hbm_gbs)" if peaks else "of fallback 6.8 TB/s"}}
    if cpu:
        from oracle import oracle as O
        o = O.oracle(10)
        qq, rr, nzz = np.zeros_like(t), np.zeros_like(t), np.zeros(nblocks, np.uint64)
        rng = np.random.default_rng(3)
        idx = rng.permutation(nblocks)
        t0, n, done_steps = time.perf_counter(), 0, 0
        while time.perf_counter() - t0 < 10.0 and n < nblocks:
            b = blocks[idx[n]]
            off = int(b["offset"])
            o.dep_quant(O.ptr(t, off), int(b["stride"]), 1 << int(b["log2_w"]), 1 << int(b["log2_h"]), int(b["qp"]),
                        int(b["comp"]), sets[int(b["ctx_set"])].ctypes.data, int(b["root_cbf"]), O.ptr(qq, off),
                        O.ptr(rr, off), O.ptr(nzz, int(idx[n])))
            done_steps += int(wsteps[idx[n]])
            n += 1
        el = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": done_steps / el / 1e9, "unit": "Gsteps/s", "cores": 1, "kind": "port",
                               "sample": f"{n} random blocks of the same list, oracle C restatement of Xin266DepQuant, "
                                         f"1 thread, {el:.1f} s (includes a ctypes call per block)"}
    return out


def preset4_ra_bench(torch, flush, frames, steps):
    """The preset-4 form in random-access order at 1080p: GOP 16 coding order
    (synth.ra_gop: each key picture from the previous key picture, each B picture
    from the nearest coded pictures before and after it), two references per
    picture named through xin_gpu_frame_submit_refs (dpb 32: the graph pattern
    repeats every two GOPs), the search by resolution levels and full sub-pel
    search per list, the bi search of Xin266InterBiSearch per CU with SATD as
    the decision's distortion, and the coded prediction (list 0, list 1 or bi)
    through every transform candidate and dependent quantisation.  Device-
    resident pictures, CUDA-event device time per picture after two GOPs of
    warm-up, L2 flushed between pictures; then end to end through the public API
    with host buffers, two pictures in flight.  Picture POC p is frame p % 30."""
    from xin26x_gb300 import _lib, synth
    lib = _lib.load(BD)
    assert lib.xin_gpu_init(torch.cuda.current_device()) == 0
    ctx = np.ascontiguousarray(synth.contexts(np.random.default_rng(4), 1)[0])
    dev = [tuple(torch.from_numpy(np.ascontiguousarray(p)).cuda() for p in f) for f in frames]
    nwarm = 32
    order = synth.ra_gop(16, (nwarm + steps + 15) // 16 + 1)

    def run_order(submit, n):
        """submit POC 0 then n pictures of the order: submit(k, poc, ref0, ref1)
        with picture numbers for the references"""
        num = {0: 0}
        submit(0, 0, -1, -1)
        for k, (poc, r0, r1) in enumerate(order[:n], start=1):
            submit(k, poc, num[r0], num[r1])
            num[poc] = k

    cfg = _lib.xin_gpu_stream_cfg(W, H, 64, SEARCH, sum(LEVELS), 0, 1, 1, IN_BD, 1, 1, 2, 32)
    h = C.c_void_p()
    assert lib.xin_gpu_stream_open(C.byref(cfg), C.byref(h)) == 0, lib.xin_gpu_last_error()
    assert lib.xin_gpu_stream_set_contexts(h, ctx.ctypes.data) == 0
    res = _lib.xin_gpu_results()
    ms, stage = [], np.zeros(4)
    launches = [0, 0]

    def submit(k, poc, r0, r1):
        pic = _lib.xin_gpu_picture()
        for i, t in enumerate(dev[poc % len(dev)]):
            pic.plane[i] = t.data_ptr()
            pic.stride[i] = t.shape[1]
        qp = QPS[k % 3]
        pic.qp, pic.uv_qp, pic.sad_lambda = qp, qp, LAMBDA_BD[qp]
        timed = k > nwarm
        if timed:
            flush.fill_(k & 255)
            torch.cuda.synchronize()
            if k == nwarm + 1:
                launches[0] = lib.xin_gpu_kernel_launches()
        assert lib.xin_gpu_frame_submit_refs(h, C.byref(pic), r0, r1) == 0, lib.xin_gpu_last_error()
        assert lib.xin_gpu_frame_wait(h, C.byref(res), -1) == 0, lib.xin_gpu_last_error()
        if timed:
            ms.append(res.gpu_ms)
            st = (C.c_float * 4)()
            lib.xin_gpu_stream_stage_ms(h, st)
            stage[:] += np.array(list(st))
            launches[1] = lib.xin_gpu_kernel_launches()

    run_order(submit, nwarm + steps)
    lib.xin_gpu_stream_close(h)
    stage /= steps
    out = {"workload": "1080p, 8-bit 4:2:0 pictures coded at 10 bits, random-access GOP 16 coding order (key pictures "
                       "from the previous key picture, B pictures from the nearest coded pictures before and after), "
                       "two references per picture: per list the search by resolution levels (+-64) and full sub-pel "
                       "search, the bi search (target 2 org - other list's prediction, +-4 integer step, sub-pel; "
                       "averaged-prediction SATD), the choice of list 0 / list 1 / bi by SATD cost, the bi average of "
                       "14-bit predictions, then per CU luma DCT2 + MTS 2..5 (CUs up to 32) and chroma DCT2 through "
                       "dependent quantisation, inverse transform and reconstruction; CU levels 64/32/16/8, TU = CU, "
                       "QP 27/32/37 cycling",
           "value": W * H * steps / (float(np.sum(ms)) * 1e-3) / 1e6, "unit": "Mpixel/s", "ms_per_picture": float(np.mean(ms)),
           "pictures_timed": steps, "warmup_pictures": nwarm + 1,
           "stage_ms": {"prep": stage[0], "integer_search": stage[1], "subpel_bi_mc_tu": stage[2], "copies": stage[3]},
           "gpu_launches_per_picture": (launches[1] - launches[0]) / steps,
           "l2": "flushed between pictures (512 MB write outside the timed events)",
           "not_covered": "the intra key picture (POC 0 is the first reference only), DMVR and BCW weights in the frame "
                          "form (built per call), more than one reference per list, BT/TT CUs, RDOQ, the host's choice "
                          "among the transform candidates"}
    from xin26x_gb300.frame import FrameStream
    fs = FrameStream(W, H, search_range=SEARCH, levels=LEVELS, out_q=True, out_rec=False, use_graph=True, bitdepth=BD,
                     input_bitdepth=IN_BD, search_mode=1, tu_mode=1, contexts=ctx, refs=2, dpb=32)
    n_e2e = max(steps, 16)
    h2d = W * H * 3 // 2
    d2h = fs.ncus * (64 + 64 + 40) + sum((W * H if p == 0 else W * H // 4) * len(LEVELS) * 4 for p in range(3))
    t0 = [0.0]
    inflight = [0]

    def e2e_submit(k, poc, r0, r1):
        if k == nwarm + 1:
            t0[0] = time.perf_counter()
        qp = QPS[k % 3]
        fs.submit(*frames[poc % len(frames)], qp=qp, uv_qp=qp, sad_lambda=LAMBDA_BD[qp], ref0=r0, ref1=r1)
        inflight[0] += 1
        if inflight[0] == 2:          # two in flight: collect the older one
            fs.wait(copy=False)
            inflight[0] -= 1

    run_order(e2e_submit, nwarm + n_e2e)
    fs.wait(copy=False)
    el = time.perf_counter() - t0[0]
    fs.close()
    out["e2e_two_in_flight"] = {"value": W * H * n_e2e / el / 1e6, "unit": "Mpixel/s", "pictures": n_e2e,
                                "ms_per_picture": el * 1e3 / n_e2e, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                                "note": "host 8-bit planes in, CU, bi and transform-candidate records and coefficient "
                                        "planes out; wall clock over the pictures (the last collected inside)"}
    return out


def pipeline_variant_bench(torch, flush, frames, steps, warmup, bitdepth, input_bitdepth, search_mode=0):
    """The headline pictures through another build or search, for comparison: the
    8-bit library (8-bit arithmetic throughout), the 10-bit library fed the
    pictures as 10-bit samples (<< 2; the search then packs two samples a word
    instead of four), or the headline configuration with the search by resolution
    levels (search_mode 1).  Device-resident pictures, device time per picture,
    L2 flushed."""
    from xin26x_gb300 import _lib
    lib = _lib.load(bitdepth)
    assert lib.xin_gpu_init(torch.cuda.current_device()) == 0
    if bitdepth == 8 or input_bitdepth == 8:
        dev = [tuple(torch.from_numpy(np.ascontiguousarray(p)).cuda() for p in f) for f in frames]
    else:
        dev = [tuple((torch.from_numpy(np.ascontiguousarray(p)).cuda().to(torch.int32) << 2).to(torch.int16) for p in f)
               for f in frames]
    lam = LAMBDA if bitdepth == 8 else LAMBDA_BD
    cfg = _lib.xin_gpu_stream_cfg(W, H, 64, SEARCH, sum(LEVELS), 0, 1, 1, input_bitdepth, search_mode)
    h = C.c_void_p()
    assert lib.xin_gpu_stream_open(C.byref(cfg), C.byref(h)) == 0, lib.xin_gpu_last_error()
    res = _lib.xin_gpu_results()

    def submit(k):
        pic = _lib.xin_gpu_picture()
        for i, t in enumerate(dev[k % len(dev)]):
            pic.plane[i] = t.data_ptr()
            pic.stride[i] = t.shape[1]
        qp = QPS[k % 3]
        pic.qp, pic.uv_qp, pic.sad_lambda = qp, qp, lam[qp]
        assert lib.xin_gpu_frame_submit(h, C.byref(pic)) == 0, lib.xin_gpu_last_error()
        assert lib.xin_gpu_frame_wait(h, C.byref(res), -1) == 0, lib.xin_gpu_last_error()

    for k in range(1 + max(3, warmup)):
        submit(k)
    ms, stage = [], np.zeros(4)
    for k in range(steps):
        flush.fill_(k & 255)
        torch.cuda.synchronize()
        submit(10 + k)
        ms.append(res.gpu_ms)
        st = (C.c_float * 4)()
        lib.xin_gpu_stream_stage_ms(h, st)
        stage += np.array(list(st))
    lib.xin_gpu_stream_close(h)
    stage /= steps
    return {"library": f"{bitdepth}-bit",
            "pictures": "8-bit" if (bitdepth == 8 or input_bitdepth == 8) else "10-bit samples (8-bit << 2)",
            "search": "by resolution levels (1/4 exhaustive, 1/2 and full +-1)" if search_mode else "exhaustive",
            "value": W * H * steps / (float(np.sum(ms)) * 1e-3) / 1e6, "unit": "Mpixel/s",
            "ms_per_picture": float(np.mean(ms)),
            "stage_ms": {"prep": stage[0], "integer_search": stage[1], "subpel_mc_tq": stage[2], "copies": stage[3]}}


def preset4_bench(torch, flush, frames, steps, warmup, cpu_seconds=8.0):
    """The preset-4 hot path at 1080p (the named configuration's search and TU
    work, as far as the frame form carries them): 8-bit pictures coded by the
    10-bit library, integer search by resolution levels (motionSearchMode 2)
    over +-64, full sub-pel search, SATD cost of the final prediction, and per
    CU every transform candidate -- luma DCT2 and the four MTS pairs up to 32,
    chroma DCT2 -- through dependent quantisation (seeded CABAC context set),
    inverse transform and reconstruction; QP 27/32/37 cycling.  Device-resident
    pictures, CUDA-event device time per picture, L2 flushed between pictures;
    beside it the oracle on a sample of the same CTUs on one host core."""
    from xin26x_gb300 import _lib, synth
    lib = _lib.load(BD)
    assert lib.xin_gpu_init(torch.cuda.current_device()) == 0
    ctx = np.ascontiguousarray(synth.contexts(np.random.default_rng(4), 1)[0])
    dev = [tuple(torch.from_numpy(np.ascontiguousarray(p)).cuda() for p in f) for f in frames]
    cfg = _lib.xin_gpu_stream_cfg(W, H, 64, SEARCH, sum(LEVELS), 0, 1, 1, IN_BD, 1, 1)
    h = C.c_void_p()
    assert lib.xin_gpu_stream_open(C.byref(cfg), C.byref(h)) == 0, lib.xin_gpu_last_error()
    assert lib.xin_gpu_stream_set_contexts(h, ctx.ctypes.data) == 0
    res = _lib.xin_gpu_results()

    def submit(k):
        pic = _lib.xin_gpu_picture()
        for i, t in enumerate(dev[k % len(dev)]):
            pic.plane[i] = t.data_ptr()
            pic.stride[i] = t.shape[1]
        qp = QPS[k % 3]
        pic.qp, pic.uv_qp, pic.sad_lambda = qp, qp, LAMBDA_BD[qp]
        assert lib.xin_gpu_frame_submit(h, C.byref(pic)) == 0, lib.xin_gpu_last_error()
        assert lib.xin_gpu_frame_wait(h, C.byref(res), -1) == 0, lib.xin_gpu_last_error()

    for k in range(1 + max(3, warmup)):
        submit(k)
    launches0 = lib.xin_gpu_kernel_launches()
    ms, stage = [], np.zeros(4)
    for k in range(steps):
        flush.fill_(k & 255)
        torch.cuda.synchronize()
        submit(10 + k)
        ms.append(res.gpu_ms)
        st = (C.c_float * 4)()
        lib.xin_gpu_stream_stage_ms(h, st)
        stage += np.array(list(st))
    launches = (lib.xin_gpu_kernel_launches() - launches0) / steps
    lib.xin_gpu_stream_close(h)
    stage /= steps
    value = W * H * steps / (float(np.sum(ms)) * 1e-3) / 1e6
    out = {"workload": "1080p, 8-bit 4:2:0 pictures coded at 10 bits, search by resolution levels (+-64), full sub-pel "
                       "search, SATD cost, per CU luma DCT2 + MTS 2..5 (CUs up to 32) and chroma DCT2, each through "
                       "dependent quantisation, inverse transform and reconstruction; CU levels 64/32/16/8, TU = CU, "
                       "QP 27/32/37 cycling, low-delay P with one reference",
           "value": value, "unit": "Mpixel/s", "ms_per_picture": float(np.mean(ms)),
           "stage_ms": {"prep": stage[0], "integer_search": stage[1], "subpel_mc_tu": stage[2], "copies": stage[3]},
           "gpu_launches_per_picture": launches, "l2": "flushed between pictures (512 MB write outside the timed events)",
           "not_covered": "random access with bi-prediction and DMVR (built per call, not in the frame form), BT/TT "
                          "and 4x4 / 128x128 CUs, RDOQ, the host's choice among the candidates"}
    # end to end through the public API with host buffers, two pictures in flight: the
    # TU stage of picture k (its own picture set, stream and TU state) runs beside the
    # search and tails of picture k + 1.  The working set of a picture (its TU state,
    # about 0.5 GB) is above L2.
    from xin26x_gb300.frame import FrameStream
    fs = FrameStream(W, H, search_range=SEARCH, levels=LEVELS, out_q=True, out_rec=False, use_graph=True, bitdepth=BD,
                     input_bitdepth=IN_BD, search_mode=1, tu_mode=1, contexts=ctx, dpb=3)
    n_e2e = max(steps, 10)
    h2d = W * H * 3 // 2
    d2h = fs.ncus * (64 + 64) + sum((W * H if p == 0 else W * H // 4) * len(LEVELS) * 4 for p in range(3))

    def e2e_submit(k):
        qp = QPS[k % 3]
        fs.submit(*frames[k % len(frames)], qp=qp, uv_qp=qp, sad_lambda=LAMBDA_BD[qp])

    e2e_submit(0)
    fs.wait(copy=False)
    e2e_submit(1)
    for k in range(max(3, warmup)):
        e2e_submit(k + 2)
        fs.wait(copy=False)
    t0 = time.perf_counter()
    for k in range(n_e2e):
        e2e_submit(k + 2 + max(3, warmup))
        fs.wait(copy=False)
    el = time.perf_counter() - t0
    fs.wait(copy=False)
    fs.close()
    out["e2e_two_in_flight"] = {"value": W * H * n_e2e / el / 1e6, "unit": "Mpixel/s", "pictures": n_e2e,
                                "ms_per_picture": el * 1e3 / n_e2e, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                                "note": "host 8-bit planes in, CU records, per-CU transform-candidate records and "
                                        "coefficient planes out; wall clock over the pictures"}
    # the oracle on the same pictures: random 64x64 CTUs, all four levels, one core
    from tests import oracle_frame
    cur, ref = [tuple(p.astype(np.uint16) << (BD - IN_BD) for p in f) for f in (frames[1], frames[0])]
    levels, first = [], 0
    for sz in LEVELS:
        levels.append((sz, first, W // sz, H // sz))
        first += (W // sz) * (H // sz)
    ctus = [(x, y) for y in range(0, H - 63, 64) for x in range(0, W - 63, 64)]
    order = np.random.default_rng(6).permutation(len(ctus))
    done, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < cpu_seconds and done < len(order):
        cx, cy = ctus[order[done]]
        cus = [f + ((cy + yy) // sz) * nx + (cx + xx) // sz for (sz, f, nx, ny) in levels
               for yy in range(0, 64, sz) for xx in range(0, 64, sz)]
        oracle_frame.run(cur, ref, levels, search_range=SEARCH, qp=32, uv_qp=32, sad_lambda=LAMBDA_BD[32], bitdepth=BD,
                         cus=cus, search_mode=1, tu_mode=1, contexts=ctx)
        done += 1
    el = time.perf_counter() - t0
    cpu = done * 64 * 64 / el / 1e6
    out["cpu_oracle"] = {"value": cpu, "unit": "Mpixel/s", "cores": 1, "kind": "port",
                         "sample": f"{done} random 64x64 CTUs of the same workload (all four levels, QP 32), "
                                   f"oracle C restatement, 1 thread, {el:.1f} s"}
    out["gpu_over_cpu_core"] = value / cpu if cpu else None
    return out


def wide_search_bench(torch, flush, pictures=3, search_mode=0):
    """3840x2160 10-bit 4:2:0, CTU 128, +-256 integer search (the reference's
    maximum picture size and a wide search; exhaustive, or by resolution levels
    with search_mode 1), full sub-pel search and TQ of CU levels 64/32/16/8;
    device-resident pictures, CUDA-event device time per picture, L2 flushed
    between pictures."""
    from xin26x_gb300 import _lib, synth
    w, h, r = 3840, 2160, 256
    g = _lib.load(10)
    assert g.xin_gpu_init(torch.cuda.current_device()) == 0
    seq = synth.sequence(w, h, pictures, seed=2160, bitdepth=10, objects=8, octaves=4)
    dev = [tuple(torch.from_numpy(np.ascontiguousarray(p)).cuda() for p in f) for f in seq]
    # the search by levels also takes the 128 x 128 CU level (CTU 128)
    mask = 120 | (128 if search_mode == 1 else 0)
    cfg = _lib.xin_gpu_stream_cfg(w, h, 128, r, mask, 0, 1, 1, 0, search_mode)
    hs = C.c_void_p()
    assert g.xin_gpu_stream_open(C.byref(cfg), C.byref(hs)) == 0, g.xin_gpu_last_error()
    res = _lib.xin_gpu_results()
    ms, stage = [], np.zeros(4)
    for k in range(pictures):
        flush.fill_(k & 255)
        torch.cuda.synchronize()
        pic = _lib.xin_gpu_picture()
        for i, t in enumerate(dev[k]):
            pic.plane[i] = t.data_ptr()
            pic.stride[i] = t.shape[1]
        pic.qp = pic.uv_qp = (27, 32, 37)[k % 3]
        pic.sad_lambda = LAMBDA[pic.qp]
        assert g.xin_gpu_frame_submit(hs, C.byref(pic)) == 0, g.xin_gpu_last_error()
        assert g.xin_gpu_frame_wait(hs, C.byref(res), -1) == 0, g.xin_gpu_last_error()
        if k:
            st = (C.c_float * 4)()
            g.xin_gpu_stream_stage_ms(hs, st)
            stage += np.array(list(st))
            ms.append(res.gpu_ms)
    g.xin_gpu_stream_close(hs)
    stage /= len(ms)
    if search_mode == 1:
        # work of the quarter-resolution level (the bulk): every CU of each level,
        # (2 * (R >> 2) + 1)^2 candidates of (S/4)^2 samples
        algo = sum((w // sz) * (h // sz) * (sz // 4) ** 2 for sz in (128, 64, 32, 16, 8)) * (2 * (r >> 2) + 1) ** 2
        return {"workload": "3840x2160 10-bit 4:2:0, CTU 128, +-256 integer search by resolution levels (1/4 "
                            "exhaustive +-64, 1/2 and full resolution +-1), full sub-pel search, CU levels "
                            "128/64/32/16/8 (128 x 128 CUs as four 64 x 64 TUs), DCT2, seeded texture (4 octaves) + 8 "
                            "moving rectangles",
                "pictures_timed": len(ms), "ms_per_picture": float(np.mean(ms)), "value": w * h / float(np.mean(ms)) / 1e3,
                "unit": "Mpixel/s", "dtype": "u16",
                "stage_ms": {"prep": stage[0], "integer_search": stage[1], "subpel_mc_tq": stage[2]},
                "search_absdiff_per_s": algo / (stage[1] * 1e-3),
                "search_algorithmic": f"every CU of the five levels x (2*64+1)^2 candidates x (S/4)^2 samples = "
                                      f"{algo:.4g} abs differences at 1/4 resolution"}
    peak = C.c_double()
    g.xin_gpu_measure_sad_peak(C.byref(peak))
    algo = (w // 8) * (h // 8) * (2 * r + 1) ** 2 * 64
    achieved = algo / (stage[1] * 1e-3)
    return {"workload": "3840x2160 10-bit 4:2:0, CTU 128, exhaustive +-256 integer search + full sub-pel search, "
                        "CU levels 64/32/16/8, DCT2 TU=CU, seeded texture (4 octaves) + 8 moving rectangles",
            "pictures_timed": len(ms), "ms_per_picture": float(np.mean(ms)), "value": w * h / float(np.mean(ms)) / 1e3,
            "unit": "Mpixel/s", "dtype": "u16",
            "stage_ms": {"prep": stage[0], "integer_search": stage[1], "subpel_mc_tq": stage[2]},
            "roofline": {"bound": "int", "kernel": "k_me_tiles (10-bit)", "achieved": achieved / 1e12,
                         "peak": peak.value / 1e12, "unit": "Tabsdiff/s", "frac": achieved / peak.value,
                         "peak_source": "xin_gpu_measure_sad_peak of the 10-bit library: packed 16-bit add-then-max "
                                        "register loop on this GPU, this run",
                         "algorithmic": f"(W/8)(H/8)(2R+1)^2*64 = {algo:.4g} abs differences per launch"}}


def _measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return None


def quant_params(qp, lg, bd=8):
    """Square-TU DCT2 quant parameters, P picture, no RDOQ (h266_trans_quant.c:104-120):
    the 10-bit build adds 12 to the QP."""
    qp = qp + (12 if bd == 10 else 0)
    qm = (26214, 23302, 20560, 18396, 16384, 14564)[qp % 6]
    iqm = (40, 45, 51, 57, 64, 72)[qp % 6] << (qp // 6)
    qs = 14 + (15 - bd) + qp // 6 - lg
    iqs = 6 - (15 - bd) + lg
    return qm, 85 << (qs - 9), qs, iqm, 1 << (iqs - 1), iqs


def percall_sample(lib, frames, seconds=6.0, bd=8):
    """Plain per-call GPU form: the same CU hot path as ~20 synchronous per-call
    launches per CU (integer search, sub-pel search, luma and chroma MC, per plane
    residual, DCT2, quant, inverse DCT2, reconstruction) on a sample of CUs;
    Mpixel/s extrapolated per CU area."""
    from xin26x_gb300 import _lib
    from xin26x_gb300.synth import pad_plane
    pix_t, coef_t = (np.uint8, np.int16) if bd == 8 else (np.uint16, np.int32)
    cur, ref = [tuple(p.astype(pix_t) << (bd - 8) for p in f) for f in (frames[1], frames[0])]
    pad = 80
    refp = [pad_plane(ref[0], pad), pad_plane(ref[1], pad // 2), pad_plane(ref[2], pad // 2)]
    rng = np.random.default_rng(3)
    me = _lib.xin_gpu_me_struct()
    pix = 0
    ncu = 0
    calls = 0
    t0 = time.perf_counter()
    P = lambda a, off=0: a.ctypes.data + off * a.itemsize  # noqa: E731
    while time.perf_counter() - t0 < seconds:
        s = int(rng.choice(LEVELS, p=[0.1, 0.2, 0.3, 0.4]))
        cx = int(rng.integers(0, W // s)) * s
        cy = int(rng.integers(0, H // s)) * s
        inp = np.ascontiguousarray(cur[0][cy:cy + s, cx:cx + s])
        me.width = me.height = s
        me.input, me.inputStride = inp.ctypes.data, s
        me.ref, me.refStride = P(refp[0], (pad + cy) * refp[0].shape[1] + pad + cx), refp[0].shape[1]
        me.searchWidth = me.searchHeight = SEARCH
        me.predMv.mvX = me.predMv.mvY = 0
        me.bestMv.mvX = me.bestMv.mvY = 0
        me.bestCost = 0xFFFFFFFF
        me.minMv.mvX, me.minMv.mvY = -cx - 72, -cy - 72
        me.maxMv.mvX, me.maxMv.mvY = W + 72 - s - cx, H + 72 - s - cy
        me.sadLambda = LAMBDA[32] << (bd - 8)
        lib.XinGpuMotionEstFull(C.byref(me))
        lib.XinGpuFullSubPelMe(C.byref(me))
        calls += 2
        mvx, mvy = me.bestMv.mvX * 4, me.bestMv.mvY * 4
        pred = np.zeros((s, s), pix_t)
        ox, oy = cx * 16 + mvx, cy * 16 + mvy
        frac = ((oy & 15) << 4) | (ox & 15)
        src = P(refp[0], (pad + (oy >> 4)) * refp[0].shape[1] + pad + (ox >> 4))
        fn = [lib.XinGpuInterpCopy, lib.XinGpuLumaInterpHor, lib.XinGpuLumaInterpVet, lib.XinGpuLumaInterpHorVet][
            (1 if frac & 15 else 0) + (2 if frac >> 4 else 0)]
        fn(src, refp[0].shape[1], pred.ctypes.data, s, frac, s, s, 0)
        calls += 1
        coef = np.zeros((s, s), coef_t)
        t = np.zeros((s, s), coef_t)
        q = np.zeros((s, s), coef_t)
        r = np.zeros((s, s), coef_t)
        rec = np.zeros((s, s), pix_t)
        nz = np.zeros(1, np.uint64)
        for p in range(3):
            bs = s if p == 0 else s // 2
            if p:
                pc = np.zeros((bs, bs), pix_t)
                cfx, cfy = (cx * 16 + mvx) & 31, (cy * 16 + mvy) & 31
                csrc = P(refp[p], (pad // 2 + ((cy * 16 + mvy) >> 5)) * refp[p].shape[1] + pad // 2 + ((cx * 16 + mvx) >> 5))
                lib.XinGpuChromaInterpHorVet(csrc, refp[p].shape[1], pc.ctypes.data, bs, (cfy << 5) | cfx, bs, bs, 0)
                pr, org = pc, np.ascontiguousarray(cur[p][cy // 2:cy // 2 + bs, cx // 2:cx // 2 + bs])
                calls += 1
            else:
                pr, org = pred, inp
            lg = bs.bit_length() - 1
            lib.XinGpuBlockSubForDct(org.ctypes.data, bs, pr.ctypes.data, bs, coef.ctypes.data, bs, bs, bs)
            lib.XinGpuFDct2WxH(coef.ctypes.data, bs, t.ctypes.data, bs, bs, bs, None, lg + bd - 9, lg + 6)
            k = min(bs, 32)
            qm, qa, qs, iqm, iqa, iqs = quant_params(32, lg, bd)
            lib.XinGpuQuantInvQuant(q.ctypes.data, t.ctypes.data, r.ctypes.data, bs, k, k, 4, 4, qm, qa, qs, iqm, iqa, iqs,
                                    nz.ctypes.data)
            lib.XinGpuIDct2WxH(r.ctypes.data, bs, coef.ctypes.data, bs, bs, bs, None, 7, 20 - bd)
            lib.XinGpuBlockAddForDct(coef.ctypes.data, bs, pr.ctypes.data, bs, rec.ctypes.data, bs, bs, bs)
            calls += 5
        _lib.check(lib, "per-call sample")
        pix += s * s
        ncu += 1
    el = time.perf_counter() - t0
    return {"value": pix / el / 1e6, "unit": "Mpixel/s", "cus": ncu, "calls": calls, "seconds": el,
            "sample": f"random CUs of the four levels (10/20/30/40 % of 64/32/16/8), ~20 synchronous C-ABI calls each, "
                      f"{bd}-bit library"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
