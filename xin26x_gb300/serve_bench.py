"""48-stream serving measurement: 16 x 640x360 + 16 x 1280x720 + 16 x 1920x1080
live streams at 30 pictures/s each (1,548.3 luma Mpixel/s offered), each with
+-64 exhaustive integer search, full sub-pel search and TQ of CU levels
64/32/16/8, low-delay P.

Streams ask to join in a seeded order at seeded times over the first 0.5 s;
the server admits a stream only if its device footprint fits and the luma
Mpixel/s already promised plus its own stays within --mpix-budget.  Each
admitted stream's pictures then arrive as a Poisson process at 30 pictures/s
(exponential gaps of mean 1/30 s, seeded) plus a seeded 0..2 ms jitter
(--arrivals periodic: a picture every 1/30 s plus 0..4 ms); a picture that
finds its stream's queue full is dropped (counted).  A
quarter of the admitted streams leave at seeded times in the last 40 % of the
run.  Reported: admitted / refused streams, luma Mpixel/s completed, and the
latency of each picture from submit to results in host memory (p50 / p99 /
max), measured inside the server.

  python -m xin26x_gb300.serve_bench [--seconds 4] [--mpix-budget 1650] [--max-inflight 6] [--arrivals poisson]
"""
from __future__ import annotations

import argparse
import heapq
import json
import threading
import time

import numpy as np

CLASSES = ((640, 360), (1280, 720), (1920, 1080))
PER_CLASS = 16
FPS = 30.0
LAMBDA = {27: 45, 32: 64, 37: 91}


def run(seconds=4.0, mpix_budget=1650.0, max_inflight=6, seed=48, search_range=64, frames_per_class=6, arrivals="poisson",
        planes=False, batch_max=0):
    from xin26x_gb300 import synth
    from xin26x_gb300.server import Admission, Server

    rng = np.random.default_rng(seed)
    content = {wh: synth.sequence(wh[0], wh[1], frames_per_class, seed=seed + i, objects=4)
               for i, wh in enumerate(CLASSES)}
    streams = [(wh, j) for wh in CLASSES for j in range(PER_CLASS)]
    order = rng.permutation(len(streams))
    join_t = np.sort(rng.uniform(0, 0.5, size=len(streams)))
    offered = sum(w * h * FPS for (w, h), _ in streams) / 1e6

    srv = Server(mpix_budget=mpix_budget, max_inflight=max_inflight, max_queue=2, batch_max=batch_max)
    admitted, refused = [], []
    lat, qms, gpu, done_px = [], [], [], 0
    dropped = 0
    failed = []
    stop = threading.Event()
    lock = threading.Lock()

    def poller():
        nonlocal done_px
        while not stop.is_set() or srv.stats()["running"] or srv.stats()["queued"]:
            for d, _ in srv.poll(timeout_ms=10):
                if d.status != 0:
                    with lock:
                        failed.append((d.stream_id, d.frame_index, d.status))
                    continue
                if d.has_results:
                    with lock:
                        lat.append(d.latency_ms)
                        qms.append(d.queue_ms)
                        gpu.append(d.gpu_ms)
                        done_px += d.user_tag
            if stop.is_set() and not srv.stats()["running"] and not srv.stats()["queued"]:
                break

    # event list: (time, kind, stream number)
    events = []
    for n, si in enumerate(order):
        heapq.heappush(events, (float(join_t[n]), 0, int(si)))
    sid_of, leave_at, qbufs = {}, {}, {}
    if planes:
        # every stream's plane buffers, allocated before the clock starts: four sets of
        # pinned host memory a stream (a picture running, two queued, one being polled)
        import torch
        tdt = torch.int16 if srv.pix == np.uint8 else torch.int32
        for si, ((w, h), _) in enumerate(streams):
            qbufs[si] = [[torch.empty((4, hh, ww), dtype=tdt, pin_memory=True).numpy()
                          for hh, ww in ((h, w), (h // 2, w // 2), (h // 2, w // 2))] for _ in range(4)]
    k_of, a_of = {}, {}             # pictures accepted / arrived per stream
    th = threading.Thread(target=poller, daemon=True)
    th.start()
    t0 = time.perf_counter()
    while events:
        t, kind, si = heapq.heappop(events)
        if t > seconds:
            continue
        now = time.perf_counter() - t0
        if t > now:
            time.sleep(t - now)
        (w, h), j = streams[si]
        if kind == 0:                      # join
            try:
                sid_of[si] = srv.join(w, h, fps=FPS, search_range=search_range, out_q=planes)
            except Admission:
                refused.append(si)
                continue
            admitted.append(si)
            k_of[si] = 0
            a_of[si] = 0
            if rng.random() < 0.25:
                leave_at[si] = float(rng.uniform(0.6, 1.0) * seconds)
                heapq.heappush(events, (leave_at[si], 2, si))
            heapq.heappush(events, (t, 1, si))
        elif kind == 1:                    # picture arrival
            if si in leave_at and t >= leave_at[si]:
                continue
            k = k_of[si]
            f = content[(w, h)][(k + j) % frames_per_class]
            qp = (27, 32, 37)[k % 3]
            st = srv.submit(sid_of[si], *f, qp=qp, sad_lambda=LAMBDA[qp], tag=w * h,
                            q_out=qbufs[si][k % 4] if planes else None)
            if st == 0:
                k_of[si] = k + 1
            elif st == -6:            # queue full (or the stream failed: reported by poll)
                dropped += 1
            else:
                raise RuntimeError(f"submit failed: {st}")
            a_of[si] += 1
            if arrivals == "poisson":
                heapq.heappush(events, (t + float(rng.exponential(1.0 / FPS)) + float(rng.uniform(0, 0.002)), 1, si))
            else:
                nxt = a_of[si] / FPS + float(rng.uniform(0, 0.004))
                heapq.heappush(events, (float(join_t[list(order).index(si)]) + nxt, 1, si))
        else:                              # leave (drains the stream's queue)
            srv.leave(sid_of[si], 60000)
    wall_submit = time.perf_counter() - t0
    stop.set()
    th.join()
    wall = time.perf_counter() - t0
    sst = srv.stats()
    srv.close()
    lat_a = np.array(lat) if lat else np.zeros(1)
    by_class = {f"{w}x{h}": sum(1 for si in admitted if streams[si][0] == (w, h)) for (w, h) in CLASSES}
    return {"workload": f"{len(streams)} streams (16 x 640x360, 16 x 1280x720, 16 x 1920x1080) at 30 fps, "
                        f"+-{search_range} exhaustive search, CU levels 64/32/16/8, {seconds:.1f} s",
            "arrivals": "Poisson at 30 pictures/s per stream + 0..2 ms jitter" if arrivals == "poisson"
                        else "every 1/30 s + 0..4 ms jitter",
            "results": "CU records and every picture's coefficient planes (all levels) copied into pinned caller buffers"
                       if planes else "CU records",
            "offered_mpix_s": offered, "mpix_budget": mpix_budget, "max_inflight": max_inflight,
            "admitted": len(admitted), "refused": len(refused), "admitted_by_class": by_class,
            "pictures": len(lat), "arrived": int(sum(a_of.values())), "dropped": dropped, "failed": len(failed), "first_failures": failed[:4],
            "completed_mpix_s": done_px / 1e6 / wall_submit,
            "latency_ms": {"p50": float(np.percentile(lat_a, 50)), "p99": float(np.percentile(lat_a, 99)),
                           "max": float(lat_a.max())},
            "queue_ms_p99": float(np.percentile(qms, 99)) if qms else None,
            "gpu_ms_mean": float(np.mean(gpu)) if gpu else None,
            "cross_stream_batches": {"batch_max": batch_max or 8, "batches": int(sst["batches"]),
                                     "pictures_in_batches": int(sst["batched_pictures"]),
                                     "share_of_pictures": sst["batched_pictures"] / max(1, sst["launched"])},
            "wall_s": wall}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--seconds", type=float, default=4.0)
    ap.add_argument("--mpix-budget", type=float, default=1650.0)
    ap.add_argument("--max-inflight", type=int, default=6)
    ap.add_argument("--seed", type=int, default=48)
    ap.add_argument("--arrivals", choices=("poisson", "periodic"), default="poisson")
    ap.add_argument("--planes", action="store_true", help="every picture's coefficient planes returned too")
    ap.add_argument("--batch-max", type=int, default=0, help="pictures a cross-stream batch may carry (1 = none)")
    a = ap.parse_args()
    print(json.dumps(run(a.seconds, a.mpix_budget, a.max_inflight, a.seed, arrivals=a.arrivals, planes=a.planes,
                         batch_max=a.batch_max)), flush=True)


if __name__ == "__main__":
    main()
