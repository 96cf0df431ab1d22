"""Oracle of the batched frame form: runs oracle/xin_oracle.c's per-CU hot path
(orc_cu_hotpath) over every CU of every level, in the library's output order.
Test infrastructure only."""
from __future__ import annotations

import ctypes as C
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from oracle import oracle as O
from xin26x_gb300.frame import BI_DTYPE, CU_DTYPE, MTS_DTYPE
from xin26x_gb300.synth import pad_plane


def downscaled(plane, o, levels=2):
    """The plane at 1/2 and 1/4 resolution by the oracle's 2x2 downscale."""
    out = []
    src = np.ascontiguousarray(plane)
    for _ in range(levels):
        h, w = src.shape[0] // 2, src.shape[1] // 2
        dst = np.zeros((h, w), src.dtype)
        o.downscale2x2(src.ctypes.data, src.shape[1], 0, 0, dst.ctypes.data, w, w, h)
        out.append(dst)
        src = dst
    return out


def run(cur, ref, levels, ctu=64, search_range=16, qp=32, uv_qp=32, sad_lambda=64, bitdepth=8, cus=None, threads=1,
        search_mode=0, tu_mode=0, contexts=None, ref1=None):
    """cur, ref: (Y, U, V) planes.  levels: [(size, first, cus_x, cus_y)] as the stream reports.
    cus: optional list of global CU indices to evaluate (others left zero).
    search_mode: 0 exhaustive integer search, 1 by resolution levels (the reference
    and the current picture downscaled by 2 and 4, the padded reference as a whole).
    tu_mode 1: the preset-4 TU (transform candidates with dependent quantisation,
    rates from contexts); the transform candidates' records are returned too.
    threads: host threads sharing the CUs (0 = every core); each CU writes only its
    own record and its own area of the level's planes, so the calls are independent.
    ref1: list 1's planes (two references and the bi search); its records
    (BI_DTYPE) are returned last.
    Returns (cu records, q planes [levels,h,w] x3, rec planes x3)."""
    o = O.oracle(bitdepth)
    h, w = cur[0].shape
    pad = ctu + 16
    refp = [pad_plane(ref[0], pad), pad_plane(ref[1], pad // 2), pad_plane(ref[2], pad // 2)]
    curc = [np.ascontiguousarray(p) for p in cur]
    f = O.orc_frame_desc()
    f.width, f.height, f.ctu = w, h, ctu
    for i in range(3):
        f.in_[i] = curc[i].ctypes.data
        pp = pad if i == 0 else pad // 2
        f.ref[i] = refp[i].ctypes.data + (pp * refp[i].shape[1] + pp) * refp[i].itemsize
    f.in_stride[0], f.in_stride[1] = w, w // 2
    f.ref_stride[0], f.ref_stride[1] = refp[0].shape[1], refp[1].shape[1]
    f.search_range, f.sad_lambda, f.qp, f.uv_qp, f.intra_frame = search_range, sad_lambda, qp, uv_qp, 0
    f.search_mode = search_mode
    f.tu_mode = tu_mode
    ref1p = None
    if ref1 is not None:
        ref1p = [pad_plane(ref1[0], pad), pad_plane(ref1[1], pad // 2), pad_plane(ref1[2], pad // 2)]
        f.refs = 2
        for i in range(3):
            pp = pad if i == 0 else pad // 2
            f.ref1[i] = ref1p[i].ctypes.data + (pp * ref1p[i].shape[1] + pp) * ref1p[i].itemsize
    ctx = None
    if tu_mode:
        ctx = np.ascontiguousarray(contexts)
        f.ctx = ctx.ctypes.data
    keep = []
    if search_mode == 1:
        ref_lo, in_lo = downscaled(refp[0], o), downscaled(curc[0], o)
        keep = ref_lo + in_lo
        for l in range(2):
            pl = pad >> (l + 1)
            f.ref_lo[l] = ref_lo[l].ctypes.data + (pl * ref_lo[l].shape[1] + pl) * ref_lo[l].itemsize
            f.ref_lo_stride[l] = ref_lo[l].shape[1]
            f.in_lo[l] = in_lo[l].ctypes.data
            f.in_lo_stride[l] = in_lo[l].shape[1]
        if ref1p is not None:
            ref1_lo = downscaled(ref1p[0], o)
            keep += ref1_lo
            for l in range(2):
                pl = pad >> (l + 1)
                f.ref1_lo[l] = ref1_lo[l].ctypes.data + (pl * ref1_lo[l].shape[1] + pl) * ref1_lo[l].itemsize
    ncu = sum(cx * cy for (_, _, cx, cy) in levels)
    recs = np.zeros(ncu, CU_DTYPE)
    mts = np.zeros(ncu, MTS_DTYPE)
    bis = np.zeros(ncu, BI_DTYPE)
    nl = len(levels)
    q = [np.zeros((nl, h, w), o.coef), np.zeros((nl, h // 2, w // 2), o.coef), np.zeros((nl, h // 2, w // 2), o.coef)]
    rec = [np.zeros((nl, h, w), o.pix), np.zeros((nl, h // 2, w // 2), o.pix), np.zeros((nl, h // 2, w // 2), o.pix)]
    want = None if cus is None else set(int(c) for c in cus)
    qs = (C.c_ssize_t * 2)(w, w // 2)
    ptrs = []
    work = []
    for li, (size, first, cx, cy) in enumerate(levels):
        ptrs.append(((C.c_void_p * 3)(*[q[p][li].ctypes.data for p in range(3)]),
                     (C.c_void_p * 3)(*[rec[p][li].ctypes.data for p in range(3)])))
        for j in range(cx * cy):
            if want is None or first + j in want:
                work.append((li, size, first, cx, j))

    def one(item):
        li, size, first, cx, j = item
        out = O.orc_cu_out()
        o.cu_hotpath(C.byref(f), (j % cx) * size, (j // cx) * size, size, ptrs[li][0], qs, ptrs[li][1], qs,
                     C.byref(out))
        r = recs[first + j]
        r["mvx"], r["mvy"], r["cost"], r["int_cost"] = out.mvx, out.mvy, out.cost, out.int_cost
        r["nz"] = list(out.nz)
        r["ssd"] = list(out.ssd)
        if ref1 is not None:
            b = bis[first + j]
            b["mvx1"], b["mvy1"], b["cost1"], b["int_cost1"] = out.mvx1, out.mvy1, out.cost1, out.int_cost1
            b["bmv"] = list(out.bmv)
            b["bi_cost"], b["inter_dir"] = out.bi_cost, out.inter_dir
        if tu_mode:
            m = mts[first + j]
            m["satd_cost"], m["ncand"] = out.satd_cost, out.ncand
            m["nz"] = list(out.nz_mts)
            m["ssd"] = list(out.ssd_mts)

    nthreads = (os.cpu_count() or 1) if threads == 0 else max(1, threads)
    if nthreads == 1 or len(work) < 2:
        for item in work:
            one(item)
    else:
        # largest CUs first so that the last ones to finish are short
        work.sort(key=lambda it: -it[1])
        one(work[0])        # the oracle builds its transform matrices on first use: once, before the threads
        with ThreadPoolExecutor(nthreads) as ex:
            list(ex.map(one, work[1:]))
    if tu_mode:
        return (recs, q, rec, mts, bis) if ref1 is not None else (recs, q, rec, mts)
    if ref1 is not None:
        return recs, q, rec, bis
    return recs, q, rec
