"""Seeded synthetic YUV 4:2:0 sequences with the shapes and statistics of the
benchmark configurations (the reference's CTC sequences are not available).

Luma texture: clamp(128 + 40 sin(x/7) + 30 cos(y/11) + N(0, 6)) (x4 for 10-bit).
Picture k is picture 0 moved by a seeded motion, bilinear resampling:
  * mode "shift":   a global (dx, dy) uniform in [-8, 8] at quarter-pel per picture
  * mode "objects": the global shift plus `objects` rectangles (64..256 px) of a
                    second texture moving with seeded velocities up to +-24 px/picture
Chroma: 2x2 average of the luma texture + N(0, 3).
"""
from __future__ import annotations

import numpy as np


def _bilinear(img: np.ndarray, dx: float, dy: float) -> np.ndarray:
    h, w = img.shape
    ys = np.clip(np.arange(h)[:, None] + dy, 0, h - 1)
    xs = np.clip(np.arange(w)[None, :] + dx, 0, w - 1)
    y0 = np.floor(ys).astype(np.int64)
    x0 = np.floor(xs).astype(np.int64)
    y1 = np.minimum(y0 + 1, h - 1)
    x1 = np.minimum(x0 + 1, w - 1)
    fy = ys - y0
    fx = xs - x0
    a = img[y0, x0] * (1 - fx) + img[y0, x1] * fx
    b = img[y1, x0] * (1 - fx) + img[y1, x1] * fx
    return a * (1 - fy) + b * fy


def sequence(width: int, height: int, frames: int, seed: int, bitdepth: int = 8, objects: int = 0,
             octaves: int = 1):
    """Returns a list of (Y, U, V) uint8/uint16 planes."""
    rng = np.random.default_rng(seed)
    scale = 1 << (bitdepth - 8)
    maxv = (1 << bitdepth) - 1
    x = np.arange(width, dtype=np.float64)[None, :]
    y = np.arange(height, dtype=np.float64)[:, None]
    tex = 128 + 40 * np.sin(x / 7) + 30 * np.cos(y / 11)
    for o in range(1, octaves):
        tex = tex + (20.0 / o) * np.sin(x / (7 / (2 ** o)) + o) * np.cos(y / (11 / (2 ** o)) + 2 * o)
    base = tex + rng.normal(0, 6, size=tex.shape)
    obj_tex = 128 + 50 * np.sin((x + y) / 5) * np.cos((x - y) / 9)
    objs = []
    for _ in range(objects):
        lo_w, hi_w = min(64, width // 4), min(256, width // 2)
        lo_h, hi_h = min(64, height // 4), min(256, height // 2)
        ow, oh = int(rng.integers(lo_w, hi_w + 1)), int(rng.integers(lo_h, hi_h + 1))
        ox, oy = float(rng.integers(0, max(1, width - ow))), float(rng.integers(0, max(1, height - oh)))
        vx, vy = float(rng.uniform(-24, 24)), float(rng.uniform(-24, 24))
        objs.append((ow, oh, ox, oy, vx, vy))
    out = []
    for k in range(frames):
        if k == 0:
            dx = dy = 0.0
        else:
            dx, dy = rng.integers(-32, 33, size=2) / 4.0
        luma = _bilinear(base, dx, dy) if k else base.copy()
        for (ow, oh, ox, oy, vx, vy) in objs:
            px, py = int(round(ox + vx * k)) % max(1, width - ow), int(round(oy + vy * k)) % max(1, height - oh)
            luma[py:py + oh, px:px + ow] = obj_tex[:oh, :ow]
        ycl = np.clip(np.rint(luma * scale), 0, maxv)
        c = 0.25 * (luma[0::2, 0::2] + luma[1::2, 0::2] + luma[0::2, 1::2] + luma[1::2, 1::2])
        u = np.clip(np.rint((c + rng.normal(0, 3, size=c.shape)) * scale), 0, maxv)
        v = np.clip(np.rint((255 - c + rng.normal(0, 3, size=c.shape)) * scale), 0, maxv)
        dt = np.uint8 if bitdepth == 8 else np.uint16
        out.append((ycl.astype(dt), u.astype(dt), v.astype(dt)))
    return out


def pad_plane(p: np.ndarray, pad: int) -> np.ndarray:
    """Edge-replicated padding (the reference-picture layout)."""
    return np.pad(p, pad, mode="edge")


TQ_BLOCK_DTYPE = np.dtype([("offset", "<u4"), ("log2w", "u1"), ("log2h", "u1"), ("mts", "u1"), ("flags", "u1"),
                           ("qp", "<i4")])     # xin_gpu_tq_block, 12 bytes


def tq_blocks(n: int, seed: int, bitdepth: int = 10, kernel_bench_mix: bool = True):
    """Seeded residual blocks for xin_gpu_tq_batch: (blocks, residuals).

    Sides 4..64 drawn per axis with P(4, 8, 16, 32, 64) = (.12, .34, .30, .16, .08),
    a geometric-like tail biased to 8 and 16.  kernel_bench_mix: residuals are
    11-bit signed Laplacian (scale 12) clipped to +-1023, DCT2 70 % and the four
    DST7/DCT8 pairs 30 % on blocks with both sides <= 32 (no 64-point DST7/DCT8
    exists), QP uniform in [22, 42], no flags.  Otherwise: Laplacian scale 60
    clipped to the bit depth, every MTS index (skip and the pairs only up to 32),
    QP 0..63 and every flag combination."""
    rng = np.random.default_rng(seed)
    p = np.array([0.12, 0.34, 0.30, 0.16, 0.08])
    b = np.zeros(n, TQ_BLOCK_DTYPE)
    lw = rng.choice(5, size=n, p=p) + 2
    lh = rng.choice(5, size=n, p=p) + 2
    small = (lw <= 5) & (lh <= 5)
    if kernel_bench_mix:
        mts = np.where((rng.random(n) < 0.3) & small, rng.integers(2, 6, size=n), 0)
        qp = rng.integers(22, 43, size=n)
        flags = np.zeros(n, np.int64)
    else:
        mts = np.where(small, rng.integers(0, 6, size=n), 0)
        qp = rng.integers(0, 64, size=n)
        flags = rng.integers(0, 32, size=n)
    area = (1 << (lw + lh)).astype(np.int64)
    off = np.concatenate(([0], np.cumsum(area)[:-1]))
    b["offset"], b["log2w"], b["log2h"], b["mts"], b["flags"], b["qp"] = off, lw, lh, mts, flags, qp
    lim = 1023 if kernel_bench_mix else (1 << bitdepth) - 1
    scale = 12 if kernel_bench_mix else 60
    resid = np.clip(np.rint(rng.laplace(0, scale, size=int(area.sum()))), -lim, lim)
    return b, resid.astype(np.int16 if bitdepth == 8 else np.int32)


DQ_BLOCK_DTYPE = np.dtype([("offset", "<u4"), ("stride", "<u2"), ("log2_w", "u1"), ("log2_h", "u1"), ("qp", "u1"),
                           ("comp", "u1"), ("root_cbf", "u1"), ("reserved", "u1"), ("ctx_set", "<u4")])   # xin_gpu_dq_block
PROB_DTYPE = np.dtype([("s0", "<u2"), ("s1", "<u2"), ("rate", "u1"), ("pad", "u1")])   # xin_gpu_prob (xin_prob_model)
NUM_CTX = 401


def contexts(rng, n_sets: int = 1) -> np.ndarray:
    """Seeded CABAC context states in the reference layout: n_sets x NUM_CTX records
    (10-bit and 14-bit probability windows, as the encoder keeps them)."""
    a = np.zeros((n_sets, NUM_CTX), PROB_DTYPE)
    a["s0"] = rng.integers(0, 1024, size=a.shape) << 5
    a["s1"] = rng.integers(0, 16384, size=a.shape) << 1
    a["rate"] = rng.integers(0, 256, size=a.shape)
    return a


def coefficients(rng, w: int, h: int, bitdepth: int, scale: float = None) -> np.ndarray:
    """Seeded transform coefficients shaped like a residual spectrum: Laplacian
    magnitudes decaying away from DC, random zero runs and sparse large values."""
    coef = np.int16 if bitdepth == 8 else np.int32
    if scale is None:
        scale = float(rng.choice([2.0, 8.0, 40.0, 200.0, 1500.0]))
    y, x = np.mgrid[0:h, 0:w]
    decay = np.exp(-(x + y) / max(1.0, rng.uniform(1.0, 12.0)))
    v = rng.laplace(0, scale, size=(h, w)) * (0.15 + decay)
    v[rng.random((h, w)) < rng.uniform(0.0, 0.6)] = 0
    big = rng.random((h, w)) < 0.01
    v[big] = rng.choice([-1, 1], size=big.sum()) * rng.uniform(2000, 30000, size=big.sum())
    return np.clip(np.rint(v), -32768, 32767).astype(coef)


def dq_blocks(n: int, seed: int, bitdepth: int = 10, n_sets: int = 1, qp_range=None, any_mix: bool = False):
    """Seeded blocks for xin_gpu_dep_quant_batch: (blocks, coefficients, context sets).

    Shapes as tq_blocks (sides 4..64, P(4, 8, 16, 32, 64) = (.12, .34, .30, .16, .08)
    per axis), blocks packed one after another (stride = width), components
    luma 2/3 and Cb / Cr 1/6 each, root cbf on half of the luma blocks.  QP: the
    QP the reference's TU driver passes to the trellis, slice QP U[22, 39]
    (+12 at 10-bit), or qp_range.  any_mix: coefficient magnitudes spread from
    near-zero to large (the parity mix); otherwise the spectrum of an
    11-bit Laplacian residual (scale 12) after a DCT2 of the block's size."""
    rng = np.random.default_rng(seed)
    p = np.array([0.12, 0.34, 0.30, 0.16, 0.08])
    lw = rng.choice(5, size=n, p=p) + 2
    lh = rng.choice(5, size=n, p=p) + 2
    b = np.zeros(n, DQ_BLOCK_DTYPE)
    area = (1 << (lw + lh)).astype(np.int64)
    off = np.concatenate(([0], np.cumsum(area)[:-1]))
    lo, hi = qp_range if qp_range else (22 + (12 if bitdepth == 10 else 0), 39 + (12 if bitdepth == 10 else 0))
    comp = rng.choice(3, size=n, p=[2 / 3, 1 / 6, 1 / 6])
    b["offset"], b["stride"], b["log2_w"], b["log2_h"] = off, 1 << lw, lw, lh
    b["qp"] = rng.integers(lo, hi + 1, size=n)
    b["comp"] = comp
    b["root_cbf"] = (comp == 0) & (rng.random(n) < 0.5)
    b["ctx_set"] = rng.integers(0, n_sets, size=n)
    coef = np.zeros(int(area.sum()), np.int16 if bitdepth == 8 else np.int32)
    for i in range(n):
        w, h = 1 << int(lw[i]), 1 << int(lh[i])
        if any_mix:
            c = coefficients(rng, w, h, bitdepth)
        else:
            # DCT2 of a Laplacian(12) residual keeps its energy: the coefficient
            # std grows with sqrt(w*h) at the transform's output scaling
            c = coefficients(rng, w, h, bitdepth, scale=12.0 * np.sqrt(w * h) / 8.0)
        coef[off[i]:off[i] + w * h] = c.ravel()
    return b, coef, contexts(rng, n_sets)


def _diag_scan(w: int, h: int):
    """up-right diagonal scan of a w x h grid: (x, y) per scan index"""
    out, x, y = [], 0, 0
    for _ in range(w * h):
        out.append((x, y))
        if x == w - 1 or y == 0:
            y += x + 1
            x = 0
            if y >= h:
                x += y - (h - 1)
                y = h - 1
        else:
            x += 1
            y -= 1
    return out


_RASTER_OF_SCAN: dict = {}


def dq_steps(blocks, t, bitdepth: int) -> np.ndarray:
    """Trellis length of each block: 1 + the highest scan index whose |t| exceeds
    the last-position threshold (thresLast / (qScale << 2) of the trellis
    parameters), 0 for blocks with none.  This is the number of coefficient
    steps the trellis walks; it is the work unit of the dependent-quantisation
    throughput figures."""
    qm = ((26214, 23302, 20560, 18396, 16384, 14564), (18396, 16384, 14564, 13107, 11651, 10280))
    out = np.zeros(len(blocks), np.int64)
    for i, b in enumerate(blocks):
        lw, lh, qp = int(b["log2_w"]), int(b["log2_h"]), int(b["qp"])
        ew, eh, st, off = min(1 << lw, 32), min(1 << lh, 32), int(b["stride"]), int(b["offset"])
        key = (ew, eh, st)
        if key not in _RASTER_OF_SCAN:
            cg = _diag_scan(ew // 4, eh // 4)
            inner = _diag_scan(4, 4)
            _RASTER_OF_SCAN[key] = np.array([(gy * 4 + iy) * st + gx * 4 + ix for gx, gy in cg for ix, iy in inner])
        lg = lw + lh
        adj, per, rem = lg & 1, (qp + 1) // 6, (qp + 1) % 6
        ts = 15 - bitdepth - (lg >> 1) - adj
        qshift = 13 + per + ts
        thr = (8 << (qshift - 1) if qshift else 4) // (qm[adj][rem] << 2)
        v = np.abs(t[off + _RASTER_OF_SCAN[key]].astype(np.int64))
        hit = np.nonzero(v > thr)[0]
        out[i] = hit[-1] + 1 if hit.size else 0
    return out

def ra_gop(gop: int, ngops: int):
    """Random-access coding order of ngops GOPs of size gop (a power of two)
    after picture 0: a list of (poc, ref0_poc, ref1_poc).  Each GOP codes its
    key picture (both references the previous key picture), then the pictures
    between, halving: a B picture's list 0 is the nearest coded picture before
    it and list 1 the nearest after it (the hierarchy of the reference's
    random-access GOP)."""
    out = []
    for gi in range(ngops):
        base = gi * gop
        key = base + gop
        out.append((key, base, base))

        def split(lo, hi):
            if hi - lo < 2:
                return
            mid = (lo + hi) // 2
            out.append((mid, lo, hi))
            split(lo, mid)
            split(mid, hi)

        split(base, key)
    return out
