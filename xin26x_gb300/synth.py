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
