"""Seeded synthetic video, flow and noise for the benchmark workloads.

The reference is tuned on external datasets that are not available here; these
generators produce inputs with the shapes, value ranges and motion of those
workloads instead:

* texture  -- a sum of 64 random 2-D cosines (frequency magnitude uniform in
  [0, 0.25] cycles/px, random orientation and phase, amplitude proportional to
  1/|f|) rescaled to [16, 240], plus 8 constant rectangles (sides 16-96 px,
  levels uniform in [16, 240]);
* motion   -- frame k+1 is frame k's background translated bilinearly by a
  seeded global shift (uniform in [-2, 2] px per axis), with 4 opaque
  rectangles moving at their own seeded velocities drawn on top;
* flow     -- the exact forward/backward displacement of that motion as
  2-channel planar float32 fields; the last forward and the first backward
  field are copies of their neighbours, as the reference's tvl1flow-seq.sh
  script does (scripts/tvl1flow-seq.sh:43,61);
* noise    -- additive white Gaussian noise of standard deviation sigma,
  not clipped.

Videos use the reference's planar layout (t, c, y, x), float32.
"""
from __future__ import annotations

import numpy as np

__all__ = ["texture", "video", "noisy", "rgb_video"]


def _rects(rng, W, H, n, smin=16, smax=96):
    out = []
    for _ in range(n):
        rw = int(rng.integers(min(smin, W), min(smax, W) + 1))
        rh = int(rng.integers(min(smin, H), min(smax, H) + 1))
        x0 = int(rng.integers(0, max(1, W - rw + 1)))
        y0 = int(rng.integers(0, max(1, H - rh + 1)))
        lvl = float(rng.uniform(16.0, 240.0))
        out.append((x0, y0, rw, rh, lvl))
    return out


def texture(W: int, H: int, seed: int, rects=None) -> np.ndarray:
    """One H x W float32 frame: cosines + constant rectangles."""
    rng = np.random.default_rng(seed)
    x = np.arange(W, dtype=np.float64)
    y = np.arange(H, dtype=np.float64)
    img = np.zeros((H, W), dtype=np.float64)
    for _ in range(64):
        fmag = rng.uniform(0.0, 0.25)
        fmag = max(fmag, 1.0 / max(W, H))          # keep 1/|f| finite
        th = rng.uniform(0.0, 2.0 * np.pi)
        ph = rng.uniform(0.0, 2.0 * np.pi)
        a, b = 2 * np.pi * fmag * np.cos(th), 2 * np.pi * fmag * np.sin(th)
        amp = 1.0 / fmag
        # cos(a x + b y + ph) = cos(a x + ph) cos(b y) - sin(a x + ph) sin(b y)
        img += amp * (np.outer(np.cos(b * y), np.cos(a * x + ph))
                      - np.outer(np.sin(b * y), np.sin(a * x + ph)))
    lo, hi = img.min(), img.max()
    img = 16.0 + (img - lo) * (224.0 / max(hi - lo, 1e-12))
    if rects is None:
        rects = _rects(rng, W, H, 8)
    for (x0, y0, rw, rh, lvl) in rects:
        img[y0:y0 + rh, x0:x0 + rw] = lvl
    return img.astype(np.float32)


def _shift_bilinear(img: np.ndarray, dx: float, dy: float) -> np.ndarray:
    """out(x, y) = img(x - dx, y - dy), bilinear, borders clamped."""
    H, W = img.shape
    xs = np.clip(np.arange(W) - dx, 0, W - 1)
    ys = np.clip(np.arange(H) - dy, 0, H - 1)
    x0 = np.floor(xs).astype(np.int64)
    y0 = np.floor(ys).astype(np.int64)
    x1 = np.minimum(x0 + 1, W - 1)
    y1 = np.minimum(y0 + 1, H - 1)
    fx = (xs - x0).astype(np.float32)[None, :]
    fy = (ys - y0).astype(np.float32)[:, None]
    r0 = img[y0][:, x0] * (1 - fx) + img[y0][:, x1] * fx
    r1 = img[y1][:, x0] * (1 - fx) + img[y1][:, x1] * fx
    return (r0 * (1 - fy) + r1 * fy).astype(np.float32)


def _motion(rng, W, H, F, n_movers=4):
    shifts = rng.uniform(-2.0, 2.0, size=(F, 2))   # shifts[k] moves frame k-1 -> k
    movers = []
    for (x0, y0, rw, rh, lvl) in _rects(rng, W, H, n_movers):
        v = rng.uniform(-2.0, 2.0, size=2)
        movers.append((x0, y0, rw, rh, lvl, float(v[0]), float(v[1])))
    return shifts, movers


def _draw(frame, mover, k, flows=None, val=None):
    x0, y0, rw, rh, lvl, vx, vy = mover
    H, W = frame.shape
    # integer raster position of the mover at frame k (exact, no resampling)
    cx = int(np.floor(x0 + k * vx + 0.5))
    cy = int(np.floor(y0 + k * vy + 0.5))
    xa, xb = max(0, cx), min(W, cx + rw)
    ya, yb = max(0, cy), min(H, cy + rh)
    if xa >= xb or ya >= yb:
        return
    frame[ya:yb, xa:xb] = lvl
    if flows is not None:
        flows[0][ya:yb, xa:xb] = val[0]
        flows[1][ya:yb, xa:xb] = val[1]


def video(W: int, H: int, F: int, seed: int, channels: int = 1):
    """Clean video (F, C, H, W) and its exact forward/backward flow (F, 2, H, W)."""
    rng = np.random.default_rng(seed)
    shifts, movers = _motion(rng, W, H, F)
    layout = _rects(np.random.default_rng(seed + 7919), W, H, 8)
    bgs = [texture(W, H, seed * 31 + 17 * c + 1, rects=layout) for c in range(channels)]
    clean = np.empty((F, channels, H, W), np.float32)
    fflow = np.empty((F, 2, H, W), np.float32)
    bflow = np.empty((F, 2, H, W), np.float32)
    for k in range(F):
        if k > 0:
            bgs = [_shift_bilinear(b, shifts[k][0], shifts[k][1]) for b in bgs]
        for c in range(channels):
            fr = bgs[c].copy()
            for m in movers:
                _draw(fr, m, k)
            clean[k, c] = fr
        # flow of the background, then of each mover (topmost last)
        nxt = shifts[k + 1] if k + 1 < F else shifts[k]
        fflow[k, 0], fflow[k, 1] = nxt[0], nxt[1]
        bflow[k, 0], bflow[k, 1] = -shifts[k][0], -shifts[k][1]
        for m in movers:
            scratch = np.zeros((H, W), np.float32)
            _draw(scratch, m, k, flows=(fflow[k, 0], fflow[k, 1]), val=(m[5], m[6]))
            _draw(scratch, m, k, flows=(bflow[k, 0], bflow[k, 1]), val=(-m[5], -m[6]))
    if F > 1:
        fflow[F - 1] = fflow[F - 2]
        bflow[0] = bflow[1]
    return clean, fflow, bflow


def noisy(clean: np.ndarray, sigma: float, seed: int) -> np.ndarray:
    """clean + N(0, sigma^2), float32, not clipped."""
    rng = np.random.default_rng(seed + 104729)
    return (clean + rng.standard_normal(clean.shape, dtype=np.float32) * np.float32(sigma)).astype(np.float32)


def rgb_video(W: int, H: int, F: int, seed: int):
    """Three-channel video: independent textures per channel, shared rectangle layout."""
    return video(W, H, F, seed, channels=3)
