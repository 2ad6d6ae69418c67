"""Seeded synthetic frame pairs with known flow.

These stand in for the Middlebury-style pairs the reference is demonstrated on
(the public benchmark data is not used).  Generator, per the workload
description:
  frame 1  mid-grey 128 + 40 Gaussian blobs (sigma U[5,40] px, amplitude
           U[-80,80]) + band-limited noise of standard deviation 10 (i.i.d.
           normal noise blurred with a 3 px Gaussian, then rescaled to sigma 10:
           blurring alone would leave sigma ~0.94, below frame 2's sensor noise,
           and the pairs would carry no texture to match)
  flow     global affine (|t| <= 4 px, rotation <= 2 deg, scale 0.97-1.03)
           plus 3-6 rectangles moving rigidly (|v| <= vmax px)
  frame 2  frame 1 warped by the flow (bilinear, backward), + i.i.d. N(0, 2)
           (2/255 of full scale), clamped to [0,255], 8-bit
Sequences redraw the flow for every pair and warp the previous frame.
"""
from __future__ import annotations

import numpy as np


def _gauss_blur(img, sigma):
    try:
        from scipy.ndimage import gaussian_filter

        return gaussian_filter(img, sigma, mode="reflect", truncate=3.0)
    except ImportError:
        pass
    r = int(np.ceil(3 * sigma))
    t = np.arange(-r, r + 1, dtype=np.float64)
    k = np.exp(-t * t / (2 * sigma * sigma))
    k /= k.sum()
    pad = np.pad(img, r, mode="reflect")
    tmp = np.zeros_like(pad)
    for i, w in enumerate(k):
        tmp += w * np.roll(pad, i - r, axis=1)
    out = np.zeros_like(pad)
    for i, w in enumerate(k):
        out += w * np.roll(tmp, i - r, axis=0)
    return out[r:-r, r:-r]


def make_frame(rng, w, h, blobs=40):
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    img = np.full((h, w), 128.0)
    for _ in range(blobs):
        cx, cy = rng.uniform(0, w), rng.uniform(0, h)
        s = rng.uniform(5, 40)
        a = rng.uniform(-80, 80)
        x0, x1 = int(max(0, cx - 4 * s)), int(min(w, cx + 4 * s + 1))
        y0, y1 = int(max(0, cy - 4 * s)), int(min(h, cy + 4 * s + 1))
        if x0 >= x1 or y0 >= y1:
            continue
        sub = ((xx[y0:y1, x0:x1] - cx) ** 2 + (yy[y0:y1, x0:x1] - cy) ** 2) / (2 * s * s)
        img[y0:y1, x0:x1] += a * np.exp(-sub)
    noise = _gauss_blur(rng.normal(0, 10, size=(h, w)), 3.0)
    img += noise * (10.0 / max(float(noise.std()), 1e-9))
    return img


def make_flow(rng, w, h, vmax=10.0):
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    cx, cy = w / 2.0, h / 2.0
    t = rng.uniform(-1, 1, size=2)
    t *= rng.uniform(0, 4) / max(np.hypot(*t), 1e-9)
    ang = np.deg2rad(rng.uniform(-2, 2))
    sc = rng.uniform(0.97, 1.03)
    X, Y = xx - cx, yy - cy
    u = sc * (np.cos(ang) * X - np.sin(ang) * Y) - X + t[0]
    v = sc * (np.sin(ang) * X + np.cos(ang) * Y) - Y + t[1]
    rects = []
    for _ in range(int(rng.integers(3, 7))):
        rw, rh = rng.uniform(0.08, 0.3) * w, rng.uniform(0.08, 0.3) * h
        x0, y0 = rng.uniform(0, w - rw), rng.uniform(0, h - rh)
        vel = rng.uniform(-1, 1, size=2)
        vel *= rng.uniform(0, vmax) / max(np.hypot(*vel), 1e-9)
        m = (xx >= x0) & (xx < x0 + rw) & (yy >= y0) & (yy < y0 + rh)
        u[m] = vel[0]
        v[m] = vel[1]
        rects.append((x0, y0, rw, rh, vel))
    return u.astype(np.float32), v.astype(np.float32), rects


def _bilinear(img, x, y):
    try:
        from scipy.ndimage import map_coordinates

        return map_coordinates(img, [np.clip(y, 0, img.shape[0] - 1), np.clip(x, 0, img.shape[1] - 1)], order=1,
                               mode="nearest")
    except ImportError:
        pass
    h, w = img.shape
    x = np.clip(x, 0, w - 1)
    y = np.clip(y, 0, h - 1)
    x0 = np.floor(x).astype(np.int64)
    y0 = np.floor(y).astype(np.int64)
    x1 = np.minimum(x0 + 1, w - 1)
    y1 = np.minimum(y0 + 1, h - 1)
    fx, fy = x - x0, y - y0
    return ((1 - fx) * (1 - fy) * img[y0, x0] + fx * (1 - fy) * img[y0, x1] + (1 - fx) * fy * img[y1, x0]
            + fx * fy * img[y1, x1])


def warp(rng, img1, u, v, noise=2.0):
    """Frame 2 with frame2(p + flow(p)) ~ frame1(p): backward warp by the flow
    (inverse approximated by the flow at the target pixel), then noise."""
    h, w = img1.shape
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    img2 = _bilinear(img1, xx - u, yy - v)
    img2 = img2 + rng.normal(0, noise, size=(h, w))
    return img2


def to_u8(img):
    return np.clip(np.rint(img), 0, 255).astype(np.uint8)


def make_pair(seed, w, h, vmax=10.0):
    """(frame1 u8, frame2 u8, u_gt, v_gt) for one pair; flow on frame 1's grid."""
    rng = np.random.default_rng(seed)
    f1 = make_frame(rng, w, h)
    u, v, _ = make_flow(rng, w, h, vmax)
    f2 = warp(rng, f1, u, v)
    return to_u8(f1), to_u8(f2), u, v


def make_sequence(seed, w, h, frames, vmax=15.0):
    """frames 8-bit frames and frames-1 ground-truth flows (flow re-drawn per pair)."""
    rng = np.random.default_rng(seed)
    cur = make_frame(rng, w, h)
    out = [to_u8(cur)]
    flows = []
    for _ in range(frames - 1):
        u, v, _ = make_flow(rng, w, h, vmax)
        nxt = warp(rng, cur, u, v)
        out.append(to_u8(nxt))
        flows.append((u, v))
        cur = np.clip(nxt, 0, 255)
    return out, flows


def make_batch_sizes(seed, count=64, wmin=320, wmax=1920, hmin=240, hmax=1080):
    """Uneven pair sizes for the batched workload: widths U[320,1920], heights
    U[240,1080], rounded to multiples of 4."""
    rng = np.random.default_rng(seed)
    ws = (np.rint(rng.uniform(wmin, wmax, size=count) / 4) * 4).astype(int)
    hs = (np.rint(rng.uniform(hmin, hmax, size=count) / 4) * 4).astype(int)
    return list(zip(ws.tolist(), hs.tolist()))
