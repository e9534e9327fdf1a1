"""Seeded synthetic clips: the stand-in for video data (no dataset is used).

A clean clip is a background of 128 plus 6-12 Gaussian blobs (sigma 5-25 px,
amplitude 40-200, random sign) and 3-6 rectangles textured with a sinusoidal
grating (period 4-16 px), each object translating at a constant random
velocity (<= vmax px/frame).  RGB clips draw each object once and jitter its
amplitude per channel.  Noise is AWGN added in float32, unclipped, from an
independent random stream.  Seeds: numpy PCG64(seed) for content and
PCG64(seed + 2**32) for noise; the benchmark uses seed = config * 1000 + clip.

Flows (optional) are the exact per-pixel displacement of the top-most
object (the last grating drawn), zero elsewhere, in the reference's flow
layout [F][2][H][W]: fflow[t] is the motion t -> t+1, bflow[t-1] the motion
t -> t-1 (src/main.cpp:353-369 loads them the same way).
"""
import numpy as np


def _blob(shape, cx, cy, s, amp):
    h, w = shape
    r = int(np.ceil(3.5 * s))
    x0, x1 = max(0, int(cx) - r), min(w, int(cx) + r + 1)
    y0, y1 = max(0, int(cy) - r), min(h, int(cy) + r + 1)
    if x0 >= x1 or y0 >= y1:
        return None
    xs = np.arange(x0, x1, dtype=np.float32) - np.float32(cx)
    ys = np.arange(y0, y1, dtype=np.float32) - np.float32(cy)
    g = np.exp(-(ys[:, None] ** 2 + xs[None, :] ** 2) / np.float32(2 * s * s)).astype(np.float32)
    return (y0, y1, x0, x1), g * np.float32(amp)


def make_clip(width, height, frames, channels, sigma, seed, vmax=3.0, with_flow=False):
    """Returns (clean, noisy, fflow, bflow) as float32 [F, C, H, W] arrays
    (flows [F, 2, H, W], or None when with_flow is False)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nrng = np.random.Generator(np.random.PCG64(seed + (1 << 32)))
    clean = np.full((frames, channels, height, width), 128.0, dtype=np.float32)

    nb = int(rng.integers(6, 13))
    blobs = []
    for _ in range(nb):
        s = rng.uniform(5, 25)
        amp = rng.uniform(40, 200) * (1 if rng.random() < 0.5 else -1)
        jit = rng.uniform(0.7, 1.3, size=channels)
        cx, cy = rng.uniform(0, width), rng.uniform(0, height)
        v = rng.uniform(-vmax, vmax, size=2)
        blobs.append((s, amp, jit, cx, cy, v))
    ng = int(rng.integers(3, 7))
    grats = []
    for _ in range(ng):
        rw = int(rng.integers(max(8, width // 10), max(9, width // 3)))
        rh = int(rng.integers(max(8, height // 10), max(9, height // 3)))
        x, y = rng.uniform(-rw / 2, width - rw / 2), rng.uniform(-rh / 2, height - rh / 2)
        period = rng.uniform(4, 16)
        theta = rng.uniform(0, np.pi)
        amp = rng.uniform(20, 80)
        base = rng.uniform(60, 200)
        jit = rng.uniform(0.7, 1.3, size=channels)
        v = rng.uniform(-vmax, vmax, size=2)
        grats.append((rw, rh, x, y, period, theta, amp, base, jit, v))

    fflow = bflow = None
    if with_flow:
        fflow = np.zeros((frames, 2, height, width), dtype=np.float32)
        bflow = np.zeros((frames, 2, height, width), dtype=np.float32)

    for t in range(frames):
        for (s, amp, jit, cx, cy, v) in blobs:
            res = _blob((height, width), cx + v[0] * t, cy + v[1] * t, s, amp)
            if res is None:
                continue
            (y0, y1, x0, x1), g = res
            for c in range(channels):
                clean[t, c, y0:y1, x0:x1] += g * np.float32(jit[c])
        for gi, (rw, rh, x, y, period, theta, amp, base, jit, v) in enumerate(grats):
            ox, oy = x + v[0] * t, y + v[1] * t
            x0, x1 = max(0, int(np.floor(ox))), min(width, int(np.floor(ox)) + rw)
            y0, y1 = max(0, int(np.floor(oy))), min(height, int(np.floor(oy)) + rh)
            if x0 >= x1 or y0 >= y1:
                continue
            xs = np.arange(x0, x1, dtype=np.float64) - ox
            ys = np.arange(y0, y1, dtype=np.float64) - oy
            ph = (np.cos(theta) * xs[None, :] + np.sin(theta) * ys[:, None]) * (2 * np.pi / period)
            tex = (base + amp * np.sin(ph)).astype(np.float32)
            for c in range(channels):
                clean[t, c, y0:y1, x0:x1] = tex * np.float32(jit[c])
            if with_flow and gi == ng - 1:
                if t + 1 < frames:
                    fflow[t, 0, y0:y1, x0:x1] = v[0]
                    fflow[t, 1, y0:y1, x0:x1] = v[1]
                if t >= 1:
                    bflow[t - 1, 0, y0:y1, x0:x1] = -v[0]
                    bflow[t - 1, 1, y0:y1, x0:x1] = -v[1]

    noise = nrng.standard_normal(size=clean.shape, dtype=np.float32)
    noisy = clean + noise * np.float32(sigma)
    return clean, noisy.astype(np.float32), fflow, bflow


def batch_specs(n=64, seed=4000, scale=1.0):
    """(width, height, frames, channels, sigma) of the uneven-batch workload:
    width uniform in 160-1280, height in 120-720, 5-40 frames, 1 or 3
    channels, sigma in {5, 10, 20, 30, 50}, drawn from PCG64(seed); clip i
    is generated with seed + i.  `scale` shrinks the sides (for small
    profiling cases)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for _ in range(n):
        w = int(rng.integers(160, 1281))
        h = int(rng.integers(120, 721))
        f = int(rng.integers(5, 41))
        c = int(rng.choice([1, 3]))
        s = float(rng.choice([5, 10, 20, 30, 50]))
        out.append((max(16, int(w * scale)), max(16, int(h * scale)), f, c, s))
    return out


def psnr(clean, est):
    """PSNR with both videos clipped to [0, 255], as VideoUtils::computePSNR
    (src/Utilities/LibVideoT.hpp:576-597); computed in double."""
    a = np.clip(clean.astype(np.float64), 0, 255)
    b = np.clip(est.astype(np.float64), 0, 255)
    rmse = np.sqrt(np.mean((a - b) ** 2))
    return float(20 * np.log10(255.0 / rmse))
