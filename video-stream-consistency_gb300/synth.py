"""Seeded synthetic video streams (the benchmark and test inputs).

The reference measures on its demo video and on frame directories that are
not part of its tree; these streams stand in for them with the same shapes
and value ranges:
  original frame 0 : sum of 64 Gaussian blobs (random centres, widths and
                     RGB amplitudes), normalised to [0, 1];
  frame t+1        : frame t advected by a smooth flow — an N(0, 1) field per
                     component, Gaussian-filtered (sigma 20 px) and scaled to
                     max |v| = 8 px, re-drawn every `redraw` frames;
  observed frame   : plus per-pixel uniform noise U(0, 0.02), quantised to RGBA8;
  processed frame  : observed / 255 + a per-frame RGB shift U(-0.05, 0.05) +
                     per-pixel flicker N(0, 0.02), quantised to RGBA8.
Random numbers come from numpy's PCG64 with a fixed seed, so the stream is
the same on every machine; the blob rendering and advection run in torch on
the requested device.
"""
from __future__ import annotations

import numpy as np


def _smooth_field(rng, w, h, sigma=20.0, vmax=8.0):
    from scipy.ndimage import gaussian_filter

    f = rng.standard_normal((2, h, w)).astype(np.float64)
    f[0] = gaussian_filter(f[0], sigma, mode="reflect")
    f[1] = gaussian_filter(f[1], sigma, mode="reflect")
    mag = np.sqrt(f[0] ** 2 + f[1] ** 2).max()
    return (f * (vmax / max(mag, 1e-12))).astype(np.float32)


def _blobs(rng, w, h, device, n=64):
    import torch

    cx = torch.tensor(rng.uniform(0, w, n), dtype=torch.float32, device=device)
    cy = torch.tensor(rng.uniform(0, h, n), dtype=torch.float32, device=device)
    sg = torch.tensor(rng.uniform(0.02, 0.12, n) * max(w, h), dtype=torch.float32, device=device)
    amp = torch.tensor(rng.uniform(0.0, 1.0, (n, 3)), dtype=torch.float32, device=device)
    ys = torch.arange(h, dtype=torch.float32, device=device).view(h, 1)
    xs = torch.arange(w, dtype=torch.float32, device=device).view(1, w)
    img = torch.zeros((h, w, 3), dtype=torch.float32, device=device)
    for k in range(n):
        g = torch.exp(-((xs - cx[k]) ** 2 + (ys - cy[k]) ** 2) / (2.0 * sg[k] ** 2))
        img += g.unsqueeze(-1) * amp[k]
    return img / img.max()


def _advect(img, flow):
    """img (h, w, 3) moved by flow (2, h, w): out(x) = img(x - v(x)), bilinear, border clamp."""
    import torch

    h, w = img.shape[:2]
    ys = torch.arange(h, dtype=torch.float32, device=img.device).view(h, 1).expand(h, w)
    xs = torch.arange(w, dtype=torch.float32, device=img.device).view(1, w).expand(h, w)
    sx = (xs - flow[0]) * (2.0 / max(w - 1, 1)) - 1.0
    sy = (ys - flow[1]) * (2.0 / max(h - 1, 1)) - 1.0
    grid = torch.stack([sx, sy], dim=-1).unsqueeze(0)
    out = torch.nn.functional.grid_sample(img.permute(2, 0, 1).unsqueeze(0), grid, mode="bilinear",
                                          padding_mode="border", align_corners=True)
    return out[0].permute(1, 2, 0).contiguous()


def _to_rgba(img01):
    rgb = np.clip(np.rint(img01 * 255.0), 0, 255).astype(np.uint8)
    out = np.empty(rgb.shape[:2] + (4,), np.uint8)
    out[..., :3] = rgb
    out[..., 3] = 255
    return out


class SyntheticStream:
    """Frames are produced in order and cached; frame(t) for t >= 0."""

    def __init__(self, width: int, height: int, seed: int = 0, redraw: int = 30, device: str = "cpu"):
        self.w, self.h, self.seed, self.redraw, self.device = width, height, seed, redraw, device
        self.rng = np.random.Generator(np.random.PCG64(seed))
        self._clean = None
        self._flow = None
        self._frames: list = []

    def _next(self):
        import torch

        t = len(self._frames)
        if t == 0:
            self._clean = _blobs(self.rng, self.w, self.h, self.device)
        else:
            if (t - 1) % self.redraw == 0:
                self._flow = torch.from_numpy(_smooth_field(self.rng, self.w, self.h)).to(self.device)
            self._clean = _advect(self._clean, self._flow)
        clean = self._clean.cpu().numpy()
        obs = clean + self.rng.uniform(0.0, 0.02, clean.shape).astype(np.float32)
        orig = _to_rgba(obs)
        shift = self.rng.uniform(-0.05, 0.05, 3).astype(np.float32)
        flick = self.rng.normal(0.0, 0.02, clean.shape).astype(np.float32)
        proc = _to_rgba(orig[..., :3].astype(np.float32) / 255.0 + shift + flick)
        self._frames.append((orig, proc))

    def frame(self, t: int):
        while len(self._frames) <= t:
            self._next()
        return self._frames[t]

    def true_flow(self, t: int):
        """The advection field that produced frame t+1 from frame t (content displacement)."""
        self.frame(t + 1)
        return None if self._flow is None else self._flow.cpu().numpy()


def feature_pyramid(width: int, height: int, seed: int = 0):
    """FP32 N(0, 1) feature pyramids of a frame pair at 1/4 .. 1/64 of the
    64-aligned size with the PWC channel counts (the Correlation op workload)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pw, ph = -(-width // 64) * 64, -(-height // 64) * 64
    out = []
    for lvl, c in zip(range(2, 7), (32, 64, 96, 128, 196)):
        lw, lh = pw >> lvl, ph >> lvl
        f1 = rng.standard_normal((1, c, lh, lw)).astype(np.float32)
        f2 = rng.standard_normal((1, c, lh, lw)).astype(np.float32)
        out.append((f1, f2))
    return out
