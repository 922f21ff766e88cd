"""Seeded synthetic grey video for the batched sigma-delta statement.

Each stream is a static seeded background plus uniform noise in [-8, 8] per
frame, with moving 32x32 bright (255) blocks; frames are uint8 planes of
width*height pixels stored column-major (NT2's of_size(height, width)),
`frame_stride` bytes apart.  Generated on the GPU with torch.
"""
from __future__ import annotations

import math

import numpy as np
import torch


def stream_sizes(nstreams: int, seed: int, lo=(320, 240), hi=(1920, 1080)):
    """Widths and heights drawn log-uniform between lo and hi, rounded to even."""
    rng = np.random.default_rng(seed)
    w = np.exp(rng.uniform(math.log(lo[0]), math.log(hi[0]), nstreams))
    h = np.exp(rng.uniform(math.log(lo[1]), math.log(hi[1]), nstreams))
    w = (np.round(w / 2) * 2).astype(int)
    h = (np.round(h / 2) * 2).astype(int)
    return list(zip(w.tolist(), h.tolist()))


def make_stream(width: int, height: int, nframes: int, seed: int, frame_stride: int | None = None,
                device: str = "cuda", blocks: int = 4) -> dict:
    npix = width * height
    fs = frame_stride if frame_stride is not None else (npix + 15) // 16 * 16
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    frames = torch.zeros(nframes * fs, dtype=torch.uint8, device=device)
    bg = torch.randint(16, 240, (npix,), generator=g, device=device, dtype=torch.int16)
    rng = np.random.default_rng(seed)
    pos = rng.integers(0, [max(1, width - 32), max(1, height - 32)], size=(blocks, 2))
    vel = rng.integers(-6, 7, size=(blocks, 2))
    for k in range(nframes):
        noise = torch.randint(-8, 9, (npix,), generator=g, device=device, dtype=torch.int16)
        img = (bg + noise).clamp_(0, 255).to(torch.uint8).view(width, height)   # [j, i]: column-major
        for b in range(blocks):
            x0 = int((pos[b, 0] + vel[b, 0] * k) % max(1, width - 32))
            y0 = int((pos[b, 1] + vel[b, 1] * k) % max(1, height - 32))
            img[x0:x0 + 32, y0:y0 + 32] = 255
        frames[k * fs:k * fs + npix] = img.reshape(-1)
    labels_per = nframes
    ls = fs
    return {
        "frames": frames, "frame_stride": fs, "width": width, "height": height,
        "bkg": torch.zeros(npix, dtype=torch.uint8, device=device),
        "var": torch.zeros(npix, dtype=torch.uint8, device=device),
        "labels": torch.zeros(labels_per * ls, dtype=torch.uint8, device=device),
        "label_stride": ls,
    }


def make_batch(nstreams: int, nframes: int, seed: int, device: str = "cuda", sizes=None) -> list[dict]:
    sizes = sizes or stream_sizes(nstreams, seed)
    return [make_stream(w, h, nframes, seed * 1000003 + i, device=device) for i, (w, h) in enumerate(sizes)]


def pixel_frames(batch: list[dict], nframes: int, init: bool) -> int:
    k = nframes - 1 if init else nframes
    return sum(e["width"] * e["height"] for e in batch) * k


def bytes_moved(batch: list[dict], nframes: int, init: bool) -> int:
    """Compulsory bytes of one batched call: every frame read once, every label plane written,
    bkg and var written (and read when continuing from a previous call)."""
    npix = sum(e["width"] * e["height"] for e in batch)
    nl = nframes - 1 if init else nframes
    return npix * (nframes + nl + 2 + (0 if init else 2))
