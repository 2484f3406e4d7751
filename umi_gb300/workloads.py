"""Seeded synthetic inputs for the benchmark workloads (numpy, host side).

No public dataset is involved: each generator draws the distributions the
workload definitions name, from numpy's PCG64 with an explicit seed.
"""
from __future__ import annotations

import numpy as np


def rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def gaussian_blur(img: np.ndarray, sigma: float) -> np.ndarray:
    """Separable Gaussian blur (radius ceil(3 sigma)), edges replicated, float32."""
    r = int(np.ceil(3 * sigma))
    t = np.arange(-r, r + 1, dtype=np.float64)
    k = np.exp(-t * t / (2 * sigma * sigma))
    k = (k / k.sum()).astype(np.float32)
    x = img.astype(np.float32)
    p = np.pad(x, ((0, 0), (r, r)), mode="edge")
    y = np.zeros_like(x)
    for i in range(2 * r + 1):
        y += k[i] * p[:, i:i + x.shape[1]]
    p = np.pad(y, ((r, r), (0, 0)), mode="edge")
    z = np.zeros_like(x)
    for i in range(2 * r + 1):
        z += k[i] * p[i:i + x.shape[0], :]
    return z


# ---- filter3x3: one float image, 3x3 weights ----

def filter_image(seed: int = 1, h: int = 1024, w: int = 1024):
    """Pixels U[0,1) float32 and 3x3 weights N(0,1) float32."""
    g = rng(seed)
    img = g.random((h, w), dtype=np.float32)
    w9 = g.standard_normal(9).astype(np.float32)
    return img, w9


# ---- integer pair: iimg frame and motion-estimation frame pair ----

def iimg_frame(seed: int = 2, h: int = 1080, w: int = 1920) -> np.ndarray:
    """uint8 pixels uniform 0..255."""
    return rng(seed).integers(0, 256, size=(h, w), dtype=np.uint8)


def me_pair(seed: int = 3, h: int = 1080, w: int = 1920, block: int = 16, shift_sigma: float = 8.0,
            max_shift: int = 32, noise_sigma: float = 2.0, blur_sigma: float = 2.0):
    """Frame pair for block motion estimation.

    ref (frame A) = clip(blur_{blur_sigma}(N(128, 40^2))) as uint8.
    cur (frame B) = per-block translation of A: inside block (by, bx) with
    shift (sy, sx) ~ round(N(0, shift_sigma^2)) clipped to +-max_shift,
    B[y, x] = A[clamp(y+sy), clamp(x+sx)] + N(0, noise_sigma^2), clipped.
    Returns (cur, ref, true_mv) with true_mv (nby*nbx, 2) = (sy, sx): searching
    the block of `cur` in `ref`, the true match sits at displacement (sy, sx).
    Pixels below / right of the last whole block use the shift of the nearest block.
    """
    g = rng(seed)
    a = g.normal(128.0, 40.0, size=(h, w)).astype(np.float32)
    a = np.clip(np.rint(gaussian_blur(a, blur_sigma)), 0, 255).astype(np.uint8)
    nby, nbx = h // block, w // block
    sh = np.clip(np.rint(g.normal(0.0, shift_sigma, size=(max(nby, 1), max(nbx, 1), 2))), -max_shift, max_shift)
    sh = sh.astype(np.int64)
    by = np.minimum(np.arange(h) // block, max(nby, 1) - 1)
    bx = np.minimum(np.arange(w) // block, max(nbx, 1) - 1)
    sy = sh[by[:, None], bx[None, :], 0]
    sx = sh[by[:, None], bx[None, :], 1]
    yy = np.clip(np.arange(h)[:, None] + sy, 0, h - 1)
    xx = np.clip(np.arange(w)[None, :] + sx, 0, w - 1)
    b = a[yy, xx].astype(np.float32) + g.normal(0.0, noise_sigma, size=(h, w)).astype(np.float32)
    b = np.clip(np.rint(b), 0, 255).astype(np.uint8)
    true_mv = sh[:nby, :nbx].reshape(-1, 2).astype(np.int32)
    return b, a, true_mv


def video_frames(seed: int = 11, n: int = 8, h: int = 1080, w: int = 1920, velocity=(3, -5),
                 noise_sigma: float = 2.0, blur_sigma: float = 2.0):
    """A panning camera over a still scene: frame t is the window of a larger
    clip(blur_{blur_sigma}(N(128, 40^2))) canvas whose origin moves by
    `velocity` (dy, dx) pixels per frame, plus N(0, noise_sigma^2) sensor
    noise per frame, as uint8.  Every block of frame t matches frame t - 1
    at displacement (dy, dx): the scene point at (y, x) of frame t sat at
    (y + dy, x + dx) one frame earlier."""
    g = rng(seed)
    vy, vx = velocity
    my, mx = abs(vy) * max(n - 1, 0), abs(vx) * max(n - 1, 0)
    canvas = g.normal(128.0, 40.0, size=(h + my, w + mx)).astype(np.float32)
    canvas = gaussian_blur(canvas, blur_sigma)
    y0, x0 = (my if vy < 0 else 0), (mx if vx < 0 else 0)
    frames = []
    for t in range(n):
        oy, ox = y0 + vy * t, x0 + vx * t
        f = canvas[oy:oy + h, ox:ox + w] + g.normal(0.0, noise_sigma, size=(h, w)).astype(np.float32)
        frames.append(np.clip(np.rint(f), 0, 255).astype(np.uint8))
    return frames


def me_pair_cuda(seed: int, h: int = 2160, w: int = 3840, block: int = 16, shift_sigma: float = 16.0,
                 max_shift: int = 64, noise_sigma: float = 2.0, blur_sigma: float = 2.0, device="cuda"):
    """me_pair's distribution drawn on the GPU (torch's Philox generator, seeded).

    Same construction as me_pair (blurred N(128, 40^2) reference, per-block
    shifts round(N(0, shift_sigma^2)) clipped to +-max_shift, edge-clamped
    gather, N(0, noise_sigma^2) noise); the random streams differ from
    numpy's, so the frames are not me_pair's frames.  Used where thousands
    of 4K pairs are needed (training the motion-proposal network).
    Returns (cur, ref, true_mv) as CUDA tensors (uint8, uint8, int32 (nblk, 2)).
    """
    import torch
    dev = torch.device(device)
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    a = torch.normal(128.0, 40.0, size=(h, w), generator=g, device=dev)
    r = int(np.ceil(3 * blur_sigma))
    t = torch.arange(-r, r + 1, dtype=torch.float64, device=dev)
    k = torch.exp(-t * t / (2 * blur_sigma * blur_sigma))
    k = (k / k.sum()).float()
    x = torch.nn.functional.pad(a[None, None], (r, r, 0, 0), mode="replicate")
    x = torch.nn.functional.conv2d(x, k.view(1, 1, 1, -1))
    x = torch.nn.functional.pad(x, (0, 0, r, r), mode="replicate")
    x = torch.nn.functional.conv2d(x, k.view(1, 1, -1, 1))[0, 0]
    ref = x.round().clamp(0, 255).to(torch.uint8)
    nby, nbx = max(h // block, 1), max(w // block, 1)
    sh = torch.normal(0.0, shift_sigma, size=(nby, nbx, 2), generator=g, device=dev)
    sh = sh.round().clamp(-max_shift, max_shift).to(torch.int64)
    by = torch.clamp(torch.arange(h, device=dev) // block, max=nby - 1)
    bx = torch.clamp(torch.arange(w, device=dev) // block, max=nbx - 1)
    sy = sh[by[:, None], bx[None, :], 0]
    sx = sh[by[:, None], bx[None, :], 1]
    yy = torch.clamp(torch.arange(h, device=dev)[:, None] + sy, 0, h - 1)
    xx = torch.clamp(torch.arange(w, device=dev)[None, :] + sx, 0, w - 1)
    b = ref[yy, xx].float() + torch.normal(0.0, noise_sigma, size=(h, w), generator=g, device=dev)
    cur = b.round().clamp(0, 255).to(torch.uint8)
    true_mv = sh[:h // block, :w // block].reshape(-1, 2).to(torch.int32).contiguous()
    return cur.contiguous(), ref.contiguous(), true_mv
