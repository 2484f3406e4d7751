"""Window operators of the UMI family on the generic operator (umi_launch).

The reference ships eight example applications; these are four more of the
same kind, each one descriptor over the closed-form generic kernel with a
built-in strategy (no specialised kernel):

* ``census``: census transform, one bit per window pixel (row-major), set
  where the pixel is below the centre (CENSUS_I32); edges replicated.
* ``box_sum``: sums over (2r+1)^2 windows clipped to the image, from the
  integral image (``iimg_u8_i32``): four corner reads of the zero-bordered
  integral image with weights +1 -1 -1 +1 (WEIGHTED_SUM_I32 over a 2 x 2
  accumulation view of stride 2r+1, coordinates clamped).
* ``gaussian``: separable Gaussian blur, a horizontal then a vertical pass
  of WEIGHTED_SUM_F32 with the normalised 1-D kernel; edges replicated.
* ``dilate`` / ``erode``: grey-level max / min over (2r+1)^2 windows
  (MAX_I32 / MIN_I32); edges replicated.

All take and return CUDA tensors of shape (h, w) and run on the current
stream.
"""
from __future__ import annotations

import math

import numpy as np

import umi_gb300 as U

PAD, WRAP = 0, 1


_CONST = {}  # small constant tensors (weights) per (device, key): made once, so calls can be graph-captured


def _const(dev, key, make):
    import torch
    k = (str(dev), key)
    if k not in _CONST:
        _CONST[k] = torch.from_numpy(np.ascontiguousarray(make())).to(dev)
    return _CONST[k]


def _p(h, w):
    return [(1, 1, 1, 1), (1, 1, 1, 1), (h, 16, 4, 1), (w, 16, 8, 1)]


def _img(h, w, mode=WRAP, a_view=None, stage=1, out=False):
    m = dict(p_view=[(), (), (2, 0, 1), (3, 0, 1)], phys=[(1, mode), (1, mode), (h, mode), (w, mode)], stage=stage)
    if a_view is not None:
        m["a_view"] = a_view
    if out:
        m["out"] = True
    return m


def _window(r):
    return [(), (), (2, -r, 1), (3, -r, 1)]


def census(img, radius: int = 1, out=None, stream=None):
    """Census transform of an int32 image over (2 radius + 1)^2 windows
    (radius <= 2 keeps every bit: at most 32)."""
    import torch
    h, w = img.shape
    k = 2 * radius + 1
    if out is None:
        out = torch.empty((h, w), dtype=torch.int32, device=img.device)
    d = U.make_desc(p=_p(h, w), a=[(1, 1), (1, 1), (k, k), (k, k)],
                    mems=[_img(h, w, stage=0), _img(h, w, a_view=_window(radius)), _img(h, w, PAD, stage=2, out=True)])
    U.launch(d, U.STRATEGY_CENSUS_I32, [img, img], [out], stream=stream)
    return out


def _extremum(img, radius, strategy, init, out, stream):
    import torch
    h, w = img.shape
    k = 2 * radius + 1
    if out is None:
        out = torch.empty((h, w), dtype=torch.int32, device=img.device)
    d = U.make_desc(p=_p(h, w), a=[(1, 1), (1, 1), (k, k), (k, k)],
                    mems=[_img(h, w, a_view=_window(radius)), _img(h, w, PAD, stage=2, out=True)])
    U.launch(d, strategy, [img], [out], consts=[init], stream=stream)
    return out


def dilate(img, radius: int = 1, out=None, stream=None):
    """Grey-level dilation (window maximum) of an int32 image."""
    return _extremum(img, radius, U.STRATEGY_MAX_I32, -(1 << 31), out, stream)


def erode(img, radius: int = 1, out=None, stream=None):
    """Grey-level erosion (window minimum) of an int32 image."""
    return _extremum(img, radius, U.STRATEGY_MIN_I32, (1 << 31) - 1, out, stream)


def box_sum(img_u8, radius: int, out=None, J=None, ii=None, workspace=None, stream=None):
    """Sums of a uint8 image over (2 radius + 1)^2 windows clipped to the
    image (int32), from its integral image.  J ((h+1, w+1) int32, first row
    and column zero), ii ((h, w) int32) and the iimg workspace may be passed
    in to avoid allocations."""
    import torch
    h, w = img_u8.shape
    k = 2 * radius + 1
    dev = img_u8.device
    if J is None:
        J = torch.zeros((h + 1, w + 1), dtype=torch.int32, device=dev)  # J[y][x] = sum of img[:y, :x]
    J[1:, 1:] = U.iimg_u8_i32(img_u8, out=ii, workspace=workspace, stream=stream)
    wts = _const(dev, "box", lambda: np.array([[1, -1], [-1, 1]], np.int32))
    if out is None:
        out = torch.empty((h, w), dtype=torch.int32, device=dev)
    # corner (a_y, a_x) of point (y, x): J[clamp(y - r + a_y k)][clamp(x - r + a_x k)]
    jmem = dict(p_view=[(), (), (2, -radius, 1), (3, -radius, 1)], a_view=[(), (), (2, 0, k), (3, 0, k)],
                phys=[(1, WRAP), (1, WRAP), (h + 1, WRAP), (w + 1, WRAP)], stage=1)
    wmem = dict(p_view=[(), (), (), ()], a_view=[(), (), (2, 0, 1), (3, 0, 1)],
                phys=[(1, PAD), (1, PAD), (2, PAD), (2, PAD)], stage=1)
    d = U.make_desc(p=_p(h, w), a=[(1, 1), (1, 1), (2, 2), (2, 2)], mems=[jmem, wmem, _img(h, w, PAD, stage=2, out=True)])
    U.launch(d, U.STRATEGY_WEIGHTED_SUM_I32, [J, wts], [out], consts=[0], stream=stream)
    return out


def gaussian_kernel(sigma: float, radius: int | None = None) -> np.ndarray:
    """Normalised 1-D Gaussian weights exp(-i^2 / (2 sigma^2)), i = -r..r
    (r = ceil(3 sigma) by default), as float32."""
    r = int(math.ceil(3 * sigma)) if radius is None else int(radius)
    t = np.arange(-r, r + 1, dtype=np.float64)
    k = np.exp(-t * t / (2.0 * sigma * sigma))
    return (k / k.sum()).astype(np.float32)


def gaussian(img, sigma: float, radius: int | None = None, out=None, tmp=None, stream=None):
    """Separable Gaussian blur of a float32 image (edges replicated)."""
    import torch
    h, w = img.shape
    kern = gaussian_kernel(sigma, radius)
    k = kern.size
    r = k // 2
    dev = img.device
    wt = _const(dev, ("gauss", float(sigma), k), lambda: kern)
    if tmp is None:
        tmp = torch.empty((h, w), dtype=torch.float32, device=dev)
    if out is None:
        out = torch.empty((h, w), dtype=torch.float32, device=dev)
    dh = U.make_desc(p=_p(h, w), a=[(1, 1), (1, 1), (1, 1), (k, k)],
                     mems=[_img(h, w, a_view=[(), (), (), (3, -r, 1)]),
                           dict(p_view=[(), (), (), ()], a_view=[(), (), (), (3, 0, 1)],
                                phys=[(1, PAD), (1, PAD), (1, PAD), (k, PAD)], stage=1),
                           _img(h, w, PAD, stage=2, out=True)])
    U.launch(dh, U.STRATEGY_WEIGHTED_SUM_F32, [img, wt], [tmp], consts=[0.0], stream=stream)
    dv = U.make_desc(p=_p(h, w), a=[(1, 1), (1, 1), (k, k), (1, 1)],
                     mems=[_img(h, w, a_view=[(), (), (2, -r, 1), ()]),
                           dict(p_view=[(), (), (), ()], a_view=[(), (), (2, 0, 1), ()],
                                phys=[(1, PAD), (1, PAD), (k, PAD), (1, PAD)], stage=1),
                           _img(h, w, PAD, stage=2, out=True)])
    U.launch(dv, U.STRATEGY_WEIGHTED_SUM_F32, [tmp, wt], [out], consts=[0.0], stream=stream)
    return out
