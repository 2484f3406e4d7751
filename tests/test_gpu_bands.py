"""Row-band split (umi_gb300/bands.py) on one GPU: the bands of 1 to 5 ranks,
run one after another through the CUDA kernels, match the CPU oracle on the
whole frame (full search and integral image bit-exact, 3x3 filter within
1e-5 of FP64) and reproduce the whole-frame GPU result bit for bit (full
search on halo slices, 3x3 filter, integral image with the carry of the bands
above); frames the whole-frame integral image refuses are refused by the
bands too."""
import functools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

WORLDS = [1, 2, 3, 5]


@functools.lru_cache(maxsize=None)
def _me_case(h, w, b, r):
    g = np.random.default_rng(h * 7 + w)
    cur = g.integers(0, 256, (h, w), dtype=np.uint8)
    ref = np.roll(cur, (5, -3), (0, 1)) ^ g.integers(0, 8, (h, w), dtype=np.uint8)
    import oracle
    return cur, ref, oracle.full_me_u8(cur, ref, b, r).reshape(-1, 3)


@functools.lru_cache(maxsize=None)
def _filter_case(h, w):
    g = np.random.default_rng(h * w)
    img = g.standard_normal((h, w)).astype(np.float32)
    w9 = g.standard_normal(9).astype(np.float32)
    import oracle
    want = oracle.filter3x3_f64(img, w9, 0.5)
    p = np.pad(np.abs(img.astype(np.float64)), 1, constant_values=0.5)
    scale = np.zeros((h, w))
    for k in range(9):
        dy, dx = divmod(k, 3)
        scale += abs(float(w9[k])) * p[dy:dy + h, dx:dx + w]
    return img, w9, want, scale


@functools.lru_cache(maxsize=None)
def _iimg_case(h, w, full):
    g = np.random.default_rng(h + w)
    img = np.full((h, w), 255, np.uint8) if full else g.integers(0, 256, (h, w), dtype=np.uint8)
    import oracle
    return img, oracle.iimg_u8_i32(img)


def _t(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


@pytest.mark.parametrize("h,w,b,r", [(272, 320, 16, 32), (130, 104, 8, 5), (1080, 1920, 16, 32), (200, 256, 16, 64)])
@pytest.mark.parametrize("world", WORLDS)
def test_me_bands(umi, dev, h, w, b, r, world):
    import torch
    from umi_gb300 import bands
    cur, ref, want = _me_case(h, w, b, r)
    c, rf = _t(cur, dev), _t(ref, dev)
    parts = torch.cat([bands.me_band(c, rf, world, k, block=b, search=r) for k in range(world)])
    assert np.array_equal(parts.cpu().numpy(), want)
    assert torch.equal(parts, umi.full_me_u8(c, rf, block=b, search=r).reshape(-1, 3))


@pytest.mark.parametrize("h,w", [(67, 129), (1, 40), (1024, 1024)])
@pytest.mark.parametrize("world", WORLDS)
def test_filter3x3_bands(umi, dev, h, w, world):
    import torch
    from umi_gb300 import bands
    x, w9, want, scale = _filter_case(h, w)  # host weights, as the C-ABI takes them
    img = _t(x, dev)
    parts = torch.cat([bands.filter3x3_band(img, w9, world, k, pad=0.5) for k in range(world)])
    got = parts.cpu().numpy().astype(np.float64)
    assert np.max(np.abs(got - want) / np.maximum(scale, 1e-30)) <= 1e-5
    assert torch.equal(parts, umi.filter3x3_f32(img, w9, 0.5))


@pytest.mark.parametrize("h,w,full", [(37, 53, False), (1080, 1920, False), (2160, 3840, True)])
@pytest.mark.parametrize("world", WORLDS)
def test_iimg_bands(umi, dev, h, w, full, world):
    import torch
    from umi_gb300 import bands
    img, want = _iimg_case(h, w, full)  # 4K of 255: the largest sums the operator takes
    x = _t(img, dev)
    locals_ = [bands.iimg_band_local(x, world, k) for k in range(world)]
    totals = [bands.band_totals(l) for l in locals_]
    parts = torch.cat([bands.add_carry(l, totals, k) for k, l in enumerate(locals_)])
    assert np.array_equal(parts.cpu().numpy(), want)
    assert torch.equal(parts, umi.iimg_u8_i32(x))


def test_iimg_band_refuses_what_the_operator_refuses(umi, dev):
    from umi_gb300 import bands
    x = _t(np.zeros((2304, 4096), np.uint8), dev)
    with pytest.raises(umi.UmiError):
        umi.iimg_u8_i32(x)
    with pytest.raises(umi.UmiError):
        bands.iimg_band_local(x, 2, 1)
