"""The window operators of umi_gb300/apps.py (census, box sums via the
integral image, separable Gaussian, dilation / erosion: four more members of
the UMI example family on the generic operator) against numpy restatements
of their definitions.  Integer outputs bit-exact; the Gaussian within
rel 1e-5 of an FP64 separable filter."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = [(37, 53), (1, 1), (16, 16), (130, 300), (5, 200)]


def _t(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def _windows(x, r, mode):
    """(k*k, h, w) stack of the window elements in row-major order."""
    p = np.pad(x, r, mode=mode) if mode == "edge" else np.pad(x, r, mode="constant")
    h, w = x.shape
    return np.stack([p[dy:dy + h, dx:dx + w] for dy in range(2 * r + 1) for dx in range(2 * r + 1)])


@pytest.mark.parametrize("h,w", SIZES)
@pytest.mark.parametrize("r", [1, 2])
def test_census(umi, dev, h, w, r):
    from umi_gb300 import apps
    x = np.random.default_rng(h * w + r).integers(0, 8, (h, w)).astype(np.int32)  # many ties
    got = apps.census(_t(x, dev), r).cpu().numpy().view(np.uint32)
    want = np.zeros((h, w), np.uint64)
    for win in _windows(x, r, "edge"):
        want = (want << np.uint64(1)) | (win < x).astype(np.uint64)
    assert np.array_equal(got, (want & np.uint64(0xffffffff)).astype(np.uint32))


@pytest.mark.parametrize("h,w", SIZES)
@pytest.mark.parametrize("r", [1, 3])
def test_dilate_erode(umi, dev, h, w, r):
    from umi_gb300 import apps
    x = np.random.default_rng(h + w * 3 + r).integers(-1000, 1000, (h, w)).astype(np.int32)
    win = _windows(x, r, "edge")
    assert np.array_equal(apps.dilate(_t(x, dev), r).cpu().numpy(), win.max(0))
    assert np.array_equal(apps.erode(_t(x, dev), r).cpu().numpy(), win.min(0))


@pytest.mark.parametrize("h,w", SIZES + [(1080, 1920)])
@pytest.mark.parametrize("r", [0, 2, 7])
def test_box_sum(umi, dev, h, w, r):
    from umi_gb300 import apps
    x = np.random.default_rng(h * 7 + w + r).integers(0, 256, (h, w), dtype=np.uint8)
    c = np.pad(x.astype(np.int64), r, mode="constant").cumsum(0).cumsum(1)
    c = np.pad(c, ((1, 0), (1, 0)))
    k = 2 * r + 1
    want = c[k:k + h, k:k + w] - c[0:h, k:k + w] - c[k:k + h, 0:w] + c[0:h, 0:w]
    got = apps.box_sum(_t(x, dev), r).cpu().numpy()
    assert np.array_equal(got, want)


@pytest.mark.parametrize("h,w", SIZES)
@pytest.mark.parametrize("sigma", [0.8, 2.0])
def test_gaussian(umi, dev, h, w, sigma):
    from umi_gb300 import apps
    x = np.random.default_rng(h + w).random((h, w), dtype=np.float32)
    k = apps.gaussian_kernel(sigma).astype(np.float64)
    r = k.size // 2
    p = np.pad(x.astype(np.float64), r, mode="edge")
    hz = sum(k[i] * p[:, i:i + w] for i in range(k.size))          # (h + 2r, w)
    want = sum(k[i] * hz[i:i + h, :] for i in range(k.size))
    got = apps.gaussian(_t(x, dev), sigma).cpu().numpy()
    assert np.max(np.abs(got - want) / np.maximum(np.abs(want), 1e-3)) <= 1e-5
