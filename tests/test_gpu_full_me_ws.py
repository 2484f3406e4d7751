"""GPU parity tests of the warp-specialised full search (16x16 blocks,
r = 32 and 64: umi_gb300/csrc/full_me_ws.cu) through the C ABI, bit-exact
against the CPU oracle (main/full_me.cu:66-87 with the argmin first in raster
order).  The shapes exercise both ways a window arrives: one TMA box (inside
the frame on a 16-byte boundary, w % 16 == 0) and 4-byte copies with rows
clamped and edge bytes replicated (frame borders, w % 16 != 0, centres that
move a window off the 16-byte grid), the ring of buffers over many
macroblocks per CTA, list searches, and ties.  After every call the
library's error word of the motion-estimation kernels must read 0."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _t(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def _no_error(umi):
    bits = ctypes.c_int32(-1)
    assert umi.lib().umi_full_me_error(ctypes.byref(bits), None) == 0, umi.lib().umi_last_error_string()
    assert bits.value == 0


@pytest.mark.parametrize("h,w,r", [(192, 256, 32), (200, 260, 32), (96, 128, 32), (16, 16, 32), (300, 400, 64),
                                   (144, 208, 64), (33, 1000, 32), (1000, 36, 64), (720, 1280, 32)])
def test_ws_search_random(umi, orc, dev, h, w, r):
    g = np.random.default_rng(h * 7 + w + r)
    cur = g.integers(0, 256, (h, w), dtype=np.uint8)
    ref = g.integers(0, 256, (h, w), dtype=np.uint8)
    got = umi.full_me_u8(_t(cur, dev), _t(ref, dev), 16, r).cpu().numpy()
    _no_error(umi)
    assert np.array_equal(got, orc.full_me_u8(cur, ref, 16, r))


@pytest.mark.parametrize("r", [32, 64])
def test_ws_search_planted_motion(umi, orc, dev, r):
    """Blurred noise shifted per block (the benchmark generator), so the
    optimum is sharp and mostly the planted shift."""
    from umi_gb300 import workloads
    cur, ref, true_mv = workloads.me_pair(seed=21 + r, h=320, w=448, shift_sigma=r / 4, max_shift=r)
    got = umi.full_me_u8(_t(cur, dev), _t(ref, dev), 16, r).cpu().numpy()
    _no_error(umi)
    assert np.array_equal(got, orc.full_me_u8(cur, ref, 16, r))


@pytest.mark.parametrize("r", [32, 64])
def test_ws_ties_and_extremes(umi, orc, dev, r):
    import torch
    # flat frames: every displacement ties and the first, (-r, -r), wins
    got = umi.full_me_u8(torch.full((160, 192), 7, dtype=torch.uint8, device=dev),
                         torch.full((160, 192), 9, dtype=torch.uint8, device=dev), 16, r).cpu().numpy()
    assert np.all(got[:, 0] == -r) and np.all(got[:, 1] == -r) and np.all(got[:, 2] == 512)
    # the largest SAD: 0 against 255
    got = umi.full_me_u8(torch.zeros((160, 192), dtype=torch.uint8, device=dev),
                         torch.full((160, 192), 255, dtype=torch.uint8, device=dev), 16, r).cpu().numpy()
    assert np.all(got[:, 2] == 255 * 256) and np.all(got[:, :2] == -r)
    _no_error(umi)


@pytest.mark.parametrize("r", [32, 64])
def test_ws_search_centers(umi, orc, dev, r):
    g = np.random.default_rng(5 + r)
    h, w = 128, 160
    cur = g.integers(0, 256, (h, w), dtype=np.uint8)
    ref = g.integers(0, 256, (h, w), dtype=np.uint8)
    n = (h // 16) * (w // 16)
    centers = g.integers(-9, 10, (n, 2)).astype(np.int32)
    centers[:3] = [[0, 0], [16, -16], [-5, 3]]
    got = umi.full_me_u8(_t(cur, dev), _t(ref, dev), 16, r, centers=_t(centers, dev)).cpu().numpy()
    _no_error(umi)
    nbx = w // 16
    for i in g.choice(n, 12, replace=False).tolist() + [0, 1, 2]:
        by, bx = divmod(i, nbx)
        best = None
        for dy in range(centers[i, 0] - r, centers[i, 0] + r + 1):
            for dx in range(centers[i, 1] - r, centers[i, 1] + r + 1):
                s = orc.block_sad_u8(cur, ref, 16, by, bx, dy, dx)
                if best is None or s < best[0]:
                    best = (s, dy, dx)
        assert tuple(got[i]) == (best[1], best[2], best[0]), i


@pytest.mark.parametrize("r", [32, 64])
def test_ws_list_search(umi, orc, dev, r):
    """Only the listed blocks are searched and written; the list's length is a
    device word; a CTA may get no block at all."""
    import torch
    g = np.random.default_rng(50 + r)
    h, w = 256, 320
    cur = g.integers(0, 256, (h, w), dtype=np.uint8)
    ref = g.integers(0, 256, (h, w), dtype=np.uint8)
    n = (h // 16) * (w // 16)
    want = orc.full_me_u8(cur, ref, 16, r)
    for count in (0, 1, 7, 150, n):
        blocks = g.permutation(n)[:max(count, 1)].astype(np.int32)
        out = torch.full((n, 3), -9, dtype=torch.int32, device=dev)
        umi.full_me_u8_list(_t(cur, dev), _t(ref, dev), _t(blocks, dev), torch.tensor([count], dtype=torch.int32,
                            device=dev), out, 16, r)
        got = out.cpu().numpy()
        _no_error(umi)
        listed = np.zeros(n, bool)
        listed[blocks[:count]] = True
        assert np.array_equal(got[listed], want[listed]), count
        assert np.all(got[~listed] == -9), count


def test_ws_1080p_benchmark_pair_twice(umi, orc, dev):
    """The benchmark pair, two calls in a row on the same output."""
    from umi_gb300 import workloads
    cur, ref, _ = workloads.me_pair(seed=3)
    want = orc.full_me_u8(cur, ref, 16, 32)
    c, rf = _t(cur, dev), _t(ref, dev)
    out = umi.full_me_u8(c, rf, 16, 32)
    assert np.array_equal(out.cpu().numpy(), want)
    umi.full_me_u8(c, rf, 16, 32, out=out)
    assert np.array_equal(out.cpu().numpy(), want)
    _no_error(umi)
