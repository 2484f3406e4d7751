"""GPU parity tests of the specialised kernels, through the C ABI, against the
CPU oracle on the same seeded inputs.

Integer work (iimg, full_me) must be bit-exact.  The float filter is compared
with the FP64 oracle at rel <= 1e-5 where
rel = |y - y64| / max(|y64|, sum |w * x|)  (the scale of the sum, so that
outputs that cancel to ~0 are judged against the magnitude of their terms).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FILTER_REL_TOL = 1e-5


def _t(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


# ---------------------------------------------------------------- filter3x3
def _filter_scale(x, w9, pad):
    p = np.pad(np.abs(x.astype(np.float64)), 1, constant_values=abs(pad))
    s = np.zeros(x.shape)
    for i in range(3):
        for j in range(3):
            s += abs(float(w9[3 * i + j])) * p[i:i + x.shape[0], j:j + x.shape[1]]
    return s


@pytest.mark.parametrize("h,w,pad", [(1024, 1024, 0.0), (1, 1, 0.0), (3, 5, 2.5), (37, 131, 0.0), (130, 257, -1.0),
                                     (64, 128, 0.0), (33, 4, 0.0)])
def test_filter3x3_f32(umi, orc, dev, h, w, pad):
    from umi_gb300 import workloads
    x, w9 = workloads.filter_image(seed=h * 7 + w, h=h, w=w)
    got = umi.filter3x3_f32(_t(x, dev), w9, pad=pad).cpu().numpy()
    want = orc.filter3x3_f64(x, w9, pad=pad)
    rel = np.abs(got - want) / np.maximum(np.abs(want), _filter_scale(x, w9, pad))
    assert rel.max() <= FILTER_REL_TOL, rel.max()


@pytest.mark.parametrize("h,w", [(100, 260), (32, 128), (35, 132), (2000, 8), (1, 4), (97, 1028), (4096, 1024)])
def test_filter3x3_tma_tiles_match_register_kernel(umi, orc, dev, h, w):
    """The TMA-staged halo tiles (umi_filter3x3_f32_tma: ragged edge tiles,
    several tiles per persistent CTA at 2000 rows) and the register kernel use
    the same (dy, dx) FMA order: they agree exactly, and both match FP64."""
    from umi_gb300 import workloads
    x, w9 = workloads.filter_image(seed=h + w, h=h, w=w)
    xt = _t(x, dev)
    tma = umi.filter3x3_f32_tma(xt, w9).cpu().numpy()
    reg = umi.filter3x3_f32(xt, w9, pad=0.0).cpu().numpy()
    assert np.array_equal(tma, reg)
    want = orc.filter3x3_f64(x, w9, pad=0.0)
    rel = np.abs(tma - want) / np.maximum(np.abs(want), _filter_scale(x, w9, 0.0))
    assert rel.max() <= FILTER_REL_TOL, rel.max()


def test_filter3x3_rejects_alias(umi, dev):
    import torch
    x = torch.zeros(8, 8, device=dev)
    with pytest.raises(umi.UmiError):
        umi.filter3x3_f32(x, [0.0] * 9, out=x)
    with pytest.raises(umi.UmiError):
        umi.filter3x3_f32_tma(torch.zeros(8, 6, device=dev), [0.0] * 9)  # w % 4 != 0


# ---------------------------------------------------------------- iimg
@pytest.mark.parametrize("h,w", [(1080, 1920), (1, 1), (1, 130), (97, 1), (31, 127), (33, 129), (256, 256),
                                 (300, 500), (517, 1023), (64, 256), (65, 257), (63, 255), (4096, 72), (2160, 3840),
                                 (4097, 8), (9, 2049), (13, 4101), (17, 6150), (7, 2048)])
def test_iimg_u8_i32(umi, orc, dev, h, w):
    from umi_gb300 import workloads
    x = workloads.iimg_frame(seed=h + w, h=h, w=w)
    got = umi.iimg_u8_i32(_t(x, dev)).cpu().numpy()
    assert np.array_equal(got, orc.iimg_u8_i32(x))


def test_iimg_all_255_max_value(umi, orc, dev):
    # the largest value of the 1080p workload: 1920*1080*255 < 2^31
    x = np.full((1080, 1920), 255, np.uint8)
    got = umi.iimg_u8_i32(_t(x, dev)).cpu().numpy()
    assert got[-1, -1] == 1920 * 1080 * 255
    assert np.array_equal(got, orc.iimg_u8_i32(x))


def test_iimg_4k_all_255_near_int32_max(umi, dev):
    # 3840 x 2160 x 255 = 2 115 072 000: the largest 4K integral, 1.5 % below 2^31
    import torch
    x = torch.full((2160, 3840), 255, dtype=torch.uint8, device=dev)
    got = umi.iimg_u8_i32(x)
    y = torch.arange(1, 2161, device=dev, dtype=torch.int64)[:, None]
    xx = torch.arange(1, 3841, device=dev, dtype=torch.int64)[None, :]
    assert int(got[-1, -1].item()) == 2160 * 3840 * 255
    assert torch.equal(got.to(torch.int64), y * xx * 255)
    got2 = torch.empty_like(got)
    assert umi.lib().umi_iimg_u8_i32_noalloc(umi._ptr(x), umi._ptr(got2), 2160, 3840, umi._stream_ptr()) == 0
    assert torch.equal(got2, got)


def test_iimg_unaligned_views(umi, orc, dev):
    import torch
    x = np.random.default_rng(7).integers(0, 256, (50, 61), dtype=np.uint8)
    big = torch.zeros(50 * 61 + 3, dtype=torch.uint8, device=dev)
    big[3:] = _t(x.ravel(), dev)
    inp = big[3:].view(50, 61)  # 3-byte offset: byte loads path
    out_big = torch.zeros(50 * 61 + 1, dtype=torch.int32, device=dev)
    out = out_big[1:].view(50, 61)  # 4-byte offset: scalar stores path
    umi.iimg_u8_i32(inp, out=out)
    assert np.array_equal(out.cpu().numpy(), orc.iimg_u8_i32(x))


def test_iimg_limits(umi, dev):
    import torch
    x = torch.zeros((8500, 1000), dtype=torch.uint8, device=dev)
    with pytest.raises(umi.UmiError) as e:
        umi.iimg_u8_i32(x)
    assert e.value.status == 3  # UMI_ERR_UNSUPPORTED: 8.5M pixels x 255 could overflow int32


def test_iimg_repeated_calls_reuse_workspace(umi, orc, dev):
    import torch
    ws = torch.empty(umi.iimg_workspace_bytes(200, 300), dtype=torch.uint8, device=dev)
    for seed in range(3):
        x = np.random.default_rng(seed).integers(0, 256, (200, 300), dtype=np.uint8)
        got = umi.iimg_u8_i32(_t(x, dev), workspace=ws).cpu().numpy()
        assert np.array_equal(got, orc.iimg_u8_i32(x))


@pytest.mark.parametrize("fill", [0x01, 0xFF])
@pytest.mark.parametrize("h,w", [(1080, 1920), (2160, 3840), (70, 600), (129, 130)])
def test_iimg_workspace_content_is_irrelevant(umi, orc, dev, fill, h, w):
    """Kernel 1 writes every group sum that kernel 2 reads: whatever the
    workspace held before the call, the result is exact."""
    import torch
    from umi_gb300 import workloads
    x = workloads.iimg_frame(seed=h * 7 + w + fill, h=h, w=w)
    ws = torch.full((umi.iimg_workspace_bytes(h, w),), fill, dtype=torch.uint8, device=dev)
    got = umi.iimg_u8_i32(_t(x, dev), workspace=ws).cpu().numpy()
    assert np.array_equal(got, orc.iimg_u8_i32(x))


def test_iimg_graph_replays(umi, orc, dev):
    """Captured once (the group sums and the dependent output launch),
    replayed on new frames copied into the same input buffer."""
    import torch
    h, w = 1080, 1920
    inp = torch.zeros((h, w), dtype=torch.uint8, device=dev)
    out = torch.empty((h, w), dtype=torch.int32, device=dev)
    ws = torch.empty(umi.iimg_workspace_bytes(h, w), dtype=torch.uint8, device=dev)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        umi.iimg_u8_i32(inp, out=out, workspace=ws)  # first call outside the capture
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            umi.iimg_u8_i32(inp, out=out, workspace=ws)
    torch.cuda.current_stream().wait_stream(s)
    for seed in range(3):
        x = np.random.default_rng(40 + seed).integers(0, 256, (h, w), dtype=np.uint8)
        inp.copy_(_t(x, dev))
        g.replay()
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), orc.iimg_u8_i32(x)), seed


# ---------------------------------------------------------------- full_me
@pytest.mark.parametrize("h,w,b,r", [(64, 64, 16, 4), (48, 80, 16, 7), (64, 96, 8, 7), (96, 128, 16, 32),
                                     (40, 56, 8, 3), (17, 33, 16, 5), (130, 70, 16, 64), (50, 70, 8, 13)])
def test_full_me_u8_random(umi, orc, dev, h, w, b, r):
    g = np.random.default_rng(h * 1000 + w + r)
    cur = g.integers(0, 256, (h, w), dtype=np.uint8)
    ref = g.integers(0, 256, (h, w), dtype=np.uint8)
    got = umi.full_me_u8(_t(cur, dev), _t(ref, dev), b, r).cpu().numpy()
    assert np.array_equal(got, orc.full_me_u8(cur, ref, b, r))


def test_full_me_u8_ties_first_in_raster_order(umi, orc, dev):
    # flat frames: every displacement ties, the first (-r, -r) must win
    cur = np.full((64, 64), 7, np.uint8)
    ref = np.full((64, 64), 9, np.uint8)
    got = umi.full_me_u8(_t(cur, dev), _t(ref, dev), 16, 6).cpu().numpy()
    assert np.all(got[:, 0] == -6) and np.all(got[:, 1] == -6) and np.all(got[:, 2] == 2 * 256)
    assert np.array_equal(got, orc.full_me_u8(cur, ref, 16, 6))


def test_full_me_u8_extremes(umi, orc, dev):
    # maximum SAD: 0 vs 255 everywhere
    cur = np.zeros((32, 32), np.uint8)
    ref = np.full((32, 32), 255, np.uint8)
    got = umi.full_me_u8(_t(cur, dev), _t(ref, dev), 16, 32).cpu().numpy()
    assert np.all(got[:, 2] == 255 * 256)
    assert np.array_equal(got, orc.full_me_u8(cur, ref, 16, 32))


def test_full_me_u8_centers(umi, orc, dev):
    import torch
    g = np.random.default_rng(11)
    cur = g.integers(0, 256, (64, 80), dtype=np.uint8)
    ref = g.integers(0, 256, (64, 80), dtype=np.uint8)
    n = (64 // 16) * (80 // 16)
    centers = g.integers(-20, 21, (n, 2)).astype(np.int32)
    got = umi.full_me_u8(_t(cur, dev), _t(ref, dev), 16, 4, centers=_t(centers, dev)).cpu().numpy()
    for i in range(n):
        by, bx = divmod(i, 80 // 16)
        best = None
        for dy in range(centers[i, 0] - 4, centers[i, 0] + 5):
            for dx in range(centers[i, 1] - 4, centers[i, 1] + 5):
                s = orc.block_sad_u8(cur, ref, 16, by, bx, dy, dx)
                if best is None or s < best[0]:
                    best = (s, dy, dx)
        assert tuple(got[i]) == (best[1], best[2], best[0])


@pytest.mark.parametrize("r", [1, 2, 3, 4, 5, 6, 7])
def test_full_me_small_range_centers(umi, orc, dev, r):
    # the register-only small-range search: centres that push windows past every frame edge
    import torch
    g = np.random.default_rng(40 + r)
    h, w = 80, 112
    cur = g.integers(0, 256, (h, w), dtype=np.uint8)
    ref = g.integers(0, 256, (h, w), dtype=np.uint8)
    n = (h // 16) * (w // 16)
    centers = g.integers(-30, 31, (n, 2)).astype(np.int32)
    centers[:4] = [[-40, -40], [40, 40], [0, -3], [5, 0]]
    got = umi.full_me_u8(_t(cur, dev), _t(ref, dev), 16, r, centers=_t(centers, dev)).cpu().numpy()
    for i in range(n):
        by, bx = divmod(i, w // 16)
        best = None
        for dy in range(centers[i, 0] - r, centers[i, 0] + r + 1):
            for dx in range(centers[i, 1] - r, centers[i, 1] + r + 1):
                s = orc.block_sad_u8(cur, ref, 16, by, bx, dy, dx)
                if best is None or s < best[0]:
                    best = (s, dy, dx)
        assert tuple(got[i]) == (best[1], best[2], best[0]), i
    # without centres: identical to the oracle's search around (0, 0); flat frames tie to the first
    assert np.array_equal(umi.full_me_u8(_t(cur, dev), _t(ref, dev), 16, r).cpu().numpy(),
                          orc.full_me_u8(cur, ref, 16, r))
    flat = umi.full_me_u8(torch.full((32, 48), 3, dtype=torch.uint8, device=dev),
                          torch.full((32, 48), 5, dtype=torch.uint8, device=dev), 16, r).cpu().numpy()
    assert np.all(flat[:, :2] == -r) and np.all(flat[:, 2] == 512)


def test_full_me_sad_volume(umi, orc, dev):
    g = np.random.default_rng(12)
    cur = g.integers(0, 256, (48, 64), dtype=np.uint8)
    ref = g.integers(0, 256, (48, 64), dtype=np.uint8)
    for b, r in [(16, 5), (8, 7), (16, 32)]:
        got = umi.full_me_sad_u8(_t(cur, dev), _t(ref, dev), b, r).cpu().numpy()
        _, want = orc.full_me_u8(cur, ref, b, r, sad_volume=True)
        assert np.array_equal(got, want)


def test_full_me_sad_volume_matches_reference_loop(umi, orc, dev):
    # the reference example's own check (main/full_me.cu:66-87) on a u8 pair
    g = np.random.default_rng(13)
    cur = g.integers(0, 256, (40, 64), dtype=np.uint8)
    ref = g.integers(0, 256, (40, 64), dtype=np.uint8)
    got = umi.full_me_sad_u8(_t(cur, dev), _t(ref, dev), 8, 7).cpu().numpy()
    want = orc.ref_full_me_i32(cur.astype(np.int32), ref.astype(np.int32), 8, -7, 15)
    assert np.array_equal(got, want)


def test_full_me_u8_1080p_workload(umi, orc, dev):
    """The benchmark workload: 1920x1080 pair, 16x16 blocks, +-32, all 8040 blocks."""
    from umi_gb300 import workloads
    cur, ref, true_mv = workloads.me_pair(seed=3)
    got = umi.full_me_u8(_t(cur, dev), _t(ref, dev), 16, 32).cpu().numpy()
    assert got.shape == (8040, 3)
    want = orc.full_me_u8(cur, ref, 16, 32)
    assert np.array_equal(got, want)
    # sanity: most blocks recover the planted translation
    assert np.mean(np.all(got[:, :2] == true_mv, axis=1)) > 0.8
