"""Row-band split (umi_gb300/bands.py) on CPU: the band plans cover every
block row once with the rows their candidates read, band searches on the
slices reproduce the whole-frame search (the oracle on both sides), and the
integral image's exchange step and the gathering of bands work across two
gloo ranks."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


@pytest.mark.parametrize("h,w,b,r", [(80, 48, 16, 7), (50, 40, 8, 5), (1080, 1920, 16, 32), (17, 16, 16, 64),
                                     (2160, 3840, 16, 64), (33, 24, 8, 1)])
@pytest.mark.parametrize("world", [1, 2, 3, 4, 7])
def test_me_band_plans(h, w, b, r, world):
    from umi_gb300 import bands
    nby, nbx = h // b, w // b
    seen = []
    for rank in range(world):
        p = bands.me_band_plan(h, w, b, r, world, rank)
        assert p.s0 % b == 0 and 0 <= p.s0 <= p.s1 <= h
        assert p.count == (p.by1 - p.by0) * nbx and p.first == (p.by0 - p.s0 // b) * nbx
        seen += list(range(p.by0, p.by1))
        if p.count:
            lo, hi = p.by0 * b - r, p.by1 * b - 1 + r  # rows the band's candidates read
            assert p.s0 == 0 if lo < 0 else p.s0 <= lo
            assert p.s1 == h if hi >= h else p.s1 > hi
            assert p.first + p.count <= ((p.s1 - p.s0) // b) * nbx
    assert seen == list(range(nby))


@pytest.mark.parametrize("h,w,b,r", [(80, 48, 16, 7), (50, 40, 8, 5), (45, 32, 8, 9)])
@pytest.mark.parametrize("world", [2, 3, 4])
def test_me_bands_reproduce_whole_frame_on_the_oracle(h, w, b, r, world):
    import oracle
    from umi_gb300 import bands
    g = np.random.default_rng(h * world + r)
    cur = g.integers(0, 256, (h, w), dtype=np.uint8)
    ref = np.roll(cur, (3, -2), (0, 1)) ^ g.integers(0, 4, (h, w), dtype=np.uint8)
    whole = oracle.full_me_u8(cur, ref, b, r)
    parts = []
    for rank in range(world):
        p = bands.me_band_plan(h, w, b, r, world, rank)
        if p.count:
            blocks = np.arange(p.first, p.first + p.count, dtype=np.int32)
            parts.append(oracle.full_me_u8(cur[p.s0:p.s1], ref[p.s0:p.s1], b, r, blocks=blocks))
    assert np.array_equal(np.concatenate(parts), whole)


def _iimg_i32(x):
    s = np.cumsum(np.cumsum(x.astype(np.int64), 0), 1)
    return ((s + 2 ** 31) % 2 ** 32 - 2 ** 31).astype(np.int32)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _band_worker(rank, world, port, frames, out_path):
    os.environ.update(WORLD_SIZE=str(world), RANK=str(rank), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist
    from umi_gb300 import bands
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ok = []
    for img in frames:
        y0, y1 = bands.split(img.shape[0], world, rank)
        local = torch.from_numpy(_iimg_i32(img[y0:y1]))  # the band's own integral image
        band = bands.add_carry(local, bands.exchange_totals(bands.band_totals(local)), rank)
        whole = bands.gather_rows(band)
        ok.append(bool(np.array_equal(whole.numpy(), _iimg_i32(img))))
    dist.destroy_process_group()
    with open(f"{out_path}.{rank}", "w") as f:
        f.write(repr(ok))


def test_iimg_exchange_and_gather_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    g = np.random.default_rng(3)
    frames = [g.integers(0, 256, (37, 53), dtype=np.uint8),  # uneven bands: 18 and 19 rows
              g.integers(0, 256, (1, 9), dtype=np.uint8),    # an empty band on rank 0
              np.full((2160, 3840), 255, np.uint8)]           # 4K of 255: sums near 2^31, the operator's limit
    out = str(tmp_path / "bands")
    mp.spawn(_band_worker, args=(2, _free_port(), frames, out), nprocs=2, join=True)
    for rank in range(2):
        assert open(f"{out}.{rank}").read() == repr([True] * len(frames))


def test_single_process_exchange_is_local():
    import torch
    from umi_gb300 import bands
    t = torch.arange(5, dtype=torch.int32)
    got = bands.exchange_totals(t)
    assert len(got) == 1 and got[0] is t
    assert bands.gather_rows(t) is t
    with pytest.raises(ValueError):
        bands.split(10, 2, 2)
