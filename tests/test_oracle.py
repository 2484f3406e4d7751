"""CPU tests of the oracle itself: pinned against the reference's own checks.

refpin.json holds, for every Execute call of the reference's example programs,
the digest of the output that the reference's own CPU assert loop accepted
(tests/golden/make_refpin_golden.py).  Here the closed-form oracle recomputes
those outputs from the same inputs and must reproduce the digests.
"""
import hashlib
import json
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLD = json.load(open(os.path.join(HERE, "golden", "refpin.json")))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _closed_form(app):
    import importlib.util
    spec = importlib.util.spec_from_file_location("mk", os.path.join(HERE, "golden", "make_refpin_golden.py"))
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    return mk.closed_form(app, GOLD["apps"][app]["params"])


@pytest.mark.parametrize("app", ["filter3x3", "wfilter3x3", "bilateral", "cost_volume", "full_me", "iimg", "gemm"])
def test_closed_form_matches_reference_checks(app, orc):
    outs = _closed_form(app)
    calls = GOLD["apps"][app]["calls"]
    assert len(outs) == len(calls)
    for got, want in zip(outs, calls):
        assert got.size == want["n"]
        assert sha(got) == want["sha256"], app


@pytest.mark.slow
def test_closed_form_fprop_matches_reference_check(orc):
    outs = _closed_form("fprop")
    assert sha(outs[0]) == GOLD["apps"]["fprop"]["calls"][0]["sha256"]


def test_fprop_input_stream(orc):
    # main/fprop.cu:41-47: default_random_engine + uniform_int_distribution(0, 10)
    a, b = orc.ref_fprop_inputs(1000, 10)
    assert a.min() >= 0 and a.max() <= 10
    a2, b2 = orc.ref_fprop_inputs(1010, 0)
    assert np.array_equal(a2[:1000], a) and np.array_equal(a2[1000:], b)


REFPIN = os.path.join(ROOT, "oracle", "_ref")
REF_SRC = os.environ.get("UMI_REFERENCE", os.path.join(os.path.dirname(ROOT), "reference"))


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF_SRC, "main")), reason="reference sources not present")
@pytest.mark.parametrize("app", ["filter3x3", "wfilter3x3", "bilateral", "cost_volume", "full_me", "iimg", "gemm"])
def test_reference_program_accepts_oracle(app):
    """The reference's own example program, compiled against the oracle shim,
    must pass its own assert loop."""
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), f"REF={REF_SRC}", f"_ref/{app}"], check=True)
    r = subprocess.run([os.path.join(REFPIN, app)], capture_output=True, timeout=300)
    assert r.returncode == 0, r.stderr


# ---- oracle self-consistency at workload types ----

def test_iimg_u8_matches_cumsum(orc):
    g = np.random.default_rng(0)
    for h, w in [(1, 1), (1, 7), (5, 1), (37, 53), (120, 200)]:
        x = g.integers(0, 256, (h, w), dtype=np.uint8)
        want = np.cumsum(np.cumsum(x.astype(np.int64), 0), 1).astype(np.int32)
        assert np.array_equal(orc.iimg_u8_i32(x), want)


def test_iimg_u8_matches_reference_loop(orc):
    # the u8 form against the reference's int32 loop (main/iimg.cu:100-111)
    x = np.random.default_rng(1).integers(0, 256, (64, 90), dtype=np.uint8)
    assert np.array_equal(orc.iimg_u8_i32(x), orc.ref_iimg_i32(x.astype(np.int32)))


def test_full_me_argmin_matches_volume(orc):
    g = np.random.default_rng(2)
    cur = g.integers(0, 256, (48, 64), dtype=np.uint8)
    ref = g.integers(0, 256, (48, 64), dtype=np.uint8)
    mv, vol = orc.full_me_u8(cur, ref, 16, 5, sad_volume=True)
    nd = 11
    flat = vol.reshape(-1, nd * nd)
    idx = flat.argmin(axis=1)  # numpy argmin returns the first minimum: raster order
    assert np.array_equal(mv[:, 2], flat.min(axis=1))
    assert np.array_equal(mv[:, 0], idx // nd - 5)
    assert np.array_equal(mv[:, 1], idx % nd - 5)


def test_full_me_u8_matches_reference_loop(orc):
    # The u8 SAD volume equals the reference's int32 loop (main/full_me.cu:68-87)
    # with the same clamping, for a (cur, ref) pair.
    g = np.random.default_rng(3)
    cur = g.integers(0, 256, (40, 56), dtype=np.uint8)
    ref = g.integers(0, 256, (40, 56), dtype=np.uint8)
    _, vol = orc.full_me_u8(cur, ref, 8, 7, sad_volume=True)
    want = orc.ref_full_me_i32(cur.astype(np.int32), ref.astype(np.int32), 8, -7, 15)
    assert np.array_equal(vol, want)


def test_full_me_blocks_subset(orc):
    g = np.random.default_rng(4)
    cur = g.integers(0, 256, (64, 64), dtype=np.uint8)
    ref = g.integers(0, 256, (64, 64), dtype=np.uint8)
    full = orc.full_me_u8(cur, ref, 16, 4)
    sub = orc.full_me_u8(cur, ref, 16, 4, blocks=np.array([3, 0, 15], np.int32))
    assert np.array_equal(sub, full[[3, 0, 15]])


def test_filter_f64_matches_numpy(orc):
    g = np.random.default_rng(5)
    x = g.random((33, 47), dtype=np.float32)
    w9 = g.standard_normal(9).astype(np.float32)
    p = np.pad(x.astype(np.float64), 1)
    want = np.zeros(x.shape)
    for i in range(3):
        for j in range(3):
            want += float(w9[3 * i + j]) * p[i:i + 33, j:j + 47]
    np.testing.assert_allclose(orc.filter3x3_f64(x, w9), want, rtol=1e-12, atol=1e-12)


def test_me_pair_true_motion_is_found(orc):
    from umi_gb300 import workloads
    cur, ref, true_mv = workloads.me_pair(seed=9, h=96, w=128, shift_sigma=3.0, max_shift=6)
    mv = orc.full_me_u8(cur, ref, 16, 8)
    # interior blocks must recover the planted translation
    nby, nbx = 6, 8
    inner = [by * nbx + bx for by in range(1, nby - 1) for bx in range(1, nbx - 1)]
    hit = np.mean([(mv[i, 0], mv[i, 1]) == tuple(true_mv[i]) for i in inner])
    assert hit > 0.9


def _coarse_numpy(cur, ref, rng):
    """The coarse proposal restated from its definition with numpy (independent of the C oracle)."""
    h, w = cur.shape
    def q(img, y, x):  # (n,) y, (n,) x -> rounded 4x4 means, coordinates clamped
        yy = np.clip(y[:, None, None] + np.arange(4)[None, :, None], 0, h - 1)
        xx = np.clip(x[:, None, None] + np.arange(4)[None, None, :], 0, w - 1)
        return (img[yy, xx].astype(np.int64).sum(axis=(1, 2)) + 8) >> 4
    nby, nbx = h // 16, w // 16
    out = np.zeros((nby * nbx, 2), np.int32)
    ii, jj = np.meshgrid(np.arange(4), np.arange(4), indexing="ij")
    for blk in range(nby * nbx):
        by, bx = divmod(blk, nbx)
        ys, xs = (16 * by + 4 * ii).ravel(), (16 * bx + 4 * jj).ravel()
        c = q(cur, ys, xs)
        best = None
        for dy in range(-rng, rng + 1, 2):
            for dx in range(-rng, rng + 1, 2):
                s = int(np.abs(c - q(ref, ys + dy, xs + dx)).sum())
                if best is None or s < best[0]:
                    best = (s, dy, dx)
        out[blk] = best[1:]
    return out


@pytest.mark.parametrize("h,w,rng", [(32, 48, 6), (48, 32, 10), (16, 16, 0), (16, 64, 2), (48, 64, 8)])
def test_coarse_centers_match_numpy(orc, h, w, rng):
    g = np.random.default_rng(h + w + rng)
    cur = g.integers(0, 256, (h, w), dtype=np.uint8)
    ref = g.integers(0, 256, (h, w), dtype=np.uint8)
    assert np.array_equal(orc.coarse_centers_u8(cur, ref, rng), _coarse_numpy(cur, ref, rng))
    if h >= 48 and w >= 48:
        # a planted displacement is found exactly: block (1, 1) of moved = ref at (+6, -4)
        moved = np.roll(ref, (-6, 4), axis=(0, 1))
        assert (orc.coarse_centers_u8(moved, ref, rng)[w // 16 + 1] == [6, -4]).all()


def test_coarse_proposal_lands_near_true_motion(orc):
    # the property the proposal exists for: on the 4K-style pairs (per-block shifts
    # N(0, 16^2) clipped to +-64) almost every block's centre lies within +-4 of the
    # planted motion, so a +-4 refine around it holds the optimum
    from umi_gb300 import workloads
    cur, ref, true_mv = workloads.me_pair(seed=21, h=544, w=960, shift_sigma=16.0, max_shift=64)
    c = orc.coarse_centers_u8(cur, ref, 60)
    near = np.all(np.abs(c - np.clip(true_mv, -60, 60)) <= 4, axis=1)
    assert near.mean() > 0.95, near.mean()
