"""Poisoned guard zones around every output (the sanitizer-free bounds check):
each output is a view into a larger buffer whose guard words before and after
hold a sentinel; after the call the guards must be intact.  Sizes are ragged
so that edge tiles, partial vectors and TMA clipping are exercised.  Also the
checked build of the generic path (-DUMI_CHECKED, tests/cpp/checked_oob.cu)."""
import json
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GUARD = 256  # elements on each side (a multiple of 4: views stay 16-byte aligned)


def _guarded(shape, dtype, dev):
    """(full buffer, view) with sentinel guards; the view starts GUARD elements in."""
    import torch
    n = int(np.prod(shape))
    full = torch.empty(n + 2 * GUARD, dtype=dtype, device=dev)
    if dtype.is_floating_point:
        full.fill_(-12345.0)
    else:
        full.fill_(-123456789 if dtype == torch.int32 else 0x5A)
    return full, full[GUARD:GUARD + n].view(shape)


def _guards_ok(full):
    import torch
    sentinel = full[0].item()
    head, tail = full[:GUARD], full[-GUARD:]
    return bool(torch.all(head == sentinel).item()) and bool(torch.all(tail == sentinel).item())


def test_guards_filter_iimg(umi, dev):
    import torch
    g = torch.Generator(device=dev).manual_seed(1)
    h, w = 37, 45
    x = torch.rand((h, w), generator=g, device=dev)
    full, out = _guarded((h, w), torch.float32, dev)
    umi.filter3x3_f32(x, [0.5] * 9, out=out)
    torch.cuda.synchronize()
    assert _guards_ok(full)
    for hh, ww in [(33, 129), (9, 2049), (17, 6150)]:
        u8 = torch.randint(0, 256, (hh, ww), generator=g, device=dev, dtype=torch.uint8)
        full, out = _guarded((hh, ww), torch.int32, dev)
        umi.iimg_u8_i32(u8, out=out)
        torch.cuda.synchronize()
        assert _guards_ok(full), (hh, ww)


def test_guards_full_me(umi, dev):
    import torch
    from umi_gb300.workloads import me_pair
    cur, ref, _ = me_pair(seed=8, h=100, w=150, shift_sigma=4.0, max_shift=8)
    c, r = torch.from_numpy(cur).to(dev), torch.from_numpy(ref).to(dev)
    nblk = (100 // 16) * (150 // 16)
    for search in (8, 32, 64):
        full, out = _guarded((nblk, 3), torch.int32, dev)
        umi.full_me_u8(c, r, 16, search, out=out)
        torch.cuda.synchronize()
        assert _guards_ok(full), search
    full, out = _guarded((nblk, 3), torch.int32, dev)
    blocks = torch.tensor([3, 7, 11], dtype=torch.int32, device=dev)
    umi.full_me_u8_list(c, r, blocks, torch.tensor([3], dtype=torch.int32, device=dev), out, 16, 16)
    torch.cuda.synchronize()
    assert _guards_ok(full)


def test_guards_batched_ops(umi, dev):
    import torch
    g = torch.Generator(device=dev).manual_seed(2)
    h, w = 61, 83
    x = torch.rand((h, w), generator=g, device=dev)
    full, out = _guarded((h, w), torch.float32, dev)
    umi.bilateral_f32(x, out=out)
    torch.cuda.synchronize()
    assert _guards_ok(full)
    wts = torch.rand((h, w, 3, 3), generator=g, device=dev)
    full, out = _guarded((h, w), torch.float32, dev)
    umi.wfilter3x3_pp_f32(x, wts, out=out)
    torch.cuda.synchronize()
    assert _guards_ok(full)
    L = torch.rand((32, 13, 77), generator=g, device=dev)
    R = torch.rand((32, 13, 77), generator=g, device=dev)
    full, out = _guarded((13, 77, 64), torch.float32, dev)
    umi.cost_volume_dot_f32(L, R, 64, out=out)
    torch.cuda.synchronize()
    assert _guards_ok(full)
    # the tensor-core cost volume (16-byte aligned rows): ragged last tile, bulk stores of partial warps
    for w in (76, 200, 4, 131):
        L = torch.rand((32, 13, w), generator=g, device=dev)
        R = torch.rand((32, 13, w), generator=g, device=dev)
        full, out = _guarded((13, w, 64), torch.float32, dev)
        umi.cost_volume_dot_f32(L, R, 64, out=out)
        torch.cuda.synchronize()
        assert _guards_ok(full), w


def test_guards_gemm_conv(umi, dev):
    import torch
    g = torch.Generator(device="cpu").manual_seed(3)
    for M, N, K in [(130, 520, 136), (200, 300, 72), (1, 1, 16)]:
        A = torch.randn(M, K, generator=g).to(torch.bfloat16).to(dev)
        B = torch.randn(N, K, generator=g).to(torch.bfloat16).to(dev)
        full, out = _guarded((M, N), torch.float32, dev)
        umi.gemm(A, B, out=out)
        torch.cuda.synchronize()
        assert _guards_ok(full), (M, N, K)
    for n, c, h, w, k, r in [(1, 64, 6, 300, 96, 3), (2, 64, 3, 129, 16, 3), (1, 64, 9, 20, 200, 5)]:
        x = torch.randn(n, h, w, c, generator=g).to(torch.bfloat16).to(dev)
        wt = (torch.randn(k, r, r, c, generator=g) / 24).to(torch.bfloat16).to(dev)
        full, out = _guarded((n, k, h, w), torch.float32, dev)
        umi.conv2d_fprop_bf16(x, wt, out=out)
        torch.cuda.synchronize()
        assert _guards_ok(full), (n, c, h, w, k, r)


def test_guards_menet(umi, dev):
    import torch
    h, w = 144, 528
    g = torch.Generator(device=dev).manual_seed(4)
    cur = torch.randint(0, 256, (h, w), generator=g, device=dev, dtype=torch.uint8)
    ref = torch.randint(0, 256, (h, w), generator=g, device=dev, dtype=torch.uint8)
    net = umi.MeNet(h, w, device=dev)
    nblk = (h // 16) * (w // 16)
    full, pred = _guarded((nblk, 2), torch.float32, dev)
    net.infer(cur, ref, pred=pred)
    torch.cuda.synchronize()
    assert _guards_ok(full)
    full, mv = _guarded((nblk, 3), torch.int32, dev)
    net.estimate(cur, ref, 4, 24, sad_threshold=500, audit_stride=7, out=mv)
    torch.cuda.synchronize()
    assert _guards_ok(full)


def test_checked_build_flags_out_of_extent_writes(umi):
    import sys
    sys.path.insert(0, os.path.join(HERE, "cpp"))
    import build_tests
    path = build_tests.binary("checked_oob")
    if not os.path.exists(path):
        build_tests.build()
    r = subprocess.run([path], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    d = json.loads(r.stdout.strip().splitlines()[-1])
    assert d["valid"] == {"status": 0, "flags": 0, "guard_ok": 1, "written": 64}
    assert d["oob"]["status"] == 0 and d["oob"]["flags"] == 1 and d["oob"]["guard_ok"] == 1
    assert d["oob"]["written"] == 22  # points 0..21 land at 0, 3, ..., 63; the rest are skipped


def test_guards_coarse_me(umi, dev):
    import torch
    h, w = 144, 528
    g = torch.Generator(device=dev).manual_seed(5)
    cur = torch.randint(0, 256, (h, w), generator=g, device=dev, dtype=torch.uint8)
    ref = torch.randint(0, 256, (h, w), generator=g, device=dev, dtype=torch.uint8)
    cme = umi.CoarseMe(h, w, device=dev)
    nblk = (h // 16) * (w // 16)
    for rng in (0, 30, 62):
        full, cen = _guarded((nblk, 2), torch.int32, dev)
        cme.centers(cur, ref, rng, out=cen)
        torch.cuda.synchronize()
        assert _guards_ok(full), rng
    full, mv = _guarded((nblk, 3), torch.int32, dev)
    cme.estimate(cur, ref, 4, 24, sad_threshold=500, audit_stride=7, out=mv)
    torch.cuda.synchronize()
    assert _guards_ok(full)
