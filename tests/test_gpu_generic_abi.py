"""The generic operator through the C ABI (umi_plan_create / umi_launch /
umi_plan_destroy) on the reference applications' descriptors and inputs
(main/*.cu, the same calls as tests/cpp/dropin_apps.cu): every integer output
must have the digest the reference's own CPU checks accepted
(tests/golden/refpin.json); bilateral is held to the reference's 0.1 %.
Plus the batch-graph API against single batched launches."""
import hashlib
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "refpin.json")))
PAD, WRAP = 0, 1


def _iota(n, dev):
    import torch
    return torch.arange(n, dtype=torch.int32, device=dev)


def _digest_ok(app, call, t):
    want = GOLD["apps"][app]["calls"][call]
    raw = t.cpu().numpy().astype(np.int32).ravel()
    assert raw.size == want["n"]
    assert hashlib.sha256(raw.tobytes()).hexdigest() == want["sha256"], (app, call)


def test_launch_filter3x3(umi, dev):
    import torch
    w, h = 500, 300
    x, out = _iota(w * h, dev), torch.zeros(w * h, dtype=torch.int32, device=dev)
    d = umi.make_desc(p=[(1, 1, 1, 1), (1, 1, 1, 1), (h, 16, 4, 1), (w, 16, 8, 1)],
                      a=[(1, 1), (1, 1), (3, 3), (3, 3)],
                      mems=[dict(p_view=[(), (), (2, 0, 1), (3, 0, 1)], a_view=[(), (), (2, -1, 1), (3, -1, 1)],
                                 phys=[(1, PAD), (1, PAD), (h, PAD), (w, PAD)], stage=1),
                            dict(p_view=[(), (), (2, 0, 1), (3, 0, 1)], phys=[(), (), (h, PAD), (w, PAD)], stage=2,
                                 out=True)], expand=0x1111)
    umi.launch(d, umi.STRATEGY_NEIGHBOUR_SUM_I32, [x], [out], pads=[999], consts=[-5, 2])
    _digest_ok("filter3x3", 0, out)


def test_launch_wfilter3x3(umi, dev):
    import torch
    w, h = 300, 250
    x, out = _iota(w * h, dev), torch.zeros(w * h, dtype=torch.int32, device=dev)
    wt = torch.tensor([1, 2, 1, 2, 4, 2, 1, 2, 1], dtype=torch.int32, device=dev)
    d = umi.make_desc(p=[(1, 1, 1, 1), (1, 1, 1, 1), (h, 16, 4, 1), (w, 16, 8, 1)],
                      a=[(1, 1), (1, 1), (3, 3), (3, 3)],
                      mems=[dict(p_view=[(), (), (2, 0, 1), (3, 0, 1)], a_view=[(), (), (2, -1, 1), (3, -1, 1)],
                                 phys=[(1, PAD), (1, PAD), (h, PAD), (w, PAD)], stage=1),
                            dict(p_view=[(), (), (), ()], a_view=[(), (), (2, 0, 1), (3, 0, 1)],
                                 phys=[(1, PAD), (1, PAD), (3, PAD), (3, PAD)], stage=1),
                            dict(p_view=[(), (), (2, 0, 1), (3, 0, 1)], phys=[(), (), (h, PAD), (w, PAD)], stage=2,
                                 out=True)], expand=0x1122)
    umi.launch(d, umi.STRATEGY_WEIGHTED_SUM_I32, [x, wt], [out], pads=[56, 0], consts=[-5])
    _digest_ok("wfilter3x3", 0, out)


def test_launch_cost_volume_and_full_me(umi, dev):
    import torch
    w, h, k, sr = 1920, 1080, 7, 15
    ko, so = k // 2, sr // 2
    f = _iota(w * h, dev)
    cv = torch.zeros(w * h * sr, dtype=torch.int32, device=dev)
    d = umi.make_desc(p=[(1, 1, 1, 1), (h, 4, 1, 1), (w, 8, 2, 1), (sr, 16, 16, 1)],
                      a=[(1, 1), (1, 1), (1, 1), (k, k)],
                      mems=[dict(p_view=[(), (2, 0, 1), (3, 0, 1), (3, -so, 1)], a_view=[(), (), (), (3, -ko, 1)],
                                 phys=[(1, WRAP), (1, WRAP), (h, WRAP), (w, WRAP)], stage=1),
                            dict(p_view=[(), (2, 0, 1), (3, 0, 1), ()], a_view=[(), (), (), (3, -ko, 1)],
                                 phys=[(1, WRAP), (1, WRAP), (h, WRAP), (w, WRAP)], stage=1),
                            dict(p_view=[(), (1, 0, 1), (2, 0, 1), (3, 0, 1)],
                                 phys=[(1, WRAP), (h, WRAP), (w, WRAP), (sr, WRAP)], stage=2, out=True)])
    umi.launch(d, umi.STRATEGY_ABS_DIFF_SUM_I32, [f, f], [cv])
    _digest_ok("cost_volume", 0, cv)
    b, so, sr = 8, -7, 15
    sad = torch.zeros((w // b) * (h // b) * sr * sr, dtype=torch.int32, device=dev)
    d = umi.make_desc(p=[(h // b, 1, 1, 1), (w // b, 1, 1, 1), (sr, 16, 2, 1), (sr, 16, 16, 1)],
                      a=[(1, 1), (1, 1), (b, b), (b, b)],
                      mems=[dict(p_view=[(2, 0, b), (3, 0, b), (2, so, 1), (3, so, 1)], a_view=[(), (), (2, 0, 1), (3, 0, 1)],
                                 phys=[(1, WRAP), (1, WRAP), (h, WRAP), (w, WRAP)], stage=1),
                            dict(p_view=[(2, 0, b), (3, 0, b), (), ()], a_view=[(), (), (2, 0, 1), (3, 0, 1)],
                                 phys=[(1, WRAP), (1, WRAP), (h, WRAP), (w, WRAP)], stage=1),
                            dict(p_view=[(0, 0, 1), (1, 0, 1), (2, 0, 1), (3, 0, 1)],
                                 phys=[(h // b, WRAP), (w // b, WRAP), (sr, WRAP), (sr, WRAP)], stage=2, out=True)],
                      expand=0x2211)
    umi.launch(d, umi.STRATEGY_ABS_DIFF_SUM_I32, [f, f], [sad])
    _digest_ok("full_me", 0, sad)


def test_launch_iimg_two_calls(umi, dev):
    import torch
    w, h = 500, 300
    x = torch.ones(w * h, dtype=torch.int32, device=dev)
    tmp = torch.zeros(w * h, dtype=torch.int32, device=dev)
    out = torch.zeros(w * h, dtype=torch.int32, device=dev)
    d1 = umi.make_desc(p=[(1, 1, 1, 1), (1, 1, 1, 1), (1, 1, 1, 1), (h, 128, 32, 1)], a=[(1, 1), (1, 1), (1, 1), (w, 32)],
                       mems=[dict(p_view=[(), (), (), (2, 0, 1)], a_view=[(), (), (), (3, 0, 1)],
                                  phys=[(1, PAD), (1, PAD), (h, PAD), (w, PAD)], stage=1),
                             dict(p_view=[(), (), (), (3, 0, 1)], a_view=[(), (), (), (2, 0, 1)],
                                  phys=[(1, PAD), (1, PAD), (w, PAD), (h, PAD)], stage=1, out=True)])
    umi.launch(d1, umi.STRATEGY_RUNNING_SUM_I32, [x], [tmp])
    _digest_ok("iimg", 0, tmp)
    # the reference's second call leaves warp_shuf at 0 (read as 1 here)
    d2 = umi.make_desc(p=[(1, 1, 1, 0), (1, 1, 1, 0), (1, 1, 1, 0), (w, 128, 32, 0)], a=[(1, 1), (1, 1), (1, 1), (h, 32)],
                       mems=[dict(p_view=[(), (), (), (2, 0, 1)], a_view=[(), (), (), (3, 0, 1)],
                                  phys=[(1, PAD), (1, PAD), (w, PAD), (h, PAD)], stage=1),
                             dict(p_view=[(), (), (), (3, 0, 1)], a_view=[(), (), (), (2, 0, 1)],
                                  phys=[(1, PAD), (1, PAD), (h, PAD), (w, PAD)], stage=1, out=True)])
    umi.launch(d2, umi.STRATEGY_RUNNING_SUM_I32, [tmp], [out])
    _digest_ok("iimg", 1, out)


def test_launch_gemm_and_fprop(umi, orc, dev):
    import torch
    m, k, n = 100, 100, 200
    A, B = _iota(m * k, dev), _iota(k * n, dev)
    C = torch.zeros(m * n, dtype=torch.int32, device=dev)
    d = umi.make_desc(p=[(1, 1, 1, 1), (1, 1, 1, 1), (m, 16, 2, 1), (n, 16, 16, 1)], a=[(1, 1), (1, 1), (1, 1), (k, 16)],
                      mems=[dict(p_view=[(), (), (2, 0, 1), ()], a_view=[(), (), (), (3, 0, 1)],
                                 phys=[(1, PAD), (1, PAD), (m, PAD), (k, PAD)], stage=1),
                            dict(p_view=[(), (), (), (3, 0, 1)], a_view=[(), (), (), (2, 0, 1)],
                                 phys=[(1, PAD), (1, PAD), (k, PAD), (n, PAD)], stage=1),
                            dict(p_view=[(), (), (2, 0, 1), (3, 0, 1)], phys=[(), (), (m, PAD), (n, PAD)], stage=2,
                                 out=True)], expand=0x1124)
    umi.launch(d, umi.STRATEGY_DOT_I32, [A, B], [C])
    _digest_ok("gemm", 0, C)
    iw, ih, f, s, ich, och, bs = 80, 64, 7, 2, 40, 60, 32
    ofs, ow, oh = -(f // 2), iw // s, ih // s  # main/fprop.cu: ofs = -f / 2 (C++ truncation)
    xin, wt = orc.ref_fprop_inputs(iw * ih * ich * bs, och * ich * f * f)
    x = torch.from_numpy(xin).to(dev)
    wd = torch.from_numpy(wt).to(dev)
    out = torch.zeros(ow * oh * och * bs, dtype=torch.int32, device=dev)
    d = umi.make_desc(p=[(bs, 1, 1, 1), (och, 4, 1, 1), (oh, 8, 4, 1), (ow, 8, 8, 1)],
                      a=[(1, 1), (ich, 6), (f, f), (f, f)],
                      mems=[dict(p_view=[(0, 0, 1), (), (2, 0, s), (3, 0, s)], a_view=[(), (1, 0, 1), (2, ofs, 1), (3, ofs, 1)],
                                 phys=[(bs, PAD), (ich, PAD), (ih, PAD), (iw, PAD)], stage=1),
                            dict(p_view=[(), (0, 0, 1), (), ()], a_view=[(), (1, 0, 1), (2, 0, 1), (3, 0, 1)],
                                 phys=[(och, PAD), (ich, PAD), (f, PAD), (f, PAD)], stage=1),
                            dict(p_view=[(0, 0, 1), (1, 0, 1), (2, 0, 1), (3, 0, 1)],
                                 phys=[(bs, PAD), (och, PAD), (oh, PAD), (ow, PAD)], stage=2, out=True)])
    umi.launch(d, umi.STRATEGY_DOT_I32, [x, wd], [out])
    _digest_ok("fprop", 0, out)


def test_launch_bilateral_within_reference_tolerance(umi, orc, dev):
    import torch
    p = GOLD["apps"]["bilateral"]["params"]
    h, w, ofs = p["h"], p["w"], p["ofs"]
    k = 2 * ofs + 1
    xn = np.arange(h * w, dtype=np.float32)
    n1 = np.float32(-1.0) / (np.float32(2.0) * np.float32(p["sigma_s"]) ** 2)
    n2 = np.float32(-1.0) / (np.float32(2.0) * np.float32(p["sigma_r"]) ** 2)
    ws = np.array([np.exp(float((i - ofs) ** 2) * float(n1)) for i in range(k)], np.float32)
    x = torch.from_numpy(xn).to(dev)
    wd = torch.from_numpy(ws).to(dev)
    out = torch.zeros(h * w, dtype=torch.float32, device=dev)
    d = umi.make_desc(p=[(1, 1, 1, 1), (1, 1, 1, 1), (h, 16, 2, 1), (w, 16, 16, 1)], a=[(1, 1), (1, 1), (k, k), (k, k)],
                      mems=[dict(p_view=[(), (), (2, 0, 1), (3, 0, 1)], phys=[(1, PAD), (1, PAD), (h, PAD), (w, PAD)],
                                 stage=0),
                            dict(p_view=[(), (), (2, 0, 1), (3, 0, 1)], a_view=[(), (), (2, -ofs, 1), (3, -ofs, 1)],
                                 phys=[(1, PAD), (1, PAD), (h, PAD), (w, PAD)], stage=1),
                            dict(a_view=[(), (), (3, 0, 1), ()], phys=[(1, PAD), (1, PAD), (1, PAD), (k, PAD)], stage=1),
                            dict(a_view=[(), (), (), (3, 0, 1)], phys=[(1, PAD), (1, PAD), (1, PAD), (k, PAD)], stage=1),
                            dict(p_view=[(), (), (2, 0, 1), (3, 0, 1)], phys=[(), (), (h, PAD), (w, PAD)], stage=2,
                                 out=True)])
    umi.launch(d, umi.STRATEGY_RANGE_WEIGHTED_F32, [x, x, wd, wd], [out], pads=[0.0, 0.0, 0.0, 0.0], consts=[n2])
    want = orc.ref_bilateral_f32(xn.reshape(h, w), ofs, ws, float(n2))
    ratio = want / out.cpu().numpy().reshape(h, w)
    assert np.all((ratio > 0.999) & (ratio < 1.001))


def test_launch_rejects_mismatched_strategy(umi, dev):
    import torch
    x = _iota(64, dev)
    d = umi.make_desc(p=[(1, 1, 1, 1), (1, 1, 1, 1), (1, 1, 1, 1), (64, 32, 32, 1)], a=[(1, 1)] * 4,
                      mems=[dict(p_view=[(), (), (), (3, 0, 1)], phys=[(1, PAD)] * 3 + [(64, PAD)], stage=1),
                            dict(p_view=[(), (), (), (3, 0, 1)], phys=[(1, PAD)] * 3 + [(64, PAD)], stage=2, out=True)])
    with pytest.raises(umi.UmiError, match="INVALID_DESC"):
        umi.launch(d, umi.STRATEGY_DOT_I32, [x], [x.clone()])  # Dot needs two Loop inputs
    with pytest.raises(umi.UmiError, match="INVALID_ARG"):
        umi.launch(d, umi.STRATEGY_NEIGHBOUR_SUM_I32, [x], [x.clone()])  # constants missing
    with pytest.raises(umi.UmiError, match="UNSUPPORTED"):
        umi.launch(d, 99, [x], [x.clone()])


def test_batch_graph_matches_batch_run(umi, dev):
    import torch
    g = torch.Generator(device=dev).manual_seed(3)
    imgs = [torch.rand((h, w), generator=g, device=dev) for h, w in [(64, 96), (130, 70), (256, 256)]]
    prm = umi.BatchParams(2, 2.0, 0.1, 0, 0)
    want = [torch.empty_like(x) for x in imgs]
    umi.batch_run(umi.OP_BILATERAL, [(x, None, o) for x, o in zip(imgs, want)], prm)
    wts = [torch.rand((x.shape[0], x.shape[1], 3, 3), generator=g, device=dev) for x in imgs]
    want2 = [torch.empty_like(x) for x in imgs]
    umi.batch_run(umi.OP_WFILTER_PP, [(x, wt, o) for x, wt, o in zip(imgs, wts, want2)])
    got = [torch.full_like(x, -1.0) for x in imgs]
    got2 = [torch.full_like(x, -1.0) for x in imgs]
    bg = umi.BatchGraph()
    bg.add(umi.OP_BILATERAL, [(x, None, o) for x, o in zip(imgs, got)], prm)
    bg.add(umi.OP_WFILTER_PP, [(x, wt, o) for x, wt, o in zip(imgs, wts, got2)])
    for _ in range(3):
        bg.launch()
    torch.cuda.synchronize()
    bg.close()
    for a, b in zip(got + got2, want + want2):
        assert torch.equal(a, b)
