"""GPU parity tests of the image operators and their batched launches, through
the C ABI, against the FP64 CPU oracle.

Floating-point tolerance: rel <= 1e-5 with
  bilateral:   rel = |y - y64| / max(|y64|, 1e-3)      (outputs are weighted means of [0,1) pixels)
  wfilter:     rel = |y - y64| / max(|y64|, sum |w x|)
  cost volume: rel = |y - y64| / max(|y64|, sum_c |L R|)
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _t(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def _bil_rel(got, want):
    return np.max(np.abs(got - want) / np.maximum(np.abs(want), 1e-3))


def _wf_scale(x, wts):
    h, w = x.shape
    p = np.pad(np.abs(x.astype(np.float64)), 1)
    s = np.zeros((h, w))
    for dy in range(3):
        for dx in range(3):
            s += np.abs(wts[:, :, dy, dx]) * p[dy:dy + h, dx:dx + w]
    return s


def _cv_scale(L, R, nd):
    c, h, w = L.shape
    Rp = np.concatenate([np.abs(R.astype(np.float64)), np.zeros((c, h, nd))], axis=2)
    La = np.abs(L.astype(np.float64))
    return np.stack([(La * Rp[:, :, d:d + w]).sum(0) for d in range(nd)], axis=-1)


@pytest.mark.parametrize("h,w,r", [(1, 1, 2), (7, 5, 2), (33, 65, 2), (256, 300, 2), (40, 70, 1), (37, 91, 3)])
def test_bilateral_f32(umi, orc, dev, h, w, r):
    x = np.random.default_rng(h * w + r).random((h, w), dtype=np.float32)
    got = umi.bilateral_f32(_t(x, dev), r, 2.0, 0.1).cpu().numpy()
    want = orc.bilateral_f64(x, r, 2.0, 0.1)
    assert _bil_rel(got, want) <= TOL


@pytest.mark.parametrize("h,w", [(1, 1), (5, 3), (64, 128), (97, 259), (300, 513)])
def test_wfilter3x3_pp_f32(umi, orc, dev, h, w):
    g = np.random.default_rng(h + w)
    x = g.random((h, w), dtype=np.float32)
    wts = g.random((h, w, 3, 3), dtype=np.float32)
    got = umi.wfilter3x3_pp_f32(_t(x, dev), _t(wts, dev)).cpu().numpy()
    want = orc.wfilter_pp_f64(x, wts)
    assert np.max(np.abs(got - want) / np.maximum(np.abs(want), _wf_scale(x, wts))) <= TOL


@pytest.mark.parametrize("c,h,w,nd", [(32, 4, 300, 64), (32, 3, 64, 64), (8, 5, 70, 32), (3, 2, 40, 16), (32, 1, 1, 64),
                                      (13, 3, 257, 64), (13, 3, 256, 64), (32, 2, 4, 64), (32, 3, 640, 64),
                                      (1, 1, 128, 64), (32, 2, 132, 64), (32, 1, 1924, 64)])
def test_cost_volume_dot_f32(umi, orc, dev, c, h, w, nd):
    g = np.random.default_rng(c * 100 + w)
    L = g.standard_normal((c, h, w)).astype(np.float32)
    R = g.standard_normal((c, h, w)).astype(np.float32)
    got = umi.cost_volume_dot_f32(_t(L, dev), _t(R, dev), nd).cpu().numpy()
    want = orc.cost_volume_dot_f64(L, R, nd)
    assert np.max(np.abs(got - want) / np.maximum(np.maximum(np.abs(want), _cv_scale(L, R, nd)), 1e-30)) <= TOL


def _uneven_sizes(seed, n, lo, hi):
    g = np.random.default_rng(seed)
    sizes = [(int(g.integers(lo, hi + 1)), int(g.integers(lo, hi + 1))) for _ in range(n)]
    sizes[1] = (0, 5)      # an empty image in the batch
    sizes[2] = (1, 1)
    return sizes


def test_batch_bilateral_all_variants(umi, orc, dev):
    import torch
    sizes = _uneven_sizes(1, 7, 16, 200)
    g = np.random.default_rng(2)
    xs = [g.random(s, dtype=np.float32) for s in sizes]
    ins = [_t(x, dev) for x in xs]
    want = [orc.bilateral_f64(x, 2, 2.0, 0.1) if x.size else None for x in xs]
    prm = umi.BatchParams(2, 2.0, 0.1, 0, 0)
    for v in range(umi.batch_variants(umi.OP_BILATERAL)):
        outs = [torch.full(s, -7.0, device=dev) for s in sizes]
        umi.batch_run(umi.OP_BILATERAL, [(i, None, o) for i, o in zip(ins, outs)], prm, variant=v)
        for o, wv in zip(outs, want):
            if wv is not None:
                assert _bil_rel(o.cpu().numpy(), wv) <= TOL, v


def test_batch_wfilter_all_variants(umi, orc, dev):
    import torch
    sizes = _uneven_sizes(3, 6, 8, 300)
    g = np.random.default_rng(4)
    xs = [g.random(s, dtype=np.float32) for s in sizes]
    ws = [g.random(s + (3, 3), dtype=np.float32) for s in sizes]
    want = [orc.wfilter_pp_f64(x, wt) if x.size else None for x, wt in zip(xs, ws)]
    for v in range(umi.batch_variants(umi.OP_WFILTER_PP)):
        outs = [torch.full(s, -7.0, device=dev) for s in sizes]
        umi.batch_run(umi.OP_WFILTER_PP, [(_t(x, dev), _t(wt, dev), o) for x, wt, o in zip(xs, ws, outs)], variant=v)
        for o, wv, x, wt in zip(outs, want, xs, ws):
            if wv is not None:
                got = o.cpu().numpy()
                assert np.max(np.abs(got - wv) / np.maximum(np.abs(wv), _wf_scale(x, wt))) <= TOL, v


def test_batch_cost_volume(umi, orc, dev):
    import torch
    sizes = _uneven_sizes(5, 5, 2, 90)
    g = np.random.default_rng(6)
    Ls = [g.standard_normal((32,) + s).astype(np.float32) for s in sizes]
    Rs = [g.standard_normal((32,) + s).astype(np.float32) for s in sizes]
    want = [orc.cost_volume_dot_f64(L, R, 64) if L.size else None for L, R in zip(Ls, Rs)]
    # variant 0: tensor cores, variant 1: FP32 pipe; ragged widths and widths cut to multiples of 4
    sizes4 = [(h, w - w % 4) for h, w in sizes]
    Ls4 = [L[:, :, :w] for L, (h, w) in zip(Ls, sizes4)]
    Rs4 = [R[:, :, :w] for R, (h, w) in zip(Rs, sizes4)]
    want4 = [orc.cost_volume_dot_f64(L, R, 64) if L.size else None for L, R in zip(Ls4, Rs4)]
    for v in range(umi.batch_variants(umi.OP_COST_VOLUME)):
        for ls, rs, sz, wn in ((Ls, Rs, sizes, want), (Ls4, Rs4, sizes4, want4)):
            outs = [torch.full(s + (64,), -7.0, device=dev) for s in sz]
            umi.batch_run(umi.OP_COST_VOLUME, [(_t(L, dev), _t(R, dev), o) for L, R, o in zip(ls, rs, outs)],
                          umi.BatchParams(0, 0.0, 0.0, 32, 64), variant=v)
            for L, R, o, wv in zip(ls, rs, outs, wn):
                if wv is not None:
                    got = o.cpu().numpy()
                    err = np.max(np.abs(got - wv) / np.maximum(np.maximum(np.abs(wv), _cv_scale(L, R, 64)), 1e-30))
                    assert err <= TOL, (v, L.shape)


def test_autotune_batch_picks_a_variant(umi, dev):
    import torch
    sizes = [(128, 200), (64, 64), (300, 100)]
    ins = [torch.rand(s, device=dev) for s in sizes]
    outs = [torch.empty(s, device=dev) for s in sizes]
    v, ms = umi.autotune_batch(umi.OP_BILATERAL, [(i, None, o) for i, o in zip(ins, outs)],
                               umi.BatchParams(2, 2.0, 0.1, 0, 0), reps=2)
    assert 0 <= v < umi.batch_variants(umi.OP_BILATERAL) and ms > 0


def test_batch_rejects_bad_arguments(umi, dev):
    import torch
    x = torch.zeros((4, 4), device=dev)
    with pytest.raises(umi.UmiError):
        umi.batch_run(umi.OP_BILATERAL, [(x, None, x)], umi.BatchParams(5, 2.0, 0.1, 0, 0))  # radius 5
    with pytest.raises(umi.UmiError):
        umi.batch_run(umi.OP_COST_VOLUME, [(x.view(1, 4, 4), x.view(1, 4, 4), x)], umi.BatchParams(0, 0, 0, 1, 48))
    with pytest.raises(umi.UmiError):
        umi.batch_run(umi.OP_WFILTER_PP, [(x, None, x)])  # missing weights


# ---------------------------------------------------------------- one fused launch for a batch step
def _fused_case(seed, n, lo, hi):
    sizes = _uneven_sizes(seed, n, lo, hi)
    g = np.random.default_rng(seed + 100)
    xs = [g.random(s, dtype=np.float32) for s in sizes]
    ws = [g.random(s + (3, 3), dtype=np.float32) for s in sizes]
    Ls = [g.standard_normal((32,) + s).astype(np.float32) for s in sizes]
    Rs = [g.standard_normal((32,) + s).astype(np.float32) for s in sizes]
    return sizes, xs, ws, Ls, Rs


def _fused_check(outs_b, outs_w, outs_c, xs, ws, Ls, Rs, want_b, want_w, want_c, tag):
    for o, wv in zip(outs_b, want_b):
        if wv is not None:
            assert _bil_rel(o.cpu().numpy(), wv) <= TOL, ("bilateral", tag)
    for o, wv, x, wt in zip(outs_w, want_w, xs, ws):
        if wv is not None:
            got = o.cpu().numpy()
            assert np.max(np.abs(got - wv) / np.maximum(np.abs(wv), _wf_scale(x, wt))) <= TOL, ("wfilter", tag)
    for o, wv, L, R in zip(outs_c, want_c, Ls, Rs):
        if wv is not None:
            got = o.cpu().numpy()
            err = np.max(np.abs(got - wv) / np.maximum(np.maximum(np.abs(wv), _cv_scale(L, R, 64)), 1e-30))
            assert err <= TOL, ("cost volume", tag)


def test_batch_fused_all_operators_every_variant(umi, orc, dev):
    """The three operators of an uneven batch (an empty and a 1x1 image
    included) in ONE fused launch, against the FP64 oracle, for every fused
    variant of the filters, and with a different variant per image."""
    import torch
    sizes, xs, ws, Ls, Rs = _fused_case(11, 7, 1, 150)
    want_b = [orc.bilateral_f64(x, 2, 2.0, 0.1) if x.size else None for x in xs]
    want_w = [orc.wfilter_pp_f64(x, wt) if x.size else None for x, wt in zip(xs, ws)]
    want_c = [orc.cost_volume_dot_f64(L, R, 64) if L.size else None for L, R in zip(Ls, Rs)]
    dx, dw, dL, dR = ([_t(a, dev) for a in arr] for arr in (xs, ws, Ls, Rs))
    nb, nw = umi.batch_fused_variants(umi.OP_BILATERAL), umi.batch_fused_variants(umi.OP_WFILTER_PP)
    assert nb >= 2 and nw >= 2
    plans = [([v] * len(sizes), [v % nw] * len(sizes)) for v in range(max(nb, nw))]
    plans.append(([i % nb for i in range(len(sizes))], [(i + 1) % nw for i in range(len(sizes))]))
    for vb, vw in plans:
        outs_b = [torch.full(s, -7.0, device=dev) for s in sizes]
        outs_w = [torch.full(s, -7.0, device=dev) for s in sizes]
        outs_c = [torch.full(s + (64,), -7.0, device=dev) for s in sizes]
        vb = [v % nb for v in vb]
        umi.batch_run_fused([(umi.OP_COST_VOLUME, list(zip(dL, dR, outs_c)), umi.BatchParams(0, 0.0, 0.0, 32, 64), None),
                             (umi.OP_WFILTER_PP, list(zip(dx, dw, outs_w)), None, vw),
                             (umi.OP_BILATERAL, [(x, None, o) for x, o in zip(dx, outs_b)],
                              umi.BatchParams(2, 2.0, 0.1, 0, 0), vb)])
        _fused_check(outs_b, outs_w, outs_c, xs, ws, Ls, Rs, want_b, want_w, want_c, (vb, vw))


@pytest.mark.parametrize("radius", [1, 3])
def test_batch_fused_filters_only_and_graph_replay(umi, orc, dev, radius):
    """Without a cost-volume job (filters only), other radii, and the fused
    launch recorded in a batch graph and replayed twice."""
    import torch
    sizes, xs, ws, _, _ = _fused_case(20 + radius, 5, 3, 260)
    want_b = [orc.bilateral_f64(x, radius, 1.5, 0.2) if x.size else None for x in xs]
    want_w = [orc.wfilter_pp_f64(x, wt) if x.size else None for x, wt in zip(xs, ws)]
    dx, dw = [_t(a, dev) for a in xs], [_t(a, dev) for a in ws]
    outs_b = [torch.full(s, -7.0, device=dev) for s in sizes]
    outs_w = [torch.full(s, -7.0, device=dev) for s in sizes]
    jobs = [(umi.OP_BILATERAL, [(x, None, o) for x, o in zip(dx, outs_b)], umi.BatchParams(radius, 1.5, 0.2, 0, 0),
             [i % umi.batch_fused_variants(umi.OP_BILATERAL) for i in range(len(sizes))]),
            (umi.OP_WFILTER_PP, list(zip(dx, dw, outs_w)), None, None)]
    g = umi.BatchGraph()
    g.add_fused(jobs)
    for _ in range(2):
        for o in outs_b + outs_w:
            o.fill_(-7.0)
        g.launch()
        torch.cuda.synchronize()
        _fused_check(outs_b, outs_w, [], xs, ws, [], [], want_b, want_w, [], radius)
    g.close()


def test_batch_fused_autotune_per_size_class(umi, dev, tmp_path, monkeypatch):
    """The autotuner picks one variant per operator and size class and fills
    every image's variant from its class."""
    import torch
    from umi_gb300 import autotune
    monkeypatch.setenv("UMI_AUTOTUNE_CACHE", str(tmp_path / "cache.json"))
    sizes = [(64, 64), (700, 600), (1100, 1000), (100, 90)]
    ins = [torch.rand(s, device=dev) for s in sizes]
    wts = [torch.rand(s + (3, 3), device=dev) for s in sizes]
    outs = [torch.empty(s, device=dev) for s in sizes]
    jobs = [(umi.OP_BILATERAL, [(i, None, o) for i, o in zip(ins, outs)], umi.BatchParams(2, 2.0, 0.1, 0, 0), None),
            (umi.OP_WFILTER_PP, list(zip(ins, wts, outs)), None, None)]
    tuned, report = autotune.tuned_fused_variants(jobs, reps=1)
    assert set(report) == {"bilateral", "wfilter_pp"}
    for (op, imgs, _, var), name in zip(tuned, ("bilateral", "wfilter_pp")):
        assert len(var) == len(imgs)
        for (inp, _, _), v in zip(imgs, var):
            cls = autotune.image_class(*inp.shape)
            assert report[name][cls]["variant"] == v
            assert len(report[name][cls]["candidates_ms"]) == umi.batch_fused_variants(op)
    # a second call is served from the cache
    tuned2, report2 = autotune.tuned_fused_variants(jobs, reps=1)
    assert [j[3] for j in tuned2] == [j[3] for j in tuned]


def test_batch_fused_rejects(umi, dev):
    import torch
    x = torch.zeros((8, 8), device=dev)
    cv_bad = (umi.OP_COST_VOLUME, [(x.view(1, 8, 8), x.view(1, 8, 8), torch.zeros((8, 8, 32), device=dev))],
              umi.BatchParams(0, 0, 0, 1, 32), None)  # nd 32: not the tensor-core form
    with pytest.raises(umi.UmiError) as e:
        umi.batch_run_fused([cv_bad])
    assert e.value.status == 3
    job = (umi.OP_BILATERAL, [(x, None, x.clone())], umi.BatchParams(2, 2.0, 0.1, 0, 0), None)
    with pytest.raises(umi.UmiError):
        umi.batch_run_fused([job, job])  # two jobs of one operator
    with pytest.raises(umi.UmiError):
        umi.batch_run_fused([(umi.OP_BILATERAL, [(x, None, x.clone())], umi.BatchParams(2, 2.0, 0.1, 0, 0), [9])])
