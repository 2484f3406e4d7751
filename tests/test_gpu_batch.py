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
