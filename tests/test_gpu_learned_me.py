"""GPU checks of the learned motion proposal: the block-list search against
the oracle, the network's forward pass and hand-written backward kernels
against the FP64 oracle, the learned entry point's refine / audit /
fallback logic, and a short training run."""
import numpy as np
import pytest

from oracle import menet

pytestmark = pytest.mark.gpu


def _t(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def _params(seed):
    import umi_gb300
    g = np.random.default_rng(seed)
    p = umi_gb300.init_params(seed)
    layers, wh, bh, _ = menet.layout()
    p[wh:bh] = g.normal(0, 0.2, bh - wh)
    for _, bo in layers:
        p[bo:bo + menet.CH] = g.normal(0, 0.05, menet.CH)
    p[bh:bh + 2] = [0.3, -0.2]
    return p.astype(np.float32)


def test_full_me_list_matches_oracle(umi, orc, dev):
    import torch
    from umi_gb300.workloads import me_pair
    cur, ref, _ = me_pair(seed=21, h=160, w=224, shift_sigma=6.0, max_shift=20)
    nblk = (160 // 16) * (224 // 16)
    g = np.random.default_rng(4)
    blocks = g.choice(nblk, 37, replace=False).astype(np.int32)
    out = torch.full((nblk, 3), -7, dtype=torch.int32, device=dev)
    bl = torch.zeros(64, dtype=torch.int32, device=dev)
    bl[:37] = _t(blocks, dev)
    n = torch.tensor([37], dtype=torch.int32, device=dev)
    umi.full_me_u8_list(_t(cur, dev), _t(ref, dev), bl, n, out, 16, 24)
    got = out.cpu().numpy()
    want = orc.full_me_u8(cur, ref, 16, 24, blocks=blocks)
    assert np.array_equal(got[blocks], want)
    untouched = np.setdiff1d(np.arange(nblk), blocks)
    assert (got[untouched] == -7).all()
    # a zero-length list touches nothing
    out2 = torch.full((nblk, 3), -7, dtype=torch.int32, device=dev)
    umi.full_me_u8_list(_t(cur, dev), _t(ref, dev), bl, torch.zeros(1, dtype=torch.int32, device=dev), out2, 16, 24)
    assert (out2.cpu().numpy() == -7).all()


@pytest.mark.parametrize("shape", [(64, 96), (80, 144)])
def test_menet_forward_matches_oracle(umi, dev, shape):
    h, w = shape
    g = np.random.default_rng(h + w)
    cur = g.integers(0, 256, (h, w), dtype=np.uint8)
    ref = g.integers(0, 256, (h, w), dtype=np.uint8)
    p = _params(7)
    net = umi.MeNet(h, w, device=dev, params=p)
    got = net.forward(_t(cur, dev), _t(ref, dev)).cpu().numpy()
    want, _ = menet.forward(p, cur, ref, bf16=True)
    # fp32 accumulation of bf16 weights vs fp64: relative to the output scale
    scale = np.abs(want).max() + 1e-3
    assert np.abs(got - want).max() <= 2e-5 * scale + 1e-6, np.abs(got - want).max()


@pytest.mark.parametrize("shape", [(64, 96), (144, 528), (272, 1040)])
def test_menet_infer_matches_oracle(umi, dev, shape):
    """Tensor-core inference pass vs the FP64 oracle with bf16 activations.
    Shapes cover partial 128-pixel tiles, several tiles per row, and rows
    where the dilation-8 taps fall outside the image."""
    import torch
    h, w = shape
    g = np.random.default_rng(h * w)
    cur = g.integers(0, 256, (h, w), dtype=np.uint8)
    ref = g.integers(0, 256, (h, w), dtype=np.uint8)
    p = _params(5)
    net = umi.MeNet(h, w, device=dev, params=p)
    # every workspace byte 0xff (bf16 NaN): the pass must write every value it
    # reads (activations, packed weights, predictions)
    net.ws.fill_(0xFF)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    got = net.infer(_t(cur, dev), _t(ref, dev), err=err).cpu().numpy()
    assert int(err.item()) == 0
    want, _ = menet.forward(p, cur, ref, bf16=True, act_bf16=True)
    scale = np.abs(want).max() + 1e-3
    d = np.abs(got - want)
    # fp32 accumulation vs fp64 can move an activation across a bf16 rounding
    # boundary (2^-8 relative); such flips stay far below this bound
    assert d.max() <= 5e-3 * scale, (d.max(), scale)
    assert np.median(d) <= 1e-4 * scale
    # and the tensor-core pass agrees with the fp32 training pass to bf16 precision
    fp32 = net.forward(_t(cur, dev), _t(ref, dev)).cpu().numpy()
    assert np.abs(fp32 - got).max() <= 0.05 * scale


def test_menet_infer_4k_equals_cropped_frame(umi, dev):
    """At 4K each CTA of a tensor-core layer runs about 29 output rows, so
    its ring of sixteen accumulators wraps (the split MMAs); a 272 x 1040
    crop (a shape checked against the oracle above) runs two rows per CTA.
    A block at least 64 pixels from the crop's edges sees the same inputs
    in both (receptive field: 15 quarter-resolution pixels), and every
    output value is summed in the same order, so its prediction must be
    bit-identical."""
    import torch
    h, w = 2160, 3840
    g = np.random.default_rng(11)
    cur = g.integers(0, 256, (h, w), dtype=np.uint8)
    ref = g.integers(0, 256, (h, w), dtype=np.uint8)
    p = _params(7)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    net = umi.MeNet(h, w, device=dev, params=p)
    full = net.infer(_t(cur, dev), _t(ref, dev), err=err).cpu().numpy().reshape(h // 16, w // 16, 2)
    y0, x0, ch, cw = 1024, 1600, 272, 1040
    small = umi.MeNet(ch, cw, device=dev, params=p)
    crop = small.infer(_t(cur[y0:y0 + ch, x0:x0 + cw], dev), _t(ref[y0:y0 + ch, x0:x0 + cw], dev),
                       err=err).cpu().numpy().reshape(ch // 16, cw // 16, 2)
    assert int(err.item()) == 0
    m = 4  # blocks of margin: 64 pixels
    a = full[y0 // 16 + m:(y0 + ch) // 16 - m, x0 // 16 + m:(x0 + cw) // 16 - m]
    b = crop[m:-m, m:-m]
    assert a.shape == (9, 57, 2) and np.isfinite(a).all()
    assert np.array_equal(a, b), np.abs(a - b).max()


def test_menet_backward_matches_oracle(umi, dev):
    import torch
    h, w = 64, 96
    g = np.random.default_rng(11)
    cur = g.integers(0, 256, (h, w), dtype=np.uint8)
    ref = g.integers(0, 256, (h, w), dtype=np.uint8)
    p = _params(3)
    nblk = (h // 16) * (w // 16)
    tgt = np.zeros((nblk, 3), np.int32)
    tgt[:, :2] = g.integers(-40, 40, (nblk, 2))
    net = umi.MeNet(h, w, device=dev, params=p)
    net.forward(_t(cur, dev), _t(ref, dev))
    grads = net.backward(_t(tgt, dev), stride=3).cpu().numpy().astype(np.float64)
    loss = float(net.loss.item())
    want_loss, want = menet.loss_and_grad(p, cur, ref, tgt, bf16=True)
    assert abs(loss - want_loss) <= 1e-5 * abs(want_loss)
    layers, wh, bh, total = menet.layout()
    segs = [(wo, bo) for wo, bo in layers] + [(bo, bo + menet.CH) for _, bo in layers] + [(wh, bh), (bh, bh + 2)]
    for a, b in segs:
        gw, ww = grads[a:b], want[a:b]
        scale = np.abs(ww).max() + 1e-12
        # fp32 accumulation over up to 384 pixels x 32 channels x 9 taps
        assert np.abs(gw - ww).max() <= 1e-4 * scale, (a, b, np.abs(gw - ww).max(), scale)
    assert np.linalg.norm(grads - want) <= 1e-5 * np.linalg.norm(want)


def test_menet_rejects_bad_frames(umi, dev):
    import torch
    assert umi.lib().umi_menet_workspace_bytes(100, 64) == 0
    assert umi.lib().umi_menet_workspace_bytes(8, 64) == 0
    net = umi.MeNet(64, 64, device=dev)
    net.ws = net.ws[:16]  # workspace too small: rejected before any launch
    z = torch.zeros((64, 64), dtype=torch.uint8, device=dev)
    with pytest.raises(umi.UmiError, match="NO_MEMORY"):
        net.forward(z, z)
    with pytest.raises(umi.UmiError, match="UNSUPPORTED"):
        umi.MeNet(64, 64, device=dev).estimate(z, z, refine_r=4, full_r=65)


def test_learned_entry_refine_audit_fallback(umi, dev):
    import torch
    from umi_gb300.workloads import me_pair
    h, w = 192, 256
    cur, ref, _ = me_pair(seed=5, h=h, w=w, shift_sigma=8.0, max_shift=24)
    c, r = _t(cur, dev), _t(ref, dev)
    nblk = (h // 16) * (w // 16)
    net = umi.MeNet(h, w, device=dev, params=_params(9))
    pred = net.infer(c, r)  # the pass umi_me_learned_u8 runs
    full_r, refine_r = 24, 4
    centers = torch.clamp(torch.round(pred * 16), -(full_r - refine_r), full_r - refine_r).to(torch.int32).contiguous()
    refined = umi.full_me_u8(c, r, 16, refine_r, centers=centers)
    full = umi.full_me_u8(c, r, 16, full_r)
    # no fallback, no audit: exactly the refine around the predicted centres
    mv, sums, nf = net.estimate(c, r, refine_r, full_r, sad_threshold=(1 << 31) - 1, audit_stride=0)
    assert torch.equal(mv, refined) and int(nf.item()) == 0
    # every block falls back: exactly the exhaustive search
    mv, sums, nf = net.estimate(c, r, refine_r, full_r, sad_threshold=-1, audit_stride=0)
    assert torch.equal(mv, full) and int(nf.item()) == nblk
    # audit every 5th block; fallback above a threshold
    thr = int(refined[:, 2].float().median().item())
    mv, sums, nf = net.estimate(c, r, refine_r, full_r, sad_threshold=thr, audit_stride=5)
    mv, refined_np, full_np = mv.cpu().numpy(), refined.cpu().numpy(), full.cpu().numpy()
    aud = np.arange(0, nblk, 5)
    assert np.array_equal(mv[aud], full_np[aud])
    s = sums.cpu().numpy()
    assert s[0] == refined_np[aud, 2].sum() and s[1] == full_np[aud, 2].sum()
    rest = np.setdiff1d(np.arange(nblk), aud)
    fb = rest[refined_np[rest, 2] > thr]
    keep = rest[refined_np[rest, 2] <= thr]
    assert int(nf.item()) == fb.size
    assert np.array_equal(mv[fb], full_np[fb]) and np.array_equal(mv[keep], refined_np[keep])


def test_menet_training_reduces_loss(umi, dev):
    import torch
    from umi_gb300.workloads import me_pair_cuda
    h, w = 256, 320
    cur, ref, _ = me_pair_cuda(17, h, w, shift_sigma=6.0, max_shift=24, device=dev)
    labels = umi.full_me_u8(cur, ref, 16, 24)
    net = umi.MeNet(h, w, device=dev, seed=2)
    losses = []
    for _ in range(60):
        net.forward(cur, ref)
        net.backward(labels, stride=3)
        losses.append(float(net.loss.item()))
        net.adam(3e-3)
    assert all(np.isfinite(losses))
    assert np.mean(losses[-5:]) < 0.7 * np.mean(losses[:5]), losses


def test_trained_network_beats_zero_and_median_proposals(umi, dev):
    """What the trained network gains over the method without it, on held-out
    4K pairs of the benchmark distribution (seeds never used in training): the
    committed weights' proposal, refined +-4, holds the exhaustive optimum for
    more blocks than the zero-vector and the neighbour-median proposals with
    the same refine, and needs fewer fallback searches at the same threshold."""
    from umi_gb300 import menet_train as T
    net = umi.MeNet(2160, 3840, device=dev, params=T.default_weights())
    r = T.evaluate(net, [T.EVAL_SEED0 + 1], refine_r=4, full_r=64)
    learned, zero, median = r["learned"], r["zero"], r["median"]
    assert learned["hit"] > 1.5 * zero["hit"], r
    assert learned["hit"] > 1.5 * median["hit"], r
    assert learned["fallback_frac"] < zero["fallback_frac"] and learned["fallback_frac"] < median["fallback_frac"], r
    # the full entry point with audit and fallback stays within the 1 % SAD regression bound
    assert learned["entry_sad_reg"] <= 0.01, r
