"""GPU checks of the coarse motion proposal through the C ABI: the proposal
centres bit-exact against the oracle (ragged and maximum ranges, unaligned
views that take the byte-load path, the 1080p and 4K workloads), the refine /
audit / fallback composition of umi_me_coarse_u8, and argument rejection."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _t(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


@pytest.mark.parametrize("h,w,rng", [(16, 16, 0), (32, 48, 6), (48, 32, 10), (64, 96, 60), (96, 160, 62),
                                     (80, 48, 2), (128, 256, 30), (272, 1040, 60)])
def test_coarse_centers_random(umi, orc, dev, h, w, rng):
    g = np.random.default_rng(h * 7 + w + rng)
    cur = g.integers(0, 256, (h, w), dtype=np.uint8)
    ref = g.integers(0, 256, (h, w), dtype=np.uint8)
    got = umi.CoarseMe(h, w, device=dev).centers(_t(cur, dev), _t(ref, dev), rng).cpu().numpy()
    assert np.array_equal(got, orc.coarse_centers_u8(cur, ref, rng))


def test_coarse_centers_flat_frames_tie_to_first(umi, orc, dev):
    # every displacement ties: the first in raster order, (-range, -range)
    cur = np.full((64, 64), 9, np.uint8)
    ref = np.full((64, 64), 200, np.uint8)
    got = umi.CoarseMe(64, 64, device=dev).centers(_t(cur, dev), _t(ref, dev), 20).cpu().numpy()
    assert np.all(got == -20)
    assert np.array_equal(got, orc.coarse_centers_u8(cur, ref, 20))


def test_coarse_centers_unaligned_views(umi, orc, dev):
    import torch
    h, w = 48, 80
    g = np.random.default_rng(3)
    cur = g.integers(0, 256, (h, w), dtype=np.uint8)
    ref = g.integers(0, 256, (h, w), dtype=np.uint8)
    bc = torch.zeros(h * w + 1, dtype=torch.uint8, device=dev)
    br = torch.zeros(h * w + 3, dtype=torch.uint8, device=dev)
    bc[1:] = _t(cur.ravel(), dev)
    br[3:] = _t(ref.ravel(), dev)
    got = umi.CoarseMe(h, w, device=dev).centers(bc[1:].view(h, w), br[3:].view(h, w), 14).cpu().numpy()
    assert np.array_equal(got, orc.coarse_centers_u8(cur, ref, 14))


def test_coarse_centers_1080p_workload(umi, orc, dev):
    from umi_gb300 import workloads
    cur, ref, true_mv = workloads.me_pair(seed=4, h=1072, w=1920, shift_sigma=16.0, max_shift=64)
    got = umi.CoarseMe(1072, 1920, device=dev).centers(_t(cur, dev), _t(ref, dev), 60).cpu().numpy()
    assert np.array_equal(got, orc.coarse_centers_u8(cur, ref, 60))
    assert np.mean(np.all(np.abs(got - np.clip(true_mv, -60, 60)) <= 4, axis=1)) > 0.95


def test_coarse_centers_4k_workload(umi, orc, dev):
    from umi_gb300.workloads import me_pair_cuda
    cur, ref, _ = me_pair_cuda(77, 2160, 3840, device=dev)
    got = umi.CoarseMe(2160, 3840, device=dev).centers(cur, ref, 60).cpu().numpy()
    assert np.array_equal(got, orc.coarse_centers_u8(cur.cpu().numpy(), ref.cpu().numpy(), 60))


def test_coarse_entry_refine_audit_fallback(umi, dev):
    import torch
    from umi_gb300.workloads import me_pair
    h, w = 192, 256
    cur, ref, _ = me_pair(seed=6, h=h, w=w, shift_sigma=12.0, max_shift=30)
    c, r = _t(cur, dev), _t(ref, dev)
    nblk = (h // 16) * (w // 16)
    cme = umi.CoarseMe(h, w, device=dev)
    full_r, refine_r = 31, 4
    centers = cme.centers(c, r, (full_r - refine_r) & ~1)
    refined = umi.full_me_u8(c, r, 16, refine_r, centers=centers)
    full = umi.full_me_u8(c, r, 16, full_r)
    mv, sums, nf = cme.estimate(c, r, refine_r, full_r, sad_threshold=(1 << 31) - 1, audit_stride=0)
    assert torch.equal(mv, refined) and int(nf.item()) == 0
    mv, sums, nf = cme.estimate(c, r, refine_r, full_r, sad_threshold=-1, audit_stride=0)
    assert torch.equal(mv, full) and int(nf.item()) == nblk
    thr = int(refined[:, 2].float().quantile(0.9).item())
    mv, sums, nf = cme.estimate(c, r, refine_r, full_r, sad_threshold=thr, audit_stride=7)
    mv, refined_np, full_np = mv.cpu().numpy(), refined.cpu().numpy(), full.cpu().numpy()
    aud = np.arange(0, nblk, 7)
    assert np.array_equal(mv[aud], full_np[aud])
    s = sums.cpu().numpy()
    assert s[0] == refined_np[aud, 2].sum() and s[1] == full_np[aud, 2].sum()
    rest = np.setdiff1d(np.arange(nblk), aud)
    fb = rest[refined_np[rest, 2] > thr]
    keep = rest[refined_np[rest, 2] <= thr]
    assert int(nf.item()) == fb.size
    assert np.array_equal(mv[fb], full_np[fb]) and np.array_equal(mv[keep], refined_np[keep])
    # the proposal holds the optimum for nearly every block of this pair
    assert np.mean(refined_np[:, 2] == full_np[:, 2]) > 0.9


def _estimate_into(cme, c, r, outs, stride):
    cme.estimate(c, r, 4, 31, sad_threshold=450, audit_stride=stride, out=outs[0], audit_sums=outs[1],
                 n_fallback=outs[2])


@pytest.mark.parametrize("h,w,stride", [(192, 256, 5), (384, 512, 3)])
def test_coarse_audit_stream_fork_eager_graph_and_fresh_thread(umi, dev, h, w, stride):
    """An audit of fewer blocks than SMs (39 here) joins the fallback
    blocks' list search; a larger one (256) runs on the calling thread's
    second stream, forked and joined inside the call.  The results are the
    same eagerly, replayed from a CUDA graph that captured the call, and when
    the first call of a fresh host thread is itself captured (no second
    stream yet: everything in order on the captured stream)."""
    import threading

    import torch
    from umi_gb300.workloads import me_pair
    cur, ref, _ = me_pair(seed=9, h=h, w=w, shift_sigma=12.0, max_shift=30)
    c, r = _t(cur, dev), _t(ref, dev)
    nblk = (h // 16) * (w // 16)
    cme = umi.CoarseMe(h, w, device=dev)

    def outs():
        return (torch.empty((nblk, 3), dtype=torch.int32, device=dev), torch.zeros(2, dtype=torch.int64, device=dev),
                torch.zeros(1, dtype=torch.int32, device=dev))

    # the definition, from the separate calls
    full = umi.full_me_u8(c, r, 16, 31)
    refined = umi.full_me_u8(c, r, 16, 4, centers=cme.centers(c, r, 26))
    aud = torch.arange(0, nblk, stride, device=dev)
    want = refined.clone()
    rest = torch.ones(nblk, dtype=torch.bool, device=dev)
    rest[aud] = False
    fb = rest & (refined[:, 2] > 450)
    want[fb] = full[fb]
    want[aud] = full[aud]
    want_sums = [int(refined[aud, 2].sum()), int(full[aud, 2].sum())]
    want_nf = int(fb.sum())

    def check(o):
        assert torch.equal(o[0], want)
        assert o[1].tolist() == want_sums and int(o[2].item()) == want_nf

    eager = outs()
    _estimate_into(cme, c, r, eager, stride)
    torch.cuda.synchronize()
    check(eager)

    graphed = outs()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        _estimate_into(cme, c, r, graphed, stride)
    for _ in range(2):
        g.replay()
    torch.cuda.synchronize()
    check(graphed)

    result, errors = {}, []

    def fresh_thread():
        try:
            torch.cuda.set_device(dev)
            o = outs()
            g2 = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g2):
                _estimate_into(cme, c, r, o, stride)  # this thread's first call: captured in order
            g2.replay()
            o2 = outs()
            _estimate_into(cme, c, r, o2, stride)  # eager: the thread's second stream is made now
            torch.cuda.synchronize()
            result["captured"], result["eager"] = o, o2
        except Exception as e:  # surfaced below
            errors.append(e)

    t = threading.Thread(target=fresh_thread)
    t.start()
    t.join()
    assert not errors, errors
    check(result["captured"])
    check(result["eager"])


def test_coarse_rejects(umi, dev):
    import torch
    assert umi.lib().umi_me_coarse_workspace_bytes(100, 64) == 0
    assert umi.lib().umi_me_coarse_workspace_bytes(0, 64) == 0
    cme = umi.CoarseMe(64, 64, device=dev)
    z = torch.zeros((64, 64), dtype=torch.uint8, device=dev)
    for rng in (-2, 3, 64):
        with pytest.raises(umi.UmiError, match="UNSUPPORTED"):
            cme.centers(z, z, rng)
    with pytest.raises(umi.UmiError, match="UNSUPPORTED"):
        cme.estimate(z, z, refine_r=4, full_r=65)
    with pytest.raises(umi.UmiError, match="INVALID_ARG"):
        cme.estimate(z, z, audit_stride=-1)
    cme.ws = cme.ws[:64]
    with pytest.raises(umi.UmiError, match="NO_MEMORY"):
        cme.centers(z, z, 4)
