"""GPU checks of the frame-pair pipeline (umi_gb300/video.py): for every
method its streamed results equal the per-pair calls of the same estimator on
the same (cropped) frames, read from a Y4M file or from arrays, with short and
long videos against the ring depth; and the planted pan is recovered."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _t(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def _video(n, h, w, seed=5, velocity=(3, -5)):
    from umi_gb300 import workloads
    return workloads.video_frames(seed=seed, n=n, h=h, w=w, velocity=velocity)


@pytest.mark.parametrize("n,depth", [(2, 3), (7, 3), (9, 4)])
def test_full_search_pipeline_matches_pairs(umi, orc, dev, n, depth):
    from umi_gb300 import video
    fr = _video(n, 70, 100)  # not multiples of 16: the full search takes the whole frame
    pipe = video.MotionPipeline(70, 100, method="full", search=12, depth=depth, device=dev)
    got = list(pipe.run(fr))
    assert [i for i, _ in got] == list(range(1, n))
    for i, mv in got:
        assert np.array_equal(mv, orc.full_me_u8(fr[i], fr[i - 1], 16, 12)), i
        inner = mv.reshape(4, 6, 3)[1:-1, 1:-1]  # blocks whose match lies inside the frame
        assert np.mean((inner[..., 0] == 3) & (inner[..., 1] == -5)) >= 0.75  # noise moves a few optima
    assert pipe.stats["pairs"] == n - 1


@pytest.mark.parametrize("method", ["coarse", "learned"])
def test_proposal_pipelines_match_pairs(umi, dev, method):
    import torch
    from umi_gb300 import video
    n, h, w = 6, 150, 290  # cropped to 144 x 288
    fr = _video(n, h, w, seed=8, velocity=(-7, 11))
    pipe = video.MotionPipeline(h, w, method=method, search=24, refine=4, audit_stride=5, device=dev)
    got = list(pipe.run(fr))
    thr = pipe.sad_threshold
    assert thr is not None and (pipe.h, pipe.w) == (144, 288)
    est = umi.CoarseMe(144, 288, device=dev) if method == "coarse" else \
        umi.MeNet(144, 288, device=dev, params=pipe.est.params.cpu().numpy())
    fb = 0
    for i, mv in got:
        c, r = _t(fr[i][:144, :288], dev), _t(fr[i - 1][:144, :288], dev)
        want, sums, nf = est.estimate(c, r, 4, 24, thr, 5)
        assert np.array_equal(mv, want.cpu().numpy()), (method, i)
        fb += int(nf.item())
    assert pipe.stats["pairs"] == n - 1 and pipe.stats["fallback_blocks"] == fb
    if method == "coarse":
        inner = got[-1][1].reshape(9, 18, 3)[1:-1, 1:-1]
        assert np.mean((inner[..., 0] == -7) & (inner[..., 1] == 11)) >= 0.9
    torch.cuda.synchronize()


def test_y4m_file_through_the_pipeline(umi, orc, dev, tmp_path):
    from umi_gb300 import video
    fr = _video(5, 64, 96, seed=2)
    p = str(tmp_path / "v.y4m")
    video.write_y4m(p, fr, colorspace="420jpeg")
    mvs = video.estimate_video(p, method="full", search=8, device=dev)
    assert len(mvs) == 4
    for i, mv in enumerate(mvs, start=1):
        assert np.array_equal(mv, orc.full_me_u8(fr[i], fr[i - 1], 16, 8))
    assert len(video.estimate_video(p, method="coarse", search=16, max_frames=3, device=dev)) == 2


def test_pipeline_rejects_wrong_frames(umi, dev):
    from umi_gb300 import video
    pipe = video.MotionPipeline(64, 64, method="full", search=4, device=dev)
    with pytest.raises(ValueError):
        list(pipe.run([np.zeros((64, 64), np.uint8), np.zeros((32, 64), np.uint8)]))
    with pytest.raises(ValueError):
        list(pipe.run([np.zeros((64, 64), np.float32)]))
