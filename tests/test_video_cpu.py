"""The YUV4MPEG2 frame reader / writer (umi_gb300/video.py) on CPU: round
trips in every supported layout, header and frame-line parameters, odd sizes
(chroma rounding), and the errors a malformed file must raise."""
import numpy as np
import pytest

from umi_gb300 import video


def _frames(n, h, w, seed=0):
    g = np.random.default_rng(seed)
    return [g.integers(0, 256, (h, w), dtype=np.uint8) for _ in range(n)]


@pytest.mark.parametrize("cs", ["mono", "420jpeg", "420", "420paldv", "420mpeg2", "422", "444"])
@pytest.mark.parametrize("h,w", [(21, 37), (16, 16), (1, 1), (48, 64)])
def test_round_trip(tmp_path, cs, h, w):
    fr = _frames(3, h, w, seed=h + w)
    p = str(tmp_path / "a.y4m")
    video.write_y4m(p, fr, fps=(25, 1), colorspace=cs)
    with video.Y4MReader(p) as r:
        assert (r.width, r.height, r.fps, r.colorspace, len(r)) == (w, h, (25, 1), cs, 3)
        c = {"mono": 0, "422": 2 * ((w + 1) // 2) * h, "444": 2 * w * h}.get(cs, 2 * ((w + 1) // 2) * ((h + 1) // 2))
        assert r.frame_bytes == w * h + c
        for i, f in enumerate(r):
            assert np.array_equal(f, fr[i])
        assert np.array_equal(r.luma(1), fr[1])
        with pytest.raises(IndexError):
            r.luma(3)


def test_header_and_frame_parameters(tmp_path):
    # tags in any order, unknown and comment tags, no C tag (4:2:0), parameters on FRAME lines
    h, w = 6, 10
    fr = _frames(2, h, w, seed=4)
    chroma = bytes([128]) * (2 * 5 * 3)
    data = b"YUV4MPEG2 F30000:1001 Ib H6 A0:0 XYSCSS=420JPEG W10 XCOLORRANGE=FULL\n"
    data += b"FRAME Ixyz XFOO=1\n" + fr[0].tobytes() + chroma
    data += b"FRAME\n" + fr[1].tobytes() + chroma
    p = tmp_path / "b.y4m"
    p.write_bytes(data)
    with video.Y4MReader(str(p)) as r:
        assert (r.width, r.height, r.fps, r.colorspace, len(r)) == (10, 6, (30000, 1001), "420jpeg", 2)
        assert np.array_equal(r.luma(0), fr[0]) and np.array_equal(r.luma(1), fr[1])


def test_empty_video_has_no_frames(tmp_path):
    p = tmp_path / "c.y4m"
    p.write_bytes(b"YUV4MPEG2 W8 H8 Cmono\n")
    with video.Y4MReader(str(p)) as r:
        assert len(r) == 0 and list(r) == []


@pytest.mark.parametrize("data,msg", [
    (b"RIFF....WAVEfmt \n", "not a YUV4MPEG2"),
    (b"YUV4MPEG2 W8 Cmono\n", "without W and H"),
    (b"YUV4MPEG2 W0 H8 Cmono\n", "frame size"),
    (b"YUV4MPEG2 W8 H8 C420p10\n", "not supported"),
    (b"YUV4MPEG2 W8 H8 Cmono\nFRAME\n" + bytes(63), "truncated"),
    (b"YUV4MPEG2 W8 H8 Cmono\nFRAME\n" + bytes(64) + b"FRAMX\n" + bytes(64), "missing FRAME"),
    (b"YUV4MPEG2 W8 H8 Cmono\nFRAME", "unterminated"),
])
def test_malformed_files_are_rejected(tmp_path, data, msg):
    p = tmp_path / "d.y4m"
    p.write_bytes(data)
    with pytest.raises(video.Y4MError, match=msg):
        video.Y4MReader(str(p))


def test_writer_rejects_mixed_sizes(tmp_path):
    with pytest.raises(video.Y4MError):
        video.write_y4m(str(tmp_path / "e.y4m"), [np.zeros((4, 4), np.uint8), np.zeros((4, 5), np.uint8)])


def test_pipeline_rejects_tiny_frames():
    with pytest.raises(ValueError):
        video.MotionPipeline(8, 64, method="coarse", device="cpu")
    with pytest.raises(ValueError):
        video.MotionPipeline(64, 64, method="nearest", device="cpu")
