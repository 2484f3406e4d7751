"""Frame-pair I/O for motion estimation over real video.

The reference has no I/O: its examples build frames in memory.  This module
reads YUV4MPEG2 ("Y4M") files -- the plain uncompressed container that video
tools write (a text header line, then per frame a "FRAME" line and the raw
planes) -- and runs the motion estimators of this package over consecutive
frame pairs with the frames streamed to the GPU.

* ``Y4MReader``: header parsing, a frame index built once, and the luma plane
  of any frame as a zero-copy view into a memory map of the file.
* ``write_y4m``: the inverse, for 8-bit luma frames (chroma planes written as
  mid-grey for the 4:2:x and 4:4:4 layouts).
* ``MotionPipeline``: pair i = (frame i, frame i - 1) as (cur, ref) through
  ``full_me_u8``, ``CoarseMe.estimate`` or ``MeNet.estimate``; uploads,
  compute and downloads run on three CUDA streams with a ring of device
  frames, so reading and copying the next frames overlaps the search of this
  pair.

Only 8-bit layouts are read (mono, 4:2:0 in any siting, 4:2:2, 4:4:4);
high-bit-depth files are rejected.
"""
from __future__ import annotations

import mmap
import os

import numpy as np

MAGIC = b"YUV4MPEG2"

# chroma plane sizes (width, height) for a luma plane of w x h, per colour space tag
_CHROMA = {
    "mono": lambda w, h: None,
    "420": lambda w, h: ((w + 1) // 2, (h + 1) // 2),
    "420jpeg": lambda w, h: ((w + 1) // 2, (h + 1) // 2),
    "420paldv": lambda w, h: ((w + 1) // 2, (h + 1) // 2),
    "420mpeg2": lambda w, h: ((w + 1) // 2, (h + 1) // 2),
    "422": lambda w, h: ((w + 1) // 2, h),
    "444": lambda w, h: (w, h),
}


class Y4MError(ValueError):
    pass


def _parse_params(tokens):
    out = {}
    for t in tokens:
        if not t:
            continue
        out.setdefault(t[:1], t[1:])
    return out


class Y4MReader:
    """Random access to the luma planes of a YUV4MPEG2 file.

    Attributes: ``width``, ``height``, ``fps`` (numerator, denominator),
    ``colorspace`` (the C tag, "420jpeg" when absent), ``frame_bytes`` (all
    planes of one frame) and ``len(reader)`` frames."""

    def __init__(self, path: str):
        self.path = path
        self._f = open(path, "rb")
        size = os.fstat(self._f.fileno()).st_size
        if size < len(MAGIC) + 1:
            self._f.close()
            raise Y4MError(f"{path}: not a YUV4MPEG2 file")
        self._mm = mmap.mmap(self._f.fileno(), 0, access=mmap.ACCESS_READ)
        try:
            self._parse(size)
        except Exception:
            self.close()
            raise

    def _parse(self, size):
        mm = self._mm
        end = mm.find(b"\n")
        if end < 0 or not mm[:end].startswith(MAGIC + b" "):
            raise Y4MError(f"{self.path}: not a YUV4MPEG2 file")
        p = _parse_params(mm[len(MAGIC) + 1:end].decode("ascii", "replace").split(" "))
        try:
            self.width, self.height = int(p["W"]), int(p["H"])
        except (KeyError, ValueError):
            raise Y4MError(f"{self.path}: header without W and H") from None
        if self.width <= 0 or self.height <= 0:
            raise Y4MError(f"{self.path}: frame size {self.width}x{self.height}")
        num, _, den = p.get("F", "30:1").partition(":")
        self.fps = (int(num or 30), int(den or 1))
        self.colorspace = p.get("C", "420jpeg")
        if self.colorspace not in _CHROMA:
            raise Y4MError(f"{self.path}: colour space C{self.colorspace} not supported (8-bit layouts only)")
        c = _CHROMA[self.colorspace](self.width, self.height)
        self.frame_bytes = self.width * self.height + (2 * c[0] * c[1] if c else 0)
        # frame index: offsets of the luma planes
        offs = []
        pos = end + 1
        while pos < size:
            if mm[pos:pos + 5] != b"FRAME":
                raise Y4MError(f"{self.path}: frame {len(offs)}: missing FRAME marker at byte {pos}")
            nl = mm.find(b"\n", pos)
            if nl < 0:
                raise Y4MError(f"{self.path}: frame {len(offs)}: unterminated FRAME line")
            data = nl + 1
            if data + self.frame_bytes > size:
                raise Y4MError(f"{self.path}: frame {len(offs)} truncated")
            offs.append(data)
            pos = data + self.frame_bytes
        self._offsets = offs

    def __len__(self):
        return len(self._offsets)

    def luma(self, i: int) -> np.ndarray:
        """The (height, width) uint8 luma plane of frame i: a read-only view
        into the memory map (valid until ``close``)."""
        if not 0 <= i < len(self._offsets):
            raise IndexError(f"frame {i} of {len(self._offsets)}")
        return np.frombuffer(self._mm, dtype=np.uint8, count=self.width * self.height,
                             offset=self._offsets[i]).reshape(self.height, self.width)

    def __iter__(self):
        for i in range(len(self)):
            yield self.luma(i)

    def close(self):
        mm, self._mm = getattr(self, "_mm", None), None
        if mm is not None:
            try:
                mm.close()
            except BufferError:
                pass  # views still alive: the map closes when they go
        f, self._f = getattr(self, "_f", None), None
        if f is not None:
            f.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def write_y4m(path: str, frames, fps=(30, 1), colorspace: str = "mono") -> None:
    """Writes 8-bit (h, w) luma frames as a YUV4MPEG2 file (progressive,
    square pixels); chroma planes, where the layout has them, are 128."""
    if colorspace not in _CHROMA:
        raise Y4MError(f"colour space C{colorspace} not supported")
    frames = [np.ascontiguousarray(f, dtype=np.uint8) for f in frames]
    if not frames:
        raise Y4MError("no frames")
    h, w = frames[0].shape
    c = _CHROMA[colorspace](w, h)
    chroma = np.full(2 * c[0] * c[1], 128, np.uint8).tobytes() if c else b""
    with open(path, "wb") as f:
        f.write(f"YUV4MPEG2 W{w} H{h} F{fps[0]}:{fps[1]} Ip A1:1 C{colorspace}\n".encode("ascii"))
        for fr in frames:
            if fr.shape != (h, w):
                raise Y4MError(f"frame of shape {fr.shape}, expected {(h, w)}")
            f.write(b"FRAME\n")
            f.write(fr.tobytes())
            f.write(chroma)


class MotionPipeline:
    """Motion estimation over consecutive frames: pair i = (frame i, frame
    i - 1) as (cur, ref), 16x16 blocks, for i = 1, 2, ...

    method "full": ``full_me_u8`` (+-search, any frame size); "coarse":
    ``CoarseMe.estimate`` and "learned": ``MeNet.estimate`` (refine +-refine,
    judge and fallback +-search, audit every audit_stride-th block); these two
    need multiples of 16, so frames are cropped to the largest such size.
    sad_threshold None: calibrated on the first pair as 1.2 x the 99th
    percentile of its exhaustive SADs.

    ``run(frames)`` takes an iterable of (h, w) uint8 frames (``Y4MReader``
    views or arrays) and yields (i, mv) with mv an (nblk, 3) int32 array
    (mv_y, mv_x, sad), in order.  Frames are copied into a ring of ``depth``
    pinned buffers and uploaded on their own stream; the search runs on the
    current stream; vectors come back on a third stream.  ``stats`` holds the
    pairs done, fallback blocks and audit sums (refined, exhaustive)."""

    METHODS = ("full", "coarse", "learned")

    def __init__(self, height: int, width: int, method: str = "coarse", search: int = 64, refine: int = 4,
                 sad_threshold: int | None = None, audit_stride: int = 64, depth: int = 3, device="cuda",
                 params=None):
        import torch
        import umi_gb300 as U
        if method not in self.METHODS:
            raise ValueError(f"method {method!r}: one of {self.METHODS}")
        self.U, self.method, self.search, self.refine = U, method, search, refine
        self.audit_stride, self.sad_threshold = audit_stride, sad_threshold
        self.device = torch.device(device)
        if method == "full":
            self.h, self.w = height, width
        else:
            self.h, self.w = height - height % 16, width - width % 16
        if self.h < 16 or self.w < 16:
            raise ValueError(f"frame {height}x{width} smaller than one 16x16 block")
        self.nblk = (self.h // 16) * (self.w // 16)
        self.depth = D = max(3, int(depth))
        dev = self.device
        self.dframes = [torch.empty((self.h, self.w), dtype=torch.uint8, device=dev) for _ in range(D)]
        self.dmv = [torch.empty((self.nblk, 3), dtype=torch.int32, device=dev) for _ in range(D)]
        self.dsums = [torch.zeros(2, dtype=torch.int64, device=dev) for _ in range(D)]
        self.dnf = [torch.zeros(1, dtype=torch.int32, device=dev) for _ in range(D)]
        self.up = [torch.empty((self.h, self.w), dtype=torch.uint8).pin_memory() for _ in range(D)]
        self.up_np = [t.numpy() for t in self.up]
        self.down = [torch.empty((self.nblk, 3), dtype=torch.int32).pin_memory() for _ in range(D)]
        self.down_stats = [torch.zeros(3, dtype=torch.int64).pin_memory() for _ in range(D)]
        self.dstats = [torch.zeros(3, dtype=torch.int64, device=dev) for _ in range(D)]
        self.s_in, self.s_out = torch.cuda.Stream(device=dev), torch.cuda.Stream(device=dev)
        if method == "coarse":
            self.est = U.CoarseMe(self.h, self.w, device=dev)
        elif method == "learned":
            if params is None:
                from umi_gb300 import menet_train
                params = menet_train.default_weights()
            self.est = U.MeNet(self.h, self.w, device=dev, params=params)
        self.stats = {"pairs": 0, "fallback_blocks": 0, "audit_refined_sad": 0, "audit_exhaustive_sad": 0}

    def _calibrate(self, cur, ref):
        import torch
        from umi_gb300.menet_train import threshold_from
        full = self.U.full_me_u8(cur, ref, 16, self.search)
        torch.cuda.current_stream().synchronize()
        self.sad_threshold = threshold_from(full)

    def _estimate(self, cur, ref, m):
        if self.method == "full":
            self.U.full_me_u8(cur, ref, 16, self.search, out=self.dmv[m])
            return
        if self.sad_threshold is None:
            self._calibrate(cur, ref)
        self.est.estimate(cur, ref, self.refine, self.search, self.sad_threshold, self.audit_stride,
                          out=self.dmv[m], audit_sums=self.dsums[m], n_fallback=self.dnf[m])
        st = self.dstats[m]
        st[0:1].copy_(self.dnf[m])
        st[1:3].copy_(self.dsums[m])

    def run(self, frames):
        """Yields (i, mv) for pairs i = 1, 2, ... of the frames, in order."""
        import collections

        import torch
        D = self.depth
        s_c = torch.cuda.current_stream(self.device)
        up_done = [None] * D   # H2D out of pinned slot k finished
        used = [None] * D      # last search reading device frame k finished
        mv_free = [None] * D   # D2H out of device vector slot m finished
        pending = collections.deque()  # (pair, slot, download event)

        def drain(keep):
            while len(pending) > keep:
                i, m, ev = pending.popleft()
                ev.synchronize()
                if self.method != "full":
                    st = self.down_stats[m].numpy()
                    self.stats["fallback_blocks"] += int(st[0])
                    self.stats["audit_refined_sad"] += int(st[1])
                    self.stats["audit_exhaustive_sad"] += int(st[2])
                self.stats["pairs"] += 1
                yield i, self.down[m].numpy().copy()

        for i, fr in enumerate(frames):
            k = i % D
            fr = np.asarray(fr)
            if fr.ndim != 2 or fr.dtype != np.uint8 or fr.shape[0] < self.h or fr.shape[1] < self.w:
                raise ValueError(f"frame {i}: expected uint8 of at least {self.h}x{self.w}, got {fr.dtype} {fr.shape}")
            if up_done[k] is not None:
                up_done[k].synchronize()  # the pinned slot's previous upload has left it
            np.copyto(self.up_np[k], fr[:self.h, :self.w])
            with torch.cuda.stream(self.s_in):
                if used[k] is not None:
                    self.s_in.wait_event(used[k])  # the device frame it replaces is no longer read
                self.dframes[k].copy_(self.up[k], non_blocking=True)
                e_in = torch.cuda.Event()
                e_in.record(self.s_in)
                up_done[k] = e_in
            if i == 0:
                continue
            kp, m = (i - 1) % D, i % D
            s_c.wait_event(up_done[k])
            s_c.wait_event(up_done[kp])
            if mv_free[m] is not None:
                s_c.wait_event(mv_free[m])
            self._estimate(self.dframes[k], self.dframes[kp], m)
            e_c = torch.cuda.Event()
            e_c.record(s_c)
            used[k] = used[kp] = e_c
            yield from drain(D - 2)  # the host slot about to be written is free
            with torch.cuda.stream(self.s_out):
                self.s_out.wait_event(e_c)
                self.down[m].copy_(self.dmv[m], non_blocking=True)
                if self.method != "full":
                    self.down_stats[m].copy_(self.dstats[m], non_blocking=True)
                e_o = torch.cuda.Event()
                e_o.record(self.s_out)
                mv_free[m] = e_o
            pending.append((i, m, e_o))
        yield from drain(0)


def estimate_video(path: str, method: str = "coarse", max_frames: int | None = None, **kw):
    """Motion vectors of every consecutive frame pair of a Y4M file: a list of
    (nblk, 3) int32 arrays, pair i at index i - 1 (``MotionPipeline`` options
    in kw)."""
    with Y4MReader(path) as r:
        n = len(r) if max_frames is None else min(len(r), max_frames)
        pipe = MotionPipeline(r.height, r.width, method=method, **kw)
        out = [mv for _, mv in pipe.run(r.luma(i) for i in range(n))]
    return out
