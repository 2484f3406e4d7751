#!/usr/bin/env python
"""Benchmark of the UMI operator hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

Default workload `int_pair_1080p` (the integer-pair configuration): one step =
the integral image of a 1920x1080 uint8 frame (umi_iimg_u8_i32, on a second
stream) beside full-search motion estimation of a 1920x1080 uint8 pair,
16x16 blocks, +-32, fused argmin (umi_full_me_u8), joined every step.
Metric: full_me Mblocks/s (8040 blocks per step).  Other workloads: `filter3x3_1024` (1024x1024 float32, 3x3 N(0,1)
weights, zero pad; metric GB/s).

Prints ONE JSON line (rank 0).  `value` is timed with CUDA events around
exactly K steps on inputs already in HBM, rotating through enough input
copies that the working set of consecutive steps exceeds L2; `e2e` repeats
the K steps from pinned host buffers with the host->device copies and the
device->host read of every result inside the timed region (uploads, compute
and downloads on three streams, so neighbouring steps' copies overlap).  `--impl
reference` times the reference's CPU loops (restated in the oracle) on the
host cores instead.  With N > 1 (torchrun) every rank runs its own replica
(the operator has no exchange step) and the time is the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L2_BYTES = 129 * 2 ** 20
PEAKS_FALLBACK = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}
# (dram__bytes_read.sum, dram__bytes_write.sum) per launch of the dominant
# kernel, from the ncu captures summarised under profiles/ (None where not
# captured).  batched_uneven's fused launch was captured on its 4-image case
# (8 725 530 px): its traffic grows with the pixel count, so it is kept per
# pixel and scaled to the configured batch.
NCU_TRAFFIC = {"int_pair_1080p": (4178432, 0), "filter3x3_1024": (4204544, 0), "gemm_4096": (72876544, 36060160),
               "fprop_n32": (72234752, 207382784), "learned_me_4k": None,
               # the proposal: cells kernel (both frames read once) + coarse search (planes and cells)
               "coarse_me_4k": (16615680 + 2795520, 0),
               "video_y4m_1080p": None, "apps_1080p": None, "serve_bilateral_8x512": None}
NCU_TRAFFIC_PER_PX = {"batched_uneven": (2616474000 / 8725530, 2272248000 / 8725530)}


def traffic_fields(rw, alg_write_bytes=None):
    """`traffic` = DRAM read + write bytes per launch (ncu), with the two
    counters beside it.  dram__bytes_write counts only the lines written back
    to DRAM while the launch runs: an output that is still dirty in L2 when
    the kernel ends is not counted, so a write figure below the algorithmic
    output bytes is flagged instead of being read as saved traffic."""
    if rw is None:
        return {"traffic": None}
    r, w = rw
    d = {"traffic": r + w, "traffic_read": r, "traffic_write": w}
    if alg_write_bytes and w < 0.9 * alg_write_bytes:
        d["traffic_note"] = (f"dram__bytes_write {w:.0f} B < {alg_write_bytes:.0f} B of output: "
                             "the rest was still dirty in L2 at kernel end (written back after the launch)")
    return d


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["int_pair_1080p", "filter3x3_1024", "batched_uneven", "gemm_4096",
                                           "fprop_n32", "learned_me_4k", "coarse_me_4k", "video_y4m_1080p",
                                           "apps_1080p", "serve_bilateral_8x512"],
                    default="int_pair_1080p")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--images", type=int, default=64, help="batched_uneven: number of images (64 in the benchmark)")
    a = ap.parse_args()
    if a.steps is None:
        a.steps = {"int_pair_1080p": 2000, "filter3x3_1024": 200000, "batched_uneven": 100,
                   "gemm_4096": 3000, "fprop_n32": 3000, "learned_me_4k": 200, "coarse_me_4k": 2000,
                   "video_y4m_1080p": 2000, "apps_1080p": 500, "serve_bilateral_8x512": 2000}[a.workload]
    return a


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return {"hbm_gbs": float(d["hbm_gbs"]), "bf16_tflops": float(d["bf16_tflops"]), "source": "measured"}
    return dict(PEAKS_FALLBACK, source="fallback")


# --------------------------------------------------------------------- dist
class Dist:
    def __init__(self, backend: str):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group(backend=backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        dev = "cuda" if self.pg.get_backend() == "nccl" else "cpu"
        t = torch.tensor([v], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def done(self):
        if self.pg:
            self.pg.destroy_process_group()


# --------------------------------------------------------------------- clocks
class Clocks:
    """nvidia-smi sampling during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    NAMES = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, device_index: int):
        self.proc = None
        self.path = None
        try:
            import torch
            uuid = str(torch.cuda.get_device_properties(device_index).uuid)
            sel = uuid if uuid.startswith("GPU-") else f"GPU-{uuid}"
        except Exception:
            sel = str(device_index)
        self.sel = sel

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", self.sel, f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.15)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sms, mx, reasons = [], None, set()
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sms.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for name, v in zip(self.NAMES, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sms) if sms else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sms)}


# --------------------------------------------------------------------- workloads
class IntPair:
    """iimg of a 1920x1080 u8 frame + full_me (16x16, +-32, argmin) of a 1080p pair."""
    name = "int_pair_1080p"
    H, W, B, R = 1080, 1920, 16, 32
    metric = "full_me Mblocks/s"
    unit = "Mblocks/s"
    dtype = "u8"

    def __init__(self, seed=3):
        from umi_gb300 import workloads
        self.cur, self.ref, self.true_mv = workloads.me_pair(seed=seed, h=self.H, w=self.W, block=self.B)
        self.nblk = (self.H // self.B) * (self.W // self.B)

    def config(self):
        return {"workload": self.name, "frame": f"{self.W}x{self.H} u8", "block": self.B, "search": f"+-{self.R}",
                "argmin": "fused, first in raster order",
                "step": "iimg(cur) on a second stream beside full_me(cur, ref), joined every step",
                "l2": "rotating input copies, consecutive steps touch > L2"}

    def units_per_step(self):
        return self.nblk / 1e6

    # device side
    def setup(self, dev):
        import torch
        import umi_gb300 as U
        self.U = U
        per = 3 * self.H * self.W + 4 * self.H * self.W
        self.n_rot = max(2, -(-2 * L2_BYTES // per))
        c = torch.from_numpy(self.cur).to(dev)
        r = torch.from_numpy(self.ref).to(dev)
        self.d_cur = [c.clone() for _ in range(self.n_rot)]
        self.d_ref = [r.clone() for _ in range(self.n_rot)]
        self.d_ii = [torch.empty((self.H, self.W), dtype=torch.int32, device=dev) for _ in range(self.n_rot)]
        self.d_mv = [torch.empty((self.nblk, 3), dtype=torch.int32, device=dev) for _ in range(self.n_rot)]
        self.ws = torch.empty(U.iimg_workspace_bytes(self.H, self.W), dtype=torch.uint8, device=dev)
        # pinned host buffers for e2e
        self.h_cur = torch.from_numpy(self.cur).pin_memory()
        self.h_ref = torch.from_numpy(self.ref).pin_memory()
        self.h_ii = torch.empty((self.H, self.W), dtype=torch.int32).pin_memory()
        self.h_mv = torch.empty((self.nblk, 3), dtype=torch.int32).pin_memory()
        self.launches_per_step = 3  # iimg: 2 kernels (group column sums, output pass), full_me: 1
        self.side = torch.cuda.Stream(device=dev)

    def step(self, i):
        """The two operators are independent: the integral image (memory-latency
        bound) runs on a second stream beside the search (integer-ALU bound),
        both through the C ABI, joined before the step ends (the workspace
        and buffers of one step are not reused before the join)."""
        import torch
        k = i % self.n_rot
        cur = torch.cuda.current_stream()
        self.side.wait_stream(cur)
        with torch.cuda.stream(self.side):
            self.U.iimg_u8_i32(self.d_cur[k], out=self.d_ii[k], workspace=self.ws)
        self.U.full_me_u8(self.d_cur[k], self.d_ref[k], self.B, self.R, out=self.d_mv[k])
        cur.wait_stream(self.side)

    def h2d(self, k):
        self.d_cur[k].copy_(self.h_cur, non_blocking=True)
        self.d_ref[k].copy_(self.h_ref, non_blocking=True)

    def d2h(self, k):
        self.h_ii.copy_(self.d_ii[k], non_blocking=True)
        self.h_mv.copy_(self.d_mv[k], non_blocking=True)

    def e2e_bytes(self):
        return 2 * self.H * self.W, 4 * self.H * self.W + 12 * self.nblk

    def check(self):
        """Cheap correctness guard on the timed outputs (full check lives in tests)."""
        mv = self.d_mv[0].cpu().numpy()
        return float(np.mean(np.all(mv[:, :2] == self.true_mv, axis=1)))

    def kernels(self, dev, peaks, n=400):
        """Average launch duration of each kernel: n back-to-back launches
        (graph replay, rotating buffers) timed by CUDA events on the stream."""
        R = self.n_rot
        fns = {
            "full_me_u8": lambda i: self.U.full_me_u8(self.d_cur[i % R], self.d_ref[i % R], self.B, self.R,
                                                      out=self.d_mv[i % R]),
            "iimg_u8_i32": lambda i: self.U.iimg_u8_i32(self.d_cur[i % R], out=self.d_ii[i % R], workspace=self.ws),
        }
        out = {name: time_launches(fn, R, n) for name, fn in fns.items()}
        absdiff = self.nblk * (2 * self.R + 1) ** 2 * self.B * self.B
        iimg_bytes = 5 * self.H * self.W
        return out, absdiff, iimg_bytes

    # CPU reference arm / baseline
    def cpu_setup(self):
        import oracle
        self.orc = oracle
        self.rng = np.random.default_rng(0)

    def cpu_step(self, nblocks, threads):
        blocks = self.rng.choice(self.nblk, size=nblocks, replace=False).astype(np.int32)
        rows = max(1, round(self.H * nblocks / self.nblk))
        self.orc.ref_iimg_u8(self.cur[:rows])
        self.orc.ref_full_me_u8_argmin(self.cur, self.ref, self.B, self.R, blocks, threads=threads)
        return nblocks / 1e6


class Filter3x3:
    """1024x1024 float32, 3x3 N(0,1) weights, zero padding."""
    name = "filter3x3_1024"
    H = W = 1024
    metric = "filter3x3 GB/s"
    unit = "GB/s"
    dtype = "f32"

    def __init__(self, seed=1):
        from umi_gb300 import workloads
        self.img, self.w9 = workloads.filter_image(seed=seed, h=self.H, w=self.W)

    def config(self):
        return {"workload": self.name, "image": f"{self.W}x{self.H} f32", "weights": "3x3 N(0,1)", "pad": 0.0,
                "bytes_per_px": 8, "l2": "rotating input/output copies, consecutive steps touch > L2"}

    def units_per_step(self):
        return 8 * self.H * self.W / 1e9

    def setup(self, dev):
        import torch
        import umi_gb300 as U
        self.U = U
        per = 8 * self.H * self.W
        self.n_rot = max(2, -(-2 * L2_BYTES // per))
        x = torch.from_numpy(self.img).to(dev)
        self.d_in = [x.clone() for _ in range(self.n_rot)]
        self.d_out = [torch.empty_like(x) for _ in range(self.n_rot)]
        self.h_in = torch.from_numpy(self.img).pin_memory()
        self.h_out = torch.empty_like(self.h_in).pin_memory()
        self.launches_per_step = 1

    def step(self, i):
        k = i % self.n_rot
        self.U.filter3x3_f32(self.d_in[k], self.w9, out=self.d_out[k])

    def h2d(self, k):
        self.d_in[k].copy_(self.h_in, non_blocking=True)

    def d2h(self, k):
        self.h_out.copy_(self.d_out[k], non_blocking=True)

    def e2e_bytes(self):
        return 4 * self.H * self.W, 4 * self.H * self.W

    def check(self):
        return None

    def kernels(self, dev, peaks, n=2000):
        return {"filter3x3_f32": time_launches(self.step, self.n_rot, n)}, None, 8 * self.H * self.W

    def cpu_setup(self):
        import oracle
        self.orc = oracle

    def cpu_step(self, rows, threads):
        self.orc.filter3x3_f64(self.img[:rows], self.w9, threads=threads)
        return 8 * rows * self.W / 1e9


class Batched:
    """64 float images, H and W uniform in [256, 2048] (seeded), all three
    operators in ONE persistent launch per step (umi_batch_run_fused,
    captured in a CUDA graph): bilateral 5x5 (sigma_s 2, sigma_r 0.1),
    per-pixel-weight 3x3 filter (weights U[0,1)), dot-product cost volume
    (32-channel N(0,1) features, right = left shifted by a per-pixel disparity
    U{0..63} plus N(0, 0.1^2), 64 disparities).  The filters' variants (tile
    shape, pixels per thread) are autotuned per operator and size class."""
    name = "batched_uneven"
    metric = "UMI batched ops GB/s"
    unit = "GB/s"
    dtype = "f32"
    BYTES = {"bilateral": 8, "wfilter_pp": 44, "cost_volume": 512}  # algorithmic bytes per pixel
    e2e_max_steps = 3  # each e2e step moves ~47 GB across the host link

    def __init__(self, seed=7, n=64, lo=256, hi=2048):
        g = np.random.default_rng(seed)
        self.seed = seed
        self.sizes = [(int(g.integers(lo, hi + 1)), int(g.integers(lo, hi + 1))) for _ in range(n)]
        self.px = sum(h * w for h, w in self.sizes)

    def config(self):
        return {"workload": self.name, "images": len(self.sizes), "sides": "U{256..2048} (seeded)",
                "total_px": self.px, "ops": "bilateral 5x5 s_s=2 s_r=0.1; wfilter3x3 per-pixel; "
                "cost volume dot C=32 D=64", "bytes_per_px": self.BYTES, "l2": "inputs far larger than L2",
                "launch": "one fused persistent kernel per step (umi_batch_run_fused)",
                "size_class_choices": getattr(self, "variants", None)}

    def units_per_step(self):
        return sum(self.BYTES.values()) * self.px / 1e9

    def setup(self, dev):
        import torch
        import umi_gb300 as U
        from umi_gb300 import autotune
        self.U = U
        gen = torch.Generator(device=dev).manual_seed(self.seed)
        self.bil, self.wf, self.cv = [], [], []
        for h, w in self.sizes:
            img = torch.rand((h, w), generator=gen, device=dev)
            wts = torch.rand((h, w, 3, 3), generator=gen, device=dev)
            L = torch.randn((32, h, w), generator=gen, device=dev)
            disp = torch.randint(0, 64, (h, w), generator=gen, device=dev)
            src = (torch.arange(w, device=dev).view(1, w) - disp).clamp(0, w - 1)
            R = torch.gather(L, 2, src.unsqueeze(0).expand(32, h, w)) + 0.1 * torch.randn((32, h, w), generator=gen,
                                                                                         device=dev)
            del src, disp
            self.bil.append((img, None, torch.empty((h, w), device=dev)))
            self.wf.append((img, wts, torch.empty((h, w), device=dev)))
            self.cv.append((L, R.contiguous(), torch.empty((h, w, 64), device=dev)))
        torch.cuda.synchronize()
        self.pb = U.BatchParams(2, 2.0, 0.1, 0, 0)
        self.pc = U.BatchParams(0, 0.0, 0.0, 32, 64)
        jobs = [(U.OP_COST_VOLUME, self.cv, self.pc, None), (U.OP_WFILTER_PP, self.wf, None, None),
                (U.OP_BILATERAL, self.bil, self.pb, None)]
        self.jobs, report = autotune.tuned_fused_variants(jobs)
        self.variants = {op: {cls: {"variant": r["variant"], "images": r["images"], "ms": r["ms"]}
                              for cls, r in rep.items()} for op, rep in report.items()}
        self.variants["cost_volume"] = "one form: tensor-core tiles of 128 px x 64 disparities"
        self.n_rot = 1
        self.launches_per_step = 1

    def _ops(self):
        """Each operator alone through the same fused kernel (for the per-operator breakdown)."""
        U = self.U
        names = {U.OP_COST_VOLUME: "cost_volume", U.OP_WFILTER_PP: "wfilter_pp", U.OP_BILATERAL: "bilateral"}
        return tuple((names[j[0]], lambda j=j: U.batch_run_fused([j])) for j in self.jobs)

    def step(self, i):
        self.U.batch_run_fused(self.jobs)

    def e2e_setup(self):
        import torch
        self.h_in = [[t.cpu().pin_memory() for t in (a, b) if t is not None] for a, b, _ in self.wf + self.cv]
        self.h_out = [o.cpu().pin_memory() for _, _, o in self.bil + self.wf + self.cv]
        torch.cuda.synchronize()

    def h2d(self, k):
        dev_in = [[t for t in (a, b) if t is not None] for a, b, _ in self.wf + self.cv]
        for hs, ds in zip(self.h_in, dev_in):
            for h, d in zip(hs, ds):
                d.copy_(h, non_blocking=True)

    def d2h(self, k):
        for h, (_, _, o) in zip(self.h_out, self.bil + self.wf + self.cv):
            h.copy_(o, non_blocking=True)

    def e2e_bytes(self):
        h2d = sum(t.numel() * 4 for a, b, _ in self.wf + self.cv for t in (a, b) if t is not None)
        d2h = sum(o.numel() * 4 for _, _, o in self.bil + self.wf + self.cv)
        return h2d, d2h

    def check(self):
        """Sampled FP64 check of the timed outputs (full parity lives in the tests)."""
        g = np.random.default_rng(0)
        worst = 0.0
        for k in g.choice(len(self.sizes), 4, replace=False):
            L, R, cv = (t.cpu().numpy() if t is not None else None for t in self.cv[k])
            h, w = L.shape[1:]
            for _ in range(50):
                y, x, d = int(g.integers(h)), int(g.integers(w)), int(g.integers(64))
                want = float(np.dot(L[:, y, x].astype(np.float64), R[:, y, x + d].astype(np.float64))) if x + d < w else 0.0
                scale = float(np.abs(L[:, y, x]).astype(np.float64) @ np.abs(R[:, y, min(x + d, w - 1)]).astype(np.float64))
                worst = max(worst, float(abs(float(cv[y, x, d]) - want) / max(abs(want), scale, 1e-30)))
        return worst

    def kernels(self, dev, peaks, n=3):
        ms = {name: time_launches(lambda i, f=fn: f(), 1, n) for name, fn in self._ops()}
        ms["fused_step"] = time_launches(self.step, 1, n)
        # the same step as three persistent launches (one per operator, their own kernels and tuned tile shapes)
        from umi_gb300 import autotune
        U = self.U
        sep = []
        for op, imgs, prm in ((U.OP_BILATERAL, self.bil, self.pb), (U.OP_WFILTER_PP, self.wf, None),
                              (U.OP_COST_VOLUME, self.cv, self.pc)):
            v, _, _ = autotune.tuned_variant(op, imgs, prm)
            sep.append(lambda op=op, imgs=imgs, prm=prm, v=v: U.batch_run(op, imgs, prm, v))
        ms["three_launches_step"] = time_launches(lambda i: [f() for f in sep], 1, n)
        return ms, None, None

    def cpu_setup(self):
        import oracle
        self.orc = oracle
        self.rng = np.random.default_rng(1)

    def cpu_step(self, rows, threads):
        """FP64 oracle of the three operators on `rows` rows of a 1024-wide crop."""
        g = self.rng
        x = g.random((rows, 1024), dtype=np.float32)
        self.orc.bilateral_f64(x, 2, 2.0, 0.1, threads=threads)
        self.orc.wfilter_pp_f64(x, g.random((rows, 1024, 3, 3), dtype=np.float32), threads=threads)
        L = g.standard_normal((32, rows, 1024)).astype(np.float32)
        self.orc.cost_volume_dot_f64(L, L, 64, threads=threads)
        return sum(self.BYTES.values()) * rows * 1024 / 1e9


class Gemm:
    """C = A @ B^T, M = N = K = 4096, A and B ~ N(0,1), bf16 operands, fp32
    accumulation on the tcgen05 tensor cores.  The f16 and bf16x3 (fp32
    emulation) variants are timed beside it; each reports max / RMS error
    against FP64 on sampled rows."""
    name = "gemm_4096"
    metric = "gemm TFLOP/s (4096^3, bf16 in, fp32 accumulate)"
    unit = "TFLOP/s"
    dtype = "bf16"
    M = N = K = 4096

    def __init__(self, seed=11, **_):
        self.seed = seed
        self.flops = 2.0 * self.M * self.N * self.K

    def config(self):
        return {"workload": self.name, "M": self.M, "N": self.N, "K": self.K, "layout": "A (M,K), B (N,K) row-major",
                "inputs": "N(0,1)", "l2": "3 rotating operand sets (384 MB)"}

    def units_per_step(self):
        return self.flops / 1e12

    def setup(self, dev):
        import torch
        import umi_gb300 as U
        self.U = U
        gen = torch.Generator(device=dev).manual_seed(self.seed)
        self.a32 = torch.randn((self.M, self.K), generator=gen, device=dev)
        self.b32 = torch.randn((self.N, self.K), generator=gen, device=dev)
        self.n_rot = 3
        self.A = [self.a32.to(torch.bfloat16) for _ in range(self.n_rot)]
        self.B = [self.b32.to(torch.bfloat16) for _ in range(self.n_rot)]
        self.C = [torch.empty((self.M, self.N), device=dev) for _ in range(self.n_rot)]
        self.err = torch.zeros(1, dtype=torch.int32, device=dev)
        self.launches_per_step = 1
        self.hA = self.A[0].cpu().pin_memory()
        self.hB = self.B[0].cpu().pin_memory()
        self.hC = torch.empty((self.M, self.N)).pin_memory()

    def step(self, i):
        k = i % self.n_rot
        self.U.gemm(self.A[k], self.B[k], out=self.C[k], err=self.err)

    def h2d(self, k):
        self.A[k].copy_(self.hA, non_blocking=True)
        self.B[k].copy_(self.hB, non_blocking=True)

    def d2h(self, k):
        self.hC.copy_(self.C[k], non_blocking=True)

    def e2e_bytes(self):
        return 2 * 2 * self.M * self.K, 4 * self.M * self.N

    @staticmethod
    def _err(C, ref, rows):
        got = C[rows].double().cpu().numpy()
        d = np.abs(got - ref)
        rel = d / np.maximum(np.abs(ref), 1e-30)
        return {"max_abs": float(d.max()), "rms_abs": float(np.sqrt((d ** 2).mean())),
                "max_rel_to_scale": None, "rms_rel": float(np.sqrt(np.mean(np.minimum(rel, 1.0) ** 2)))}

    @staticmethod
    def _errors(got, ref, scale):
        """Error of one variant against FP64: elementwise max / median of
        |C - C64| / |C64|, normwise RMS ||C - C64||_F / ||C64||_F, and the
        largest error over the condition scale sum_k |a b|."""
        d = np.abs(got - ref)
        rel = d / np.maximum(np.abs(ref), 1e-300)
        return {"max_rel": float(rel.max()), "median_rel": float(np.median(rel)),
                "rms_rel": float(np.sqrt((d ** 2).sum() / (ref ** 2).sum())),
                "max_err_over_scale": float((d / scale).max())}

    def check(self):
        """Max and RMS relative error against FP64 for every variant, on 32
        complete sampled rows of C (4096 x 32 outputs), all from the same fp32
        inputs: bf16 / f16 (inputs rounded to 16 bits), bf16x3, f16x3 (the
        FP32-level product), and the plain FP32 UMI path (the generic operator
        with the reference's Gemm strategy, main/gemm.cu:8-15, fp32 FMA)."""
        import torch
        rows = np.random.default_rng(0).choice(self.M, 32, replace=False)
        a32 = self.a32[rows].double().cpu().numpy()
        b32 = self.b32.double().cpu().numpy()
        ref32 = a32 @ b32.T
        scale = np.abs(a32) @ np.abs(b32).T
        ridx = torch.from_numpy(rows).to(self.a32.device)
        out = {"rows_checked": len(rows), "reference": "FP64 product of the fp32 inputs"}
        variants = {
            "bf16": lambda: self.U.gemm(self.a32.to(torch.bfloat16), self.b32.to(torch.bfloat16))[ridx],
            "f16": lambda: self.U.gemm(self.a32.to(torch.float16), self.b32.to(torch.float16))[ridx],
            "bf16x3": lambda: self.U.gemm_f32_bf16x3(self.a32, self.b32)[ridx],
            "f16x3": lambda: self.U.gemm_f32_f16x3(self.a32, self.b32)[ridx],
            "fp32_umi_generic": lambda: self.U.gemm_f32_generic(self.a32[ridx].contiguous(), self.b32),
        }
        for name, fn in variants.items():
            out[name] = self._errors(fn().double().cpu().numpy(), ref32, scale)
        out["err_word"] = int(self.err.item())
        return out

    def kernels(self, dev, peaks, n=30):
        import torch
        R = self.n_rot
        A16 = [a.to(torch.float16) for a in self.A]
        B16 = [b.to(torch.float16) for b in self.B]
        ws = torch.empty(self.U.lib().umi_gemm_f32_bf16x3_workspace_bytes(self.M, self.N, self.K), dtype=torch.uint8,
                         device=dev)
        a32, b32 = self.a32, self.b32
        ws16 = torch.empty(self.U.lib().umi_gemm_f32_f16x3_workspace_bytes(self.M, self.N, self.K),
                           dtype=torch.uint8, device=dev)
        fns = {"gemm_bf16": lambda i: self.U.gemm(self.A[i % R], self.B[i % R], out=self.C[i % R], err=self.err),
               "gemm_f16": lambda i: self.U.gemm(A16[i % R], B16[i % R], out=self.C[i % R], err=self.err),
               "gemm_f32_bf16x3": lambda i: self.U.gemm_f32_bf16x3(a32, b32, out=self.C[i % R], workspace=ws,
                                                                   err=self.err),
               "gemm_f32_f16x3": lambda i: self.U.gemm_f32_f16x3(a32, b32, out=self.C[i % R], workspace=ws16,
                                                                 err=self.err)}
        ms = {k: time_launches(f, R, n) for k, f in fns.items()}
        # the plain FP32 UMI path on a 256-row slice of C (the whole product
        # through the generic operator would take seconds)
        rows = 256
        a_sl = a32[:rows].contiguous()
        c_sl = torch.empty((rows, self.N), device=dev)
        ms["gemm_f32_umi_generic_256rows"] = time_launches(lambda i: self.U.gemm_f32_generic(a_sl, b32, out=c_sl), 1, 3)
        return ms, None, None

    def cpu_setup(self):
        import oracle
        self.orc = oracle
        g = np.random.default_rng(1)
        self.ha = g.standard_normal((256, self.K)).astype(np.float32)
        self.hb = g.standard_normal((self.N, self.K)).astype(np.float32)

    def cpu_step(self, rows, threads):
        """The reference's gemm loop (main/gemm.cu:69-78, restated with FP64 accumulation) on `rows` rows of C."""
        self.orc.gemm_f64(self.ha[:rows], self.hb, b_is_nk=True, threads=threads)
        return 2.0 * rows * self.N * self.K / 1e12


class Fprop:
    """Convolution forward pass N=32, C=64, H=W=128, K=128, 3x3, stride 1,
    pad 1: bf16 NHWC input ~ N(0,1), bf16 KRSC weights ~ N(0, 1/576), fp32
    accumulation and NCHW fp32 output (implicit GEMM on the tensor cores)."""
    name = "fprop_n32"
    metric = "fprop TFLOP/s (N32 C64 128x128 K128 3x3, bf16 in, fp32 accumulate)"
    unit = "TFLOP/s"
    dtype = "bf16"
    N, C, H, W, K, R = 32, 64, 128, 128, 128, 3

    def __init__(self, seed=13, **_):
        self.seed = seed
        self.flops = 2.0 * self.N * self.K * self.H * self.W * self.C * self.R * self.R

    def config(self):
        return {"workload": self.name, "N": self.N, "C": self.C, "H": self.H, "W": self.W, "K": self.K,
                "filter": "3x3 s1 p1", "layout": "x NHWC bf16, w KRSC bf16, out NCHW fp32",
                "l2": "4 rotating input/output sets (>= 1 GB)"}

    def units_per_step(self):
        return self.flops / 1e12

    def setup(self, dev):
        import torch
        import umi_gb300 as U
        self.U = U
        gen = torch.Generator(device=dev).manual_seed(self.seed)
        self.x32 = torch.randn((self.N, self.H, self.W, self.C), generator=gen, device=dev)
        self.w32 = torch.randn((self.K, self.R, self.R, self.C), generator=gen, device=dev) / 24.0
        x = self.x32.to(torch.bfloat16)
        w = self.w32.to(torch.bfloat16)
        self.n_rot = 4
        self.x = [x.clone() for _ in range(self.n_rot)]
        self.w = w
        self.out = [torch.empty((self.N, self.K, self.H, self.W), device=dev) for _ in range(self.n_rot)]
        self.err = torch.zeros(1, dtype=torch.int32, device=dev)
        self.launches_per_step = 1
        self.hx = x.cpu().pin_memory()
        self.hout = torch.empty((self.N, self.K, self.H, self.W)).pin_memory()

    def step(self, i):
        k = i % self.n_rot
        self.U.conv2d_fprop_bf16(self.x[k], self.w, out=self.out[k], err=self.err)

    def h2d(self, k):
        self.x[k].copy_(self.hx, non_blocking=True)

    def d2h(self, k):
        self.hout.copy_(self.out[k], non_blocking=True)

    def e2e_bytes(self):
        return 2 * self.N * self.H * self.W * self.C, 4 * self.N * self.K * self.H * self.W

    def check(self):
        """Max and RMS relative error against an FP64 convolution (on the GPU,
        2 images) of the bf16 product (against its bf16 inputs) and of the
        FP32-level split product f16x3 (against fp32 inputs)."""
        import torch

        def errs(got, xd, wd):
            ref = torch.nn.functional.conv2d(xd, wd, padding=1)
            scale = torch.nn.functional.conv2d(xd.abs(), wd.abs(), padding=1)
            d = (got.double() - ref).abs()
            return {"max_rel": float((d / ref.abs().clamp_min(1e-300)).max()),
                    "median_rel": float((d / ref.abs().clamp_min(1e-300)).median()),
                    "rms_rel": float((d.pow(2).sum() / ref.pow(2).sum()).sqrt()),
                    "max_err_over_scale": float((d / scale.clamp_min(1e-30)).max())}
        out = {"images_checked": 2, "reference": "FP64 convolution of the same inputs"}
        out["bf16"] = errs(self.out[0][:2], self.x[0][:2].permute(0, 3, 1, 2).double(),
                           self.w.permute(0, 3, 1, 2).double())
        x32, w32 = self.x32[:2].contiguous(), self.w32
        got = self.U.conv2d_fprop_f32_f16x3(x32, w32)
        out["f16x3_fp32_inputs"] = errs(got, x32.permute(0, 3, 1, 2).double(), w32.permute(0, 3, 1, 2).double())
        out["err_word"] = int(self.err.item())
        return out

    def kernels(self, dev, peaks, n=30):
        import torch
        ws = torch.empty(self.U.lib().umi_conv2d_fprop_f32_f16x3_workspace_bytes(self.N, self.C, self.H, self.W,
                                                                               self.K, self.R), dtype=torch.uint8,
                         device=dev)
        o32 = torch.empty_like(self.out[0])
        return {"conv2d_fprop_bf16": time_launches(self.step, self.n_rot, n),
                "conv2d_fprop_f32_f16x3": time_launches(
                    lambda i: self.U.conv2d_fprop_f32_f16x3(self.x32, self.w32, out=o32, workspace=ws, err=self.err),
                    1, n)}, None, None

    def cpu_setup(self):
        import oracle
        self.orc = oracle
        g = np.random.default_rng(1)
        self.hxn = g.standard_normal((1, self.C, self.H, self.W)).astype(np.float32)
        self.hwn = (g.standard_normal((self.K, self.C, self.R, self.R)) / 24.0).astype(np.float32)

    def cpu_step(self, rows, threads):
        """The reference's direct convolution loop (main/fprop.cu:84-108, FP64) on `rows` output rows of one image."""
        self.orc.conv2d_f64(np.ascontiguousarray(self.hxn[:, :, :rows + 2]), self.hwn, 1, 1, threads=threads)
        return 2.0 * self.K * (rows + 2) * self.W * self.C * 9 / 1e12


class LearnedMe:
    """Learned motion proposal on 3840x2160 u8 pairs (per-block shifts
    round(N(0, 16^2)) clipped to +-64, 16x16 blocks): proposal network,
    +-4 refine, audit of every 64th block by +-64 exhaustive search,
    fallback to +-64 exhaustive search above the SAD threshold
    (umi_me_learned_u8).  The plain +-64 exhaustive search on the same pairs
    is timed beside it (kernels.full_me_u8_r64)."""
    name = "learned_me_4k"
    metric = "learned ME Mblocks/s (4K, +-64 judge, +-4 refine, <= 1% mean SAD regression)"
    unit = "Mblocks/s"
    dtype = "u8 (search), bf16 weights / fp32 accumulation (network)"
    H, W, B, FULL_R, REFINE_R, AUDIT = 2160, 3840, 16, 64, 4, 64
    data = "synthetic (seeded torch Philox generator on the GPU; the network's weights trained on 2000 such pairs)"

    def __init__(self, seed=0, **_):
        self.nblk = (self.H // self.B) * (self.W // self.B)

    def config(self):
        return {"workload": self.name, "frame": f"{self.W}x{self.H} u8", "block": self.B,
                "shifts": "round(N(0,16^2)) per block, clipped +-64", "judge": f"+-{self.FULL_R} exhaustive",
                "refine": f"+-{self.REFINE_R}", "audit": f"every {self.AUDIT}th block",
                "threshold": "1.2 x p99 of the optimal SAD of a calibration pair",
                "network": "4 x conv3x3 32ch dil 1,2,4,8 + per-block linear head, trained on 2000 pairs",
                "l2": "16 distinct pairs rotated (265 MB > L2)"}

    def units_per_step(self):
        return self.nblk / 1e6

    def setup(self, dev):
        import torch
        import umi_gb300 as U
        from umi_gb300 import menet_train as T
        from umi_gb300.workloads import me_pair_cuda
        self.U, self.T = U, T
        self.n_rot = 16
        pairs = [me_pair_cuda(T.EVAL_SEED0 + k, self.H, self.W, device=dev) for k in range(self.n_rot)]
        self.d_cur = [p[0] for p in pairs]
        self.d_ref = [p[1] for p in pairs]
        self.net = U.MeNet(self.H, self.W, device=dev, params=T.default_weights())
        self.trained = os.path.exists(T.WEIGHTS)
        self.full0 = U.full_me_u8(self.d_cur[0], self.d_ref[0], self.B, self.FULL_R)
        self.thr = T.threshold_from(self.full0)
        self.d_mv = [torch.empty((self.nblk, 3), dtype=torch.int32, device=dev) for _ in range(self.n_rot)]
        self.d_sums = [torch.zeros(2, dtype=torch.int64, device=dev) for _ in range(self.n_rot)]
        self.d_nf = [torch.zeros(1, dtype=torch.int32, device=dev) for _ in range(self.n_rot)]
        self.h_cur = self.d_cur[0].cpu().pin_memory()
        self.h_ref = self.d_ref[0].cpu().pin_memory()
        self.h_mv = torch.empty((self.nblk, 3), dtype=torch.int32).pin_memory()
        # audit list + audit search (second stream) + inference (downsample, 4 weight packs, layer 1,
        # 3 tensor-core layers, head) + centres + refine + flag + fallback list search + audit merge
        # (memsets, event waits and the count copy are not kernels)
        self.launches_per_step = 17

    def _estimate(self, k):
        self.net.estimate(self.d_cur[k], self.d_ref[k], self.REFINE_R, self.FULL_R, self.thr, self.AUDIT,
                          out=self.d_mv[k], audit_sums=self.d_sums[k], n_fallback=self.d_nf[k])

    def step(self, i):
        self._estimate(i % self.n_rot)

    def h2d(self, k):
        self.d_cur[k].copy_(self.h_cur, non_blocking=True)
        self.d_ref[k].copy_(self.h_ref, non_blocking=True)

    def d2h(self, k):
        self.h_mv.copy_(self.d_mv[k], non_blocking=True)

    def e2e_bytes(self):
        return 2 * self.H * self.W, 12 * self.nblk

    def check(self):
        """Quality of the timed results against exhaustive search, plus the ablation."""
        import torch
        regs, fbs = [], []
        for k in range(2):
            full = self.U.full_me_u8(self.d_cur[k], self.d_ref[k], self.B, self.FULL_R)
            self._estimate(k)
            regs.append((self.d_mv[k][:, 2].long().sum() / full[:, 2].long().sum()).item() - 1.0)
            fbs.append(int(self.d_nf[k].item()) / self.nblk)
        ab = self.T.evaluate(self.net, [self.T.EVAL_SEED0 + 2], self.REFINE_R, self.FULL_R, self.thr, self.AUDIT,
                             coarse=getattr(self, "cme", None))
        return {"mean_sad_regression": float(np.mean(regs)), "fallback_fraction": float(np.mean(fbs)),
                "sad_threshold": self.thr, "trained_weights": self.trained,
                "ablation_hit_rate_within_refine": {m: ab[m]["hit"] for m in ab},
                "ablation_fallback_fraction": {m: ab[m]["fallback_frac"] for m in ab},
                "ablation_sad_regression_without_fallback": {m: ab[m]["sad_reg_no_fallback"] for m in ab}}

    def kernels(self, dev, peaks, n=20):
        R = self.n_rot
        fns = {
            "me_learned_u8": self.step,
            "full_me_u8_r64": lambda i: self.U.full_me_u8(self.d_cur[i % R], self.d_ref[i % R], self.B, self.FULL_R,
                                                          out=self.d_mv[i % R]),
            "menet_forward_fp32_training_pass": lambda i: self.net.forward(self.d_cur[i % R], self.d_ref[i % R]),
            "menet_infer_tensor_cores": lambda i: self.net.infer(self.d_cur[i % R], self.d_ref[i % R]),
            "refine_r4": lambda i: self.U.full_me_u8(self.d_cur[i % R], self.d_ref[i % R], self.B, self.REFINE_R,
                                                     out=self.d_mv[i % R]),
        }
        out = {name: time_launches(fn, R, n) for name, fn in fns.items()}
        absdiff = self.nblk * (2 * self.FULL_R + 1) ** 2 * self.B * self.B
        return out, absdiff, None

    def cpu_setup(self):
        import oracle
        from umi_gb300.workloads import me_pair
        self.orc = oracle
        self.rng = np.random.default_rng(0)
        # the reference's CPU path is the exhaustive search; a 4K numpy pair of the same distribution
        self.hc, self.hr, _ = me_pair(seed=5, h=self.H, w=self.W, block=self.B, shift_sigma=16.0, max_shift=64)

    def cpu_step(self, nblocks, threads):
        blocks = self.rng.choice(self.nblk, size=nblocks, replace=False).astype(np.int32)
        self.orc.ref_full_me_u8_argmin(self.hc, self.hr, self.B, self.FULL_R, blocks, threads=threads)
        return nblocks / 1e6


class CoarseMe4k(LearnedMe):
    """Coarse-to-fine motion estimation on the same 4K pairs: 4x4-mean cells
    searched on a 2-pixel grid within +-60, then the same +-4 refine, audit
    and fallback (umi_me_coarse_u8).  The learned pipeline and the plain
    +-64 exhaustive search are timed beside it."""
    name = "coarse_me_4k"
    metric = "coarse-to-fine ME Mblocks/s (4K, +-64 judge, +-4 refine, <= 1% mean SAD regression)"
    dtype = "u8 (search)"
    step_kernel = "me_coarse_u8"

    def config(self):
        c = super().config()
        c.pop("network")
        c["proposal"] = "rounded 4x4-mean cells, even displacements within +-60 (2-pixel grid), packed SAD, first-min"
        return c

    def setup(self, dev):
        super().setup(dev)
        self.cme = self.U.CoarseMe(self.H, self.W, device=dev)
        # audit list + audit search (second stream) + cells + search + refine + flag + fallback list
        # search + audit merge
        self.launches_per_step = 8

    def _estimate(self, k):
        self.cme.estimate(self.d_cur[k], self.d_ref[k], self.REFINE_R, self.FULL_R, self.thr, self.AUDIT,
                          out=self.d_mv[k], audit_sums=self.d_sums[k], n_fallback=self.d_nf[k])

    def kernels(self, dev, peaks, n=20):
        R = self.n_rot
        rng = (self.FULL_R - self.REFINE_R) & ~1
        fns = {
            "me_coarse_u8": self.step,
            "coarse_centers": lambda i: self.cme.centers(self.d_cur[i % R], self.d_ref[i % R], rng),
            "full_me_u8_r64": lambda i: self.U.full_me_u8(self.d_cur[i % R], self.d_ref[i % R], self.B, self.FULL_R,
                                                          out=self.d_mv[i % R]),
            "me_learned_u8": lambda i: LearnedMe._estimate(self, i % R),
            "refine_r4": lambda i: self.U.full_me_u8(self.d_cur[i % R], self.d_ref[i % R], self.B, self.REFINE_R,
                                                     out=self.d_mv[i % R]),
        }
        out = {name: time_launches(fn, R, n) for name, fn in fns.items()}
        absdiff = self.nblk * (rng + 1) ** 2 * 16  # the coarse search: 16 cells per candidate
        return out, absdiff, None


class VideoY4M:
    """Motion estimation over a YUV4MPEG2 video: 64 frames of 1920x1080
    (a panning camera over a blurred-noise scene, workloads.video_frames,
    6 and -10 pixels per frame, N(0, 2^2) sensor noise) written to a
    temporary 4:2:0 Y4M file; every consecutive pair through the coarse
    proposal (frames cropped to 1920x1072, +-64 judge, +-4 refine, audit
    every 64th block).  value: pairs/s with the frames resident in HBM; e2e:
    pairs/s through video.MotionPipeline from the file (memory map, pinned
    copy, upload, search, download; wall clock around whole passes)."""
    name = "video_y4m_1080p"
    metric = "video motion estimation pairs/s (1080p Y4M, coarse proposal, +-64 judge, +-4 refine)"
    unit = "pairs/s"
    dtype = "u8 (search)"
    data = "synthetic (seeded numpy: panning camera over a blurred-noise scene), written as a Y4M file"
    H, W, N, B, REFINE_R, FULL_R, AUDIT, VEL = 1080, 1920, 64, 16, 4, 64, 64, (6, -10)
    e2e_max_steps = 630  # ten passes over the file

    def __init__(self, seed=11, **_):
        self.seed = seed
        self.h16 = self.H - self.H % 16
        self.nblk = (self.h16 // 16) * (self.W // 16)

    def config(self):
        return {"workload": self.name, "frame": f"{self.W}x{self.H} u8 (4:2:0 Y4M, luma searched, cropped to "
                f"{self.W}x{self.h16})", "frames": self.N, "motion": f"pan {self.VEL} px/frame + N(0,2^2) noise",
                "block": self.B, "judge": f"+-{self.FULL_R} exhaustive", "refine": f"+-{self.REFINE_R}",
                "audit": f"every {self.AUDIT}th block", "l2": "64 resident frames (133 MB > L2)"}

    def units_per_step(self):
        return 1.0

    def setup(self, dev):
        import atexit
        import shutil
        import tempfile
        import torch
        import umi_gb300 as U
        from umi_gb300 import menet_train as T
        from umi_gb300 import video, workloads
        self.U, self.video, self.dev = U, video, dev
        frames = workloads.video_frames(seed=self.seed, n=self.N, h=self.H, w=self.W, velocity=self.VEL)
        self.tmp = tempfile.mkdtemp(prefix="umi_video_")
        atexit.register(shutil.rmtree, self.tmp, True)
        self.path = os.path.join(self.tmp, "pan_1080p.y4m")
        video.write_y4m(self.path, frames, colorspace="420jpeg")
        self.frames = frames
        self.d = [torch.from_numpy(f[:self.h16]).to(dev) for f in frames]
        self.cme = U.CoarseMe(self.h16, self.W, device=dev)
        self.thr = T.threshold_from(U.full_me_u8(self.d[1], self.d[0], self.B, self.FULL_R))
        self.n_rot = self.N - 1
        self.d_mv = [torch.empty((self.nblk, 3), dtype=torch.int32, device=dev) for _ in range(self.n_rot)]
        self.d_sums = [torch.zeros(2, dtype=torch.int64, device=dev) for _ in range(self.n_rot)]
        self.d_nf = [torch.zeros(1, dtype=torch.int32, device=dev) for _ in range(self.n_rot)]
        # cells + search + refine + flag + one list search (the 126 audited blocks, fewer than the
        # SMs, join the fallback blocks' list) + audit sum
        self.launches_per_step = 6

    def _pair(self, j):
        self.cme.estimate(self.d[j + 1], self.d[j], self.REFINE_R, self.FULL_R, self.thr, self.AUDIT,
                          out=self.d_mv[j], audit_sums=self.d_sums[j], n_fallback=self.d_nf[j])

    def step(self, i):
        self._pair(i % self.n_rot)

    def e2e_bytes(self):
        return self.h16 * self.W, 12 * self.nblk + 24

    def e2e_run(self, steps, warmup):
        """ms for `steps` pairs through MotionPipeline reading the Y4M file."""
        import torch
        pipe = self.video.MotionPipeline(self.H, self.W, method="coarse", search=self.FULL_R, refine=self.REFINE_R,
                                         sad_threshold=self.thr, audit_stride=self.AUDIT, device=self.dev)
        with self.video.Y4MReader(self.path) as r:
            for _ in pipe.run(r.luma(i) for i in range(min(len(r), warmup + 2))):
                pass
            torch.cuda.synchronize()
            passes = max(1, -(-steps // (len(r) - 1)))
            t0 = time.perf_counter()
            done = 0
            for _ in range(passes):
                for _ in pipe.run(r):
                    done += 1
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
        self.e2e_pairs = done
        return dt * 1e3 * steps / done

    def check(self):
        """Quality on two pairs against exhaustive search, and the pan recovered."""
        regs, fbs, pan = [], [], []
        for j in (0, self.N // 2):
            self._pair(j)
            full = self.U.full_me_u8(self.d[j + 1], self.d[j], self.B, self.FULL_R)
            regs.append((self.d_mv[j][:, 2].long().sum() / full[:, 2].long().sum()).item() - 1.0)
            fbs.append(int(self.d_nf[j].item()) / self.nblk)
            mv = self.d_mv[j].cpu().numpy().reshape(self.h16 // 16, self.W // 16, 3)[1:-1, 1:-1]
            pan.append(float(np.mean((mv[..., 0] == self.VEL[0]) & (mv[..., 1] == self.VEL[1]))))
        return {"mean_sad_regression": float(np.mean(regs)), "fallback_fraction": float(np.mean(fbs)),
                "interior_blocks_at_true_pan": float(np.mean(pan)), "sad_threshold": self.thr}

    def kernels(self, dev, peaks, n=20):
        R = self.n_rot
        rng = (self.FULL_R - self.REFINE_R) & ~1
        fns = {
            "me_coarse_u8": self.step,
            "coarse_centers": lambda i: self.cme.centers(self.d[i % R + 1], self.d[i % R], rng),
            "full_me_u8_r64": lambda i: self.U.full_me_u8(self.d[i % R + 1], self.d[i % R], self.B, self.FULL_R,
                                                          out=self.d_mv[i % R]),
        }
        out = {name: time_launches(fn, R, n) for name, fn in fns.items()}
        return out, self.nblk * (rng + 1) ** 2 * 16, None

    def cpu_setup(self):
        import oracle
        from umi_gb300 import workloads
        self.orc = oracle
        self.rng = np.random.default_rng(0)
        fr = workloads.video_frames(seed=self.seed, n=2, h=self.H, w=self.W, velocity=self.VEL)
        self.hc, self.hr = np.ascontiguousarray(fr[1][:self.h16]), np.ascontiguousarray(fr[0][:self.h16])

    def cpu_step(self, nblocks, threads):
        blocks = self.rng.choice(self.nblk, size=nblocks, replace=False).astype(np.int32)
        self.orc.ref_full_me_u8_argmin(self.hc, self.hr, self.B, self.FULL_R, blocks, threads=threads)
        return nblocks / self.nblk


class Apps1080p:
    """Four window operators of the UMI family on the generic operator
    (umi_gb300/apps.py, umi_launch with built-in strategies) over one
    1920x1080 frame per step: census 5x5 (int32), grey-level dilation 3x3
    (int32), box sums 15x15 via the integral image (uint8 -> int32) and a
    separable Gaussian, sigma 2, 13 taps (float32, two passes)."""
    name = "apps_1080p"
    metric = "UMI window apps Mpx/s (1080p: census 5x5 + dilate 3x3 + box 15x15 via iimg + gaussian sigma 2)"
    unit = "Mpx/s"
    dtype = "i32 / u8 / f32"
    H, W = 1080, 1920
    # bytes moved per pixel as implemented (read + write of every launch)
    BYTES = {"census": 8, "dilate": 8, "box_sum": 5 + 8 + 8, "gaussian": 16}

    def __init__(self, seed=21, **_):
        self.seed = seed
        self.px = self.H * self.W

    def config(self):
        return {"workload": self.name, "frame": f"{self.W}x{self.H}", "ops": "census r2, dilate r1, box r7 "
                "(integral image + 4 corner reads), gaussian sigma 2 (13 taps, two passes)",
                "bytes_per_px": self.BYTES, "l2": "4 frame sets rotated (> L2)",
                "streams": "census + dilate | box | gaussian, joined every step"}

    def units_per_step(self):
        return self.px / 1e6

    def setup(self, dev):
        import torch
        import umi_gb300 as U
        from umi_gb300 import apps
        self.U, self.apps = U, apps
        self.n_rot = 4
        g = np.random.default_rng(self.seed)
        frames = [g.integers(0, 256, (self.H, self.W), dtype=np.uint8) for _ in range(self.n_rot)]
        self.h_u8 = [torch.from_numpy(f).pin_memory() for f in frames]
        self.u8 = [t.to(dev) for t in self.h_u8]
        self.i32 = [t.to(torch.int32) for t in self.u8]
        self.f32 = [t.to(torch.float32) * (1.0 / 255.0) for t in self.u8]
        mk = lambda dt: [torch.empty((self.H, self.W), dtype=dt, device=dev) for _ in range(self.n_rot)]
        self.o_census, self.o_dil, self.o_box, self.ii = mk(torch.int32), mk(torch.int32), mk(torch.int32), mk(torch.int32)
        self.o_g, self.tmp = mk(torch.float32), mk(torch.float32)
        self.J = [torch.zeros((self.H + 1, self.W + 1), dtype=torch.int32, device=dev) for _ in range(self.n_rot)]
        self.ws = torch.empty(U.iimg_workspace_bytes(self.H, self.W), dtype=torch.uint8, device=dev)
        self.h_out = torch.empty((self.H, self.W), dtype=torch.int32).pin_memory()
        # census + dilate + (iimg 2 kernels + J copy + box) + gaussian 2
        self.launches_per_step = 1 + 1 + 4 + 2
        self.s1, self.s2 = torch.cuda.Stream(device=dev), torch.cuda.Stream(device=dev)
        for k in range(self.n_rot):  # constants made before any graph capture
            self.step(k)

    def _op(self, name, k):
        a = self.apps
        if name == "census":
            a.census(self.i32[k], 2, out=self.o_census[k])
        elif name == "dilate":
            a.dilate(self.i32[k], 1, out=self.o_dil[k])
        elif name == "box_sum":
            a.box_sum(self.u8[k], 7, out=self.o_box[k], J=self.J[k], ii=self.ii[k], workspace=self.ws)
        else:
            a.gaussian(self.f32[k], 2.0, out=self.o_g[k], tmp=self.tmp[k])

    def step(self, i):
        """The four operators are independent: census and dilation on one
        stream, the box sums (integral image, copy, generic launch) on a
        second, the Gaussian passes on the caller's, joined every step."""
        import torch
        k = i % self.n_rot
        cur = torch.cuda.current_stream()
        self.s1.wait_stream(cur)
        self.s2.wait_stream(cur)
        with torch.cuda.stream(self.s1):
            self._op("census", k)
            self._op("dilate", k)
        with torch.cuda.stream(self.s2):
            self._op("box_sum", k)
        self._op("gaussian", k)
        cur.wait_stream(self.s1)
        cur.wait_stream(self.s2)

    def h2d(self, k):
        self.u8[k].copy_(self.h_u8[k], non_blocking=True)
        self.i32[k].copy_(self.u8[k])
        self.f32[k].copy_(self.u8[k])
        self.f32[k].mul_(1.0 / 255.0)

    def d2h(self, k):
        self.h_out.copy_(self.o_box[k], non_blocking=True)

    def e2e_bytes(self):
        return self.px, 4 * self.px

    def check(self):
        """Sampled rows against numpy restatements of the four definitions."""
        import torch
        k = 0
        self.step(k)
        torch.cuda.synchronize()
        x = self.u8[k].cpu().numpy()
        rows = [0, 1, 539, 1078, 1079]
        errs = {}
        xi = x.astype(np.int64)
        p2 = np.pad(xi, 2, mode="edge")
        cen = np.zeros((len(rows), self.W), np.uint64)
        for dy in range(5):
            for dx in range(5):
                nb = np.stack([p2[r + dy, dx:dx + self.W] for r in rows])
                cen = (cen << np.uint64(1)) | (nb < xi[rows]).astype(np.uint64)
        errs["census_rows_exact"] = bool(np.array_equal(self.o_census[k].cpu().numpy()[rows].view(np.uint32),
                                                       cen.astype(np.uint32)))
        p1 = np.pad(xi, 1, mode="edge")
        dil = np.max([[p1[r + dy, dx:dx + self.W] for r in rows] for dy in range(3) for dx in range(3)], axis=0)
        errs["dilate_rows_exact"] = bool(np.array_equal(self.o_dil[k].cpu().numpy()[rows], dil))
        c = np.pad(np.pad(xi, 7).cumsum(0).cumsum(1), ((1, 0), (1, 0)))
        box = np.stack([c[r + 15, 15:15 + self.W] - c[r, 15:15 + self.W] - c[r + 15, :self.W] + c[r, :self.W]
                        for r in rows])
        errs["box_rows_exact"] = bool(np.array_equal(self.o_box[k].cpu().numpy()[rows], box))
        kern = self.apps.gaussian_kernel(2.0).astype(np.float64)
        pf = np.pad(x.astype(np.float64) / 255.0, 6, mode="edge")
        hz = sum(kern[i] * pf[:, i:i + self.W] for i in range(13))
        gw = np.stack([sum(kern[i] * hz[r + i] for i in range(13)) for r in rows])
        got = self.o_g[k].cpu().numpy()[rows]
        errs["gaussian_max_rel_err"] = float(np.max(np.abs(got - gw) / np.maximum(np.abs(gw), 1e-3)))
        return errs

    def kernels(self, dev, peaks, n=20):
        fns = {name: (lambda nm: (lambda i: self._op(nm, i % self.n_rot)))(name)
               for name in ("census", "dilate", "box_sum", "gaussian")}
        return {name: time_launches(fn, self.n_rot, n) for name, fn in fns.items()}, None, None

    def cpu_setup(self):
        from umi_gb300 import apps
        self.apps_np = apps
        self.cx = np.random.default_rng(self.seed).integers(0, 256, (self.H, self.W), dtype=np.uint8)
        self.row = 0

    def cpu_step(self, nrows, threads):
        """The four operators on `nrows` rows of the frame in numpy (FP64 Gaussian)."""
        r0 = self.row % (self.H - nrows)
        self.row += nrows
        x = self.cx[max(r0 - 7, 0):r0 + nrows + 7].astype(np.int64)
        p2 = np.pad(x, 2, mode="edge")
        h, w = x.shape
        bits = np.zeros((h, w), np.uint64)
        for dy in range(5):
            for dx in range(5):
                bits = (bits << np.uint64(1)) | (p2[dy:dy + h, dx:dx + w] < x).astype(np.uint64)
        p1 = np.pad(x, 1, mode="edge")
        np.max([p1[dy:dy + h, dx:dx + w] for dy in range(3) for dx in range(3)], axis=0)
        c = np.pad(np.pad(x, 7).cumsum(0).cumsum(1), ((1, 0), (1, 0)))
        _ = c[15:15 + h, 15:15 + w] - c[:h, 15:15 + w] - c[15:15 + h, :w] + c[:h, :w]
        kern = self.apps_np.gaussian_kernel(2.0).astype(np.float64)
        pf = np.pad(x / 255.0, 6, mode="edge")
        hz = sum(kern[i] * pf[:, i:i + w] for i in range(13))
        _ = sum(kern[i] * hz[i:i + h] for i in range(13))
        return nrows * self.W / 1e6


class ServeBilateral:
    """Serving small batches (umi_gb300/serve.py): a request is 8 float32
    images of 512x512 through the batched bilateral 5x5 (sigma_s 2, sigma_r
    0.1).  value: requests/s of the recorded batch graph replayed with the
    images resident in HBM (8 rotating buffer sets); e2e: requests/s through
    BatchServer with 4 instances (streams) from host arrays: copy into pinned
    staging, upload, replay, download per request (wall clock); the same
    server with 1 instance is timed beside it."""
    name = "serve_bilateral_8x512"
    metric = "served requests/s (8 x 512x512 float32 bilateral 5x5 per request)"
    unit = "requests/s"
    dtype = "f32"
    N_IMG, S, INSTANCES = 8, 512, 4
    e2e_max_steps = 2000

    def __init__(self, seed=31, **_):
        self.seed = seed
        self.px = self.N_IMG * self.S * self.S

    def config(self):
        return {"workload": self.name, "request": f"{self.N_IMG} x {self.S}x{self.S} f32",
                "op": "bilateral r2 sigma_s 2 sigma_r 0.1", "instances": self.INSTANCES,
                "l2": "8 resident request buffers rotated (134 MB > L2)"}

    def units_per_step(self):
        return 1.0

    def setup(self, dev):
        import torch
        import umi_gb300 as U
        from umi_gb300 import serve
        self.U, self.serve, self.dev = U, serve, dev
        self.prm = U.BatchParams(2, 2.0, 0.1, 0, 0)
        g = np.random.default_rng(self.seed)
        shp = (self.S, self.S)
        self.reqs = [[g.random(shp, dtype=np.float32) for _ in range(self.N_IMG)] for _ in range(8)]
        self.n_rot = 8
        self.d_in = [[torch.from_numpy(x).to(dev) for x in r] for r in self.reqs]
        self.d_out = [[torch.empty(shp, dtype=torch.float32, device=dev) for _ in range(self.N_IMG)]
                      for _ in range(self.n_rot)]
        self.tables = [list(zip(self.d_in[k], [None] * self.N_IMG, self.d_out[k])) for k in range(self.n_rot)]
        self.launches_per_step = 1

    def step(self, i):
        # the batched launch a request's graph holds (the timed steps are themselves replayed from a graph)
        self.U.batch_run(self.U.OP_BILATERAL, self.tables[i % self.n_rot], self.prm)

    def e2e_bytes(self):
        return 4 * self.px, 4 * self.px

    def _serve(self, instances, n):
        import torch
        slots = [((self.S, self.S), None, (self.S, self.S))] * self.N_IMG
        srv = self.serve.BatchServer(self.U.OP_BILATERAL, slots, self.prm, instances=instances, device=self.dev)
        for r in self.reqs[:instances]:  # warm-up: graphs instantiated
            srv.submit(r)
        srv.drain()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        inflight = []
        for i in range(n):
            inflight.append(srv.submit(self.reqs[i % len(self.reqs)]))
            if len(inflight) == instances:  # consumed in place, before its instance is reused
                srv.result(inflight.pop(0), copy=False)
        for t in inflight:
            srv.result(t, copy=False)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        srv.close()
        return dt

    def e2e_run(self, steps, warmup):
        """ms for `steps` requests through BatchServer with INSTANCES streams."""
        dt = self._serve(self.INSTANCES, steps)
        self.one_instance_rps = steps / self._serve(1, steps)
        return dt * 1e3

    def check(self):
        """Every output of one served request against the direct call."""
        import torch
        srv = self.serve.BatchServer(self.U.OP_BILATERAL, [((self.S, self.S), None, (self.S, self.S))] * self.N_IMG,
                                     self.prm, instances=2, device=self.dev)
        out = srv.result(srv.submit(self.reqs[3]))
        srv.close()
        same = all(np.array_equal(o, self.U.bilateral_f32(torch.from_numpy(x).to(self.dev), 2, 2.0, 0.1).cpu().numpy())
                   for x, o in zip(self.reqs[3], out))
        return {"served_equals_direct": bool(same)}

    def kernels(self, dev, peaks, n=50):
        return {"bilateral_batch": time_launches(self.step, self.n_rot, n)}, None, 8 * self.px

    def cpu_setup(self):
        import oracle
        self.orc = oracle
        self.k = 0

    def cpu_step(self, nrows, threads):
        """FP64 bilateral of `nrows` rows of one 512x512 image of a request; units = requests."""
        x = self.reqs[self.k % len(self.reqs)][0] if hasattr(self, "reqs") else \
            np.random.default_rng(self.seed).random((self.S, self.S), dtype=np.float32)
        self.k += 1
        r0 = (self.k * nrows) % (self.S - nrows - 4)
        self.orc.bilateral_f64(np.ascontiguousarray(x[r0:r0 + nrows + 4]), 2, 2.0, 0.1, threads=threads)
        return nrows / (self.S * self.N_IMG)


WORKLOADS = {"int_pair_1080p": IntPair, "filter3x3_1024": Filter3x3, "batched_uneven": Batched, "gemm_4096": Gemm,
             "fprop_n32": Fprop, "learned_me_4k": LearnedMe, "coarse_me_4k": CoarseMe4k,
             "video_y4m_1080p": VideoY4M, "apps_1080p": Apps1080p, "serve_bilateral_8x512": ServeBilateral}


def time_launches(fn, period: int, n: int) -> float:
    """ms per launch of fn over n launches replayed from CUDA graphs."""
    import torch
    g = StepGraphs(fn, period)
    g.prepare(n)
    g.run(period)
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(st)
    g.run(n)
    b.record(st)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / n


def copy_gbs(dev, nbytes: int, n: int = 400) -> float:
    """GB/s of a device-to-device copy moving `nbytes` (read + write) per launch,
    rotating buffers so that consecutive copies touch more than L2: the
    bandwidth a memory-bound kernel of that size can reach at most."""
    import torch
    half = max(16, nbytes // 2)
    n_rot = max(2, -(-2 * L2_BYTES // (2 * half)))
    src = [torch.empty(half, dtype=torch.uint8, device=dev) for _ in range(n_rot)]
    dst = [torch.empty(half, dtype=torch.uint8, device=dev) for _ in range(n_rot)]
    ms = time_launches(lambda i: dst[i % n_rot].copy_(src[i % n_rot]), n_rot, n)
    return 2 * half / (ms * 1e-3) / 1e9


# --------------------------------------------------------------------- arms
def sad4_peak(dev):
    """Denominator of the integer-pipe roofline (byte absdiffs/s) and its
    source: the larger of the measured throughput of a loop of nothing but
    `vabsdiff4.add` (probe/sad4_peak.cu) and the issue-rate figure 64 SAD
    instructions/clk/SM x 4 bytes x SMs x the maximum SM clock (the ALU pipe
    takes a 32-lane warp instruction every 2 cycles per sub-partition)."""
    import torch
    measured = probe_sad4_peak(dev)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    mhz = 2070.0
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        mhz = float(json.load(open(path)).get("sm_max_mhz", mhz))
    derived = 64 * 4 * sms * mhz * 1e6
    peak = max(measured, derived)
    src = (f"max(measured vabsdiff4.add loop {measured / 1e9:.0f} G/s (probe/libumi_probe.so), "
           f"issue rate 64/clk/SM x 4 B x {sms} SMs x {mhz:.0f} MHz = {derived / 1e9:.0f} G/s)")
    return peak, src


def probe_sad4_peak(dev):
    """Measured throughput (byte absdiffs/s) of the packed SAD instruction."""
    import ctypes
    import torch
    from umi_gb300 import build
    L = ctypes.CDLL(build.PROBE_LIB)
    L.umi_probe_sad4_peak.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    L.umi_probe_sad4_ops.argtypes = [ctypes.c_int, ctypes.c_int]
    L.umi_probe_sad4_ops.restype = ctypes.c_double
    ctas, iters = torch.cuda.get_device_properties(dev).multi_processor_count * 8, 2048
    out = torch.empty(ctas * 256, dtype=torch.int32, device=dev)
    st = torch.cuda.current_stream()
    best = 0.0
    for _ in range(5):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(st)
        rc = L.umi_probe_sad4_peak(0, ctas, iters, ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(st.cuda_stream))
        b.record(st)
        torch.cuda.synchronize()
        assert rc == 0
        best = max(best, L.umi_probe_sad4_ops(ctas, iters) / (a.elapsed_time(b) * 1e-3))
    return best


class StepGraphs:
    """The steps of a workload captured in CUDA graphs (through the same C-ABI
    calls a user makes), so that the timed loop measures the GPU and not the
    Python launch path.  `run(k)` replays exactly k steps."""

    def __init__(self, fn, period: int):
        import torch
        self.period = period
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            for i in range(3):
                fn(i)
        torch.cuda.current_stream().wait_stream(side)
        torch.cuda.synchronize()
        self.graphs = {}
        self.fn = fn

    def graph(self, n: int):
        import torch
        if n not in self.graphs:
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                for i in range(n):
                    self.fn(i)
            self.graphs[n] = g
        return self.graphs[n]

    def run(self, k: int):
        full, rest = divmod(k, self.period)
        if full:
            g = self.graph(self.period)
            for _ in range(full):
                g.replay()
        if rest:
            self.graph(rest).replay()

    def prepare(self, k: int):
        """Capture every graph run(k) needs (capture outside the timed region)."""
        full, rest = divmod(k, self.period)
        if full:
            self.graph(self.period)
        if rest:
            self.graph(rest)


def e2e_pipelined(wl, steps: int, warmup: int, dist) -> float:
    """ms for `steps` end-to-end steps: every step copies its inputs from
    pinned host memory (wl.h2d), runs the operators through the C ABI
    (wl.step) and copies its results back (wl.d2h).  Uploads, compute and
    downloads run on three streams, ordered per buffer by events, so the
    copies of neighbouring steps overlap the compute of this one, as a
    serving loop would; all of every step's copies are inside the timed
    region."""
    import torch
    R = wl.n_rot
    s_c = torch.cuda.current_stream()
    s_in, s_out = torch.cuda.Stream(), torch.cuda.Stream()
    computed = [None] * R  # compute of the last step that used buffer k
    read = [None] * R      # download of the last step that used buffer k

    def one(i):
        k = i % R
        with torch.cuda.stream(s_in):
            if computed[k] is not None:
                s_in.wait_event(computed[k])  # its inputs are no longer read
            wl.h2d(k)
            e_in = torch.cuda.Event()
            e_in.record(s_in)
        s_c.wait_event(e_in)
        if read[k] is not None:
            s_c.wait_event(read[k])  # its outputs have been copied out
        wl.step(k)
        e_c = torch.cuda.Event()
        e_c.record(s_c)
        computed[k] = e_c
        with torch.cuda.stream(s_out):
            s_out.wait_event(e_c)
            wl.d2h(k)
            e_o = torch.cuda.Event()
            e_o.record(s_out)
            read[k] = e_o

    for i in range(warmup):
        one(i)
    torch.cuda.synchronize()
    dist.barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s_c)
    s_in.wait_event(e0)
    s_out.wait_event(e0)
    for i in range(warmup, warmup + steps):
        one(i)
    done = torch.cuda.Event()
    done.record(s_out)
    s_c.wait_event(done)
    e1.record(s_c)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def run_ours(args, wl, dist):
    import torch
    import umi_gb300 as U
    U.lib()  # the CUDA library must be present: no fallback
    torch.cuda.set_device(dist.local)
    dev = torch.device("cuda", dist.local)
    pk = peaks()
    wl.setup(dev)
    st = torch.cuda.current_stream()
    steps = StepGraphs(wl.step, wl.n_rot)
    steps.prepare(args.steps)
    steps.prepare(args.warmup)
    steps.run(args.warmup)
    torch.cuda.synchronize()
    clocks = Clocks(dist.local)
    clocks.start()
    dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.profiler.start()  # a profiler started with --profile-from-start off sees only the timed steps
    e0.record(st)
    steps.run(args.steps)
    e1.record(st)
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    dist.barrier()
    clk = clocks.stop()
    ms = dist.max(e0.elapsed_time(e1))
    value = wl.units_per_step() * args.steps * dist.world / (ms * 1e-3)
    sanity = wl.check()

    # e2e: host buffers, copies inside the timed region (eager C-ABI calls)
    if hasattr(wl, "e2e_setup"):
        wl.e2e_setup()
    e2e_steps = min(args.steps, getattr(wl, "e2e_max_steps", args.steps))
    if hasattr(wl, "e2e_run"):  # the workload's own public-API loop (host wall clock)
        ms_e2e = dist.max(wl.e2e_run(e2e_steps, min(args.warmup, 2)))
    else:
        ms_e2e = dist.max(e2e_pipelined(wl, e2e_steps, min(args.warmup, 2), dist))
    e2e_value = wl.units_per_step() * e2e_steps * dist.world / (ms_e2e * 1e-3)
    h2d, d2h = wl.e2e_bytes()

    # dominant kernel roofline
    kms, absdiff, hbm_bytes = wl.kernels(dev, pk)
    kernels = {}
    if isinstance(wl, IntPair):
        sad_peak, sad_src = sad4_peak(dev)
        ach = absdiff / (kms["full_me_u8"] * 1e-3)
        roof = {"bound": "int", "kernel": "full_me_u8", "achieved": ach / 1e9, "peak": sad_peak / 1e9,
                "unit": "Gabsdiff/s", "frac": ach / sad_peak, **traffic_fields(NCU_TRAFFIC[wl.name]),
                "peak_source": sad_src, "work_per_launch": absdiff, "ms_per_launch": kms["full_me_u8"]}
        ig = hbm_bytes / (kms["iimg_u8_i32"] * 1e-3) / 1e9
        cg = copy_gbs(dev, hbm_bytes)
        kernels["iimg_u8_i32"] = {"ms_per_launch": kms["iimg_u8_i32"], "achieved": ig, "unit": "GB/s",
                                  "peak": pk["hbm_gbs"], "frac": ig / pk["hbm_gbs"], "bytes_per_launch": hbm_bytes,
                                  "peak_source": pk["source"], "size_matched_copy_gbs": cg,
                                  "frac_of_size_matched_copy": ig / cg}
    elif isinstance(wl, Gemm):
        for name, kt in kms.items():
            if name == "gemm_f32_umi_generic_256rows":
                f = wl.flops * 256 / wl.M
                kernels[name] = {"ms_per_launch": kt, "fp32_gemm_tflops": f / (kt * 1e-3) / 1e12,
                                 "note": "plain fp32 FMA through the generic operator, 256 of the 4096 rows"}
                continue
            f = wl.flops * (3 if name in ("gemm_f32_bf16x3", "gemm_f32_f16x3") else 1)
            kernels[name] = {"ms_per_launch": kt, "achieved": f / (kt * 1e-3) / 1e12, "unit": "TFLOP/s",
                             "frac": f / (kt * 1e-3) / 1e12 / pk["bf16_tflops"],
                             "note": "3 half-precision products per fp32 product (plus the operand split); "
                                     "achieved counts tensor FLOPs"
                             if name in ("gemm_f32_bf16x3", "gemm_f32_f16x3") else None}
        for name in ("gemm_f32_bf16x3", "gemm_f32_f16x3"):
            kernels[name]["fp32_gemm_tflops"] = wl.flops / (kms[name] * 1e-3) / 1e12
        roof = dict(kernels["gemm_bf16"], bound="tensor", kernel="gemm_tc_kernel (bf16)", peak=pk["bf16_tflops"],
                    **traffic_fields(NCU_TRAFFIC.get(wl.name), 4 * wl.M * wl.N), peak_source=pk["source"] + " (burst)",
                    flops_per_launch=wl.flops)
    elif isinstance(wl, Fprop):
        kt = kms["conv2d_fprop_bf16"]
        ach = wl.flops / (kt * 1e-3) / 1e12
        # compulsory bytes: bf16 NHWC input + bf16 weights read once, fp32 NCHW output written once
        nbytes = 2 * wl.N * wl.H * wl.W * wl.C + 2 * wl.K * wl.R * wl.R * wl.C + 4 * wl.N * wl.K * wl.H * wl.W
        gbs = nbytes / (kt * 1e-3) / 1e9
        kernels["conv2d_fprop_bf16"] = {"ms_per_launch": kt, "achieved": ach, "unit": "TFLOP/s",
                                        "frac": ach / pk["bf16_tflops"], "bytes_per_launch": nbytes,
                                        "achieved_gbs": gbs, "frac_of_hbm": gbs / pk["hbm_gbs"],
                                        "tensor_floor_ms": wl.flops / (pk["bf16_tflops"] * 1e12) * 1e3,
                                        "hbm_floor_ms": nbytes / (pk["hbm_gbs"] * 1e9) * 1e3}
        kt3 = kms["conv2d_fprop_f32_f16x3"]
        kernels["conv2d_fprop_f32_f16x3"] = {"ms_per_launch": kt3, "fp32_conv_tflops": wl.flops / (kt3 * 1e-3) / 1e12,
                                             "tensor_tflops": 3 * wl.flops / (kt3 * 1e-3) / 1e12,
                                             "note": "fp32 inputs split f16 hi/lo (3 products), fp32-level accuracy"}
        k = kernels["conv2d_fprop_bf16"]
        if k["hbm_floor_ms"] >= k["tensor_floor_ms"]:  # the fp32 output makes the launch HBM-bound
            roof = {"bound": "hbm", "kernel": "strip_run_kernel<ConvRun> (bf16)", "achieved": gbs, "peak": pk["hbm_gbs"],
                    "unit": "GB/s", "frac": gbs / pk["hbm_gbs"],
                    **traffic_fields(NCU_TRAFFIC.get(wl.name), 4 * wl.N * wl.K * wl.H * wl.W),
                    "peak_source": pk["source"], "bytes_per_launch": nbytes, "ms_per_launch": kt,
                    "tensor_frac": k["frac"]}
        else:
            roof = dict(k, bound="tensor", kernel="strip_run_kernel<ConvRun> (bf16)", peak=pk["bf16_tflops"],
                        **traffic_fields(NCU_TRAFFIC.get(wl.name), 4 * wl.N * wl.K * wl.H * wl.W),
                        peak_source=pk["source"] + " (burst)",
                        flops_per_launch=wl.flops)
    elif isinstance(wl, LearnedMe):
        sad_peak, sad_src = sad4_peak(dev)
        for name, kt in kms.items():
            kernels[name] = {"ms_per_launch": kt, "Mblocks_per_s": wl.nblk / (kt * 1e-3) / 1e6}
        kernels["speedup_learned_vs_full_search"] = kms["full_me_u8_r64"] / kms["me_learned_u8"]
        if isinstance(wl, CoarseMe4k):
            kernels["speedup_coarse_vs_full_search"] = kms["full_me_u8_r64"] / kms["me_coarse_u8"]
            roof_k, roof_name = "coarse_centers", "coarse_cells + coarse_search (the proposal)"
        else:
            roof_k, roof_name = "full_me_u8_r64", "full_me_u8 +-64 (judge and fallback)"
        ach = absdiff / (kms[roof_k] * 1e-3)
        roof = {"bound": "int", "kernel": roof_name, "achieved": ach / 1e9,
                "peak": sad_peak / 1e9, "unit": "Gabsdiff/s", "frac": ach / sad_peak,
                **traffic_fields(NCU_TRAFFIC[wl.name]), "peak_source": sad_src,
                "work_per_launch": absdiff, "ms_per_launch": kms[roof_k]}
    elif isinstance(wl, ServeBilateral):
        kt = kms["bilateral_batch"]
        ach = hbm_bytes / (kt * 1e-3) / 1e9
        kernels["bilateral_batch"] = {"ms_per_launch": kt, "achieved": ach, "unit": "GB/s", "frac": ach / pk["hbm_gbs"],
                                      "bytes_per_launch": hbm_bytes, "ex2_per_s": 25 * wl.px / (kt * 1e-3)}
        kernels["served_requests_per_s_one_instance"] = getattr(wl, "one_instance_rps", None)
        roof = dict(kernels["bilateral_batch"], bound="hbm", kernel="batch_kernel<Bilateral> (graph replay)",
                    peak=pk["hbm_gbs"], traffic=None, peak_source=pk["source"])
    elif isinstance(wl, Apps1080p):
        for name, kt in kms.items():
            b = wl.BYTES[name] * wl.px
            kernels[name] = {"ms_per_launch": kt, "achieved": b / (kt * 1e-3) / 1e9, "unit": "GB/s",
                             "frac": b / (kt * 1e-3) / 1e9 / pk["hbm_gbs"], "bytes_per_launch": b}
        dom = max(kms, key=kms.get)
        cg = copy_gbs(dev, wl.BYTES[dom] * wl.px)
        roof = dict(kernels[dom], bound="hbm", kernel=f"generic_kernel ({dom})", peak=pk["hbm_gbs"], traffic=None,
                    peak_source=pk["source"], size_matched_copy_gbs=cg,
                    frac_of_size_matched_copy=kernels[dom]["achieved"] / cg)
    elif isinstance(wl, VideoY4M):
        sad_peak, sad_src = sad4_peak(dev)
        for name, kt in kms.items():
            kernels[name] = {"ms_per_launch": kt, "pairs_per_s": 1e3 / kt}
        kernels["speedup_coarse_vs_full_search"] = kms["full_me_u8_r64"] / kms["me_coarse_u8"]
        ach = absdiff / (kms["coarse_centers"] * 1e-3)
        roof = {"bound": "int", "kernel": "coarse_cells + coarse_search (the proposal)", "achieved": ach / 1e9,
                "peak": sad_peak / 1e9, "unit": "Gabsdiff/s", "frac": ach / sad_peak, "traffic": None,
                "peak_source": sad_src,
                "work_per_launch": absdiff, "ms_per_launch": kms["coarse_centers"]}
    elif isinstance(wl, Batched):
        for name, kt in kms.items():
            b = (sum(wl.BYTES.values()) if name.endswith("_step") else wl.BYTES[name]) * wl.px
            kernels[name] = {"ms_per_launch": kt, "achieved": b / (kt * 1e-3) / 1e9, "unit": "GB/s",
                             "frac": b / (kt * 1e-3) / 1e9 / pk["hbm_gbs"], "bytes_per_launch": b}
        kernels["bilateral"]["ex2_per_s"] = 25 * wl.px / (kms["bilateral"] * 1e-3)
        kernels["fused_step"]["note"] = "the three operators in one launch; the others are each operator alone"
        kernels["three_launches_step"]["note"] = "the same step as three launches (one kernel per operator)"
        roof = dict(kernels["fused_step"], bound="hbm", kernel="batch_fused_kernel (all three operators)",
                    peak=pk["hbm_gbs"],
                    **traffic_fields(tuple(v * wl.px for v in NCU_TRAFFIC_PER_PX["batched_uneven"]),
                                     (256 + 4 + 4) * wl.px),
                    peak_source=pk["source"])
    else:
        ach = hbm_bytes / (kms["filter3x3_f32"] * 1e-3) / 1e9
        cg = copy_gbs(dev, hbm_bytes)
        roof = {"bound": "hbm", "kernel": "filter3x3_f32", "achieved": ach, "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": ach / pk["hbm_gbs"], **traffic_fields(NCU_TRAFFIC[wl.name], hbm_bytes // 2),
                "peak_source": pk["source"], "bytes_per_launch": hbm_bytes, "ms_per_launch": kms["filter3x3_f32"],
                "size_matched_copy_gbs": cg, "frac_of_size_matched_copy": ach / cg}

    line = {
        "metric": wl.metric, "value": value, "unit": wl.unit, "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": wl.dtype, "data": getattr(wl, "data", "synthetic (seeded numpy generators)"),
        "config": dict(wl.config(), parallelism=f"replicas x{dist.world}"),
        "e2e": {"value": e2e_value, "unit": wl.unit, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": ms_e2e / e2e_steps, "steps": e2e_steps,
                "schedule": "pinned host buffers; upload, compute, download on three streams"},
        "gpu_launches": wl.launches_per_step * args.steps,
        "roofline": roof, "kernels": kernels, "clocks": clk,
        "impl": "ours",
    }
    if sanity is not None:
        key = {IntPair: "sanity_true_mv_recovered", Gemm: "errors_vs_fp64_sampled_rows",
               Fprop: "errors_vs_fp64", LearnedMe: "quality_vs_exhaustive_search",
               CoarseMe4k: "quality_vs_exhaustive_search", VideoY4M: "quality_vs_exhaustive_search"}.get(
                   type(wl), "sanity_max_rel_err_sampled")
        line[key] = sanity
    if dist.rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(wl, sample_s=10.0)
    return line


def cpu_baseline(wl, sample_s=10.0):
    """The reference's CPU loop (oracle restatement) on a bounded sample, all host threads."""
    threads = os.cpu_count() or 1
    wl.cpu_setup()
    if isinstance(wl, ServeBilateral):
        chunk, what = 16, "rows of one 512x512 request image through the FP64 bilateral 5x5 (units = requests of 8 images)"
    elif isinstance(wl, Apps1080p):
        chunk, what = 16, "rows of the 1080p frame through numpy restatements of census 5x5, dilation 3x3, box 15x15 (integral image) and the FP64 separable Gaussian (the reference has none of these: its operator has no CPU path)"
    elif isinstance(wl, VideoY4M):
        chunk, what = 8, "random blocks of a 1080p pair of the video, +-64 full search with per-pixel clamp (main/full_me.cu:68-87) + argmin (the reference has no I/O and no proposal), units = pairs"
    elif isinstance(wl, LearnedMe):
        chunk, what = 8, "random blocks of a 4K pair, +-64 full search with per-pixel clamp (main/full_me.cu:68-87) + argmin (the reference has no learned path)"
    elif isinstance(wl, IntPair):
        chunk, what = 256, "random blocks of the 1080p pair, +-32 full search with per-pixel clamp (main/full_me.cu:68-87) + argmin, plus the matching rows of iimg (main/iimg.cu:100-111)"
    elif isinstance(wl, Fprop):
        chunk, what = 8, "output rows of one 64-channel 128x128 image through the reference's direct convolution loop (main/fprop.cu:84-108), FP64"
    elif isinstance(wl, Gemm):
        chunk, what = 4, "rows of the 4096^3 product, the reference's gemm loop (main/gemm.cu:69-78) with FP64 accumulation"
    elif isinstance(wl, Batched):
        chunk, what = 8, "rows of 1024-wide crops through the FP64 restatements of bilateral 5x5, per-pixel wfilter3x3 and the 32x64 dot cost volume"
    else:
        chunk, what = 128, "rows of the 1024x1024 image, 3x3 weighted sum in FP64"
    units, t0 = 0.0, time.perf_counter()
    n = 0
    while time.perf_counter() - t0 < sample_s and n < 4096:
        units += wl.cpu_step(chunk, threads)
        n += 1
    dt = time.perf_counter() - t0
    return {"value": units / dt, "unit": wl.unit, "cores": threads, "kind": "port",
            "sample": f"{n} x {chunk} {what}; {dt:.1f} s"}


def run_reference(args, wl, dist):
    """The reference's own CPU implementation of the path (restated in the oracle), host cores only."""
    if dist.rank != 0:
        return None
    threads = os.cpu_count() or 1
    wl.cpu_setup()
    base = {IntPair: 32, Batched: 2, Gemm: 2, Fprop: 2, LearnedMe: 8, CoarseMe4k: 8, VideoY4M: 8}.get(type(wl), 16)
    cap = {IntPair: 8040, Batched: 512, Gemm: 256, Fprop: 126, LearnedMe: 32400, CoarseMe4k: 32400,
           VideoY4M: 8040}.get(type(wl), 1024)
    # each step a bounded sample of the workload: calibrate on one call, then
    # size the sample to about 0.4 s per step (at most 90 s for the whole run)
    t0 = time.perf_counter()
    wl.cpu_step(base, threads)
    dt1 = max(time.perf_counter() - t0, 1e-6)
    target = min(0.4, 90.0 / max(1, args.steps + args.warmup))
    per_step = int(min(cap, max(base, base * target / dt1)))
    for _ in range(args.warmup):
        wl.cpu_step(per_step, threads)
    t0 = time.perf_counter()
    units = 0.0
    for _ in range(args.steps):
        units += wl.cpu_step(per_step, threads)
    dt = time.perf_counter() - t0
    v = units / dt
    return {
        "metric": wl.metric, "value": v, "unit": wl.unit, "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": wl.dtype, "data": "synthetic (seeded numpy generators)",
        "config": dict(wl.config(), parallelism="host cores"), "impl": "reference",
        "cpu_baseline": {"value": v, "unit": wl.unit, "cores": threads, "kind": "port",
                         "sample": f"{per_step} {'blocks' if isinstance(wl, (IntPair, LearnedMe, VideoY4M)) else 'rows'} per step"},
        "e2e": {"value": v, "unit": wl.unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
    }


def main():
    args = parse()
    wl = WORKLOADS[args.workload](n=args.images) if args.workload == "batched_uneven" else WORKLOADS[args.workload]()
    if args.impl == "reference":
        dist = Dist("gloo")
        line = run_reference(args, wl, dist)
    else:
        dist = Dist("nccl")
        line = run_ours(args, wl, dist)
    if dist.rank == 0 and line is not None:
        print(json.dumps(line, default=float), flush=True)
    dist.done()


if __name__ == "__main__":
    main()
