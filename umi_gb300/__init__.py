"""umi_gb300: GB300 (sm_103a) implementation of the UMI operator.

Python bindings over the C ABI of libumi_gb300.so (include/umi_gb300.h).
Every call goes straight to a CUDA kernel of this library on the caller's
current torch CUDA stream; there is no CPU fallback.  If the library is
missing, importing works but the first call raises UmiLibraryMissing (build
it with `python -m umi_gb300.build`).

torch is used only as the device-memory and stream provider: tensors are
passed to the C ABI as raw pointers.
"""
from __future__ import annotations

import ctypes
import os
import re

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
LIB_PATH = os.path.join(PKG, "libumi_gb300.so")
HEADER = os.path.join(ROOT, "include", "umi_gb300.h")

UMI_OK = 0
UMI_ERR_UNSUPPORTED = 3
STATUS_NAMES = {
    0: "UMI_OK", 1: "UMI_ERR_INVALID_DESC", 2: "UMI_ERR_INVALID_ARG", 3: "UMI_ERR_UNSUPPORTED",
    4: "UMI_ERR_CUDA", 5: "UMI_ERR_NO_MEMORY", 6: "UMI_ERR_TIMEOUT",
}


class UmiLibraryMissing(RuntimeError):
    pass


class UmiError(RuntimeError):
    def __init__(self, status: int, fn: str, detail: str):
        self.status = status
        super().__init__(f"{fn}: {STATUS_NAMES.get(status, status)}: {detail}")


_LIB = None

_vp = ctypes.c_void_p
_i32 = ctypes.c_int32
_f32 = ctypes.c_float
_sz = ctypes.c_size_t

# C signatures (argtypes, restype) of every entry point in include/umi_gb300.h.
SIGNATURES = {
    "umi_status_string": ([ctypes.c_int], ctypes.c_char_p),
    "umi_last_error_string": ([], ctypes.c_char_p),
    "umi_version": ([], ctypes.c_int),
    "umi_plan_build": ([_vp, _vp], ctypes.c_int),
    "umi_plan_create": ([_vp, _vp], ctypes.c_int),
    "umi_plan_destroy": ([_vp], None),
    "umi_launch": ([_vp, _i32, _vp, _vp, _vp, _vp, _sz, _vp], ctypes.c_int),
    "umi_batch_graph_create": ([_vp], ctypes.c_int),
    "umi_batch_graph_add": ([_vp, _i32, _vp, _i32, _vp, _i32], ctypes.c_int),
    "umi_batch_graph_launch": ([_vp, _vp], ctypes.c_int),
    "umi_batch_fused_variants": ([_i32], _i32),
    "umi_batch_run_fused": ([_vp, _i32, _vp], ctypes.c_int),
    "umi_batch_graph_add_fused": ([_vp, _vp, _i32], ctypes.c_int),
    "umi_batch_graph_destroy": ([_vp], None),
    "umi_filter3x3_f32": ([_vp, _vp, _i32, _i32, _vp, _f32, _vp], ctypes.c_int),
    "umi_filter3x3_f32_tma": ([_vp, _vp, _i32, _i32, _vp, _vp], ctypes.c_int),
    "umi_iimg_u8_i32_workspace_bytes": ([_i32, _i32], _sz),
    "umi_iimg_u8_i32": ([_vp, _vp, _i32, _i32, _vp, _sz, _vp], ctypes.c_int),
    "umi_iimg_u8_i32_noalloc": ([_vp, _vp, _i32, _i32, _vp], ctypes.c_int),
    "umi_iimg_noalloc_forget": ([], None),
    "umi_full_me_u8": ([_vp, _vp, _i32, _i32, _i32, _i32, _vp, _vp, _vp], ctypes.c_int),
    "umi_full_me_sad_u8": ([_vp, _vp, _i32, _i32, _i32, _i32, _vp, _vp], ctypes.c_int),
    "umi_full_me_error": ([_vp, _vp], ctypes.c_int),
    "umi_full_me_u8_list": ([_vp, _vp, _i32, _i32, _i32, _i32, _vp, _vp, _vp, _i32, _vp, _vp], ctypes.c_int),
    "umi_menet_param_count": ([], _i32),
    "umi_menet_workspace_bytes": ([_i32, _i32], _sz),
    "umi_menet_forward": ([_vp, _vp, _i32, _i32, _vp, _vp, _vp, _sz, _vp], ctypes.c_int),
    "umi_menet_backward": ([_vp, _i32, _i32, _i32, _vp, _vp, _vp, _vp, _sz, _vp], ctypes.c_int),
    "umi_menet_adam": ([_vp, _vp, _vp, _vp, _i32, _f32, _vp], ctypes.c_int),
    "umi_menet_infer": ([_vp, _vp, _i32, _i32, _vp, _vp, _vp, _vp, _sz, _vp], ctypes.c_int),
    "umi_me_learned_u8": ([_vp, _vp, _i32, _i32, _vp, _i32, _i32, _i32, _i32, _vp, _vp, _vp, _vp, _sz, _vp],
                          ctypes.c_int),
    "umi_me_coarse_workspace_bytes": ([_i32, _i32], _sz),
    "umi_me_coarse_centers_u8": ([_vp, _vp, _i32, _i32, _i32, _vp, _vp, _sz, _vp], ctypes.c_int),
    "umi_me_coarse_u8": ([_vp, _vp, _i32, _i32, _i32, _i32, _i32, _i32, _vp, _vp, _vp, _vp, _sz, _vp], ctypes.c_int),
    "umi_bilateral_f32": ([_vp, _vp, _i32, _i32, _i32, _f32, _f32, _vp], ctypes.c_int),
    "umi_wfilter3x3_pp_f32": ([_vp, _vp, _vp, _i32, _i32, _vp], ctypes.c_int),
    "umi_cost_volume_dot_f32": ([_vp, _vp, _vp, _i32, _i32, _i32, _i32, _vp], ctypes.c_int),
    "umi_gemm_bf16": ([_vp, _vp, _vp, _i32, _i32, _i32, _vp, _vp], ctypes.c_int),
    "umi_gemm_f16": ([_vp, _vp, _vp, _i32, _i32, _i32, _vp, _vp], ctypes.c_int),
    "umi_gemm_bf16_wait_limit": ([_vp, _vp, _vp, _i32, _i32, _i32, _vp, ctypes.c_ulonglong, _vp], ctypes.c_int),
    "umi_err_status": ([_i32], ctypes.c_int),
    "umi_gemm_f32_bf16x3_workspace_bytes": ([_i32, _i32, _i32], _sz),
    "umi_gemm_f32_bf16x3": ([_vp, _vp, _vp, _i32, _i32, _i32, _vp, _sz, _vp, _vp], ctypes.c_int),
    "umi_gemm_f32_f16x3_workspace_bytes": ([_i32, _i32, _i32], _sz),
    "umi_gemm_f32_f16x3": ([_vp, _vp, _vp, _i32, _i32, _i32, _i32, _vp, _sz, _vp, _vp], ctypes.c_int),
    "umi_conv2d_fprop_f32_f16x3_workspace_bytes": ([_i32, _i32, _i32, _i32, _i32, _i32], _sz),
    "umi_conv2d_fprop_f32_f16x3": ([_vp, _vp, _vp, _i32, _i32, _i32, _i32, _i32, _i32, _i32, _vp, _sz, _vp, _vp],
                                   ctypes.c_int),
    "umi_conv2d_fprop_bf16": ([_vp, _vp, _vp, _i32, _i32, _i32, _i32, _i32, _i32, _vp, _vp], ctypes.c_int),
    "umi_batch_variants": ([_i32], _i32),
    "umi_batch_run": ([_i32, _vp, _i32, _vp, _i32, _vp], ctypes.c_int),
    "umi_autotune_batch": ([_i32, _vp, _i32, _vp, _i32, _vp, _vp, _vp], ctypes.c_int),
}


# ---- descriptor structs (mirror include/umi_gb300.h) ----

class PDim(ctypes.Structure):
    _fields_ = [("total_size", _i32), ("block_size", _i32), ("warp_size", _i32), ("warp_shuf", _i32)]


class ADim(ctypes.Structure):
    _fields_ = [("total_size", _i32), ("block_size", _i32)]


class VDim(ctypes.Structure):
    _fields_ = [("physical_dim_id", _i32), ("ofs", _i32), ("stride", _i32)]


class PhyDim(ctypes.Structure):
    _fields_ = [("size", _i32), ("mode", _i32)]


class MemDesc(ctypes.Structure):
    _fields_ = [("p_view", VDim * 4), ("a_view", VDim * 4), ("phys", PhyDim * 4), ("stage", _i32), ("n_ptr", _i32)]


class Desc(ctypes.Structure):
    _fields_ = [("p", PDim * 4), ("a", ADim * 4), ("expand", ctypes.c_uint32), ("n_in", _i32), ("n_out", _i32),
                ("mem", MemDesc * 16)]


class MemPlan(ctypes.Structure):
    _fields_ = [("base", _i32 * 4), ("pcoef", (_i32 * 4) * 4), ("acoef", (_i32 * 4) * 4), ("size", _i32 * 4),
                ("rowstride", ctypes.c_int64 * 4), ("pad_mask", _i32), ("stage", _i32), ("n_ptr", _i32),
                ("is_output", _i32)]


class Plan(ctypes.Structure):
    _fields_ = [("ptotal", _i32 * 4), ("block", _i32 * 4), ("expand", _i32 * 4), ("grid", _i32 * 4),
                ("n_cta", ctypes.c_int64), ("n_threads", _i32), ("atotal", _i32 * 4), ("ablock", _i32 * 4),
                ("agrid", _i32 * 4), ("n_ablock", _i32), ("ablock_size", _i32), ("n_in", _i32), ("n_out", _i32),
                ("mem", MemPlan * 16)]


PAD, WRAP = 0, 1


def make_desc(p, a, mems, expand: int = 0x1111, n_in: int | None = None) -> Desc:
    """Build a Desc from python lists.

    p: 4 tuples (total, block, warp, shuf); a: 4 tuples (total, block);
    mems: list of dicts {p_view: 4 (dim, ofs, stride), a_view: ..., phys: 4 (size, mode),
    stage: 0/1/2, n_ptr: int, out: bool}; inputs must precede outputs."""
    d = Desc()
    for i, t in enumerate(p):
        t = tuple(t) + (0,) * (4 - len(t))
        d.p[i] = PDim(*t)
    for i, t in enumerate(a):
        d.a[i] = ADim(*t)
    d.expand = expand
    ins = [m for m in mems if not m.get("out")]
    outs = [m for m in mems if m.get("out")]
    d.n_in = len(ins) if n_in is None else n_in
    d.n_out = len(outs)
    for i, m in enumerate(ins + outs):
        md = d.mem[i]
        for k, v in enumerate(m.get("p_view", [()] * 4)):
            md.p_view[k] = VDim(*(tuple(v) + (0,) * (3 - len(v))))
        for k, v in enumerate(m.get("a_view", [()] * 4)):
            md.a_view[k] = VDim(*(tuple(v) + (0,) * (3 - len(v))))
        for k, v in enumerate(m.get("phys", [()] * 4)):
            md.phys[k] = PhyDim(*(tuple(v) + (0,) * (2 - len(v))))
        md.stage = m.get("stage", 1)
        md.n_ptr = m.get("n_ptr", 1)
    return d


def plan_build(desc: Desc) -> Plan:
    """Validate a descriptor and return its launch plan (umi_plan_build)."""
    plan = Plan()
    check(lib().umi_plan_build(ctypes.byref(desc), ctypes.byref(plan)), "umi_plan_build")
    return plan


(STRATEGY_NEIGHBOUR_SUM_I32, STRATEGY_WEIGHTED_SUM_I32, STRATEGY_RANGE_WEIGHTED_F32, STRATEGY_ABS_DIFF_SUM_I32,
 STRATEGY_RUNNING_SUM_I32, STRATEGY_DOT_I32, STRATEGY_DOT_F32, STRATEGY_CENSUS_I32, STRATEGY_WEIGHTED_SUM_F32,
 STRATEGY_MAX_I32, STRATEGY_MIN_I32) = range(11)
_STRATEGY_FLOAT = {STRATEGY_RANGE_WEIGHTED_F32, STRATEGY_DOT_F32, STRATEGY_WEIGHTED_SUM_F32}


def launch(desc: Desc, strategy: int, ins, outs, pads=None, consts=None, stream=None) -> None:
    """Generic operator with a built-in strategy (umi_plan_create + umi_launch + umi_plan_destroy).

    ins / outs: CUDA tensors (int32 or float32, per the strategy), one per
    memory in the descriptor's order; pads: one padding value per input;
    consts: the strategy's constants as a sequence of numbers (int32 or
    float32 by strategy)."""
    import numpy as np
    import torch
    is_f = strategy in _STRATEGY_FLOAT
    et = torch.float32 if is_f else torch.int32
    for i, t in enumerate(list(ins) + list(outs)):
        _need(t, et, f"memory {i}")
    plan = ctypes.c_void_p()
    check(lib().umi_plan_create(ctypes.byref(desc), ctypes.byref(plan)), "umi_plan_create")
    try:
        inp = (ctypes.c_void_p * max(1, len(ins)))(*[t.data_ptr() for t in ins])
        outp = (ctypes.c_void_p * max(1, len(outs)))(*[t.data_ptr() for t in outs])
        pad = None
        if pads is not None:
            pad = np.ascontiguousarray(pads, dtype=np.float32 if is_f else np.int32)
        uc = None
        if consts is not None:
            uc = np.ascontiguousarray(consts, dtype=np.float32 if is_f else np.int32)
        check(lib().umi_launch(plan, strategy, inp, pad.ctypes.data_as(ctypes.c_void_p) if pad is not None else None,
                               outp, uc.ctypes.data_as(ctypes.c_void_p) if uc is not None else None,
                               uc.nbytes if uc is not None else 0, _stream_ptr(stream)), "umi_launch")
    finally:
        lib().umi_plan_destroy(plan)


class BatchGraph:
    """A sequence of batched launches recorded once and replayed (umi_batch_graph_*)."""

    def __init__(self):
        self._h = ctypes.c_void_p()
        check(lib().umi_batch_graph_create(ctypes.byref(self._h)), "umi_batch_graph_create")
        self._keep = []

    def add(self, op: int, images, params=None, variant: int = -1):
        """Record one batched launch: images = [(in, aux_or_None, out), ...] as batch_run."""
        table = _batch_table(images)
        prm = params if params is not None else BatchParams()
        check(lib().umi_batch_graph_add(self._h, op, table, len(images), ctypes.byref(prm), variant),
              "umi_batch_graph_add")
        self._keep.append((table, prm))

    def add_fused(self, jobs):
        """Record one fused launch (batch_run_fused's job list)."""
        arr, keep = _fused_jobs(jobs)
        check(lib().umi_batch_graph_add_fused(self._h, arr, len(jobs)), "umi_batch_graph_add_fused")
        self._keep.append((arr, keep))

    def launch(self, stream=None):
        check(lib().umi_batch_graph_launch(self._h, _stream_ptr(stream)), "umi_batch_graph_launch")

    def close(self):
        if self._h:
            lib().umi_batch_graph_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def header_functions() -> list[str]:
    """Names of the functions declared in include/umi_gb300.h."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*(umi_[a-z0-9_]+)\s*\(", text, flags=re.M)


def lib():
    """Load libumi_gb300.so (raises UmiLibraryMissing if it was not built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise UmiLibraryMissing(f"{LIB_PATH} not built: run `python -m umi_gb300.build`")
        L = ctypes.CDLL(LIB_PATH)
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _LIB = L
    return _LIB


def check(status: int, fn: str) -> None:
    if status != UMI_OK:
        detail = lib().umi_last_error_string().decode(errors="replace")
        raise UmiError(status, fn, detail)


def _stream_ptr(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _need(t, dtype, name):
    import torch
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype}, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")


def filter3x3_f32(inp, w9, pad: float = 0.0, out=None, stream=None):
    """3x3 weighted filter of a float32 (h, w) CUDA tensor (umi_filter3x3_f32)."""
    import torch
    _need(inp, torch.float32, "inp")
    h, w = inp.shape
    if out is None:
        out = torch.empty_like(inp)
    _need(out, torch.float32, "out")
    wv = (ctypes.c_float * 9)(*[float(v) for v in list(w9)])
    check(lib().umi_filter3x3_f32(_ptr(inp), _ptr(out), h, w, wv, float(pad), _stream_ptr(stream)),
          "umi_filter3x3_f32")
    return out


def filter3x3_f32_tma(inp, w9, out=None, stream=None):
    """The zero-padded 3x3 filter through TMA-staged halo tiles (umi_filter3x3_f32_tma)."""
    import torch
    _need(inp, torch.float32, "inp")
    h, w = inp.shape
    if out is None:
        out = torch.empty_like(inp)
    _need(out, torch.float32, "out")
    wv = (ctypes.c_float * 9)(*[float(v) for v in list(w9)])
    check(lib().umi_filter3x3_f32_tma(_ptr(inp), _ptr(out), h, w, wv, _stream_ptr(stream)), "umi_filter3x3_f32_tma")
    return out


def iimg_workspace_bytes(h: int, w: int) -> int:
    return int(lib().umi_iimg_u8_i32_workspace_bytes(h, w))


def iimg_u8_i32(inp, out=None, workspace=None, stream=None):
    """Integral image of a uint8 (h, w) CUDA tensor into int32 (umi_iimg_u8_i32)."""
    import torch
    _need(inp, torch.uint8, "inp")
    h, w = inp.shape
    if out is None:
        out = torch.empty((h, w), dtype=torch.int32, device=inp.device)
    _need(out, torch.int32, "out")
    nbytes = iimg_workspace_bytes(h, w)
    if workspace is None:
        workspace = torch.empty(max(nbytes, 16), dtype=torch.uint8, device=inp.device)
    check(lib().umi_iimg_u8_i32(_ptr(inp), _ptr(out), h, w, _ptr(workspace), workspace.numel(),
                                _stream_ptr(stream)), "umi_iimg_u8_i32")
    return out


def full_me_u8(cur, ref, block: int = 16, search: int = 32, centers=None, out=None, stream=None):
    """Full-search motion estimation with argmin (umi_full_me_u8).

    Returns an int32 (h//block * w//block, 3) tensor of (mv_y, mv_x, sad)."""
    import torch
    _need(cur, torch.uint8, "cur")
    _need(ref, torch.uint8, "ref")
    if cur.shape != ref.shape:
        raise ValueError("cur and ref differ in shape")
    h, w = cur.shape
    n = (h // block) * (w // block)
    if out is None:
        out = torch.empty((n, 3), dtype=torch.int32, device=cur.device)
    _need(out, torch.int32, "out")
    if centers is not None:
        _need(centers, torch.int32, "centers")
    check(lib().umi_full_me_u8(_ptr(cur), _ptr(ref), h, w, block, search, _ptr(centers), _ptr(out),
                               _stream_ptr(stream)), "umi_full_me_u8")
    return out


def full_me_u8_list(cur, ref, blocks, n_blocks, out, block: int = 16, search: int = 32, centers=None,
                    stream=None):
    """Full search of the listed blocks only (umi_full_me_u8_list).

    blocks: int32 CUDA tensor of block indices; n_blocks: int32 CUDA tensor
    whose first element is how many of them to search; out: the (nblk, 3)
    int32 tensor whose listed rows are overwritten."""
    import torch
    _need(cur, torch.uint8, "cur")
    _need(ref, torch.uint8, "ref")
    _need(blocks, torch.int32, "blocks")
    _need(n_blocks, torch.int32, "n_blocks")
    _need(out, torch.int32, "out")
    if centers is not None:
        _need(centers, torch.int32, "centers")
    h, w = cur.shape
    check(lib().umi_full_me_u8_list(_ptr(cur), _ptr(ref), h, w, block, search, _ptr(centers), _ptr(blocks),
                                    _ptr(n_blocks), blocks.numel(), _ptr(out), _stream_ptr(stream)),
          "umi_full_me_u8_list")
    return out


class MeNet:
    """Learned motion proposal network (umi_menet_* / umi_me_learned_u8).

    Holds the fp32 parameters, Adam moments and a workspace for one frame
    size on one CUDA device."""

    def __init__(self, h: int, w: int, device="cuda", params=None, seed: int = 0):
        import torch
        self.h, self.w = h, w
        self.n = param_count()
        self.device = torch.device(device)
        if params is None:
            params = init_params(seed)
        self.params = torch.as_tensor(params, dtype=torch.float32).to(self.device).contiguous()
        if self.params.numel() != self.n:
            raise ValueError(f"expected {self.n} parameters, got {self.params.numel()}")
        self.grads = torch.zeros_like(self.params)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.step = 0
        nbytes = lib().umi_menet_workspace_bytes(h, w)
        if nbytes == 0:
            raise ValueError(f"frame {h}x{w} unsupported (h, w must be multiples of 16)")
        self.ws = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        self.nblk = (h // 16) * (w // 16)
        self.loss = torch.zeros(1, dtype=torch.float32, device=self.device)

    def forward(self, cur, ref, pred=None, stream=None):
        import torch
        _need(cur, torch.uint8, "cur")
        _need(ref, torch.uint8, "ref")
        if pred is None:
            pred = torch.empty((self.nblk, 2), dtype=torch.float32, device=self.device)
        check(lib().umi_menet_forward(_ptr(cur), _ptr(ref), self.h, self.w, _ptr(self.params), _ptr(pred),
                                      _ptr(self.ws), self.ws.numel(), _stream_ptr(stream)), "umi_menet_forward")
        return pred

    def infer(self, cur, ref, pred=None, err=None, stream=None):
        """Inference forward pass, layers 2-4 on the tensor cores (umi_menet_infer)."""
        import torch
        _need(cur, torch.uint8, "cur")
        _need(ref, torch.uint8, "ref")
        if pred is None:
            pred = torch.empty((self.nblk, 2), dtype=torch.float32, device=self.device)
        check(lib().umi_menet_infer(_ptr(cur), _ptr(ref), self.h, self.w, _ptr(self.params), _ptr(pred), _ptr(err),
                                    _ptr(self.ws), self.ws.numel(), _stream_ptr(stream)), "umi_menet_infer")
        return pred

    def backward(self, target, stride: int = 2, stream=None):
        import torch
        _need(target, torch.int32, "target")
        check(lib().umi_menet_backward(_ptr(target), stride, self.h, self.w, _ptr(self.params), _ptr(self.grads),
                                       _ptr(self.loss), _ptr(self.ws), self.ws.numel(), _stream_ptr(stream)),
              "umi_menet_backward")
        return self.grads

    def adam(self, lr: float, stream=None):
        self.step += 1
        check(lib().umi_menet_adam(_ptr(self.params), _ptr(self.grads), _ptr(self.m), _ptr(self.v), self.step,
                                   lr, _stream_ptr(stream)), "umi_menet_adam")

    def estimate(self, cur, ref, refine_r: int = 4, full_r: int = 64, sad_threshold: int = (1 << 31) - 1,
                 audit_stride: int = 0, out=None, audit_sums=None, n_fallback=None, stream=None):
        """Learned proposal + refine + audit + fallback (umi_me_learned_u8).

        Returns (mv (nblk, 3) int32, audit_sums (2,) int64, n_fallback (1,) int32)."""
        import torch
        if out is None:
            out = torch.empty((self.nblk, 3), dtype=torch.int32, device=self.device)
        if audit_sums is None:
            audit_sums = torch.zeros(2, dtype=torch.int64, device=self.device)
        if n_fallback is None:
            n_fallback = torch.zeros(1, dtype=torch.int32, device=self.device)
        _need(cur, torch.uint8, "cur")
        _need(ref, torch.uint8, "ref")
        check(lib().umi_me_learned_u8(_ptr(cur), _ptr(ref), self.h, self.w, _ptr(self.params), refine_r, full_r,
                                      sad_threshold, audit_stride, _ptr(out), _ptr(audit_sums), _ptr(n_fallback),
                                      _ptr(self.ws), self.ws.numel(), _stream_ptr(stream)), "umi_me_learned_u8")
        return out, audit_sums, n_fallback


class CoarseMe:
    """Coarse-to-fine motion proposal (umi_me_coarse_centers_u8 / umi_me_coarse_u8):
    the even displacement minimising the SAD of 4x4-mean cells, then the same
    refine / audit / fallback stage as the learned proposal.  Holds a workspace
    for one frame size on one CUDA device."""

    def __init__(self, h: int, w: int, device="cuda"):
        import torch
        self.h, self.w = h, w
        self.device = torch.device(device)
        nbytes = lib().umi_me_coarse_workspace_bytes(h, w)
        if nbytes == 0:
            raise ValueError(f"frame {h}x{w} unsupported (h, w must be multiples of 16)")
        self.ws = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        self.nblk = (h // 16) * (w // 16)

    def centers(self, cur, ref, rng: int = 60, out=None, stream=None):
        """Proposal centres (nblk, 2) int32, even, within +-rng."""
        import torch
        _need(cur, torch.uint8, "cur")
        _need(ref, torch.uint8, "ref")
        if out is None:
            out = torch.empty((self.nblk, 2), dtype=torch.int32, device=self.device)
        check(lib().umi_me_coarse_centers_u8(_ptr(cur), _ptr(ref), self.h, self.w, rng, _ptr(out), _ptr(self.ws),
                                             self.ws.numel(), _stream_ptr(stream)), "umi_me_coarse_centers_u8")
        return out

    def estimate(self, cur, ref, refine_r: int = 4, full_r: int = 64, sad_threshold: int = (1 << 31) - 1,
                 audit_stride: int = 0, out=None, audit_sums=None, n_fallback=None, stream=None):
        """Coarse proposal + refine + audit + fallback (umi_me_coarse_u8); the
        proposal range is (full_r - refine_r) rounded down to even.

        Returns (mv (nblk, 3) int32, audit_sums (2,) int64, n_fallback (1,) int32)."""
        import torch
        if out is None:
            out = torch.empty((self.nblk, 3), dtype=torch.int32, device=self.device)
        if audit_sums is None:
            audit_sums = torch.zeros(2, dtype=torch.int64, device=self.device)
        if n_fallback is None:
            n_fallback = torch.zeros(1, dtype=torch.int32, device=self.device)
        _need(cur, torch.uint8, "cur")
        _need(ref, torch.uint8, "ref")
        check(lib().umi_me_coarse_u8(_ptr(cur), _ptr(ref), self.h, self.w, refine_r, full_r, sad_threshold,
                                     audit_stride, _ptr(out), _ptr(audit_sums), _ptr(n_fallback), _ptr(self.ws),
                                     self.ws.numel(), _stream_ptr(stream)), "umi_me_coarse_u8")
        return out, audit_sums, n_fallback


def param_count() -> int:
    return int(lib().umi_menet_param_count())


MENET_CH = 32
MENET_CIN = (2, 32, 32, 32)
MENET_DIL = (1, 2, 4, 8)


def param_layout():
    """Offsets of the parameter array: [(w_off, b_off) per layer], head_w_off, head_b_off, total."""
    o = 0
    layers = []
    for cin in MENET_CIN:
        wo = o
        o += MENET_CH * cin * 9
        layers.append((wo, o))
        o += MENET_CH
    wh = o
    o += 2 * MENET_CH * 16
    bh = o
    o += 2
    return layers, wh, bh, o


def init_params(seed: int = 0):
    """He-normal conv weights, zero biases, small head weights (numpy float32)."""
    import numpy as np
    g = np.random.Generator(np.random.PCG64(seed))
    layers, wh, bh, total = param_layout()
    p = np.zeros(total, dtype=np.float32)
    for (wo, bo), cin in zip(layers, MENET_CIN):
        p[wo:bo] = g.normal(0.0, np.sqrt(2.0 / (cin * 9)), size=bo - wo)
    p[wh:bh] = g.normal(0.0, 0.01, size=bh - wh)
    return p


def full_me_sad_u8(cur, ref, block: int = 16, search: int = 32, out=None, stream=None):
    """Whole SAD volume (h//b, w//b, 2r+1, 2r+1) int32 (umi_full_me_sad_u8)."""
    import torch
    _need(cur, torch.uint8, "cur")
    _need(ref, torch.uint8, "ref")
    h, w = cur.shape
    nd = 2 * search + 1
    if out is None:
        out = torch.empty((h // block, w // block, nd, nd), dtype=torch.int32, device=cur.device)
    _need(out, torch.int32, "out")
    check(lib().umi_full_me_sad_u8(_ptr(cur), _ptr(ref), h, w, block, search, _ptr(out), _stream_ptr(stream)),
          "umi_full_me_sad_u8")
    return out


# ---- image operators and batches ----

OP_BILATERAL, OP_WFILTER_PP, OP_COST_VOLUME = 0, 1, 2
BATCH_MAX_IMAGES = 256


class BatchImage(ctypes.Structure):
    _fields_ = [("inp", _vp), ("aux", _vp), ("out", _vp), ("h", _i32), ("w", _i32)]


class BatchParams(ctypes.Structure):
    _fields_ = [("radius", _i32), ("sigma_s", _f32), ("sigma_r", _f32), ("channels", _i32), ("nd", _i32)]


def bilateral_f32(inp, radius=2, sigma_s=2.0, sigma_r=0.1, out=None, stream=None):
    """Bilateral filter of a float32 (h, w) CUDA tensor (umi_bilateral_f32)."""
    import torch
    _need(inp, torch.float32, "inp")
    h, w = inp.shape
    out = torch.empty_like(inp) if out is None else out
    _need(out, torch.float32, "out")
    check(lib().umi_bilateral_f32(_ptr(inp), _ptr(out), h, w, radius, sigma_s, sigma_r, _stream_ptr(stream)),
          "umi_bilateral_f32")
    return out


def wfilter3x3_pp_f32(inp, wts, out=None, stream=None):
    """Per-pixel-weight 3x3 filter; wts is (h, w, 3, 3) float32 (umi_wfilter3x3_pp_f32)."""
    import torch
    _need(inp, torch.float32, "inp")
    _need(wts, torch.float32, "wts")
    h, w = inp.shape
    if tuple(wts.shape) != (h, w, 3, 3):
        raise ValueError("wts must be (h, w, 3, 3)")
    out = torch.empty_like(inp) if out is None else out
    _need(out, torch.float32, "out")
    check(lib().umi_wfilter3x3_pp_f32(_ptr(inp), _ptr(wts), _ptr(out), h, w, _stream_ptr(stream)),
          "umi_wfilter3x3_pp_f32")
    return out


def cost_volume_dot_f32(left, right, nd=64, out=None, stream=None):
    """Dot-product cost volume of (c, h, w) features into (h, w, nd) (umi_cost_volume_dot_f32)."""
    import torch
    _need(left, torch.float32, "left")
    _need(right, torch.float32, "right")
    c, h, w = left.shape
    out = torch.empty((h, w, nd), dtype=torch.float32, device=left.device) if out is None else out
    _need(out, torch.float32, "out")
    check(lib().umi_cost_volume_dot_f32(_ptr(left), _ptr(right), _ptr(out), c, h, w, nd, _stream_ptr(stream)),
          "umi_cost_volume_dot_f32")
    return out


def _batch_table(images):
    n = len(images)
    if n > BATCH_MAX_IMAGES:
        raise ValueError("too many images")
    tab = (BatchImage * max(n, 1))()
    for i, (inp, aux, out) in enumerate(images):
        h, w = inp.shape[-2], inp.shape[-1]
        tab[i] = BatchImage(inp.data_ptr(), aux.data_ptr() if aux is not None else None, out.data_ptr(), h, w)
    return tab


def batch_run(op, images, params=None, variant=-1, stream=None):
    """One persistent launch over a batch: images = [(in, aux_or_None, out), ...] (umi_batch_run)."""
    tab = _batch_table(images)
    prm = params if params is not None else BatchParams()
    check(lib().umi_batch_run(op, tab, len(images), ctypes.byref(prm), variant, _stream_ptr(stream)), "umi_batch_run")


def batch_variants(op):
    return int(lib().umi_batch_variants(op))


class BatchJob(ctypes.Structure):
    _fields_ = [("op", _i32), ("images", _vp), ("n_images", _i32), ("params", BatchParams), ("variants", _vp)]


def batch_fused_variants(op):
    """Variants (tile shape, pixels per thread) of `op` inside the fused launch."""
    return int(lib().umi_batch_fused_variants(op))


def _fused_jobs(jobs):
    """jobs: [(op, images, params_or_None, variants_or_None), ...] -> (BatchJob array, objects to keep alive)."""
    arr = (BatchJob * max(len(jobs), 1))()
    keep = []
    for k, (op, images, params, variants) in enumerate(jobs):
        tab = _batch_table(images)
        var = None
        if variants is not None:
            if len(variants) != len(images):
                raise ValueError("one variant per image")
            var = (_i32 * max(len(variants), 1))(*[int(v) for v in variants])
        prm = params if params is not None else BatchParams()
        arr[k] = BatchJob(op, ctypes.cast(tab, _vp), len(images), prm, ctypes.cast(var, _vp) if var is not None else None)
        keep += [tab, var]
    return arr, keep


def batch_run_fused(jobs, stream=None):
    """One persistent launch for a whole batch step (umi_batch_run_fused):
    jobs = [(op, [(in, aux_or_None, out), ...], params_or_None, per-image variants_or_None), ...],
    at most one job per operator."""
    arr, keep = _fused_jobs(jobs)
    check(lib().umi_batch_run_fused(arr, len(jobs), _stream_ptr(stream)), "umi_batch_run_fused")


def autotune_batch(op, images, params=None, reps=3, stream=None):
    """Time every tile variant of `op` on this batch; returns (variant, ms) (umi_autotune_batch)."""
    tab = _batch_table(images)
    prm = params if params is not None else BatchParams()
    v = ctypes.c_int32(-1)
    ms = ctypes.c_float(0)
    check(lib().umi_autotune_batch(op, tab, len(images), ctypes.byref(prm), reps, ctypes.byref(v), ctypes.byref(ms),
                                   _stream_ptr(stream)), "umi_autotune_batch")
    return v.value, ms.value


# ---- tensor-core GEMM ----

def gemm(A, B, out=None, err=None, stream=None):
    """C = A @ B.T on the tensor cores: A (M,K), B (N,K) bf16 or f16 CUDA tensors -> fp32 (M,N)."""
    import torch
    if A.dtype not in (torch.bfloat16, torch.float16) or B.dtype != A.dtype:
        raise TypeError("A and B must both be bfloat16 or both float16")
    _need(A, A.dtype, "A")
    _need(B, B.dtype, "B")
    M, K = A.shape
    N = B.shape[0]
    if B.shape[1] != K:
        raise ValueError("B must be (N, K)")
    out = torch.empty((M, N), dtype=torch.float32, device=A.device) if out is None else out
    _need(out, torch.float32, "out")
    fn = lib().umi_gemm_bf16 if A.dtype == torch.bfloat16 else lib().umi_gemm_f16
    check(fn(_ptr(A), _ptr(B), _ptr(out), M, N, K, _ptr(err), _stream_ptr(stream)), fn.__name__)
    return out


def check_err(err, fn: str = "kernel") -> None:
    """Raise UmiError(UMI_ERR_TIMEOUT) if a kernel left error bits in the
    device word `err` (synchronises with the word's stream first)."""
    import torch
    torch.cuda.synchronize(err.device)
    check(lib().umi_err_status(int(err.item())), fn)


def gemm_bf16_wait_limit(A, B, epilogue_wait_ns, out=None, err=None, stream=None):
    """umi_gemm_bf16 with the epilogue's accumulator wait limited to
    epilogue_wait_ns (the timeout path's test hook)."""
    import torch
    _need(A, torch.bfloat16, "A")
    _need(B, torch.bfloat16, "B")
    M, K = A.shape
    N = B.shape[0]
    out = torch.empty((M, N), dtype=torch.float32, device=A.device) if out is None else out
    check(lib().umi_gemm_bf16_wait_limit(_ptr(A), _ptr(B), _ptr(out), M, N, K, _ptr(err), int(epilogue_wait_ns),
                                         _stream_ptr(stream)), "umi_gemm_bf16_wait_limit")
    return out


def gemm_f32_bf16x3(A, B, out=None, workspace=None, err=None, stream=None):
    """C = A @ B.T for fp32 A (M,K), B (N,K) via bf16x3 split precision on the tensor cores."""
    import torch
    _need(A, torch.float32, "A")
    _need(B, torch.float32, "B")
    M, K = A.shape
    N = B.shape[0]
    out = torch.empty((M, N), dtype=torch.float32, device=A.device) if out is None else out
    nb = int(lib().umi_gemm_f32_bf16x3_workspace_bytes(M, N, K))
    workspace = torch.empty(max(nb, 256), dtype=torch.uint8, device=A.device) if workspace is None else workspace
    check(lib().umi_gemm_f32_bf16x3(_ptr(A), _ptr(B), _ptr(out), M, N, K, _ptr(workspace), workspace.numel(),
                                    _ptr(err), _stream_ptr(stream)), "umi_gemm_f32_bf16x3")
    return out


def gemm_f32_f16x3(A, B, out=None, workspace=None, chunk=0, err=None, stream=None):
    """C = A @ B.T for fp32 A (M,K), B (N,K) at fp32-level accuracy: f16 hi/lo
    split with error correction on the tensor cores, the large product added
    in fp32 registers every `chunk` K-slices of 64 (umi_gemm_f32_f16x3)."""
    import torch
    _need(A, torch.float32, "A")
    _need(B, torch.float32, "B")
    M, K = A.shape
    N = B.shape[0]
    if B.shape[1] != K:
        raise ValueError("B must be (N, K)")
    out = torch.empty((M, N), dtype=torch.float32, device=A.device) if out is None else out
    _need(out, torch.float32, "out")
    nb = int(lib().umi_gemm_f32_f16x3_workspace_bytes(M, N, K))
    workspace = torch.empty(max(nb, 256), dtype=torch.uint8, device=A.device) if workspace is None else workspace
    check(lib().umi_gemm_f32_f16x3(_ptr(A), _ptr(B), _ptr(out), M, N, K, int(chunk), _ptr(workspace),
                                   workspace.numel(), _ptr(err), _stream_ptr(stream)), "umi_gemm_f32_f16x3")
    return out


def conv2d_fprop_f32_f16x3(x_nhwc, w_krsc, out=None, workspace=None, chunk=0, err=None, stream=None):
    """Stride-1 'same' convolution of fp32 x (N,H,W,C) with fp32 w (K,R,R,C) ->
    (N,K,H,W) fp32 at fp32-level accuracy (umi_conv2d_fprop_f32_f16x3)."""
    import torch
    _need(x_nhwc, torch.float32, "x")
    _need(w_krsc, torch.float32, "w")
    n, h, w, c = x_nhwc.shape
    k, r = w_krsc.shape[0], w_krsc.shape[1]
    out = torch.empty((n, k, h, w), dtype=torch.float32, device=x_nhwc.device) if out is None else out
    _need(out, torch.float32, "out")
    nb = int(lib().umi_conv2d_fprop_f32_f16x3_workspace_bytes(n, c, h, w, k, r))
    workspace = torch.empty(max(nb, 256), dtype=torch.uint8, device=x_nhwc.device) if workspace is None else workspace
    check(lib().umi_conv2d_fprop_f32_f16x3(_ptr(x_nhwc), _ptr(w_krsc), _ptr(out), n, c, h, w, k, r, int(chunk),
                                           _ptr(workspace), workspace.numel(), _ptr(err), _stream_ptr(stream)),
          "umi_conv2d_fprop_f32_f16x3")
    return out


def gemm_f32_generic(A, B, out=None, stream=None):
    """C = A @ B.T in plain fp32 through the generic UMI operator with the
    reference's Gemm strategy (main/gemm.cu:8-15: accum += a * b over a
    blocked K loop, fp32 FMA), for A (M,K) and B (N,K) fp32: the plain FP32
    UMI path that the split-precision products are measured against."""
    import torch
    _need(A, torch.float32, "A")
    _need(B, torch.float32, "B")
    M, K = A.shape
    N = B.shape[0]
    out = torch.empty((M, N), dtype=torch.float32, device=A.device) if out is None else out
    _need(out, torch.float32, "out")
    # P = (row m, column n), A = K; A row-major (M,K), B row-major (N,K): both read along K
    d = make_desc(p=[(1, 1, 1, 1), (1, 1, 1, 1), (M, 16, 2, 1), (N, 16, 16, 1)], a=[(1, 1), (1, 1), (1, 1), (K, 16)],
                  mems=[dict(p_view=[(), (), (2, 0, 1), ()], a_view=[(), (), (), (3, 0, 1)],
                             phys=[(1, PAD), (1, PAD), (M, PAD), (K, PAD)], stage=1),
                        dict(p_view=[(), (), (), (2, 0, 1)], a_view=[(), (), (), (3, 0, 1)],
                             phys=[(1, PAD), (1, PAD), (N, PAD), (K, PAD)], stage=1),
                        dict(p_view=[(), (), (2, 0, 1), (3, 0, 1)], phys=[(), (), (M, PAD), (N, PAD)], stage=2,
                             out=True)])
    launch(d, STRATEGY_DOT_F32, [A, B], [out], stream=stream)
    return out


def conv2d_fprop_bf16(x_nhwc, w_krsc, out=None, err=None, stream=None):
    """Stride-1 'same' convolution on the tensor cores: x (N,H,W,C) bf16, w (K,R,R,C) bf16 -> (N,K,H,W) fp32."""
    import torch
    _need(x_nhwc, torch.bfloat16, "x")
    _need(w_krsc, torch.bfloat16, "w")
    n, h, w, c = x_nhwc.shape
    k, r, r2, c2 = w_krsc.shape
    if r != r2 or c2 != c:
        raise ValueError("w must be (K, R, R, C) with the input's C")
    out = torch.empty((n, k, h, w), dtype=torch.float32, device=x_nhwc.device) if out is None else out
    _need(out, torch.float32, "out")
    check(lib().umi_conv2d_fprop_bf16(_ptr(x_nhwc), _ptr(w_krsc), _ptr(out), n, c, h, w, k, r, _ptr(err),
                                      _stream_ptr(stream)), "umi_conv2d_fprop_bf16")
    return out
