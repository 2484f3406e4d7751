"""CPU oracle for the UMI operator hot path (ctypes bindings over liboracle.so).

TEST INFRASTRUCTURE ONLY.  This package is the checker: the test suite, the
smoke entry and the bench's CPU-baseline leg use it; the product library never
imports it.  Each function names the reference lines it restates (see
umi_oracle.h for the C contract).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_I = ctypes.c_int


def build() -> str:
    """Compile liboracle.so in place (make -C oracle)."""
    subprocess.run(["make", "-s", "-C", _HERE, "liboracle.so"], check=True)
    return os.path.join(_HERE, "liboracle.so")


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        sig = {
            "oracle_ref_filter3x3_i32": [_i32p, _i32p, _I, _I, _I, _I, _I],
            "oracle_ref_wfilter3x3_i32": [_i32p, _i32p, _I, _I, _i32p, _I, _I],
            "oracle_ref_bilateral_f32": [_f32p, _f32p, _I, _I, _I, _f32p, ctypes.c_float],
            "oracle_ref_cost_volume_i32": [_i32p, _i32p, _I, _I, _I, _I],
            "oracle_ref_full_me_i32": [_i32p, _i32p, _i32p, _I, _I, _I, _I, _I],
            "oracle_ref_iimg_i32": [_i32p, _i32p, _I, _I],
            "oracle_ref_gemm_i32": [_i32p, _i32p, _i32p, _I, _I, _I],
            "oracle_ref_fprop_i32": [_i32p, _i32p, _i32p, _I, _I, _I, _I, _I, _I, _I, _I, _I],
            "oracle_ref_fprop_inputs": [_i32p, ctypes.c_size_t, _i32p, ctypes.c_size_t],
            "oracle_filter3x3_f64": [_f32p, _f64p, _I, _I, _f32p, ctypes.c_float, _I],
            "oracle_iimg_u8_i32": [_u8p, _i32p, _I, _I, _I],
            "oracle_full_me_u8": [_u8p, _u8p, _I, _I, _I, _I, ctypes.c_void_p, _I, _i32p, ctypes.c_void_p, _I],
            "oracle_block_sad_u8": [_u8p, _u8p, _I, _I, _I, _I, _I, _I, _I],
            "oracle_coarse_centers_u8": [_u8p, _u8p, _I, _I, _I, _i32p, _I],
            "oracle_ref_full_me_u8_argmin": [_u8p, _u8p, _I, _I, _I, _I, _i32p, _I, _i32p, _I],
            "oracle_ref_iimg_u8": [_u8p, _i32p, _I, _I],
            "oracle_bilateral_f64": [_f32p, _f64p, _I, _I, _I, ctypes.c_double, ctypes.c_double, _I],
            "oracle_wfilter_pp_f64": [_f32p, _f32p, _f64p, _I, _I, _I],
            "oracle_cost_volume_dot_f64": [_f32p, _f32p, _f64p, _I, _I, _I, _I, _I],
            "oracle_gemm_f64": [_f32p, _f32p, _f64p, _I, _I, _I, _I, _I],
            "oracle_conv2d_f64": [_f32p, _f32p, _f64p, _I, _I, _I, _I, _I, _I, _I, _I, _I],
        }
        for name, args in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int32 if name == "oracle_block_sad_u8" else None
        _LIB = L
    return _LIB


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


# ---- the reference's own CPU checks (main/<app>.cu) ----

def ref_filter3x3_i32(img, init, mul, pad):
    img = _c(img, np.int32); out = np.empty_like(img)
    lib().oracle_ref_filter3x3_i32(img, out, img.shape[0], img.shape[1], init, mul, pad)
    return out


def ref_wfilter3x3_i32(img, w9, init, pad):
    img = _c(img, np.int32); out = np.empty_like(img)
    lib().oracle_ref_wfilter3x3_i32(img, out, img.shape[0], img.shape[1], _c(w9, np.int32), init, pad)
    return out


def ref_bilateral_f32(img, ofs, ws, norm):
    img = _c(img, np.float32); out = np.empty_like(img)
    lib().oracle_ref_bilateral_f32(img, out, img.shape[0], img.shape[1], ofs, _c(ws, np.float32), norm)
    return out


def ref_cost_volume_i32(frame, k, sr):
    frame = _c(frame, np.int32); h, w = frame.shape
    out = np.empty((h, w, sr), np.int32)
    lib().oracle_ref_cost_volume_i32(frame, out, h, w, k, sr)
    return out


def ref_full_me_i32(cur, ref, b, sr_ofs, sr):
    cur = _c(cur, np.int32); ref = _c(ref, np.int32); h, w = cur.shape
    out = np.empty((h // b, w // b, sr, sr), np.int32)
    lib().oracle_ref_full_me_i32(cur, ref, out, h, w, b, sr_ofs, sr)
    return out


def ref_iimg_i32(img):
    img = _c(img, np.int32); out = np.empty_like(img)
    lib().oracle_ref_iimg_i32(img, out, img.shape[0], img.shape[1])
    return out


def ref_gemm_i32(A, B):
    A = _c(A, np.int32); B = _c(B, np.int32)
    m, k = A.shape; n = B.shape[1]
    C = np.empty((m, n), np.int32)
    lib().oracle_ref_gemm_i32(A, B, C, m, k, n)
    return C


def ref_fprop_i32(x, wt, f, s, ofs, threads=0):
    x = _c(x, np.int32); wt = _c(wt, np.int32)
    n, c, ih, iw = x.shape; k = wt.shape[0]
    out = np.empty((n, k, ih // s, iw // s), np.int32)
    lib().oracle_ref_fprop_i32(x, wt, out, n, c, ih, iw, k, f, s, ofs, threads)
    return out


def ref_fprop_inputs(n_in, n_wt):
    a = np.empty(n_in, np.int32); b = np.empty(n_wt, np.int32)
    lib().oracle_ref_fprop_inputs(a, n_in, b, n_wt)
    return a, b


# ---- benchmark workloads ----

def filter3x3_f64(img, w9, pad=0.0, threads=0):
    img = _c(img, np.float32); out = np.empty(img.shape, np.float64)
    lib().oracle_filter3x3_f64(img, out, img.shape[0], img.shape[1], _c(w9, np.float32).ravel(), pad, threads)
    return out


def iimg_u8_i32(img):
    img = _c(img, np.uint8); out = np.empty(img.shape, np.int32)
    lib().oracle_iimg_u8_i32(img, out, img.shape[0], img.shape[1], 1)
    return out


def full_me_u8(cur, ref, b, r, blocks=None, sad_volume=False, threads=0):
    """Returns mv (n, 3) int32 [mv_y, mv_x, sad] (and the SAD volume if asked)."""
    cur = _c(cur, np.uint8); ref = _c(ref, np.uint8); h, w = cur.shape
    nby, nbx, nd = h // b, w // b, 2 * r + 1
    if blocks is not None:
        blocks = _c(blocks, np.int32)
        n = len(blocks)
        bp = blocks.ctypes.data_as(ctypes.c_void_p)
    else:
        n = nby * nbx
        bp = None
    mv = np.empty((n, 3), np.int32)
    vol = np.empty((nby, nbx, nd, nd), np.int32) if (sad_volume and blocks is None) else None
    lib().oracle_full_me_u8(cur, ref, h, w, b, r, bp, n, mv,
                            vol.ctypes.data_as(ctypes.c_void_p) if vol is not None else None, threads)
    return (mv, vol) if sad_volume else mv


def ref_full_me_u8_argmin(cur, ref, b, r, blocks, threads=0):
    """The reference's full_me check loop as written (main/full_me.cu:68-87)
    plus argmin, on the listed blocks: the timed CPU baseline."""
    cur = _c(cur, np.uint8); ref = _c(ref, np.uint8); h, w = cur.shape
    blocks = _c(blocks, np.int32)
    mv = np.empty((len(blocks), 3), np.int32)
    lib().oracle_ref_full_me_u8_argmin(cur, ref, h, w, b, r, blocks, len(blocks), mv, threads)
    return mv


def ref_iimg_u8(img):
    """The reference's iimg check loop (main/iimg.cu:100-111) on a uint8 frame."""
    img = _c(img, np.uint8); out = np.empty(img.shape, np.int32)
    lib().oracle_ref_iimg_u8(img, out, img.shape[0], img.shape[1])
    return out


def coarse_centers_u8(cur, ref, rng, threads=0):
    """Coarse proposal centres (nblk, 2) int32: the even displacement within
    +-rng minimising the SAD of 4x4-mean cells (umi_oracle.h)."""
    cur = _c(cur, np.uint8); ref = _c(ref, np.uint8); h, w = cur.shape
    out = np.empty(((h // 16) * (w // 16), 2), np.int32)
    lib().oracle_coarse_centers_u8(cur, ref, h, w, rng, out, threads)
    return out


def block_sad_u8(cur, ref, b, by, bx, dy, dx):
    cur = _c(cur, np.uint8); ref = _c(ref, np.uint8); h, w = cur.shape
    return int(lib().oracle_block_sad_u8(cur, ref, h, w, b, by, bx, dy, dx))


def bilateral_f64(img, r, sigma_s, sigma_r, threads=0):
    img = _c(img, np.float32); out = np.empty(img.shape, np.float64)
    lib().oracle_bilateral_f64(img, out, img.shape[0], img.shape[1], r, sigma_s, sigma_r, threads)
    return out


def wfilter_pp_f64(img, wts, threads=0):
    img = _c(img, np.float32); wts = _c(wts, np.float32); out = np.empty(img.shape, np.float64)
    lib().oracle_wfilter_pp_f64(img, wts, out, img.shape[0], img.shape[1], threads)
    return out


def cost_volume_dot_f64(L, R, nd, threads=0):
    L = _c(L, np.float32); R = _c(R, np.float32); c, h, w = L.shape
    out = np.empty((h, w, nd), np.float64)
    lib().oracle_cost_volume_dot_f64(L, R, out, c, h, w, nd, threads)
    return out


def gemm_f64(A, B, b_is_nk=False, threads=0):
    A = _c(A, np.float32); B = _c(B, np.float32)
    m, k = A.shape
    n = B.shape[0] if b_is_nk else B.shape[1]
    C = np.empty((m, n), np.float64)
    lib().oracle_gemm_f64(A, B, C, m, n, k, int(b_is_nk), threads)
    return C


def conv2d_f64(x, wt, stride=1, pad=1, threads=0):
    x = _c(x, np.float32); wt = _c(wt, np.float32)
    n, c, h, w = x.shape; k, _, r, _ = wt.shape
    oh = (h + 2 * pad - r) // stride + 1; ow = (w + 2 * pad - r) // stride + 1
    out = np.empty((n, k, oh, ow), np.float64)
    lib().oracle_conv2d_f64(x, wt, out, n, c, h, w, k, r, stride, pad, threads)
    return out
