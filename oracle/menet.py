"""FP64 CPU oracle of the learned motion-proposal network (numpy).

TEST INFRASTRUCTURE ONLY: the tests use it to check the GPU forward pass and
the hand-written backward kernels; the product library never imports it.

The reference has no learned component (its full_me, main/full_me.cu, only
searches exhaustively), so nothing here restates reference code: this is the
mathematical definition of the network that the CUDA kernels implement.
The oracle itself is pinned by central finite differences in the tests.

Network (parameters in the flat layout of umi_gb300.param_layout()):
  x0[0] = (boxmean4(cur) - 128)/32, x0[1] = (boxmean4(ref) - 128)/32
  a_l   = ReLU(b_l + sum_{ci,tap} W_l[co, ci, tap] * a_{l-1}[ci, p + dil_l * off(tap)])
          (zero outside the image; off(tap) = (tap // 3 - 1, tap % 3 - 1); dil 1, 2, 4, 8)
  pred[k, j] = bh[j] + sum_f Wh[j, f] * a_4[f // 16, 4 by + (f // 4) % 4, 4 bx + f % 4]
  loss  = mean_k sum_j smoothL1(pred[k, j] - target[k, j] / 16)
With bf16=True the weights (not the biases) are rounded to bfloat16 before
use, as the GPU kernels do; the gradient is then taken with respect to the
rounded weights (straight-through), which is what the GPU backward returns.
"""
from __future__ import annotations

import numpy as np

CH = 32
CIN = (2, 32, 32, 32)
DIL = (1, 2, 4, 8)


def layout():
    o = 0
    layers = []
    for cin in CIN:
        wo = o
        o += CH * cin * 9
        layers.append((wo, o))
        o += CH
    wh = o
    o += 2 * CH * 16
    bh = o
    o += 2
    return layers, wh, bh, o


def to_bf16(x):
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float64."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def downsample(cur, ref):
    h, w = cur.shape
    H4, W4 = h // 4, w // 4
    out = np.empty((2, H4, W4), np.float64)
    for c, f in enumerate((cur, ref)):
        s = f[:4 * H4, :4 * W4].astype(np.float64).reshape(H4, 4, W4, 4).sum(axis=(1, 3))
        out[c] = s / 512.0 - 4.0
    return out


def _shift(x, dy, dx):
    """y[:, i, j] = x[:, i + dy, j + dx], zero outside."""
    C, H, W = x.shape
    y = np.zeros_like(x)
    ys, ye = max(0, -dy), min(H, H - dy)
    xs, xe = max(0, -dx), min(W, W - dx)
    if ys < ye and xs < xe:
        y[:, ys:ye, xs:xe] = x[:, ys + dy:ye + dy, xs + dx:xe + dx]
    return y


def conv(x, w, b, dil):
    """w: (cout, cin, 9); returns the pre-activation (cout, H, W)."""
    out = np.zeros((w.shape[0],) + x.shape[1:], np.float64)
    for t in range(9):
        dy, dx = (t // 3 - 1) * dil, (t % 3 - 1) * dil
        out += np.einsum("oc,chw->ohw", w[:, :, t], _shift(x, dy, dx))
    if b is not None:
        out += b[:, None, None]
    return out


def conv_wgrad(x, d, dil):
    """dW[co, ci, t] = sum_p d[co, p] * x[ci, p + dil off(t)]."""
    g = np.zeros((d.shape[0], x.shape[0], 9), np.float64)
    for t in range(9):
        dy, dx = (t // 3 - 1) * dil, (t % 3 - 1) * dil
        g[:, :, t] = np.einsum("ohw,chw->oc", d, _shift(x, dy, dx))
    return g


def conv_dgrad(d, w, dil):
    """dx[ci, q] = sum_{co,t} w[co, ci, t] * d[co, q - dil off(t)]."""
    out = np.zeros((w.shape[1],) + d.shape[1:], np.float64)
    for t in range(9):
        dy, dx = (t // 3 - 1) * dil, (t % 3 - 1) * dil
        out += np.einsum("oc,ohw->chw", w[:, :, t], _shift(d, -dy, -dx))
    return out


def _weights(params, bf16):
    layers, wh, bh, _ = layout()
    p = np.asarray(params, np.float32)
    rnd = to_bf16 if bf16 else (lambda a: a.astype(np.float64))
    ws = [rnd(p[wo:bo]).reshape(CH, cin, 9) for (wo, bo), cin in zip(layers, CIN)]
    bs = [p[bo:bo + CH].astype(np.float64) for (_, bo) in layers]
    return ws, bs, rnd(p[wh:bh]).reshape(2, CH * 16), p[bh:bh + 2].astype(np.float64)


def head_features(a4, nby, nbx):
    """(nblk, 512): feature f of block k = a4[f // 16, 4 by + (f // 4) % 4, 4 bx + f % 4]."""
    C = a4.shape[0]
    t = a4[:, :4 * nby, :4 * nbx].reshape(C, nby, 4, nbx, 4)
    return t.transpose(1, 3, 0, 2, 4).reshape(nby * nbx, C * 16)


def forward(params, cur, ref, bf16=True, act_bf16=False):
    """Returns (pred (nblk, 2), activations [x0, a1..a4]).

    act_bf16: round each layer's output (after ReLU) to bfloat16, as the
    tensor-core inference pass stores its activations."""
    ws, bs, whm, bhv = _weights(params, bf16)
    acts = [downsample(cur, ref)]
    for l in range(4):
        a = np.maximum(conv(acts[-1], ws[l], bs[l], DIL[l]), 0.0)
        acts.append(to_bf16(a.astype(np.float32)) if act_bf16 else a)
    h, w = cur.shape
    feat = head_features(acts[-1], h // 16, w // 16)
    return feat @ whm.T + bhv, acts


def loss_and_grad(params, cur, ref, target, bf16=True):
    """Mean smooth-L1 loss against target/16 and its gradient (flat, float64)."""
    layers, wh, bh, total = layout()
    ws, bs, whm, bhv = _weights(params, bf16)
    pred, acts = forward(params, cur, ref, bf16)
    n = pred.shape[0]
    e = pred - np.asarray(target, np.float64)[:, :2] / 16.0
    ae = np.abs(e)
    loss = np.where(ae < 1.0, 0.5 * e * e, ae - 0.5).sum() / n
    gp = np.clip(e, -1.0, 1.0) / n  # dL/dpred
    grad = np.zeros(total, np.float64)
    h, w = cur.shape
    nby, nbx = h // 16, w // 16
    feat = head_features(acts[-1], nby, nbx)
    grad[wh:bh] = (gp.T @ feat).ravel()
    grad[bh:bh + 2] = gp.sum(axis=0)
    dfeat = gp @ whm  # (nblk, 512)
    C, H4, W4 = acts[-1].shape
    da = np.zeros_like(acts[-1])
    da[:, :4 * nby, :4 * nbx] = dfeat.reshape(nby, nbx, C, 4, 4).transpose(2, 0, 3, 1, 4).reshape(C, 4 * nby, 4 * nbx)
    for l in range(3, -1, -1):
        d = da * (acts[l + 1] > 0)
        wo, bo = layers[l]
        grad[wo:bo] = conv_wgrad(acts[l], d, DIL[l]).ravel()
        grad[bo:bo + CH] = d.sum(axis=(1, 2))
        if l > 0:
            da = conv_dgrad(d, ws[l], DIL[l])
    return loss, grad


def adam_step(p, g, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (Kingma & Ba, 2015) in float32, as umi_menet_adam; returns (p, m, v)."""
    p = np.asarray(p, np.float32); g = np.asarray(g, np.float32)
    m = (np.float32(b1) * m + np.float32(1 - b1) * g).astype(np.float32)
    v = (np.float32(b2) * v + np.float32(1 - b2) * g * g).astype(np.float32)
    c1 = np.float32(1 - b1 ** step); c2 = np.float32(1 - b2 ** step)
    p = (p - np.float32(lr) * (m / c1) / (np.sqrt(v / c2) + np.float32(eps))).astype(np.float32)
    return p, m, v
