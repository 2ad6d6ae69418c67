"""FP32 CPU restatement of the proposal network's forward and backward passes
(TEST INFRASTRUCTURE: the tensor-core kernels are compared with it).

It rounds to BF16 exactly where the GPU stores BF16 (weights, the network input,
every ReLU activation, every activation gradient), so that the GPU and this
restatement differ only by the order of FP32 accumulation.
"""
from __future__ import annotations

import numpy as np

CIN = [32, 32, 32, 32, 32, 32]
COUT = [32, 32, 32, 32, 32, 3]
DIL = [1, 2, 4, 8, 1, 1]   # dilation of each layer's 3x3 taps


def bf16(x):
    """Round float32 to the nearest bfloat16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((a + 0x7FFF + ((a >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).reshape(np.shape(x))


def reduce_frame(f, r):
    """An 8-bit frame reduced by r (bm_net.cu k_net_input_reduced): pixel (X, Y) is the
    mean of the r x r input pixels (r*X + a, r*Y + b), rounded half to even; a ragged
    right or bottom edge is dropped."""
    f = np.asarray(f)
    if r == 1:
        return f.astype(np.uint8)
    h, w = f.shape[0] // r, f.shape[1] // r
    s = f[:h * r, :w * r].astype(np.int64).reshape(h, r, w, r).sum(axis=(1, 3))
    return np.rint(s / float(r * r)).astype(np.uint8)


def net_input(f0, f1, reduce=1):
    """The network input of bm_net_prepare_reduced (bm_net.cu k_net_input /
    k_net_input_reduced) as float32 before BF16 rounding, [h4][w4][32]: channel
    4*j + i of cell (x, y) is pixel (4x + i, 4y + j) of reduced frame 0 scaled to
    [-1, 1], channels 16..31 the same for frame 1; h4 x w4 = (H // reduce // 4) x
    (W // reduce // 4)."""
    out = []
    for f in (f0, f1):
        g = reduce_frame(f, reduce)
        h4, w4 = g.shape[0] // 4, g.shape[1] // 4
        c = g[:h4 * 4, :w4 * 4].reshape(h4, 4, w4, 4).transpose(0, 2, 1, 3).reshape(h4, w4, 16)
        out.append(c.astype(np.float32) / np.float32(127.5) - np.float32(1.0))
    return np.concatenate(out, axis=2)


def unpack(params):
    out, k = [], 0
    for ci, co in zip(CIN, COUT):
        nw = co * 9 * ci
        W = params[k:k + nw].reshape(co, 9, ci)
        b = params[k + nw:k + nw + co]
        out.append((W, b))
        k += nw + co
    assert k == params.size
    return out


def _shifts(x, d=1):
    """The 9 zero-padded 3x3 neighbours at dilation d of NHWC x: list of [B,h,w,C]
    (tap = dy*3+dx, offset d*(dy-1, dx-1))."""
    B, h, w, C = x.shape
    p = np.zeros((B, h + 2 * d, w + 2 * d, C), np.float32)
    p[:, d:d + h, d:d + w] = x
    return [p[:, dy * d:dy * d + h, dx * d:dx * d + w] for dy in range(3) for dx in range(3)]


def conv(x, W, b=None, d=1):
    sh = _shifts(x, d)
    y = sum(np.einsum("bhwc,oc->bhwo", sh[t], W[:, t, :], optimize=True) for t in range(9))
    return y + (b if b is not None else 0)


def _r(x, rounding):
    return bf16(x) if rounding else np.asarray(x, np.float32)


def forward(params, x0, rounding=True):
    layers = unpack(params)
    acts = []
    x = _r(x0, rounding)
    for l in range(5):
        W, b = layers[l]
        x = _r(np.maximum(conv(x, _r(W, rounding), b, DIL[l]), 0), rounding)
        acts.append(x)
    W, b = layers[5]
    return conv(x, _r(W, rounding), b, DIL[5]).astype(np.float32), acts


def loss_grad(out, target, tau=1.0, wconf=0.25, rounding=True):
    n = out.shape[0] * out.shape[1] * out.shape[2]
    u, v, c = out[..., 0], out[..., 1], out[..., 2]
    tu, tv, valid = target[..., 0], target[..., 1], target[..., 2]
    du, dv = u - tu, v - tv

    def sl1(d):
        a = np.abs(d)
        return np.where(a < 1, 0.5 * d * d, a - 0.5), np.where(a < 1, d, np.sign(d))

    lu, gu = sl1(du)
    lv, gv = sl1(dv)
    label = ((np.abs(du) + np.abs(dv)) < tau).astype(np.float32)
    sig = 1 / (1 + np.exp(-c))
    lc = valid * (np.maximum(c, 0) - c * label + np.log1p(np.exp(-np.abs(c))))
    dY = np.zeros(out.shape[:3] + (3,), np.float32)
    dY[..., 0] = gu * valid / n
    dY[..., 1] = gv * valid / n
    dY[..., 2] = wconf * (sig - label) * valid / n
    losses = (float(((lu + lv) * valid).sum() / n), float(lc.sum() / n), float((valid * label).sum() / n))
    return _r(dY, rounding), losses


def backward(params, x0, acts, dY, rounding=True):
    """FP32 gradient vector (same layout as params)."""
    layers = unpack(params)
    grads = []
    xs = [_r(x0, rounding)] + acts
    for l in range(5, -1, -1):
        W, _ = layers[l]
        X = xs[l]
        sh = _shifts(X, DIL[l])
        dW = np.stack([np.einsum("bhwo,bhwc->oc", dY, sh[t], optimize=True) for t in range(9)], axis=1)
        db = dY.sum(axis=(0, 1, 2))
        grads.append((dW, db))
        if l > 0:
            # dX[q] = sum_t dY[q - off(t)] W[:, t, :]: correlation with the flipped kernel
            Wf = _r(W, rounding)[:, ::-1, :]
            shd = _shifts(dY, DIL[l])
            dX = sum(np.einsum("bhwo,oc->bhwc", shd[t], Wf[:, t, :], optimize=True) for t in range(9))
            dY = _r(dX * (acts[l - 1] > 0), rounding)
    grads = grads[::-1]
    return np.concatenate([np.concatenate([dW.ravel(), db]) for dW, db in grads]).astype(np.float32)
