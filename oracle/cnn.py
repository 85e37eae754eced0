"""FP64 numpy restatement of the learned-initial-guess network, test infrastructure only.

The reference has no network (its initial values come from
``models/galaxy_model_object.py:60-113`` and ``models/_shared_methods.py:116-166``); this file
is the CPU checker of the library's own CNN kernels: the same layers, parameter layout and
loss, in float64, with an explicit backward pass.  Parity is therefore against this
restatement and finite differences, not against the reference.

Layers (activations NHWC): four 3x3 stride-2 pad-1 convolutions 1->32->64->128->256 with
ReLU (64x64 -> 4x4), fc 4096->192 with ReLU, fc 192->16 (8 outputs used).  Each layer's
parameters are W[N][K] then b[N] in one flat vector; the convolution reduction index is
k = (ky * 3 + kx) * C + c; layer 1 pads K from 9 to 16 with zero columns.
"""

from __future__ import annotations

import numpy as np

# (cin, cout, hin, hout, K, N)
LAYERS = (
    (1, 32, 64, 32, 16, 32),
    (32, 64, 32, 16, 288, 64),
    (64, 128, 16, 8, 576, 128),
    (128, 256, 8, 4, 1152, 256),
    (4096, 192, 1, 1, 4096, 192),
    (192, 16, 1, 1, 192, 16),
)
N_CONV = 4


def offsets():
    w, b, o = [], [], 0
    for (_, _, _, _, K, N) in LAYERS:
        w.append(o)
        o += N * K
        b.append(o)
        o += N
    return w, b, o


W_OFF, B_OFF, PARAM_COUNT = offsets()


def weights(params, l):
    _, _, _, _, K, N = LAYERS[l]
    return params[W_OFF[l] : W_OFF[l] + N * K].reshape(N, K), params[B_OFF[l] : B_OFF[l] + N]


def im2col(x, kpad=None):
    """x [B, H, W, C] -> [B * Ho * Wo, 9C (or kpad)], 3x3 stride 2 pad 1."""
    B, H, W, C = x.shape
    Ho = H // 2
    xp = np.zeros((B, H + 2, W + 2, C), dtype=x.dtype)
    xp[:, 1:-1, 1:-1] = x
    cols = []
    for ky in range(3):
        for kx in range(3):
            cols.append(xp[:, ky : ky + 2 * Ho : 2, kx : kx + 2 * Ho : 2, :])
    col = np.stack(cols, axis=3).reshape(B * Ho * Ho, 9 * C)
    if kpad is not None and kpad > col.shape[1]:
        col = np.concatenate([col, np.zeros((col.shape[0], kpad - col.shape[1]))], axis=1)
    return col


def col2im(dcol, B, H, C):
    """Adjoint of ``im2col``: [B * Ho * Wo, 9C] -> [B, H, W, C]."""
    Ho = H // 2
    d = dcol[:, : 9 * C].reshape(B, Ho, Ho, 9, C)
    dxp = np.zeros((B, H + 2, H + 2, C))
    for ky in range(3):
        for kx in range(3):
            dxp[:, ky : ky + 2 * Ho : 2, kx : kx + 2 * Ho : 2, :] += d[:, :, :, ky * 3 + kx, :]
    return dxp[:, 1:-1, 1:-1]


def bf16(x):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def _id(x):
    return x


def forward(params, x, round_bf16=False):
    """x [B, 64, 64] -> out [B, 16] and the cache for ``backward``.  ``round_bf16`` rounds
    what the kernels keep in bfloat16 (im2col matrices, activations; the caller passes
    bf16-rounded weights), so that the result differs from the kernels' only by the order of
    the fp32 sums."""
    rnd = bf16 if round_bf16 else _id
    B = x.shape[0]
    a = x.reshape(B, 64, 64, 1).astype(np.float64)
    cache = []
    for l, (cin, cout, hin, hout, K, N) in enumerate(LAYERS):
        W, b = weights(params, l)
        if l < N_CONV:
            col = im2col(a, K)
            if l == 0:
                col = rnd(col)
        else:
            col = a.reshape(B, -1)
        pre = col @ W.T + b
        last = l == len(LAYERS) - 1
        act = pre if last else rnd(np.maximum(pre, 0.0))
        cache.append((col, act, a.shape))
        a = act.reshape(B, hout, hout, N) if l < N_CONV else act
    return a, cache


def backward(params, cache, dout, round_bf16=False):
    """Flat gradient of a loss with d loss / d out = dout [B, 16] (``round_bf16``: the
    pre-activation gradients are rounded to bfloat16 as the kernels keep them)."""
    rnd = bf16 if round_bf16 else _id
    grads = np.zeros(PARAM_COUNT)
    dA = dout
    B = dout.shape[0]
    for l in range(len(LAYERS) - 1, -1, -1):
        cin, cout, hin, hout, K, N = LAYERS[l]
        col, act, in_shape = cache[l]
        W, _ = weights(params, l)
        last = l == len(LAYERS) - 1
        dpre = rnd(dA.reshape(-1, N) * (1.0 if last else (act.reshape(-1, N) > 0)))
        grads[W_OFF[l] : W_OFF[l] + N * K] = (dpre.T @ col).reshape(-1)
        grads[B_OFF[l] : B_OFF[l] + N] = dpre.sum(axis=0)
        if l == 0:
            break
        dcol = dpre @ W
        if l < N_CONV:
            dA = col2im(dcol, B, in_shape[1], in_shape[3])
        else:
            dA = dcol.reshape(in_shape)
    return grads


def mse(out, targets):
    """Mean squared error over the 8 used outputs and its d / d out."""
    B = out.shape[0]
    d = out[:, :8] - targets
    dout = np.zeros_like(out)
    dout[:, :8] = 2.0 * d / (B * 8)
    return float(np.mean(d**2)), dout
