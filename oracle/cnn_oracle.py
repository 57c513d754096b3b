"""FP64 numpy oracle of the warm-start network (test infrastructure only).

Restates the network of ``reconflow_gb300/csrc/rf_cnn.cu`` (layers c1, c2,
c3, h16, c4, h8 with their parameter layout [Cout][3][3][Cin] then [Cout])
and its masked L1 loss, forward and backward, in float64, rounding to BF16
exactly where the GPU kernels hold BF16 values: the input, the weights, the
ReLU activations and the gradients fed to the matrix products.  The GPU
accumulates in FP32, so the two agree to a few 1e-3 relative, not bitwise.
Only the tests import this module.
"""
from __future__ import annotations

import numpy as np

LAYERS = [  # (cin, cout, stride, relu)
    (16, 32, 1, True), (32, 96, 2, True), (96, 96, 1, True), (96, 8, 1, False),
    (128, 64, 1, True), (64, 8, 1, False),
]


# BF16 rounding at the GPU's rounding points; the finite-difference self-check
# of the backward pass switches it off (rounding makes the loss piecewise
# constant at that scale).
ROUND = True


def bf(a):
    """Round float32 values to bfloat16 (round to nearest even), as float64."""
    if not ROUND:
        return np.asarray(a, np.float64)
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def unpack(params):
    out, off = [], 0
    for cin, cout, _, _ in LAYERS:
        n = cout * 9 * cin
        W = params[off:off + n].reshape(cout, 3, 3, cin)
        off += n
        b = params[off:off + cout]
        off += cout
        out.append((W.astype(np.float32) if ROUND else W.astype(np.float64), b.astype(np.float64)))
    return out


def conv(x, W, stride):
    B, H, Wd, C = x.shape
    Ho, Wo = (H + stride - 1) // stride, (Wd + stride - 1) // stride
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    y = np.zeros((B, Ho, Wo, W.shape[0]))
    for ky in range(3):
        for kx in range(3):
            patch = xp[:, ky:ky + (Ho - 1) * stride + 1:stride, kx:kx + (Wo - 1) * stride + 1:stride]
            y += np.einsum("bhwc,oc->bhwo", patch, W[:, ky, kx, :])
    return y


def conv_bwd(x, W, dy, stride, need_dx=True):
    B, H, Wd, C = x.shape
    Ho, Wo = dy.shape[1], dy.shape[2]
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    dW = np.zeros(W.shape)
    dxp = np.zeros(xp.shape) if need_dx else None
    for ky in range(3):
        for kx in range(3):
            sl = (slice(None), slice(ky, ky + (Ho - 1) * stride + 1, stride),
                  slice(kx, kx + (Wo - 1) * stride + 1, stride))
            dW[:, ky, kx, :] = np.einsum("bhwo,bhwc->oc", dy, xp[sl])
            if need_dx:
                dxp[sl] += np.einsum("bhwo,oc->bhwc", dy, W[:, ky, kx, :])
    dx = dxp[:, 1:H + 1, 1:Wd + 1] if need_dx else None
    return dW, dx


def up2(a, H, W):
    return a[:, np.arange(H) // 2][:, :, np.arange(W) // 2]


def forward(params, x):
    L = unpack(params)
    Wb = [(bf(W), b) for W, b in L]
    xb = bf(x)
    a1 = bf(np.maximum(conv(xb, Wb[0][0], 1) + Wb[0][1], 0))
    a2 = bf(np.maximum(conv(a1, Wb[1][0], 2) + Wb[1][1], 0))
    a3 = bf(np.maximum(conv(a2, Wb[2][0], 1) + Wb[2][1], 0))
    o16 = conv(a3, Wb[3][0], 1) + Wb[3][1]
    H, W = x.shape[1], x.shape[2]
    cat = np.concatenate([up2(a3, H, W), a1], axis=-1)
    a4 = bf(np.maximum(conv(cat, Wb[4][0], 1) + Wb[4][1], 0))
    o8 = conv(a4, Wb[5][0], 1) + Wb[5][1]
    return dict(x=xb, a1=a1, a2=a2, a3=a3, cat=cat, a4=a4, o16=o16, o8=o8, W=Wb)


def l1_grad(pred, tgt, mask, w):
    P = pred.shape[0] * pred.shape[1] * pred.shape[2]
    d = pred - tgt
    g = np.zeros_like(pred)
    loss = 0.0
    for c in range(3):
        m = mask > 0
        g[..., c] = np.where(m, w[c] * np.sign(d[..., c]), 0.0) / P
        loss += float(np.sum(np.where(m, w[c] * np.abs(d[..., c]), 0.0))) / P
    return g, loss


def backward(params, x, t16, m16, t8, m8, w=(1.0, 1.0, 10.0)):
    """Returns (flat gradient, loss, forward state)."""
    f = forward(params, x)
    Wb = f["W"]
    g16, l16 = l1_grad(f["o16"], t16, m16, w)
    g8, l8 = l1_grad(f["o8"], t8, m8, w)
    grads = [None] * 6

    def layer(i, xin, dy, stride, need_dx=True):
        dW, dx = conv_bwd(xin, Wb[i][0], bf(dy), stride, need_dx)
        grads[i] = (dW, dy.sum(axis=(0, 1, 2)))
        return dx

    g_a4 = layer(5, f["a4"], g8, 1)
    g_a4 = g_a4 * (f["a4"] > 0)
    g_cat = layer(4, f["cat"], g_a4, 1)
    H, W = x.shape[1], x.shape[2]
    H2, W2 = f["a3"].shape[1], f["a3"].shape[2]
    g_up = g_cat[..., :96]
    g_a3 = np.zeros(f["a3"].shape)
    for y in range(H):
        for xx in range(W):
            g_a3[:, y // 2, xx // 2] += g_up[:, y, xx]
    g_a1 = g_cat[..., 96:].copy()
    g_a3 += layer(3, f["a3"], g16, 1)
    g_a3 = g_a3 * (f["a3"] > 0)
    g_a2 = layer(2, f["a2"], g_a3, 1)
    g_a2 = g_a2 * (f["a2"] > 0)
    g_a1 += layer(1, f["a1"], g_a2, 2)
    g_a1 = g_a1 * (f["a1"] > 0)
    layer(0, f["x"], g_a1, 1, need_dx=False)
    flat = np.concatenate([np.concatenate([dW.ravel(), db.ravel()]) for dW, db in grads])
    return flat, l16 + l8, f
