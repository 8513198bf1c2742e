"""CPU restatement (numpy, float64) of the learned-proposal network and its layers.

TEST INFRASTRUCTURE ONLY: the checker for the tensor-core convolution kernels and the
U-Net forward / backward of multiview-reconstruction_gb300/csrc/unet.cu.  The network has
no counterpart in the reference, so there is nothing of the reference to pin it to; it
is pinned by these independent float64 restatements with BF16 rounding applied at the
same points as the device code (weights, activations, BF16 gradients).

Layouts: volumes [B][z][y][x][C]; weights W[co][27][ci] with tap t = 9 (dz+1) +
3 (dy+1) + (dx+1).
"""
from __future__ import annotations

import numpy as np

TAPS = [(t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1) for t in range(27)]
LAYERS = [(16, 16), (16, 32), (32, 64), (96, 32), (48, 16)]  # (ci, co)


def bf16(a):
    """Round to bfloat16 (nearest even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32).reshape(a.shape)


def bf16_bits(a):
    """bfloat16 bit patterns (uint16) of a."""
    return (bf16(a).view(np.uint32) >> 16).astype(np.uint16)


def _pad(x):
    return np.pad(x, ((0, 0), (1, 1), (1, 1), (1, 1), (0, 0)))


def _shift(xp, dz, dy, dx, shape):
    _, D, H, W, _ = shape
    return xp[:, 1 + dz:1 + dz + D, 1 + dy:1 + dy + H, 1 + dx:1 + dx + W, :]


def conv_fwd(x, w, b=None, relu=False):
    """y[n][co] = sum_t sum_ci x[n + off(t)][ci] w[co][t][ci] (+ b, ReLU), float64."""
    x = np.asarray(x, np.float64)
    w = np.asarray(w, np.float64)
    xp = _pad(x)
    y = np.zeros(x.shape[:4] + (w.shape[0],))
    for t, (dz, dy, dx) in enumerate(TAPS):
        y += np.einsum("bzyxc,oc->bzyxo", _shift(xp, dz, dy, dx, x.shape), w[:, t, :], optimize=True)
    if b is not None:
        y += np.asarray(b, np.float64)
    return np.maximum(y, 0.0) if relu else y


def conv_dgrad(g, w):
    """dx[m][ci] = sum_t sum_co g[m - off(t)][co] w[co][t][ci]."""
    g = np.asarray(g, np.float64)
    w = np.asarray(w, np.float64)
    gp = _pad(g)
    dx = np.zeros(g.shape[:4] + (w.shape[2],))
    for t, (dz, dy, dxo) in enumerate(TAPS):
        dx += np.einsum("bzyxo,oc->bzyxc", _shift(gp, -dz, -dy, -dxo, g.shape), w[:, t, :], optimize=True)
    return dx


def conv_wgrad(x, g):
    """dw[co][t][ci] = sum_n g[n][co] x[n + off(t)][ci]."""
    x = np.asarray(x, np.float64)
    g = np.asarray(g, np.float64)
    xp = _pad(x)
    dw = np.zeros((g.shape[4], 27, x.shape[4]))
    for t, (dz, dy, dx) in enumerate(TAPS):
        dw[:, t, :] = np.einsum("bzyxo,bzyxc->oc", g, _shift(xp, dz, dy, dx, x.shape), optimize=True)
    return dw


def pool(x):
    B, D, H, W, C = x.shape
    return x.reshape(B, D // 2, 2, H // 2, 2, W // 2, 2, C).mean(axis=(2, 4, 6))


def up(x):
    return x.repeat(2, axis=1).repeat(2, axis=2).repeat(2, axis=3)


def up_back(g):
    B, D, H, W, C = g.shape
    return g.reshape(B, D // 2, 2, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4, 6))


def unpack(params):
    """Split the flat parameter vector (layer W[co][27][ci], b[co], ..., head w[16], b)."""
    out, o = [], 0
    for ci, co in LAYERS:
        w = params[o:o + co * 27 * ci].reshape(co, 27, ci)
        o += co * 27 * ci
        b = params[o:o + co]
        o += co
        out.append((w, b))
    wh = params[o:o + 16]
    bh = params[o + 16]
    return out, wh, bh


def features(psi, psi_next):
    """[log(psi / mean psi), log(psi_next / psi), 0 x 14] per patch (float32 [B][z][y][x])."""
    psi = np.maximum(np.asarray(psi, np.float32), 1e-12)
    m = psi.reshape(psi.shape[0], -1).astype(np.float64).mean(axis=1).astype(np.float32)
    f = np.zeros(psi.shape + (16,), np.float32)
    f[..., 0] = np.log(psi / m[:, None, None, None])
    f[..., 1] = np.log(np.maximum(np.asarray(psi_next, np.float32), 1e-12) / psi)
    return bf16(f)


def forward_backward(params, x16, target, round_bf16=True):
    """Loss and parameter gradients of the U-Net, rounding to BF16 where the device does
    (round_bf16=False: plain float64, for finite-difference checks)."""
    global bf16
    rnd = bf16
    if not round_bf16:
        bf16 = lambda a: np.asarray(a, np.float64)  # noqa: E731
    try:
        return _forward_backward(params, x16, target)
    finally:
        bf16 = rnd


def _forward_backward(params, x16, target):
    layers, wh, bh = unpack(np.asarray(params, np.float64))
    wb = [(bf16(w), b) for w, b in layers]
    e1 = bf16(conv_fwd(x16, wb[0][0], wb[0][1], True))
    p1 = bf16(pool(e1))
    e2 = bf16(conv_fwd(p1, wb[1][0], wb[1][1], True))
    p2 = bf16(pool(e2))
    b3 = bf16(conv_fwd(p2, wb[2][0], wb[2][1], True))
    c2 = np.concatenate([up(b3), e2], axis=-1)
    d2 = bf16(conv_fwd(c2, wb[3][0], wb[3][1], True))
    c1 = np.concatenate([up(d2), e1], axis=-1)
    d1 = bf16(conv_fwd(c1, wb[4][0], wb[4][1], True))
    out = d1.astype(np.float64) @ wh.astype(np.float64) + float(bh)
    n = out.size
    diff = out - target
    loss = float((diff ** 2).sum() / n)
    gout = 2.0 * diff / n
    grads = []
    gwh = np.einsum("bzyx,bzyxc->c", gout, d1)
    gbh = gout.sum()
    G5 = np.where(d1 > 0, gout[..., None] * wh.astype(np.float64), 0.0)
    db5 = G5.reshape(-1, 16).sum(0)
    G5 = bf16(G5)
    dW5 = conv_wgrad(c1, G5)
    gc1 = conv_dgrad(G5, wb[4][0])
    G4 = np.where(d2 > 0, up_back(gc1[..., :32]), 0.0)
    db4 = G4.reshape(-1, 32).sum(0)
    G4 = bf16(G4)
    dW4 = conv_wgrad(c2, G4)
    gc2 = conv_dgrad(G4, wb[3][0])
    G3 = np.where(b3 > 0, up_back(gc2[..., :64]), 0.0)
    db3 = G3.reshape(-1, 64).sum(0)
    G3 = bf16(G3)
    dW3 = conv_wgrad(p2, G3)
    gp2 = conv_dgrad(G3, wb[2][0])
    G2 = np.where(e2 > 0, gc2[..., 64:] + up(gp2) / 8.0, 0.0)
    db2 = G2.reshape(-1, 32).sum(0)
    G2 = bf16(G2)
    dW2 = conv_wgrad(p1, G2)
    gp1 = conv_dgrad(G2, wb[1][0])
    G1 = np.where(e1 > 0, gc1[..., 32:] + up(gp1) / 8.0, 0.0)
    db1 = G1.reshape(-1, 16).sum(0)
    G1 = bf16(G1)
    dW1 = conv_wgrad(x16, G1)
    for dw, db in [(dW1, db1), (dW2, db2), (dW3, db3), (dW4, db4), (dW5, db5)]:
        grads += [dw.ravel(), db.ravel()]
    grads += [gwh.ravel(), np.array([gbh])]
    return loss, np.concatenate(grads), out
