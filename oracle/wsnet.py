"""ORACLE -- test infrastructure only: float64 restatement of the warm-start
network (four 3x3x3 convolutions, 16 channels, ReLU between them) and of its
backward pass, used to check the GPU gradients.

It rounds to BF16 wherever the GPU stores BF16 (weights, activations, the
gradients passed between layers) and computes everything else in float64,
so GPU/oracle differences are accumulation order only.
"""
from __future__ import annotations

import numpy as np

BLOCKS = 5   # 3 hidden layers + the two 16-channel halves of the output layer
NW = 27 * 16 * 16


def bf16(a: np.ndarray) -> np.ndarray:
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params: np.ndarray):
    ws, bs = [], []
    for b in range(BLOCKS):
        base = b * (NW + 16)
        ws.append(params[base:base + NW].reshape(27, 16, 16).astype(np.float64))
        bs.append(params[base + NW:base + NW + 16].astype(np.float64))
    return ws, bs


def _pad(x):
    nz, nx, ny, c = x.shape
    xp = np.zeros((nz + 2, nx + 2, ny + 2, c))
    xp[1:-1, 1:-1, 1:-1] = x
    return xp


def conv(x, w, b=None):
    nz, nx, ny, _ = x.shape
    xp = _pad(x)
    out = np.zeros((nz, nx, ny, w.shape[2]))
    for t in range(27):
        dz, dx, dy = t // 9, (t // 3) % 3, t % 3
        out += np.einsum("zxyc,cd->zxyd", xp[dz:dz + nz, dx:dx + nx, dy:dy + ny], w[t])
    if b is not None:
        out += b
    return out


def conv_transpose(g, w):
    """Gradient of conv w.r.t. its input."""
    nz, nx, ny, _ = g.shape
    gp = _pad(g)
    out = np.zeros((nz, nx, ny, 16))
    for t in range(27):
        dz, dx, dy = 2 - t // 9, 2 - (t // 3) % 3, 2 - t % 3
        out += np.einsum("zxyd,cd->zxyc", gp[dz:dz + nz, dx:dx + nx, dy:dy + ny], w[t])
    return out


def wgrad(a, g):
    nz, nx, ny, _ = a.shape
    ap = _pad(a)
    dw = np.zeros((27, 16, 16))
    for t in range(27):
        dz, dx, dy = t // 9, (t // 3) % 3, t % 3
        dw[t] = np.einsum("zxyc,zxyd->cd", ap[dz:dz + nz, dx:dx + nx, dy:dy + ny], g)
    return dw


def loss_and_grads(params, x, target, L):
    """x: [nz, nx, ny, 16] network input (BF16 values); target: [.., 32]
    (u, ps, pt, flows/alpha).  Returns (loss, flat gradient in the parameter
    layout, 32-channel output)."""
    ws, bs = unpack(params)
    wq = [bf16(w) for w in ws]
    acts = [bf16(x)]
    for l in range(3):
        acts.append(bf16(np.maximum(conv(acts[-1], wq[l], bs[l]), 0.0)))
    out = np.concatenate([conv(acts[3], wq[3], bs[3]), conv(acts[3], wq[4], bs[4])], axis=-1)
    used = 5 * L + 1
    vox = x.shape[0] * x.shape[1] * x.shape[2]
    scale = 1.0 / (vox * used)
    d = np.zeros_like(out)
    d[..., :used] = out[..., :used] - target[..., :used]
    loss = float(np.sum(d * d) * scale)
    g = bf16(2.0 * d * scale)
    grads = np.zeros(BLOCKS * (NW + 16))

    def put(b, a, gg):
        base = b * (NW + 16)
        grads[base:base + NW] = wgrad(a, gg).ravel()
        grads[base + NW:base + NW + 16] = gg.sum(axis=(0, 1, 2))

    put(3, acts[3], g[..., :16])
    put(4, acts[3], g[..., 16:])
    gh = conv_transpose(g[..., :16], wq[3]) + conv_transpose(g[..., 16:], wq[4])
    gh = bf16(np.where(acts[3] > 0, gh, 0.0))
    for l in range(2, -1, -1):
        put(l, acts[l], gh)
        if l == 0:
            break
        gh = bf16(np.where(acts[l] > 0, conv_transpose(gh, wq[l]), 0.0))
    return loss, grads, out
