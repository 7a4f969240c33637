"""ORACLE -- test infrastructure only: numpy restatement of the grid transfer
of the multilevel solve (restriction of the inputs, prolongation of a solved
state).  The multilevel solve has no counterpart in the reference; this
fixes its arithmetic (float32, the same summation order) so that the GPU
transfer can be checked bit for bit.

Arrays are flat float32 in Matlab layout, label slowest.  Internally they are
viewed in the kernel's axes (labels, s, c, r): 3D (L, z, x, y), 2D (L, x, 1, y).
"""
from __future__ import annotations

import numpy as np


def coarse_dims(dims, dim):
    ny, nx, nz = (tuple(dims) + (1,))[:3]
    return ((ny + 1) // 2, (nx + 1) // 2, (nz + 1) // 2 if dim == 3 else 1)


def _view(a, dims, dim):
    ny, nx, nz = (tuple(dims) + (1,))[:3]
    a = np.asarray(a, np.float32).reshape(-1)
    if dim == 3:
        return a.reshape(-1, nz, nx, ny)
    return a.reshape(-1, nx, 1, ny)


def restrict(a, dims, dim, scale):
    """Coarse cell = scale * mean of its fine block; sums in the order
    s, c, r (outer to inner), float32."""
    v = _view(a, dims, dim)
    L, ns, nc, nr = v.shape
    cs, cc, cr = (ns + 1) // 2, (nc + 1) // 2 if nc > 1 else 1, (nr + 1) // 2
    total = np.zeros((L, cs, cc, cr), np.float32)
    cnt = np.zeros((cs, cc, cr), np.float32)
    for ds in (0, 1) if ns > 1 else (0,):
        for dc in (0, 1) if nc > 1 else (0,):
            for dr in (0, 1):
                blk = v[:, ds::2, dc::2, dr::2] if nc > 1 else v[:, ds::2, :, dr::2]
                m = blk.shape[1:]
                total[:, :m[0], :m[1], :m[2]] += blk
                cnt[:m[0], :m[1], :m[2]] += 1
    out = (total / cnt) * np.float32(scale)
    return out.astype(np.float32).reshape(-1)


def _cell(v, shape):
    L, ns, nc, nr = shape
    out = v.repeat(2, axis=3)[:, :, :, :nr]
    out = out.repeat(2, axis=1)[:, :ns] if ns > 1 else out
    out = out.repeat(2, axis=2)[:, :, :nc] if nc > 1 else out
    return out


def prolong(a, coarse, fine, dim, scale=1.0, axis=None):
    """Fine array from a coarse one.  axis None: a cell quantity (copied);
    axis 'r' / 'c' / 's': a flow along that kernel axis (coarse face at even
    fine faces, the mean of the two neighbouring coarse faces at odd ones,
    zero beyond the last)."""
    v = _view(a, coarse, dim)
    fv = np.zeros((v.shape[0],) + _view(np.zeros(int(np.prod(fine)) * v.shape[0]), fine, dim).shape[1:],
                  np.float32)
    shape = fv.shape
    near = _cell(v, shape)
    if axis is None:
        return (near * np.float32(scale)).astype(np.float32).reshape(-1)
    ax = {"s": 1, "c": 2, "r": 3}[axis]
    if shape[ax] == 1:  # an axis of one cell is not coarsened
        return (near * np.float32(scale)).astype(np.float32).reshape(-1)
    nxt = np.concatenate([np.take(v, np.arange(1, v.shape[ax]), axis=ax),
                          np.zeros_like(np.take(v, [0], axis=ax))], axis=ax)
    mid = ((v + nxt) * np.float32(0.5)).astype(np.float32)
    mid_f = _cell(mid, shape)
    idx = np.arange(shape[ax]) % 2 == 1
    sel = idx.reshape([-1 if i == ax else 1 for i in range(4)])
    out = np.where(sel, mid_f, near)
    return (out * np.float32(scale)).astype(np.float32).reshape(-1)


def flow_axes(dim):
    """Kernel axis of the reference's (bx, by, bz)."""
    return ("c", "r", "s") if dim == 3 else ("s", "r")
