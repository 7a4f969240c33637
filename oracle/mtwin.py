"""ORACLE -- test infrastructure only: numpy restatement of the Matlab
twins of the six solvers (maxflow/asetsBinaryMF2D.m, asetsBinaryMF3D.m,
asetsPotts2D.m, asetsPotts3D.m, asetsIshikawa2D.m, asetsIshikawa3D.m), in
the class of Ct (float32 or float64) and in Matlab's evaluation order, to
check the GPU's Matlab-semantics solvers (csrc/mtwin.cu).  Scalars (cc,
steps, 1/cc, ...) are rounded to the class of Ct as Matlab does when it
combines a double scalar with a single array.  erriter is summed in float64.

Arrays: (rows, cols[, slices][, labels]).  Flow faces: pp1 along columns
(rows x cols+1), pp2 along rows (rows+1 x cols), pp3 along slices.
"""
from __future__ import annotations

import numpy as np


def _flow(ud, pps, steps, alpha, binary_form):
    """Gradient step, projection and rescale of one flow label; returns divp.
    pps: [pp1, pp2(, pp3)] face arrays (modified in place)."""
    t = ud.dtype.type
    st = t(steps)
    axes = [1, 0, 2][:len(pps)]  # pp1: columns, pp2: rows, pp3: slices
    for pp, ax in zip(pps, axes):
        n = ud.shape[ax]
        inner = [slice(None)] * ud.ndim
        inner[ax] = slice(1, n)
        hi = np.take(ud, range(1, n), axis=ax)
        lo = np.take(ud, range(0, n - 1), axis=ax)
        if binary_form:   # pp1(:,2:cols) + steps*(pts(:,2:cols) - pts(:,1:cols-1))
            pp[tuple(inner)] = pp[tuple(inner)] + st * (hi - lo)
        else:             # steps*(ud(:,2:cols) - ud(:,1:cols-1)) + pp1(:,2:cols,k)
            pp[tuple(inner)] = st * (hi - lo) + pp[tuple(inner)]
    s = None
    for pp, ax in zip(pps, axes):
        n = pp.shape[ax]
        a = np.take(pp, range(0, n - 1), axis=ax)
        b = np.take(pp, range(1, n), axis=ax)
        s = a * a if s is None else s + a * a
        s = s + b * b
    gk = np.sqrt(s * t(0.5))
    le = gk <= alpha
    with np.errstate(divide="ignore", invalid="ignore"):
        gk = np.where(le, t(1), gk / alpha).astype(ud.dtype)
        gk = (t(1) / gk).astype(ud.dtype)
    for pp, ax in zip(pps, axes):
        n = ud.shape[ax]
        inner = [slice(None)] * ud.ndim
        inner[ax] = slice(1, n)
        hi = np.take(gk, range(1, n), axis=ax)
        lo = np.take(gk, range(0, n - 1), axis=ax)
        pp[tuple(inner)] = (t(0.5) * (hi + lo)) * pp[tuple(inner)]
    dv = None
    for pp, ax in zip(pps, axes):
        n = pp.shape[ax]
        b = np.take(pp, range(1, n), axis=ax)
        a = np.take(pp, range(0, n - 1), axis=ax)
        dv = (b - a) if dv is None else (dv + b) - a
    return dv


def _faces(shape, dt):
    out = [np.zeros((shape[0], shape[1] + 1) + shape[2:], dt),
           np.zeros((shape[0] + 1,) + shape[1:], dt)]
    if len(shape) == 3:
        out.append(np.zeros(shape[:2] + (shape[2] + 1,), dt))
    return out


def _mn(a, b):
    return np.where((a <= b) | np.isnan(a), a, b)


def binary(Cs, Ct, alpha, iterNum, beta, cc, steps):
    """asetsBinaryMF2D.m / asetsBinaryMF3D.m; returns (u, erriter, i)."""
    Ct = np.asarray(Ct)
    dt = Ct.dtype
    t = dt.type
    Cs = np.asarray(Cs, dt)
    alpha = np.asarray(alpha, dt)
    shape = Ct.shape
    ccT = t(cc)
    u = ((Cs - Ct) >= 0).astype(dt)
    ps = _mn(Cs, Ct).astype(dt)
    pt = ps.copy()
    pps = _faces(shape, dt)
    divp = np.zeros(shape, dt)
    erriter = np.zeros(iterNum, dt)
    i = 0
    for i in range(1, iterNum + 1):
        pts = divp - ((ps - pt) + u / ccT)
        divp = _flow(pts, pps, steps, alpha, True)
        pts = ((divp + pt) - u / ccT) + t(1 / cc)
        ps = _mn(pts, Cs)
        pts = ((-divp) + ps) + u / ccT
        pt = _mn(pts, Ct)
        erru = ccT * ((divp + pt) - ps)
        u = u - erru
        erriter[i - 1] = t(np.sum(np.abs(erru), dtype=np.float64) / Ct.size)
        if erriter[i - 1] < beta:
            break
    return u, erriter, i


def potts(Ct, alpha, iterNum, beta, cc, steps):
    """asetsPotts2D.m / asetsPotts3D.m (labels last)."""
    Ct = np.asarray(Ct)
    dt = Ct.dtype
    t = dt.type
    alpha = np.asarray(alpha, dt)
    L = Ct.shape[-1]
    shape = Ct.shape[:-1]
    ccT = t(cc)
    ps = Ct.min(axis=-1)
    I = Ct.argmin(axis=-1)
    pt = np.stack([ps] * L, axis=-1).astype(dt)
    u = np.stack([(I == k) for k in range(L)], axis=-1).astype(dt)
    divp = np.zeros(shape + (L,), dt)
    pps = [_faces(shape, dt) for _ in range(L)]
    erriter = np.zeros(iterNum, dt)
    vol = Ct.size
    i = 0
    for i in range(1, iterNum + 1):
        pd = np.zeros(shape, dt)
        for k in range(L):
            ud = divp[..., k] - ((ps - pt[..., k]) + u[..., k] / ccT)
            divp[..., k] = _flow(ud, pps[k], steps, alpha[..., k], False)
            ud = ((-divp[..., k]) + ps) + u[..., k] / ccT
            pt[..., k] = _mn(ud, Ct[..., k])
            pd = pd + ((divp[..., k] + pt[..., k]) - u[..., k] / ccT)
        ps = pd / t(L) + t(1 / (cc * L))
        s = 0.0
        for k in range(L):
            erru = ccT * ((divp[..., k] + pt[..., k]) - ps)
            u[..., k] = u[..., k] - erru
            s += np.sum(np.abs(erru), dtype=np.float64)
        erriter[i - 1] = t(s / vol)
        if erriter[i - 1] < beta:
            break
    return u, erriter, i


def ishikawa(Ct, alpha, iterNum, beta, cc, steps):
    """asetsIshikawa2D.m / asetsIshikawa3D.m (labels last; alpha: at least
    L-1 label slices)."""
    Ct = np.asarray(Ct)
    dt = Ct.dtype
    t = dt.type
    alpha = np.asarray(alpha, dt)
    L = Ct.shape[-1]
    shape = Ct.shape[:-1]
    ccT = t(cc)
    um = Ct.min(axis=-1)
    init = Ct.argmin(axis=-1) + 1  # Matlab's 1-based index
    pt = np.stack([um] * L, axis=-1).astype(dt)
    u = np.stack([(init > k) for k in range(1, L)], axis=-1).astype(dt)
    divp = np.zeros(shape + (L - 1,), dt)
    pps = [_faces(shape, dt) for _ in range(L - 1)]
    erriter = np.zeros(iterNum, dt)
    vol = Ct.size - 1  # rows*cols*nlab-1, as the .m files
    i = 0
    for i in range(1, iterNum + 1):
        for k in range(L - 1):
            ud = divp[..., k] - ((pt[..., k] - pt[..., k + 1]) + u[..., k] / ccT)
            divp[..., k] = _flow(ud, pps[k], steps, alpha[..., k], False)
        for k in range(L):
            if k == 0:
                ud = ((divp[..., 0] + pt[..., 1]) - u[..., 0] / ccT) + t(1 / cc)
            elif k < L - 1:
                ud = ((-divp[..., k - 1]) + pt[..., k - 1]) + u[..., k - 1] / ccT
                ud = ((ud + divp[..., k]) + pt[..., k + 1]) - u[..., k] / ccT
                ud = ud / t(2)
            else:
                ud = ((-divp[..., L - 2]) + pt[..., L - 2]) + u[..., L - 2] / ccT
            pt[..., k] = _mn(ud, Ct[..., k])
        s = 0.0
        for k in range(L - 1):
            erru = ccT * ((divp[..., k] + pt[..., k + 1]) - pt[..., k])
            u[..., k] = u[..., k] - erru
            s += np.sum(np.abs(erru), dtype=np.float64)
        erriter[i - 1] = t(s / vol)
        if erriter[i - 1] < beta:
            break
    return u, erriter, i
