"""The reference's Matlab solvers (maxflow/asets*.m, the gpuArray path) on
the GPU, with their signatures: [u, erriter, i, timet] = f(Cs, Ct, alpha,
pars) or f(Ct, alpha, pars).  They compute in the class of Ct (float32 or
float64; other types as float64), with the .m files' initialisation,
expression order and `<` break rule -- unlike the mex files, which
asetsmatlabmaxflow_gb300.solvers mirrors."""
from __future__ import annotations

import ctypes

import numpy as np

from . import native as N

BINARY, POTTS, ISHIKAWA = 0, 1, 2


def _solve(model, dim, Cs, Ct, alpha, rows, cols, slices, nlab, iterNum, beta, cc, steps,
           ctx=None):
    Ct = np.asarray(Ct)
    dt = Ct.dtype if Ct.dtype in (np.float32, np.float64) else np.dtype(np.float64)
    n = rows * cols * slices
    L = 1 if model == BINARY else nlab
    nflow = L - 1 if model == ISHIKAWA else L

    def flat(a, labels):
        a = np.asarray(a, dt).reshape(-1, order="F")
        return np.ascontiguousarray(a[:n * labels])

    ct = flat(Ct, L)
    al = flat(alpha, nflow)
    cs = flat(Cs, 1) if model == BINARY else None
    nu = nflow
    u = np.empty(n * nu, dt)
    err = np.empty(iterNum, dt)
    it = ctypes.c_int(0)
    secs = ctypes.c_float(0)
    N.check(N.lib().asets_matlab_solve((ctx or N.Context.default()).handle, model, dt.itemsize,
                                       dim, rows, cols, slices, L,
                                       None if cs is None else cs.ctypes.data, ct.ctypes.data,
                                       al.ctypes.data, iterNum, beta, cc, steps, u.ctypes.data,
                                       err.ctypes.data, ctypes.byref(it), ctypes.byref(secs)))
    shape = (rows, cols) + ((slices,) if dim == 3 else ()) + ((nu,) if model != BINARY else ())
    return u.reshape(shape, order="F"), err.reshape(-1, 1), it.value, secs.value


def _ints(pars, k):
    return [int(round(float(v))) for v in pars[:k]]


def asetsBinaryMF2D(Cs, Ct, alpha, pars, *, ctx=None):
    """pars = [rows, cols, iterNum, beta, cc, steps] (asetsBinaryMF2D.m)."""
    rows, cols, iterNum = _ints(pars, 3)
    beta, cc, steps = (float(v) for v in pars[3:6])
    return _solve(BINARY, 2, Cs, Ct, alpha, rows, cols, 1, 1, iterNum, beta, cc, steps, ctx)


def asetsBinaryMF3D(Cs, Ct, alpha, pars, *, ctx=None):
    """pars = [rows, cols, slices, iterNum, beta, cc, steps] (asetsBinaryMF3D.m)."""
    rows, cols, slices, iterNum = _ints(pars, 4)
    beta, cc, steps = (float(v) for v in pars[4:7])
    return _solve(BINARY, 3, Cs, Ct, alpha, rows, cols, slices, 1, iterNum, beta, cc, steps, ctx)


def asetsPotts2D(Ct, alpha, pars, *, ctx=None):
    """pars = [rows, cols, nlab, iterNum, beta, cc, steps] (asetsPotts2D.m)."""
    rows, cols, nlab, iterNum = _ints(pars, 4)
    beta, cc, steps = (float(v) for v in pars[4:7])
    return _solve(POTTS, 2, None, Ct, alpha, rows, cols, 1, nlab, iterNum, beta, cc, steps, ctx)


def asetsPotts3D(Ct, alpha, pars, *, ctx=None):
    """pars = [rows, cols, slices, nlab, iterNum, beta, cc, steps] (asetsPotts3D.m)."""
    rows, cols, slices, nlab, iterNum = _ints(pars, 5)
    beta, cc, steps = (float(v) for v in pars[5:8])
    return _solve(POTTS, 3, None, Ct, alpha, rows, cols, slices, nlab, iterNum, beta, cc, steps,
                  ctx)


def asetsIshikawa2D(Ct, alpha, pars, *, ctx=None):
    """pars = [rows, cols, nlab, iterNum, beta, cc, steps]; alpha with at
    least nlab-1 label slices (asetsIshikawa2D.m)."""
    rows, cols, nlab, iterNum = _ints(pars, 4)
    beta, cc, steps = (float(v) for v in pars[4:7])
    return _solve(ISHIKAWA, 2, None, Ct, alpha, rows, cols, 1, nlab, iterNum, beta, cc, steps,
                  ctx)


def asetsIshikawa3D(Ct, alpha, pars, *, ctx=None):
    """pars = [rows, cols, slices, nlab, iterNum, beta, cc, steps] (asetsIshikawa3D.m)."""
    rows, cols, slices, nlab, iterNum = _ints(pars, 5)
    beta, cc, steps = (float(v) for v in pars[5:8])
    return _solve(ISHIKAWA, 3, None, Ct, alpha, rows, cols, slices, nlab, iterNum, beta, cc,
                  steps, ctx)
