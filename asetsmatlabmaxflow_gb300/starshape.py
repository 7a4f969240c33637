"""Star-shape Potts 2D on the GPU, with the Matlab function's signature
(maxflow/asetsPotts2D_starShape.m): [u, erriter, i, timet] =
asetsPotts2D_starShape(Ct, alpha, pars, ss_initPoints)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import native as N


def asetsPotts2D_starShape(Ct, alpha, pars, ss_initPoints, *, ctx=None):
    """pars = [rows, cols, nlab, iterNum, beta, cc, steps, stepv];
    ss_initPoints: nlab x 2 of 1-based (column, row) seed points.  Computes
    in double precision, as the Matlab function does."""
    rows, cols, nlab, iterNum = (int(v) for v in pars[:4])
    beta, cc, steps, stepv = (float(v) for v in pars[4:8])
    ct = np.ascontiguousarray(np.asarray(Ct, np.float64).reshape(rows, cols, nlab)
                              .ravel(order="F"))
    al = np.ascontiguousarray(np.asarray(alpha, np.float64).reshape(rows, cols, nlab)
                              .ravel(order="F"))
    pts = np.ascontiguousarray(np.asarray(ss_initPoints, np.int32).reshape(nlab, 2))
    u = np.empty(rows * cols * nlab, np.float64)
    err = np.empty(iterNum, np.float64)
    it = ctypes.c_int(0)
    secs = ctypes.c_float(0)
    h = (ctx or N.Context.default()).handle
    N.check(N.lib().asets_potts2d_starshape(h, ct.ctypes.data, al.ctypes.data, rows, cols, nlab,
                                            iterNum, beta, cc, steps, stepv, pts.ctypes.data,
                                            u.ctypes.data, err.ctypes.data, ctypes.byref(it),
                                            ctypes.byref(secs)))
    return u.reshape((rows, cols, nlab), order="F"), err.reshape(-1, 1), it.value, secs.value
