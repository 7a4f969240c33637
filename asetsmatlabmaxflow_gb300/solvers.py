"""Python mirror of the six ASETS mex entry points, running on the GPU.

    u, erriter, i, timet = asetsBinaryMF3D_mex(Cs, Ct, alpha, pars)

Same inputs, pars layout and outputs as the reference mex files
(maxflow/asets*_mex.c mexFunction): arrays are single precision in Matlab
shape (numpy, column-major indexing), `erriter` is maxIt x 1, `i` a 1x1
uint16, `timet` a 1x1 single.  alpha <= 0 raises the reference's message.
Calls go through the C ABI (asets_binary_mf2d & co.) on the default context.

`mex_dropin(name)` instead loads the compiled drop-in mex file
(lib/<name>.so) and calls its mexFunction through the mex host emulation,
exactly as Matlab would.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import build as _build
from . import native as N
from .mexhost import MexError, MexFunction


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32).ravel(order="F"))


def _parse(pars, dim: int, labelled: bool):
    p = np.asarray(pars, dtype=np.float32).ravel()
    i = 0
    ny = int(p[i]); i += 1
    nx = int(p[i]); i += 1
    nz = 1
    if dim == 3:
        nz = int(p[i]); i += 1
    nlab = 1
    if labelled:
        nlab = int(p[i]); i += 1
    max_it = int(p[i]); err = float(p[i + 1]); cc = float(p[i + 2]); steps = float(p[i + 3])
    return ny, nx, nz, nlab, max_it, np.float32(err), np.float32(cc), np.float32(steps)


def _call(fn_name, model, dim, Cs, Ct, alpha, pars, exact=False):
    labelled = model != "binary"
    ny, nx, nz, nlab, max_it, errb, cc, steps = _parse(pars, dim, labelled)
    n = ny * nx * nz
    nu = n if model == "binary" else (n * nlab if model == "potts" else n * (nlab - 1))
    u = np.zeros(nu, np.float32)
    cvg = np.zeros(max(max_it, 1), np.float32)
    it = ctypes.c_int(0)
    secs = ctypes.c_float(0)
    opt = N.Options(flags=N.FLAG_EXACT if exact else 0)
    ct = _f32(Ct)
    al = _f32(alpha)
    fn = getattr(N.lib(), fn_name)
    p = N._ptr
    if model == "binary":
        cs = _f32(Cs)
        args = [None, ctypes.addressof(opt), p(al), p(cs), p(ct), nx, ny]
        if dim == 3:
            args.append(nz)
    else:
        args = [None, ctypes.addressof(opt), p(al), p(ct), nx, ny]
        if dim == 3:
            args.append(nz)
        args.append(nlab)
    args += [max_it, errb, cc, steps, p(u), p(cvg), ctypes.addressof(it), ctypes.addressof(secs)]
    st = fn(*args)
    if st == N.ASETS_ERR_ALPHA:
        raise MexError("alpha(x) must be positive. Exiting..." if model == "binary"
                       else "alpha(x,l) must be positive. Exiting...")
    N.check(st)
    shape = (ny, nx) + ((nz,) if dim == 3 else ())
    if model == "potts":
        shape += (nlab,)
    elif model == "ishikawa":
        shape += (nlab - 1,)
    return (u.reshape(shape, order="F"), cvg[:max_it].reshape(max_it, 1),
            np.array([[it.value]], dtype=np.uint16), np.array([[secs.value]], dtype=np.float32))


def asetsBinaryMF2D_mex(Cs, Ct, alpha, pars, *, exact=False):
    """maxflow/asetsBinaryMF2D_mex.c:36-129; pars = [rows, cols, maxIt, errBound, cc, steps]."""
    return _call("asets_binary_mf2d", "binary", 2, Cs, Ct, alpha, pars, exact)


def asetsBinaryMF3D_mex(Cs, Ct, alpha, pars, *, exact=False):
    """maxflow/asetsBinaryMF3D_mex.c:39-134; pars = [rows, cols, slices, maxIt, errBound, cc, steps]."""
    return _call("asets_binary_mf3d", "binary", 3, Cs, Ct, alpha, pars, exact)


def asetsPotts2D_mex(Ct, alpha, pars, *, exact=False):
    """maxflow/asetsPotts2D_mex.c:42-135; pars = [rows, cols, nLab, maxIt, errBound, cc, steps]."""
    return _call("asets_potts2d", "potts", 2, None, Ct, alpha, pars, exact)


def asetsPotts3D_mex(Ct, alpha, pars, *, exact=False):
    """maxflow/asetsPotts3D_mex.c:44-141; pars = [rows, cols, slices, nLab, maxIt, errBound, cc, steps]."""
    return _call("asets_potts3d", "potts", 3, None, Ct, alpha, pars, exact)


def asetsIshikawa2D_mex(Ct, alpha, pars, *, exact=False):
    """maxflow/asetsIshikawa2D_mex.c:40-133; pars = [rows, cols, nLab, maxIt, errBound, cc, steps]."""
    return _call("asets_ishikawa2d", "ishikawa", 2, None, Ct, alpha, pars, exact)


def asetsIshikawa3D_mex(Ct, alpha, pars, *, exact=False):
    """maxflow/asetsIshikawa3D_mex.c:42-138; pars = [rows, cols, slices, nLab, maxIt, errBound, cc, steps]."""
    return _call("asets_ishikawa3d", "ishikawa", 3, None, Ct, alpha, pars, exact)


MEX_FUNCTIONS = {
    "asetsBinaryMF2D_mex": asetsBinaryMF2D_mex,
    "asetsBinaryMF3D_mex": asetsBinaryMF3D_mex,
    "asetsPotts2D_mex": asetsPotts2D_mex,
    "asetsPotts3D_mex": asetsPotts3D_mex,
    "asetsIshikawa2D_mex": asetsIshikawa2D_mex,
    "asetsIshikawa3D_mex": asetsIshikawa3D_mex,
}

_dropins: dict[str, MexFunction] = {}


def mex_dropin(name: str) -> MexFunction:
    """The compiled GPU mex file `name`, callable like the reference's."""
    if name not in _dropins:
        N.lib()  # make libasetscuda resolvable for the mex file
        _dropins[name] = MexFunction(_build.LIB / f"{name}.so")
    return _dropins[name]
