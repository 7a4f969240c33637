"""Call mex entry points without Matlab, through libmexshim.so.

`MexFunction(path)` loads a mex shared object (RTLD_LOCAL: every ASETS mex
file exports the same global names, `mexFunction` and `runMaxFlow`) and calls
it the way the interpreter does: numpy arrays in, Matlab-shaped
(column-major) numpy arrays out, mexErrMsgTxt raised as `MexError`.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

from . import build as _build

_CLASS_TO_DTYPE = {
    6: np.float64,
    7: np.float32,
    8: np.int8,
    9: np.uint8,
    10: np.int16,
    11: np.uint16,
    12: np.int32,
    13: np.uint32,
}
_DTYPE_TO_CLASS = {np.dtype(v): k for k, v in _CLASS_TO_DTYPE.items()}

_ENTRY = ctypes.CFUNCTYPE(None, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p), ctypes.c_int,
                          ctypes.POINTER(ctypes.c_void_p))


class MexError(RuntimeError):
    """An error raised by a mex function through mexErrMsgTxt."""


_shim = None


def shim() -> ctypes.CDLL:
    global _shim
    if _shim is None:
        path = _build.LIB / "libmexshim.so"
        if not path.exists():
            raise RuntimeError(f"{path} is missing: run asetsmatlabmaxflow_gb300.build first")
        lib = ctypes.CDLL(str(path), mode=os.RTLD_GLOBAL | os.RTLD_NOW)
        lib.mxCreateNumericArray.restype = ctypes.c_void_p
        lib.mxCreateNumericArray.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                             ctypes.c_int, ctypes.c_int]
        lib.mxDestroyArray.argtypes = [ctypes.c_void_p]
        lib.mxGetData.restype = ctypes.c_void_p
        lib.mxGetData.argtypes = [ctypes.c_void_p]
        lib.mxGetNumberOfElements.restype = ctypes.c_size_t
        lib.mxGetNumberOfElements.argtypes = [ctypes.c_void_p]
        lib.mxGetNumberOfDimensions.restype = ctypes.c_int
        lib.mxGetNumberOfDimensions.argtypes = [ctypes.c_void_p]
        lib.mxGetDimensions.restype = ctypes.POINTER(ctypes.c_int)
        lib.mxGetDimensions.argtypes = [ctypes.c_void_p]
        lib.mxGetClassID.restype = ctypes.c_int
        lib.mxGetClassID.argtypes = [ctypes.c_void_p]
        lib.mexshim_call.restype = ctypes.c_int
        lib.mexshim_call.argtypes = [ctypes.c_void_p, ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_void_p), ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p,
                                     ctypes.c_size_t]
        lib.mexshim_last_print.restype = ctypes.c_char_p
        _shim = lib
    return _shim


def to_mx(arr: np.ndarray) -> int:
    """Copy a numpy array into a new mxArray (Matlab column-major)."""
    lib = shim()
    a = np.asarray(arr)
    if a.dtype not in _DTYPE_TO_CLASS:
        raise TypeError(f"unsupported dtype {a.dtype}")
    dims = list(a.shape) if a.ndim >= 2 else ([a.shape[0], 1] if a.ndim == 1 else [1, 1])
    cdims = (ctypes.c_int * len(dims))(*dims)
    mx = lib.mxCreateNumericArray(len(dims), cdims, _DTYPE_TO_CLASS[a.dtype], 0)
    if not mx:
        raise MemoryError("mxCreateNumericArray failed")
    flat = np.asfortranarray(a).ravel(order="F")
    if flat.size:
        ctypes.memmove(lib.mxGetData(mx), flat.ctypes.data, flat.nbytes)
    return mx


def from_mx(mx: int) -> np.ndarray:
    """Copy an mxArray out as a numpy array with Matlab's shape."""
    lib = shim()
    cls = lib.mxGetClassID(mx)
    nd = lib.mxGetNumberOfDimensions(mx)
    dptr = lib.mxGetDimensions(mx)
    dims = tuple(dptr[i] for i in range(nd))
    n = lib.mxGetNumberOfElements(mx)
    dt = np.dtype(_CLASS_TO_DTYPE[cls])
    out = np.empty(n, dtype=dt)
    if n:
        ctypes.memmove(out.ctypes.data, lib.mxGetData(mx), n * dt.itemsize)
    return out.reshape(dims, order="F")


class MexFunction:
    """A loaded mex file, callable with numpy arrays."""

    def __init__(self, path: str | Path, nlhs: int = 4):
        shim()
        self.path = Path(path)
        if not self.path.exists():
            raise FileNotFoundError(self.path)
        self._lib = ctypes.CDLL(str(self.path), mode=os.RTLD_LOCAL | os.RTLD_NOW)
        self._fn = ctypes.cast(self._lib.mexFunction, ctypes.c_void_p).value
        self.nlhs = nlhs

    def __call__(self, *args: np.ndarray) -> tuple[np.ndarray, ...]:
        lib = shim()
        prhs_list = [to_mx(a) for a in args]
        prhs = (ctypes.c_void_p * max(1, len(prhs_list)))(*prhs_list)
        plhs = (ctypes.c_void_p * self.nlhs)()
        err = ctypes.create_string_buffer(1024)
        try:
            rc = lib.mexshim_call(self._fn, self.nlhs, plhs, len(prhs_list), prhs, err,
                                  ctypes.sizeof(err))
            if rc != 0:
                raise MexError(err.value.decode(errors="replace"))
            outs = []
            for i in range(self.nlhs):
                if plhs[i]:
                    outs.append(from_mx(plhs[i]))
                    lib.mxDestroyArray(plhs[i])
                else:
                    outs.append(None)
            return tuple(outs)
        finally:
            for mx in prhs_list:
                lib.mxDestroyArray(mx)

    @staticmethod
    def last_print() -> str:
        return shim().mexshim_last_print().decode(errors="replace")
