"""ORACLE -- test infrastructure only: Python access to the C restatement
(liboracle.so) and to the compiled reference mex solvers (oracle/_ref).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs use
this module, and only as the checker or the timed CPU baseline.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import build as _build

BINARY, POTTS, ISHIKAWA = 0, 1, 2
MODELS = {"binary": BINARY, "potts": POTTS, "ishikawa": ISHIKAWA}

_FP = ctypes.POINTER(ctypes.c_float)


class OracleProblem(ctypes.Structure):
    _fields_ = [
        ("model", ctypes.c_int), ("dim", ctypes.c_int),
        ("ny", ctypes.c_int), ("nx", ctypes.c_int), ("nz", ctypes.c_int), ("nlab", ctypes.c_int),
        ("max_it", ctypes.c_int), ("err_bound", ctypes.c_float), ("cc", ctypes.c_float),
        ("steps", ctypes.c_float), ("erru_double", ctypes.c_int),
        ("alpha", _FP), ("cs", _FP), ("ct", _FP),
        ("u0", _FP), ("ps0", _FP), ("pt0", _FP),
        ("u", _FP), ("cvg", _FP), ("it_num", ctypes.POINTER(ctypes.c_int)),
        ("ps_out", _FP), ("pt_out", _FP),
    ]


class OracleError(RuntimeError):
    pass


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        path = _build.build_port()
        _lib = ctypes.CDLL(str(path))
        _lib.oracle_solve.restype = ctypes.c_int
        _lib.oracle_solve.argtypes = [ctypes.POINTER(OracleProblem)]
    return _lib


def _fptr(a: np.ndarray | None):
    if a is None:
        return ctypes.cast(None, _FP)
    return a.ctypes.data_as(_FP)


def _flat(a) -> np.ndarray | None:
    if a is None:
        return None
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32).ravel(order="F"))


def solve(model: str, dims: tuple[int, ...], ct, alpha, *, cs=None, nlab: int = 1,
          max_it: int, err_bound: float, cc: float, steps: float, erru_double: bool = False,
          u0=None, ps0=None, pt0=None, want_state: bool = False) -> dict:
    """Run the restatement.  `dims` is (ny, nx) or (ny, nx, nz); arrays are in
    Matlab column-major order (any numpy layout is accepted and flattened
    with order='F').  Returns u/cvg/it (+ps/pt when want_state)."""
    m = MODELS[model]
    dim = len(dims)
    ny, nx = dims[0], dims[1]
    nz = dims[2] if dim == 3 else 1
    n = ny * nx * nz
    nu = n if m == BINARY else (n * nlab if m == POTTS else n * (nlab - 1))
    bufs = {
        "alpha": _flat(alpha), "cs": _flat(cs), "ct": _flat(ct),
        "u0": _flat(u0), "ps0": _flat(ps0), "pt0": _flat(pt0),
    }
    u = np.zeros(nu, np.float32)
    cvg = np.zeros(max(max_it, 1), np.float32)
    it = ctypes.c_int(0)
    ps = np.zeros(n, np.float32) if want_state and m != ISHIKAWA else None
    npt = n if m == BINARY else n * nlab
    pt = np.zeros(npt, np.float32) if want_state else None
    prob = OracleProblem(
        model=m, dim=dim, ny=ny, nx=nx, nz=nz, nlab=nlab, max_it=max_it,
        err_bound=np.float32(err_bound), cc=np.float32(cc), steps=np.float32(steps),
        erru_double=int(erru_double),
        alpha=_fptr(bufs["alpha"]), cs=_fptr(bufs["cs"]), ct=_fptr(bufs["ct"]),
        u0=_fptr(bufs["u0"]), ps0=_fptr(bufs["ps0"]), pt0=_fptr(bufs["pt0"]),
        u=_fptr(u), cvg=_fptr(cvg), it_num=ctypes.pointer(it),
        ps_out=_fptr(ps), pt_out=_fptr(pt),
    )
    rc = lib().oracle_solve(ctypes.byref(prob))
    if rc == 1:
        raise OracleError("alpha(x) must be positive. Exiting...")
    if rc != 0:
        raise OracleError(f"oracle_solve failed with code {rc}")
    out = {"u": u, "cvg": cvg[:max_it], "it": it.value}
    if want_state:
        out["ps"] = ps
        out["pt"] = pt
    return out


# ---------------------------------------------------------------- reference

def reference_available() -> bool:
    return all((_build.REF_OUT / f"{s}.so").exists() for s in _build.REF_SOLVERS)


_ref_cache: dict[str, object] = {}


def reference(name: str):
    """The compiled reference mex function `name` (e.g. 'asetsBinaryMF3D_mex')."""
    from asetsmatlabmaxflow_gb300.mexhost import MexFunction

    if name not in _ref_cache:
        path = _build.REF_OUT / f"{name}.so"
        if not path.exists():
            _build.build_reference()
        if not path.exists():
            raise FileNotFoundError(f"{path}: reference sources unavailable on this machine")
        _ref_cache[name] = MexFunction(path)
    return _ref_cache[name]
