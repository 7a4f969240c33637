"""ctypes binding of libasetscuda (include/asets.h).

The library must have been built in-tree (asetsmatlabmaxflow_gb300.build);
there is no fallback: every solve runs the CUDA kernels or raises.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

from . import build as _build

ASETS_OK = 0
ASETS_ERR_INVALID_ARG = 1
ASETS_ERR_ALPHA = 2
ASETS_ERR_CUDA = 3
ASETS_ERR_OUT_OF_MEMORY = 4
ASETS_ERR_TIMEOUT = 5
ASETS_ERR_NO_DEVICE = 6
ASETS_ERR_UNSUPPORTED = 7

BINARY, POTTS, ISHIKAWA = 0, 1, 2
MODELS = {"binary": BINARY, "potts": POTTS, "ishikawa": ISHIKAWA}
HOST, DEVICE = 0, 1
FLAG_EXACT = 0x1
FLAG_NO_ALPHA_CHECK = 0x2
FLAG_AUTOTUNE = 0x4

_FP = ctypes.POINTER(ctypes.c_float)
_VP = ctypes.c_void_p


class AsetsError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status
        self.message = message


class AlphaError(AsetsError):
    """alpha(x) <= 0, the reference's mexErrMsgTxt case."""


class Options(ctypes.Structure):
    _fields_ = [("flags", ctypes.c_int), ("tile_config", ctypes.c_int),
                ("reserved", ctypes.c_int * 6)]


_lib = None

# ASETS_LIB_DIR selects another in-tree build (the bounds-check flavour in
# lib_check/); the default is the release build in lib/.
LIB_PATH = Path(os.environ["ASETS_LIB_DIR"]) / "libasetscuda.so" if os.environ.get(
    "ASETS_LIB_DIR") else _build.LIB / "libasetscuda.so"

# name -> (restype, argtypes)
_SIGS = {
    "asets_abi_version": (ctypes.c_int, []),
    "asets_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "asets_last_error": (ctypes.c_char_p, []),
    "asets_context_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(_VP)]),
    "asets_context_destroy": (None, [_VP]),
    "asets_default_context": (ctypes.c_int, [ctypes.POINTER(_VP)]),
    "asets_context_set_stream": (ctypes.c_int, [_VP, _VP]),
    "asets_binary_mf2d": (ctypes.c_int, [_VP, _VP, _VP, _VP, _VP, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                         ctypes.c_float, _VP, _VP, _VP, _VP]),
    "asets_binary_mf3d": (ctypes.c_int, [_VP, _VP, _VP, _VP, _VP, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                         ctypes.c_float, ctypes.c_float, _VP, _VP, _VP, _VP]),
    "asets_potts2d": (ctypes.c_int, [_VP, _VP, _VP, _VP, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                     ctypes.c_float, _VP, _VP, _VP, _VP]),
    "asets_potts3d": (ctypes.c_int, [_VP, _VP, _VP, _VP, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                     ctypes.c_float, ctypes.c_float, _VP, _VP, _VP, _VP]),
    "asets_ishikawa2d": (ctypes.c_int, [_VP, _VP, _VP, _VP, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                        ctypes.c_float, ctypes.c_float, _VP, _VP, _VP, _VP]),
    "asets_ishikawa3d": (ctypes.c_int, [_VP, _VP, _VP, _VP, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                        ctypes.c_float, ctypes.c_float, _VP, _VP, _VP, _VP]),
    "asets_solver_create": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.POINTER(_VP)]),
    "asets_solver_destroy": (None, [_VP]),
    "asets_solver_set_inputs": (ctypes.c_int, [_VP, ctypes.c_int, _VP, _VP, _VP]),
    "asets_solver_set_initial": (ctypes.c_int, [_VP, ctypes.c_int, _VP, _VP, _VP]),
    "asets_solver_run": (ctypes.c_int, [_VP, _VP, ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                        ctypes.c_float, ctypes.POINTER(ctypes.c_int)]),
    "asets_solver_get_u": (ctypes.c_int, [_VP, ctypes.c_int, _VP]),
    "asets_solver_get_cvg": (ctypes.c_int, [_VP, ctypes.c_int, _VP, ctypes.c_int]),
    "asets_solver_get_flows": (ctypes.c_int, [_VP, ctypes.c_int, _VP, _VP]),
    "asets_solver_run_multilevel": (ctypes.c_int, [_VP, _VP, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                                    ctypes.c_float, ctypes.c_float,
                                                    ctypes.POINTER(ctypes.c_int)]),
    "asets_solver_multilevel_prepare": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    "asets_solver_level": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.POINTER(_VP)]),
    "asets_solver_multilevel_stats": (ctypes.c_int, [_VP, ctypes.c_int, _VP, _VP, ctypes.POINTER(ctypes.c_int)]),
    "asets_selftest_wait_timeout": (ctypes.c_int, [_VP]),
    "asets_matlab_solve": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          _VP, _VP, _VP, ctypes.c_int, ctypes.c_double,
                                          ctypes.c_double, ctypes.c_double, _VP, _VP,
                                          ctypes.POINTER(ctypes.c_int),
                                          ctypes.POINTER(ctypes.c_float)]),
    "asets_dag_full_flow": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_int, ctypes.c_int, _VP, _VP,
                                           _VP, _VP, _VP, ctypes.c_int, ctypes.c_double,
                                           ctypes.c_double, _VP, _VP, _VP, _VP, _VP, _VP, _VP,
                                           _VP]),
    "asets_dag_run": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_int, _VP, _VP, _VP, _VP, _VP, _VP,
                                     _VP, _VP, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                     _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP]),
    "asets_hmf_run": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_int, _VP, _VP, _VP, _VP,
                                     _VP, _VP, _VP, ctypes.c_int, ctypes.c_double,
                                     ctypes.c_double, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP,
                                     _VP]),
    "asets_hmf_full_flow": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_int, ctypes.c_int, _VP, _VP,
                                           _VP, _VP, ctypes.c_int, ctypes.c_double,
                                           ctypes.c_double, _VP, _VP, _VP, _VP, _VP, _VP, _VP,
                                           _VP, _VP]),
    "asets_potts2d_starshape": (ctypes.c_int, [_VP, _VP, _VP, ctypes.c_int, ctypes.c_int,
                                               ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                               ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                               _VP, _VP, _VP, ctypes.POINTER(ctypes.c_int),
                                               ctypes.POINTER(ctypes.c_float)]),
    "asets_cost_l1": (ctypes.c_int, [_VP, ctypes.c_int, _VP, ctypes.c_longlong, _VP, ctypes.c_int,
                                     ctypes.c_int, _VP]),
    "asets_cost_neglog": (ctypes.c_int, [_VP, ctypes.c_int, _VP, ctypes.c_longlong, ctypes.c_int,
                                         ctypes.c_float, _VP]),
    "asets_cost_histogram_ll": (ctypes.c_int, [_VP, ctypes.c_int, _VP, _VP, ctypes.c_longlong,
                                               ctypes.c_int, ctypes.c_double, _VP, _VP]),
    "asets_alpha_contrast": (ctypes.c_int, [_VP, ctypes.c_int, _VP, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                            ctypes.c_float, ctypes.c_float, ctypes.c_int,
                                            ctypes.c_int, _VP]),
    "asets_solver_get_inputs": (ctypes.c_int, [_VP, ctypes.c_int, _VP, _VP, _VP]),
    "asets_solver_set_initial_flows": (ctypes.c_int, [_VP, ctypes.c_int, _VP, _VP, _VP]),
    "asets_solver_get_spatial_flows": (ctypes.c_int, [_VP, ctypes.c_int, _VP, _VP, _VP]),
    "asets_solver_last_run_stats": (ctypes.c_int, [_VP, ctypes.POINTER(ctypes.c_float),
                                                   ctypes.POINTER(ctypes.c_int)]),
    "asets_batch_create": (ctypes.c_int, [_VP, ctypes.POINTER(_VP)]),
    "asets_batch_destroy": (None, [_VP]),
    "asets_batch_add": (ctypes.c_int, [_VP, _VP]),
    "asets_batch_run": (ctypes.c_int, [_VP, _VP, ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                       ctypes.c_float, _VP]),
    "asets_batch_last_run_stats": (ctypes.c_int, [_VP, ctypes.POINTER(ctypes.c_float),
                                                  ctypes.POINTER(ctypes.c_int),
                                                  ctypes.POINTER(ctypes.c_int), _VP]),
    "asets_batch_run_multilevel": (ctypes.c_int, [_VP, _VP, ctypes.c_int, ctypes.c_int,
                                                  ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                                  _VP]),
    "asets_conv3d_bf16": (ctypes.c_int, [_VP, _VP, _VP, _VP, _VP, _VP, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "asets_wsnet_num_params": (ctypes.c_int, []),
    "asets_wsnet_create": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_ulonglong, ctypes.POINTER(_VP)]),
    "asets_wsnet_destroy": (None, [_VP]),
    "asets_wsnet_get_params": (ctypes.c_int, [_VP, _VP]),
    "asets_wsnet_set_params": (ctypes.c_int, [_VP, _VP]),
    "asets_wsnet_predict": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_int, ctypes.c_int]
                            + [_VP] * 8),
    "asets_wsnet_gradients": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_int, ctypes.c_int]
                              + [_VP] * 9 + [ctypes.POINTER(ctypes.c_float)]),
    "asets_wsnet_train_step": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_int, ctypes.c_int]
                               + [_VP] * 8 + [ctypes.c_float, ctypes.POINTER(ctypes.c_float)]),
    "asets_binary_mf3d_noalloc": (ctypes.c_int, [_VP, _VP, _VP, _VP, ctypes.c_int, ctypes.c_int,
                                                 ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                                 ctypes.c_float, ctypes.c_float, _VP, _VP,
                                                 ctypes.POINTER(ctypes.c_int), _VP]),
}


def exported_symbols() -> list[str]:
    return list(_SIGS)


def lib() -> ctypes.CDLL:
    """Load libasetscuda.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} not found: build it with "
                               "`python -m asetsmatlabmaxflow_gb300.build` (needs nvcc)")
        l = ctypes.CDLL(str(LIB_PATH), mode=os.RTLD_GLOBAL | os.RTLD_NOW)
        for name, (res, args) in _SIGS.items():
            fn = getattr(l, name)
            fn.restype = res
            fn.argtypes = args
        _lib = l
    return _lib


def check(status: int) -> None:
    if status == ASETS_OK:
        return
    msg = lib().asets_last_error().decode(errors="replace")
    if status == ASETS_ERR_ALPHA:
        raise AlphaError(status, msg)
    raise AsetsError(status, msg or lib().asets_status_string(status).decode())


def _ptr(a) -> int | None:
    """Address of a numpy array, a torch tensor, or anything exposing
    __cuda_array_interface__ / an integer address."""
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    if hasattr(a, "__cuda_array_interface__"):
        return a.__cuda_array_interface__["data"][0]
    raise TypeError(f"cannot take the address of {type(a)}")


def _host_f32(a) -> np.ndarray | None:
    if a is None:
        return None
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32).ravel(order="F"))


class Context:
    def __init__(self, device: int = 0, handle: int | None = None):
        if handle is not None:
            self._h = handle
            self._own = False
        else:
            h = _VP()
            check(lib().asets_context_create(device, ctypes.byref(h)))
            self._h = h.value
            self._own = True

    @staticmethod
    def default() -> "Context":
        h = _VP()
        check(lib().asets_default_context(ctypes.byref(h)))
        return Context(handle=h.value)

    @property
    def handle(self) -> int:
        return self._h

    def set_stream(self, stream_ptr: int | None) -> None:
        check(lib().asets_context_set_stream(self._h, stream_ptr))

    def close(self) -> None:
        if self._own and self._h:
            lib().asets_context_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Solver:
    """A device-resident problem (asets_solver_*)."""

    def __init__(self, ctx: Context, model: str, dims: tuple[int, ...], nlab: int = 1):
        self.ctx = ctx
        self.model = model
        self.dim = len(dims)
        self.ny, self.nx = dims[0], dims[1]
        self.nz = dims[2] if self.dim == 3 else 1
        self.nlab = nlab if model != "binary" else 1
        h = _VP()
        check(lib().asets_solver_create(ctx.handle, MODELS[model], self.dim, self.ny, self.nx,
                                        self.nz, self.nlab, ctypes.byref(h)))
        self._h = h.value
        self._keep = []
        self.last_max_it = 0

    @property
    def n(self) -> int:
        return self.ny * self.nx * self.nz

    @property
    def u_labels(self) -> int:
        return {"binary": 1, "potts": self.nlab, "ishikawa": self.nlab - 1}[self.model]

    @property
    def pt_labels(self) -> int:
        return 1 if self.model == "binary" else self.nlab

    def set_inputs(self, Ct, alpha, Cs=None, where: int = HOST) -> None:
        if where == HOST:
            Ct, alpha, Cs = _host_f32(Ct), _host_f32(alpha), _host_f32(Cs)
            self._keep = [Ct, alpha, Cs]
        check(lib().asets_solver_set_inputs(self._h, where, _ptr(Cs), _ptr(Ct), _ptr(alpha)))

    def get_inputs(self, Cs=None, Ct=None, alpha=None, where: int = HOST):
        """(Cs, Ct, alpha) as set (restricted, on a coarse level); with
        where=DEVICE the caller provides the buffers."""
        if where == HOST:
            al = {"binary": 1, "potts": self.nlab, "ishikawa": self.nlab - 1}[self.model]
            Cs = np.empty(self.n, np.float32) if self.model == "binary" else None
            Ct = np.empty(self.n * (1 if self.model == "binary" else self.nlab), np.float32)
            alpha = np.empty(self.n * al, np.float32)
        check(lib().asets_solver_get_inputs(self._h, where, _ptr(Cs), _ptr(Ct), _ptr(alpha)))
        return Cs, Ct, alpha

    def set_initial(self, u0=None, ps0=None, pt0=None, where: int = HOST) -> None:
        if where == HOST:
            u0, ps0, pt0 = _host_f32(u0), _host_f32(ps0), _host_f32(pt0)
        check(lib().asets_solver_set_initial(self._h, where, _ptr(u0), _ptr(ps0), _ptr(pt0)))

    def run(self, max_it: int, err_bound: float, cc: float, steps: float, *, exact: bool = False,
            tile_config: int = 0, flags: int = 0, autotune: bool = False) -> int:
        flags |= (FLAG_EXACT if exact else 0) | (FLAG_AUTOTUNE if autotune else 0)
        opt = Options(flags=flags, tile_config=tile_config)
        it = ctypes.c_int(0)
        check(lib().asets_solver_run(self._h, ctypes.byref(opt), max_it, err_bound, cc, steps,
                                     ctypes.byref(it)))
        self.last_max_it = max_it
        return it.value

    def get_u(self, out=None, where: int = HOST) -> np.ndarray:
        if out is None:
            out = np.empty(self.n * self.u_labels, np.float32)
        check(lib().asets_solver_get_u(self._h, where, _ptr(out)))
        return out

    def get_cvg(self, n: int | None = None) -> np.ndarray:
        n = self.last_max_it if n is None else n
        out = np.empty(max(n, 0), np.float32)
        check(lib().asets_solver_get_cvg(self._h, HOST, _ptr(out) if n else None, n))
        return out

    def get_flows(self, ps=None, pt=None, where: int = HOST):
        """Final (ps, pt); with where=DEVICE, ps/pt are caller-provided device
        buffers (ps may be None)."""
        if where == HOST:
            ps = None if self.model == "ishikawa" else np.empty(self.n, np.float32)
            pt = np.empty(self.n * self.pt_labels, np.float32)
        check(lib().asets_solver_get_flows(self._h, where, _ptr(ps), _ptr(pt)))
        return ps, pt

    def run_multilevel(self, levels: int, max_it: int, err_bound: float, cc: float, steps: float,
                       *, exact: bool = False, tile_config: int = 0, flags: int = 0,
                       autotune: bool = False) -> int:
        flags |= (FLAG_EXACT if exact else 0) | (FLAG_AUTOTUNE if autotune else 0)
        opt = Options(flags=flags, tile_config=tile_config)
        it = ctypes.c_int(0)
        check(lib().asets_solver_run_multilevel(self._h, ctypes.byref(opt), levels, max_it,
                                                err_bound, cc, steps, ctypes.byref(it)))
        self.last_max_it = max_it
        return it.value

    def multilevel_prepare(self, levels: int) -> int:
        n = ctypes.c_int(0)
        check(lib().asets_solver_multilevel_prepare(self._h, levels, ctypes.byref(n)))
        return n.value

    def level(self, k: int) -> "Solver":
        """Level k of the multilevel chain (0 = self), a borrowed solver."""
        h = _VP()
        check(lib().asets_solver_level(self._h, k, ctypes.byref(h)))
        if k == 0:
            return self
        s = Solver.__new__(Solver)
        s.ctx, s.model, s.dim, s.nlab = self.ctx, self.model, self.dim, self.nlab
        ny, nx, nz = self.ny, self.nx, self.nz
        for _ in range(k):
            ny, nx = (ny + 1) // 2, (nx + 1) // 2
            nz = (nz + 1) // 2 if self.dim == 3 else 1
        s.ny, s.nx, s.nz = ny, nx, nz
        s._h, s._keep, s.last_max_it, s._borrowed = h.value, [], 0, True
        return s

    def multilevel_stats(self) -> tuple[list[int], list[float]]:
        it = (ctypes.c_int * 8)()
        ms = (ctypes.c_float * 8)()
        n = ctypes.c_int(0)
        check(lib().asets_solver_multilevel_stats(self._h, 8, ctypes.cast(it, _VP),
                                                  ctypes.cast(ms, _VP), ctypes.byref(n)))
        return list(it[:n.value]), list(ms[:n.value])

    @property
    def flow_labels(self) -> int:
        return {"binary": 1, "potts": self.nlab, "ishikawa": self.nlab - 1}[self.model]

    def set_initial_flows(self, bx=None, by=None, bz=None, where: int = HOST) -> None:
        if where == HOST:
            bx, by, bz = _host_f32(bx), _host_f32(by), _host_f32(bz)
        check(lib().asets_solver_set_initial_flows(self._h, where, _ptr(bx), _ptr(by), _ptr(bz)))

    def get_spatial_flows(self, bx=None, by=None, bz=None, where: int = HOST):
        """(bx, by, bz) after the last run, reference layout (bz None in 2D)."""
        if where == HOST:
            m = self.n * self.flow_labels
            bx, by = np.empty(m, np.float32), np.empty(m, np.float32)
            bz = np.empty(m, np.float32) if self.dim == 3 else None
        check(lib().asets_solver_get_spatial_flows(self._h, where, _ptr(bx), _ptr(by), _ptr(bz)))
        return bx, by, bz

    def last_run_stats(self) -> tuple[float, int]:
        ms = ctypes.c_float(0)
        n = ctypes.c_int(0)
        check(lib().asets_solver_last_run_stats(self._h, ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    def close(self) -> None:
        if self._h and not getattr(self, "_borrowed", False):
            lib().asets_solver_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many solvers run together (asets_batch_*): binary and labelled models,
    2D and 3D, each converging on its own."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        h = _VP()
        check(lib().asets_batch_create(ctx.handle, ctypes.byref(h)))
        self._h = h.value
        self.members: list[Solver] = []

    def add(self, s: Solver) -> None:
        check(lib().asets_batch_add(self._h, s._h))
        self.members.append(s)

    def run(self, max_it: int, err_bound: float, cc: float, steps: float, *, exact: bool = False,
            autotune: bool = False, tile_config: int = 0) -> list[int]:
        flags = (FLAG_EXACT if exact else 0) | (FLAG_AUTOTUNE if autotune else 0)
        opt = Options(flags=flags, tile_config=tile_config)
        its = (ctypes.c_int * max(len(self.members), 1))()
        check(lib().asets_batch_run(self._h, ctypes.byref(opt), max_it, err_bound, cc, steps,
                                    ctypes.addressof(its)))
        for s in self.members:
            s.last_max_it = max_it
        return list(its[:len(self.members)])

    def run_multilevel(self, levels: int, max_it: int, err_bound: float, cc: float, steps: float,
                       *, exact: bool = False, autotune: bool = False) -> list[int]:
        """Coarse-to-fine solve of every member (asets_batch_run_multilevel);
        full-resolution itNum per member, per-level ones in each member's
        multilevel_stats()."""
        opt = Options(flags=(FLAG_EXACT if exact else 0) | (FLAG_AUTOTUNE if autotune else 0),
                      tile_config=0)
        its = (ctypes.c_int * max(len(self.members), 1))()
        check(lib().asets_batch_run_multilevel(self._h, ctypes.byref(opt), levels, max_it,
                                               err_bound, cc, steps, ctypes.addressof(its)))
        for s in self.members:
            s.last_max_it = max_it
        return list(its[:len(self.members)])

    def last_run_stats(self) -> dict:
        ms = ctypes.c_float(0)
        n = ctypes.c_int(0)
        iters = ctypes.c_int(0)
        tc = (ctypes.c_int * 2)()
        check(lib().asets_batch_last_run_stats(self._h, ctypes.byref(ms), ctypes.byref(n),
                                               ctypes.byref(iters), ctypes.addressof(tc)))
        return {"ms": ms.value, "launches": n.value, "iterations": iters.value,
                "tile_config_2d": tc[0], "tile_config_3d": tc[1]}

    def close(self) -> None:
        if self._h:
            lib().asets_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class WarmStartNet:
    """The learned warm start (asets_wsnet_*): a 4-layer 3x3x3 convolutional
    net, (Ct_1..L, alpha) -> (u_1..L, ps, pt_1..L, bx, by, bz), on the tensor
    cores.
    Array arguments are device pointers / CUDA tensors in Matlab layout
    (label slowest)."""

    def __init__(self, ctx: Context, nlab: int = 6, seed: int = 0):
        self.ctx = ctx
        self.nlab = nlab
        h = _VP()
        check(lib().asets_wsnet_create(ctx.handle, nlab, seed, ctypes.byref(h)))
        self._h = h.value

    @staticmethod
    def num_params() -> int:
        return lib().asets_wsnet_num_params()

    def get_params(self) -> np.ndarray:
        out = np.empty(self.num_params(), np.float32)
        check(lib().asets_wsnet_get_params(self._h, out.ctypes.data))
        return out

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.num_params()
        check(lib().asets_wsnet_set_params(self._h, p.ctypes.data))

    def predict(self, dims, ct, alpha, u0, ps0, pt0, bx0=None, by0=None, bz0=None) -> None:
        ny, nx, nz = dims
        check(lib().asets_wsnet_predict(self._h, ny, nx, nz, _ptr(ct), _ptr(alpha), _ptr(u0),
                                        _ptr(ps0), _ptr(pt0), _ptr(bx0), _ptr(by0), _ptr(bz0)))

    def gradients(self, dims, ct, alpha, u, ps, pt, bx, by, bz):
        ny, nx, nz = dims
        g = np.empty(self.num_params(), np.float32)
        loss = ctypes.c_float(0)
        check(lib().asets_wsnet_gradients(self._h, ny, nx, nz, _ptr(ct), _ptr(alpha), _ptr(u),
                                          _ptr(ps), _ptr(pt), _ptr(bx), _ptr(by), _ptr(bz),
                                          g.ctypes.data, ctypes.byref(loss)))
        return loss.value, g

    def train_step(self, dims, ct, alpha, u, ps, pt, bx, by, bz, lr: float) -> float:
        ny, nx, nz = dims
        loss = ctypes.c_float(0)
        check(lib().asets_wsnet_train_step(self._h, ny, nx, nz, _ptr(ct), _ptr(alpha), _ptr(u),
                                           _ptr(ps), _ptr(pt), _ptr(bx), _ptr(by), _ptr(bz), lr,
                                           ctypes.byref(loss)))
        return loss.value

    def close(self) -> None:
        if self._h:
            lib().asets_wsnet_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
