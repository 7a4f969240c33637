"""The C ABI library and the drop-in mex files load and export what
include/asets.h declares; without a GPU every entry point fails cleanly."""
import ctypes
import os
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _declared():
    text = (ROOT / "include" / "asets.h").read_text()
    return sorted(set(re.findall(r"ASETS_API\s+[\w\s\*]+?\b(asets_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from asetsmatlabmaxflow_gb300 import build, native

    build.build_all()
    return native.lib()


def test_every_declared_symbol_is_exported(lib):
    from asetsmatlabmaxflow_gb300 import native

    names = _declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    # the Python binding covers the whole header
    assert set(names) == set(native.exported_symbols())


def test_status_strings_and_version(lib):
    assert lib.asets_abi_version() == 1
    assert b"alpha(x) must be positive" in lib.asets_status_string(2)
    assert lib.asets_status_string(99) == b"unknown status"


def test_no_gpu_or_bad_args_fail_cleanly(lib):
    from asetsmatlabmaxflow_gb300 import native as N

    h = ctypes.c_void_p()
    st = lib.asets_context_create(0, ctypes.byref(h))
    if st == N.ASETS_OK:
        lib.asets_context_destroy(h)
        pytest.skip("a GPU is present")
    assert st == N.ASETS_ERR_NO_DEVICE and not h.value
    assert lib.asets_last_error()
    assert lib.asets_context_create(0, None) == N.ASETS_ERR_INVALID_ARG
    assert lib.asets_solver_create(None, 0, 3, 4, 4, 4, 1, None) == N.ASETS_ERR_INVALID_ARG


def test_dropin_mex_files_export_mexFunction(lib):
    from asetsmatlabmaxflow_gb300 import build

    for name in build.MEX_SOLVERS:
        so = ctypes.CDLL(str(build.LIB / f"{name}.so"), mode=os.RTLD_LOCAL)
        assert hasattr(so, "mexFunction")


def test_dropin_mex_reports_missing_device_as_mex_error(lib):
    from asetsmatlabmaxflow_gb300 import native as N
    from asetsmatlabmaxflow_gb300.mexhost import MexError
    from asetsmatlabmaxflow_gb300.solvers import mex_dropin
    import numpy as np

    h = ctypes.c_void_p()
    if lib.asets_context_create(0, ctypes.byref(h)) == N.ASETS_OK:
        lib.asets_context_destroy(h)
        pytest.skip("a GPU is present")
    a = np.ones((4, 3), np.float32)
    pars = np.array([4, 3, 5, 0.0, 0.3, 0.16], np.float32)
    with pytest.raises(MexError, match="libasetscuda"):
        mex_dropin("asetsBinaryMF2D_mex")(a, a, a, pars)
    with pytest.raises(MexError, match="single"):
        mex_dropin("asetsBinaryMF2D_mex")(a.astype(np.float64), a, a, pars)
