"""Device arithmetic building blocks checked on the GPU."""
import ctypes
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def div_lib(tmp_path_factory):
    from asetsmatlabmaxflow_gb300 import build

    out = tmp_path_factory.mktemp("divcheck") / "libdivcheck.so"
    subprocess.run([build.nvcc(), *build.ARCH, *build.NVCC_FLAGS, f"-I{build.CSRC}",
                    f"-I{build.INCLUDE}", "-shared", "-o", str(out),
                    str(ROOT / "tests" / "cuda" / "div_check.cu")], check=True)
    lib = ctypes.CDLL(str(out))
    lib.div_check.argtypes = [ctypes.c_float, ctypes.POINTER(ctypes.c_ulonglong),
                              ctypes.POINTER(ctypes.c_uint)]
    lib.div_check.restype = ctypes.c_int
    return lib


@pytest.mark.parametrize("d", [0.35, 0.3, 0.25, 0.2, 0.75, 0.1, 1.0 / 3.0, 0.123456, 3.0, 0.9999999])
def test_reciprocal_division_is_correctly_rounded_for_all_dividends(div_lib, d):
    m = ctypes.c_ulonglong(0)
    f = ctypes.c_uint(0)
    assert div_lib.div_check(d, ctypes.byref(m), ctypes.byref(f)) == 0
    assert m.value == 0, f"{m.value} mismatches, first dividend bits {f.value:#010x}"
