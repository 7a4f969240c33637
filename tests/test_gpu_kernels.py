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


@pytest.fixture(scope="module")
def norm_lib(tmp_path_factory):
    from asetsmatlabmaxflow_gb300 import build

    out = tmp_path_factory.mktemp("normcheck") / "libnormcheck.so"
    subprocess.run([build.nvcc(), *build.ARCH, *build.NVCC_FLAGS, f"-I{build.CSRC}",
                    f"-I{build.INCLUDE}", "-shared", "-o", str(out),
                    str(ROOT / "tests" / "cuda" / "norm_check.cu")], check=True)
    lib = ctypes.CDLL(str(out))
    lib.norm_check.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_ulonglong,
                               ctypes.POINTER(ctypes.c_ulonglong)]
    lib.norm_check.restype = ctypes.c_int
    return lib


@pytest.mark.parametrize("mode", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("nfaces", [4, 6])
def test_exact_projection_factor_equals_the_double_computation(norm_lib, nfaces, mode):
    """The EXACT kernels' projection factor (float pre-check, the double norm
    reproduced in float, double only where float cannot decide) is bit for
    bit the reference's double computation, on 2^25 seeded cases per mode:
    unit-range flows, a wide exponent range, one dominant face, few-bit
    values (half of these with the capacity within a few ulps of the norm),
    and norms within a few ulps of a capacity of exactly 1 or 0.5."""
    m = ctypes.c_ulonglong(0)
    assert norm_lib.norm_check(nfaces, mode, 1 << 25, ctypes.byref(m)) == 0
    assert m.value == 0, f"{m.value} mismatches"


def test_bounded_wait_times_out_and_context_survives():
    """A device-side wait on a barrier that nothing completes gives up after
    its budget, the host gets ASETS_ERR_TIMEOUT, and the next solve on the
    same context runs normally."""
    import time

    import numpy as np

    from asetsmatlabmaxflow_gb300 import native as N

    ctx = N.Context.default()
    t0 = time.perf_counter()
    st = N.lib().asets_selftest_wait_timeout(ctx.handle)
    dt = time.perf_counter() - t0
    assert st == N.ASETS_ERR_TIMEOUT, N.lib().asets_last_error()
    assert 0.9 < dt < 10.0
    g = np.random.default_rng(0)
    n = 24 * 20 * 8
    img = g.random(n).astype(np.float32)
    s = N.Solver(ctx, "binary", (24, 20, 8))
    s.set_inputs(np.abs(img - 0.8).astype(np.float32), np.full(n, 0.3, np.float32),
                 np.abs(img - 0.2).astype(np.float32))
    it = s.run(50, 1e-4, 0.35, 0.11)
    assert 0 < it <= 50 and np.all(np.isfinite(s.get_u()))
    s.close()
