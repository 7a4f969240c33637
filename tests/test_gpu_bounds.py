"""The bounds-check build of libasetscuda (-DASETS_BOUNDS_CHECK: the
iteration kernels check every global store against its array and every
shared-memory index against its box, and report a violation as an error
instead of making the access), built in-tree into lib_check/ and run in a
child process on the odd shapes of tests/bounds_cases.py: no access flagged,
EXACT results bit-identical to the oracle."""
import os
import subprocess
import sys
from pathlib import Path

import pytest

from tests.gpu_helpers import require_gpu

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


def test_bounds_checked_kernels_run_odd_shapes_clean():
    require_gpu()
    env = dict(os.environ, ASETS_BOUNDS_CHECK="1")
    subprocess.run([sys.executable, "-c",
                    "from asetsmatlabmaxflow_gb300 import build; print(build.build_cuda())"],
                   env=env, cwd=ROOT, check=True, capture_output=True, timeout=900)
    env = dict(os.environ, ASETS_LIB_DIR=str(ROOT / "asetsmatlabmaxflow_gb300" / "lib_check"))
    env.pop("ASETS_BOUNDS_CHECK", None)
    r = subprocess.run([sys.executable, str(ROOT / "tests" / "bounds_cases.py")], env=env, cwd=ROOT,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
