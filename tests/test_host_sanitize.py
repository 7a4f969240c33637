"""The host-side boundary code -- the six mex drop-ins, the MEX host
emulation (mexshim.c) and the C oracle -- built with AddressSanitizer and
UndefinedBehaviorSanitizer and driven by tests/c/sanitize_driver.c, with the
GPU library replaced by a fake that answers from the oracle: regular solves
on odd and degenerate shapes, maxIt 0, alpha <= 0, wrong input class,
missing inputs, arrays of every class.  No GPU needed."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
MEX = ROOT / "asetsmatlabmaxflow_gb300" / "mex"


def _sanitizer_works(tmp: Path) -> bool:
    src = tmp / "probe.c"
    src.write_text("int main(void) { return 0; }\n")
    r = subprocess.run(["gcc", "-fsanitize=address,undefined", "-o", str(tmp / "probe"), str(src)],
                       capture_output=True)
    return r.returncode == 0


def test_boundary_code_is_clean_under_asan_and_ubsan(tmp_path):
    if shutil.which("gcc") is None or not _sanitizer_works(tmp_path):
        pytest.skip("gcc with AddressSanitizer/UBSan is not available on this machine")
    flags = ["-std=gnu11", "-g", "-O1", "-fno-omit-frame-pointer", "-fsanitize=address,undefined",
             "-fno-sanitize-recover=all", "-ffp-contract=off", f"-I{ROOT / 'include'}", f"-I{MEX}",
             f"-I{ROOT / 'oracle'}"]
    objs = []
    for name, sym in [("asetsBinaryMF2D_mex", "b2"), ("asetsBinaryMF3D_mex", "b3"),
                      ("asetsPotts2D_mex", "p2"), ("asetsPotts3D_mex", "p3"),
                      ("asetsIshikawa2D_mex", "i2"), ("asetsIshikawa3D_mex", "i3")]:
        obj = tmp_path / f"{name}.o"
        subprocess.run(["gcc", *flags, f"-DmexFunction=mexFunction_{sym}", "-c", "-o", str(obj),
                        str(MEX / f"{name}.c")], check=True)
        objs.append(str(obj))
    exe = tmp_path / "sanitize_driver"
    subprocess.run(["gcc", *flags, "-o", str(exe), str(ROOT / "tests" / "c" / "sanitize_driver.c"),
                    str(MEX / "mexshim.c"), str(ROOT / "oracle" / "asets_oracle.c"), *objs, "-lm"],
                   check=True)
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0",
               UBSAN_OPTIONS="print_stacktrace=1:halt_on_error=1")
    r = subprocess.run([str(exe)], capture_output=True, text=True, env=env, timeout=300)
    if r.returncode != 0 and "LeakSanitizer has encountered a fatal error" in r.stderr:
        env["ASAN_OPTIONS"] = "detect_leaks=0"  # LSan needs ptrace, which some sandboxes deny
        r = subprocess.run([str(exe)], capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "runtime error" not in r.stderr and "AddressSanitizer" not in r.stderr
    assert "all cases ok" in r.stdout
