"""Build recipe for the oracle (test infrastructure only).

Produces
  oracle/_build/liboracle.so  -- the C restatement in asets_oracle.c
  oracle/_ref/<solver>.so      -- the unmodified reference mex sources
                                  (maxflow/asets*_mex.c), compiled from where
                                  they lie, against the package's mex host
                                  emulation (mex.h + libmexshim.so); only when
                                  the reference tree is present
                                  ($ASETS_REFERENCE_DIR, or ../reference
                                  beside the repository).

Both are compiled with -ffp-contract=off: on x86-64 this is what gcc does
anyway (no FMA without -mfma), and on aarch64 it stops gcc from fusing a*b+c,
so the restatement, the reference and the GPU kernels all evaluate the same
IEEE float expressions on either host.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
# The reference tree: $ASETS_REFERENCE_DIR, else a checkout named `reference`
# beside this repository.
REF_SRC = Path(os.environ.get("ASETS_REFERENCE_DIR", REPO.parent / "reference")) / "maxflow"

REF_SOLVERS = (
    "asetsBinaryMF2D_mex",
    "asetsBinaryMF3D_mex",
    "asetsPotts2D_mex",
    "asetsPotts3D_mex",
    "asetsIshikawa2D_mex",
    "asetsIshikawa3D_mex",
)

CFLAGS = ["-std=gnu99", "-O2", "-ffp-contract=off", "-fPIC", "-shared"]


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_port() -> Path:
    """Compile the restatement into oracle/_build/liboracle.so."""
    BUILD.mkdir(exist_ok=True)
    out = BUILD / "liboracle.so"
    src = HERE / "asets_oracle.c"
    if _stale(out, [src, HERE / "asets_oracle.h"]):
        _run(["gcc", *CFLAGS, "-o", str(out), str(src), "-lm"])
    return out


def build_reference() -> list[Path]:
    """Compile the six reference mex solvers into oracle/_ref/ (if present)."""
    if not REF_SRC.is_dir():
        return []
    sys.path.insert(0, str(REPO))
    from asetsmatlabmaxflow_gb300 import build as pkg_build

    shim = pkg_build.build_mexshim()
    REF_OUT.mkdir(exist_ok=True)
    mex_inc = pkg_build.MEX_DIR

    def one(name: str) -> Path:
        src = REF_SRC / f"{name}.c"
        out = REF_OUT / f"{name}.so"
        if _stale(out, [src, mex_inc / "mex.h", shim]):
            _run(["gcc", *CFLAGS, "-w", f"-I{mex_inc}", "-o", str(out), str(src),
                  f"-L{shim.parent}", "-lmexshim", f"-Wl,-rpath,{shim.parent}", "-lm"])
        return out

    with ThreadPoolExecutor(max_workers=6) as ex:
        return list(ex.map(one, REF_SOLVERS))


def build() -> None:
    build_port()
    build_reference()


if __name__ == "__main__":
    build()
    print("oracle built:", BUILD / "liboracle.so")
    if REF_OUT.is_dir():
        print("reference built:", sorted(p.name for p in REF_OUT.glob("*.so")))
