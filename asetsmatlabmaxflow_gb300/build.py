"""In-tree build of the native libraries.

  lib/libasetscuda.so   CUDA solvers + C ABI (include/asets.h), sm_103a only
  lib/libmexshim.so     host emulation of the MEX API (mex/mex.h)
  lib/<solver>.so       the six drop-in mex entry points, linked to both

Compiled with nvcc/gcc directly (no cmake); translation units are built in
parallel so a clean build takes about a minute.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
MEX_DIR = PKG / "mex"
INCLUDE = REPO / "include"
# ASETS_BOUNDS_CHECK=1 builds the debug flavour (-DASETS_BOUNDS_CHECK: the
# iteration kernels check every store and shared-memory index and report a
# violation as an error instead of making the access) into lib_check/;
# native.py loads it when ASETS_LIB_DIR points there.
BOUNDS_CHECK = os.environ.get("ASETS_BOUNDS_CHECK", "0") not in ("", "0")
LIB = PKG / ("lib_check" if BOUNDS_CHECK else "lib")
OBJ = PKG / ("_build_check" if BOUNDS_CHECK else "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
    # IEEE division and square root, no FMA contraction unless written
    # explicitly: the kernels reproduce the reference's float arithmetic.
    "-prec-div=true", "-prec-sqrt=true", "-ftz=false", "--fmad=false",
]

# The fast kernel variants are held to the parity tolerance, not to
# bit-exactness: they may contract a*b+c into FMA and flush denormals.
FAST_FLAGS = [f for f in NVCC_FLAGS if f not in ("-ftz=false", "--fmad=false")] + [
    "-ftz=true", "--fmad=true"]
if BOUNDS_CHECK:
    NVCC_FLAGS = NVCC_FLAGS + ["-DASETS_BOUNDS_CHECK"]
    FAST_FLAGS = FAST_FLAGS + ["-DASETS_BOUNDS_CHECK"]

CU_SOURCES = (
    "runtime.cu",
    "stencil_setup.cu",
    "init_kernels.cu",
    "binary3d_fast.cu",
    "binary3d_exact.cu",
    "binary2d_fast.cu",
    "binary2d_exact.cu",
    "flow3d_fast.cu",
    "flow3d_exact.cu",
    "flow2d_fast.cu",
    "flow2d_exact.cu",
    "potts2d_fused_fast.cu",
    "potts2d_fused_exact.cu",
    "ishikawa2d_fused_fast.cu",
    "ishikawa2d_fused_exact.cu",
    "label_kernels.cu",
    "noalloc.cu",
    "conv_tc.cu",
    "warmstart.cu",
    "multilevel.cu",
    "costs.cu",
    "starshape.cu",
    "hmf.cu",
    "mtwin.cu",
)

MEX_SOLVERS = (
    "asetsBinaryMF2D_mex",
    "asetsBinaryMF3D_mex",
    "asetsPotts2D_mex",
    "asetsPotts3D_mex",
    "asetsIshikawa2D_mex",
    "asetsIshikawa3D_mex",
)


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libasetscuda")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.exists() and d.stat().st_mtime > t for d in deps)


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(INCLUDE.glob("*.h"))


def build_mexshim() -> Path:
    LIB.mkdir(exist_ok=True)
    out = LIB / "libmexshim.so"
    src = MEX_DIR / "mexshim.c"
    if _stale(out, [src, MEX_DIR / "mex.h"]):
        _run(["gcc", "-std=gnu11", "-O2", "-fPIC", "-shared", f"-I{MEX_DIR}",
              "-o", str(out), str(src)])
    return out


def build_cuda(jobs: int | None = None) -> Path:
    LIB.mkdir(exist_ok=True)
    OBJ.mkdir(exist_ok=True)
    out = LIB / "libasetscuda.so"
    hdrs = _headers()
    nv = nvcc()

    def compile_one(name: str) -> Path:
        src = CSRC / name
        obj = OBJ / (Path(name).stem + ".o")
        if _stale(obj, [src, *hdrs, Path(__file__)]):
            flags = FAST_FLAGS if name.endswith("_fast.cu") else NVCC_FLAGS
            _run([nv, *ARCH, *flags, f"-I{INCLUDE}", f"-I{CSRC}", "-c",
                  "-o", str(obj), str(src)])
        return obj

    jobs = jobs or min(len(CU_SOURCES), os.cpu_count() or 4)
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(compile_one, CU_SOURCES))
    if _stale(out, objs):
        _run([nv, *ARCH, "-shared", "-o", str(out), *map(str, objs), "-lcudart_static",
              "-Xcompiler", "-fvisibility=hidden", "-lpthread", "-ldl", "-lrt"])
    return out


def build_mex_dropins(cuda_lib: Path, shim: Path) -> list[Path]:
    outs = []

    def one(name: str) -> Path:
        src = MEX_DIR / f"{name}.c"
        out = LIB / f"{name}.so"
        deps = [src, MEX_DIR / "mex.h", MEX_DIR / "asets_mex_common.h", INCLUDE / "asets.h",
                cuda_lib, shim]
        if _stale(out, deps):
            _run(["gcc", "-std=gnu11", "-O2", "-fPIC", "-shared", f"-I{MEX_DIR}",
                  f"-I{INCLUDE}", "-o", str(out), str(src),
                  f"-L{LIB}", "-lasetscuda", "-lmexshim", "-Wl,-rpath,$ORIGIN"])
        return out

    with ThreadPoolExecutor(max_workers=len(MEX_SOLVERS)) as ex:
        outs = list(ex.map(one, MEX_SOLVERS))
    return outs


def build_all() -> dict[str, Path]:
    shim = build_mexshim()
    cuda_lib = build_cuda()
    mex = build_mex_dropins(cuda_lib, shim)
    return {"libasetscuda": cuda_lib, "libmexshim": shim, **{p.stem: p for p in mex}}


if __name__ == "__main__":
    for k, v in build_all().items():
        print(k, v)
