"""GB300-native continuous max-flow / min-cut solvers (ASETS).

Entry points
  solvers   -- asetsBinaryMF2D_mex(...) & co.: the reference mex interface
  native    -- ctypes binding of the C ABI (Context, Solver)
  synth     -- seeded synthetic problems
  build     -- in-tree build of libasetscuda.so, libmexshim.so and the mex files
"""
from . import build  # noqa: F401

__all__ = ["build", "native", "solvers", "synth", "mexhost"]


def __getattr__(name):
    import importlib

    if name in ("native", "solvers", "synth", "mexhost"):
        return importlib.import_module(f".{name}", __name__)
    if name in ("asetsBinaryMF2D_mex", "asetsBinaryMF3D_mex", "asetsPotts2D_mex",
                "asetsPotts3D_mex", "asetsIshikawa2D_mex", "asetsIshikawa3D_mex"):
        from . import solvers
        return getattr(solvers, name)
    raise AttributeError(name)
