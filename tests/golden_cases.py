"""Loader for the golden vectors in tests/golden/*.npz (made by
tests/golden/make_golden.py from the compiled reference mex solvers)."""
from __future__ import annotations

from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"


def names() -> list[str]:
    return sorted(p.stem for p in GOLDEN.glob("*.npz"))


def load(name: str) -> dict:
    z = np.load(GOLDEN / f"{name}.npz")
    d = {k: z[k] for k in z.files}
    for k in ("name", "model", "solver"):
        d[k] = str(d[k])
    d["dims"] = tuple(int(v) for v in d["dims"])
    d["nlab"] = int(d["nlab"])
    d["it"] = int(d["it"])
    p = d["pars"]
    off = len(d["dims"]) + (0 if d["model"] == "binary" else 1)
    d["max_it"] = int(p[off])
    d["err_bound"] = float(p[off + 1])
    d["cc"] = float(p[off + 2])
    d["steps"] = float(p[off + 3])
    return d
