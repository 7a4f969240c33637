"""Odd-shape solves run by test_gpu_bounds.py in a child process against the
bounds-check build of libasetscuda (ASETS_LIB_DIR=.../lib_check): every
kernel variant of every model on shapes that are odd, below one tile or a
single row, EXACT results bit-identical to the oracle, no access flagged.
Not collected by pytest (no test_ prefix)."""
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent.parent))

from oracle import oracle as O  # noqa: E402


def _rand(model, dims, L, seed):
    from scipy.ndimage import gaussian_filter

    g = np.random.default_rng(seed)
    sm = lambda shp: np.asfortranarray(gaussian_filter(g.random(shp), 1.0).astype(np.float32))  # noqa: E731
    if model == "binary":
        return dict(Cs=sm(dims), Ct=sm(dims), alpha=(0.1 + 0.6 * g.random(dims)).astype(np.float32))
    la = L if model == "potts" else L - 1
    return dict(Ct=sm(dims + (L,)), alpha=(0.1 + 0.4 * g.random(dims + (la,))).astype(np.float32))


CASES = [
    ("binary", (33, 41, 29), 1, 5, 4), ("binary", (5, 7, 3), 1, 5, 4), ("binary", (1, 9, 8), 1, 5, 4),
    ("binary", (121, 13, 6), 1, 5, 4), ("binary", (301, 170), 1, 9, 8), ("binary", (1, 9), 1, 9, 8),
    ("binary", (450, 5), 1, 9, 8), ("potts", (48, 40, 20), 4, 6, 6), ("potts", (130, 97), 5, 9, 9),
    ("potts", (7, 33), 2, 9, 9), ("ishikawa", (40, 33, 17), 4, 6, 6),
    ("ishikawa", (160, 120), 8, 9, 9), ("ishikawa", (61, 9), 3, 9, 9),
]
# (model, shape, labels, fast variants, EXACT variants): the variant counts of
# the tables in csrc/{binary,flow}{2d,3d}_{fast,exact}.cu, plus the one-pass
# kernel (csrc/{potts,ishikawa}2d_fused_*.cu) ahead of the 2D multi-label tables


def main() -> int:
    from asetsmatlabmaxflow_gb300 import native as N

    assert "lib_check" in str(N.LIB_PATH), N.LIB_PATH
    ctx = N.Context.default()
    for model, dims, L, n_fast, n_exact in CASES:
        inp = _rand(model, dims, L, 3)
        cc, steps = 0.3, (0.16 if len(dims) == 2 else 0.11)
        ref = O.solve(model, dims, inp["Ct"], inp["alpha"], cs=inp.get("Cs"), nlab=L, max_it=12,
                      err_bound=0.0, cc=cc, steps=steps)
        s = N.Solver(ctx, model, dims, L)
        s.set_inputs(inp["Ct"], inp["alpha"], inp.get("Cs"))
        for tc in range(1, n_exact + 1):
            s.run(12, 0.0, cc, steps, exact=True, tile_config=tc)  # raises on a flagged access
            u = s.get_u()
            if not np.array_equal(u.view(np.uint32), ref["u"].view(np.uint32)):
                print(f"EXACT mismatch: {model} {dims} variant {tc}")
                return 1
        for tc in range(1, n_fast + 1):
            s.run(12, 0.0, cc, steps, tile_config=tc)
            if float(np.max(np.abs(s.get_u() - ref["u"]))) > 1e-3:
                print(f"fast mismatch: {model} {dims} variant {tc}")
                return 1
        s.run(40, 1e-4, cc, steps)  # a stopping run (two-iteration passes roll back)
        s.close()
        print("ok", model, dims)
    return 0


if __name__ == "__main__":
    sys.exit(main())
