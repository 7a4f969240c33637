"""Generate the golden vectors in tests/golden/*.npz from the reference.

Each case draws seeded inputs (random costs smoothed with a Gaussian, as the
reference's own tests do with rand + imfilter, tests/runTestBinaryMF.m:35-41)
and runs the UNMODIFIED reference mex solver, compiled from
maxflow/asets*_mex.c by oracle/build.py, through the mex host emulation.
The .npz stores the inputs, the pars vector and the reference outputs
(u, erriter, i).  The reference tree is only needed to regenerate them:

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
from scipy.ndimage import gaussian_filter

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from oracle import oracle as O  # noqa: E402

SOLVER = {
    ("binary", 2): "asetsBinaryMF2D_mex", ("binary", 3): "asetsBinaryMF3D_mex",
    ("potts", 2): "asetsPotts2D_mex", ("potts", 3): "asetsPotts3D_mex",
    ("ishikawa", 2): "asetsIshikawa2D_mex", ("ishikawa", 3): "asetsIshikawa3D_mex",
}

# name, model, dims, labels, maxIt, errBound, cc, steps, alpha kind, seed
CASES = [
    # reference test parameters (tests/runTestBinaryMF.m:20-26, :44-48, :100-105)
    ("binary2d_reftest", "binary", (64, 64), 1, 300, 1e-5, 0.2, 0.16, 0.25, 1),
    ("binary3d_reftest", "binary", (48, 40, 16), 1, 60, 1e-5, 0.25, 0.11, 0.1, 2),
    # odd sizes that cross tile borders with partial tiles
    ("binary2d_odd", "binary", (301, 37), 1, 50, 0.0, 0.3, 0.16, "rand", 3),
    ("binary3d_odd", "binary", (70, 35, 13), 1, 30, 0.0, 0.35, 0.11, "rand", 4),
    ("binary3d_conv", "binary", (40, 36, 20), 1, 400, 2e-3, 0.35, 0.11, "rand", 5),
    # degenerate shapes
    ("binary2d_1x1", "binary", (1, 1), 1, 10, 0.0, 0.3, 0.16, "rand", 6),
    ("binary2d_1xN", "binary", (1, 29), 1, 20, 0.0, 0.3, 0.16, "rand", 7),
    ("binary2d_Nx1", "binary", (33, 1), 1, 20, 0.0, 0.3, 0.16, "rand", 8),
    ("binary3d_357", "binary", (3, 5, 7), 1, 25, 0.0, 0.3, 0.11, "rand", 9),
    ("binary3d_1x1x1", "binary", (1, 1, 1), 1, 5, 0.0, 0.3, 0.11, "rand", 10),
    ("binary3d_maxit0", "binary", (8, 6, 4), 1, 0, 0.0, 0.3, 0.11, "rand", 11),
    # Potts (tests/runTestPotts.m:242-249: L=10, alpha 0.05*i per label)
    ("potts2d_reftest", "potts", (48, 40), 10, 80, 1e-5, 0.2, 0.16, "label", 12),
    ("potts2d_odd", "potts", (133, 21), 4, 40, 0.0, 0.3, 0.16, "rand", 13),
    ("potts3d_small", "potts", (37, 19, 9), 3, 30, 0.0, 0.3, 0.11, "rand", 14),
    ("potts3d_conv", "potts", (24, 20, 12), 4, 300, 2e-3, 0.3, 0.11, 0.3, 15),
    ("potts2d_ties", "potts", (17, 13), 3, 20, 0.0, 0.3, 0.16, "rand", 16),
    # Ishikawa (tests/runTestIshikawa.m:19-26: L=6, cc .75, alpha 0.8/i, 0.3/i)
    ("ishikawa2d_reftest", "ishikawa", (64, 64), 6, 120, 1e-11, 0.75, 0.16, "label", 17),
    ("ishikawa2d_conv", "ishikawa", (50, 30), 5, 400, 1e-4, 0.3, 0.16, 0.2, 18),
    ("ishikawa2d_L2", "ishikawa", (29, 23), 2, 30, 0.0, 0.3, 0.16, "rand", 19),
    ("ishikawa3d_reftest", "ishikawa", (40, 36, 10), 6, 40, 1e-11, 0.75, 0.1, "label", 20),
    ("ishikawa3d_odd", "ishikawa", (45, 17, 6), 3, 30, 0.0, 0.3, 0.11, "rand", 21),
]


def make_inputs(model, dims, L, alpha_kind, seed):
    g = np.random.Generator(np.random.PCG64(seed))

    def smooth(shape):
        a = g.random(shape)
        sig = [1.0] * len(dims) + [0.0] * (len(shape) - len(dims))
        return np.asfortranarray(gaussian_filter(a, sigma=sig, mode="nearest").astype(np.float32))

    nal = 1 if model == "binary" else (L if model == "potts" else L - 1)
    ashape = dims if model == "binary" else dims + (nal,)
    if alpha_kind == "rand":
        alpha = (0.1 + 0.6 * g.random(ashape)).astype(np.float32)
    elif alpha_kind == "label":
        base = 0.05 if model == "potts" else (0.8 if len(dims) == 2 else 0.3)
        alpha = np.empty(ashape, np.float32)
        for i in range(nal):
            alpha[..., i] = base * (i + 1) if model == "potts" else base / (i + 1)
    else:
        alpha = np.full(ashape, alpha_kind, np.float32)
    alpha = np.asfortranarray(alpha)
    if model == "binary":
        return {"Cs": smooth(dims), "Ct": smooth(dims), "alpha": alpha}
    ct = smooth(dims + (L,))
    return {"Ct": ct, "alpha": alpha}


def run_case(case):
    name, model, dims, L, maxit, errb, cc, steps, akind, seed = case
    inp = make_inputs(model, dims, L, akind, seed)
    if name == "potts2d_ties":
        # equal costs on several labels: init must pick the FIRST argmin
        ct = inp["Ct"]
        ct[..., 2] = ct[..., 0]
        ct[::2, :, 1] = ct[::2, :, 0]
    solver = SOLVER[(model, len(dims))]
    if model == "binary":
        pars = np.array(list(dims) + [maxit, errb, cc, steps], np.float32)
        out = O.reference(solver)(inp["Cs"], inp["Ct"], inp["alpha"], pars)
    else:
        pars = np.array(list(dims) + [L, maxit, errb, cc, steps], np.float32)
        out = O.reference(solver)(inp["Ct"], inp["alpha"], pars)
    u, cvg, it = out[0], out[1], out[2]
    rec = dict(inp)
    rec.update(
        name=np.array(name), model=np.array(model), solver=np.array(solver),
        dims=np.array(dims, np.int32), nlab=np.array(L, np.int32), pars=pars,
        u=u, cvg=cvg.ravel(), it=np.array(int(it.ravel()[0]), np.int32),
    )
    return rec


def main():
    if not O.reference_available():
        from oracle import build as ob
        ob.build_reference()
    total = 0
    for case in CASES:
        rec = run_case(case)
        path = HERE / f"{case[0]}.npz"
        np.savez_compressed(path, **rec)
        total += path.stat().st_size
        it = int(rec["it"])
        c = rec["cvg"]
        margin = ""
        if 0 < it < c.size:
            # break iteration: how far cvg sits from errBound on either side
            margin = f" break cvg[{it}]={c[it]:.4e} prev={c[it-1]:.4e} errBound={case[5]:.1e}"
        print(f"{case[0]:22s} it={it:4d} size={path.stat().st_size/1024:.0f}KiB{margin}")
    print(f"total {total/1024:.0f} KiB")


if __name__ == "__main__":
    main()
