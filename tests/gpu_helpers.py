"""Shared helpers of the GPU parity tests."""
from __future__ import annotations

import numpy as np
import pytest


def require_gpu():
    from asetsmatlabmaxflow_gb300 import native as N

    try:
        N.Context.default()
    except Exception as e:  # noqa: BLE001
        pytest.fail(f"GPU test without a usable GB300: {e}")


def bits(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32).ravel(order="F").view(np.uint32)


def labels_of(model: str, u: np.ndarray, dims, nlab: int) -> np.ndarray:
    """Discrete labelling as the reference tests form it: u>0.5 (binary),
    argmax over labels (Potts), count of u>0.5 layers (Ishikawa)."""
    n = int(np.prod(dims))
    if model == "binary":
        return (u.ravel(order="F") > 0.5).astype(np.int32)
    if model == "potts":
        return np.argmax(u.reshape(n, nlab, order="F"), axis=1)
    return (u.reshape(n, nlab - 1, order="F") > 0.5).sum(axis=1)


# erriter below 1e-6 (a hundredth of the workloads' errBound 1e-4) is the
# mean over voxels of |e|, e = cc*((pt + dv) - ps) the per-voxel change of u,
# with e within a few float32 ulps of the O(0.1..1) terms it is formed from:
# there a change of rounding alone (FMA contraction, the hardware reciprocal
# square root of the fast kernels) moves erriter by a few percent.  So the
# relative bar holds down to 1e-6, and below it an absolute one of 1e-3 of
# 1e-6.  EXACT mode, bit-identical to the reference, is compared at 1e-4
# relative all the way down.
ERRITER_RTOL = 1e-3
ERRITER_ATOL = 1e-9


def assert_parity_bar(model, dims, nlab, u_gpu, u_ref, cvg_gpu, cvg_ref, *, it=None):
    """max|u_gpu - u_ref| <= 1e-3, >= 99.99% label agreement, erriter
    within 1e-3 relative (1e-9 absolute below erriter 1e-6, the float32
    rounding floor of the multiplier update): the parity bar of the port."""
    du = float(np.max(np.abs(u_gpu.ravel(order="F") - u_ref.ravel(order="F")))) if u_gpu.size else 0.0
    assert du <= 1e-3, f"max|du| = {du}"
    la = labels_of(model, u_gpu, dims, nlab)
    lb = labels_of(model, u_ref, dims, nlab)
    agree = float(np.mean(la == lb)) if la.size else 1.0
    assert agree >= 0.9999, f"label agreement {agree}"
    n = len(cvg_ref) if it is None else it
    if n:
        np.testing.assert_allclose(np.asarray(cvg_gpu).ravel()[:n], np.asarray(cvg_ref).ravel()[:n],
                                   rtol=ERRITER_RTOL, atol=ERRITER_ATOL)
    return du, agree
