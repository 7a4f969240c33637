"""Cost terms and regularisation weights on the GPU (asets_cost_* and
asets_alpha_contrast): the step before the solvers in the reference's
applications.  Host arrays in Matlab index order (Fortran), label last;
torch CUDA tensors are accepted as device arrays (flat, Matlab layout)."""
from __future__ import annotations

import numpy as np

from . import native as N


def _ctx(ctx):
    return (ctx or N.Context.default()).handle


def _f(a):
    return np.ascontiguousarray(np.asarray(a, np.float32).ravel(order="F"))


def l1(img, models, *, normalize: bool = True, ctx=None) -> np.ndarray:
    """|I' - m_l| for each model intensity (L1IntensitySegmentation2D.m)."""
    img = np.asarray(img)
    x = _f(img)
    m = np.ascontiguousarray(models, np.float32)
    out = np.empty(x.size * m.size, np.float32)
    N.check(N.lib().asets_cost_l1(_ctx(ctx), N.HOST, x.ctypes.data, x.size, m.ctypes.data,
                                  m.size, int(normalize), out.ctypes.data))
    return out.reshape(img.shape + (m.size,), order="F")


def neglog(prob, eps: float = 1e-10, *, ctx=None) -> np.ndarray:
    """-log(p + eps) of probability maps shaped (..., L)
    (atlasProbabilityMapsRegularization3D.m)."""
    prob = np.asarray(prob)
    x = _f(prob)
    L = prob.shape[-1]
    out = np.empty_like(x)
    N.check(N.lib().asets_cost_neglog(_ctx(ctx), N.HOST, x.ctypes.data, x.size // L, L, eps,
                                      out.ctypes.data))
    return out.reshape(prob.shape, order="F")


def histogram_ll(img, scribbles, L: int, eps: float = 1e-10, *, ctx=None):
    """Histogram log-likelihood costs from scribbles 1..L
    (interactiveGraphCutSegmentation3D.m).  Returns (Ct, counts[L, 256])."""
    img = np.asarray(img)
    x = _f(img)
    s = np.ascontiguousarray(np.asarray(scribbles).ravel(order="F"), np.int32)
    out = np.empty(x.size * L, np.float32)
    counts = np.empty(L * 256, np.uint32)
    N.check(N.lib().asets_cost_histogram_ll(_ctx(ctx), N.HOST, x.ctypes.data, s.ctypes.data,
                                            x.size, L, eps, out.ctypes.data, counts.ctypes.data))
    return out.reshape(img.shape + (L,), order="F"), counts.reshape(L, 256)


def alpha_contrast(img, a: float = 0.0, b: float = 0.2, c: float = 10.0, *,
                   squared: bool = False, normalize: bool = True, labels: int = 1,
                   ctx=None) -> np.ndarray:
    """a + b*exp(-c*|grad I'|^p) (smoothManualSegmentations2D.m; the binary
    3D workload uses a = 0.1, b = 0.9, c = 10, squared)."""
    img = np.asarray(img)
    dims = (tuple(img.shape) + (1, 1))[:3]
    x = _f(img)
    out = np.empty(x.size * labels, np.float32)
    N.check(N.lib().asets_alpha_contrast(_ctx(ctx), N.HOST, x.ctypes.data, dims[0], dims[1],
                                         dims[2], int(normalize), a, b, c, int(squared), labels,
                                         out.ctypes.data))
    shape = img.shape + ((labels,) if labels > 1 else ())
    return out.reshape(shape, order="F")


def load_mat(path, *names):
    """Arrays of a Matlab .mat file (the reference's data/ volumes) as
    float32 Fortran arrays (scipy.io; MAT v5)."""
    from scipy.io import loadmat

    d = loadmat(path)
    keys = names or [k for k in d if not k.startswith("__")]
    return {k: np.asfortranarray(np.asarray(d[k], np.float32)) for k in keys}
