"""ORACLE -- test infrastructure only: numpy restatement of the cost-term and
regularisation-weight construction in the reference's applications, in the
float32 arithmetic of the GPU kernels (asetsmatlabmaxflow_gb300/csrc/costs.cu).

Arrays are in Matlab index order (Fortran), label last.
"""
from __future__ import annotations

import numpy as np

F32 = np.float32


def normalize(img):
    """(I - min I)/(max I - min I) in float32 (L1IntensitySegmentation2D.m:36)."""
    x = np.asarray(img, F32)
    lo, hi = F32(np.nanmin(x)), F32(np.nanmax(x))
    return ((x - lo) / (hi - lo)).astype(F32)


def cost_l1(img, models, normalize_img=True):
    """Ct(:,:,i) = abs(img - imgModels(i)) (L1IntensitySegmentation2D.m:42-45)."""
    x = normalize(img) if normalize_img else np.asarray(img, F32)
    return np.stack([np.abs(x - F32(m)) for m in models], axis=-1).astype(F32)


def cost_neglog(prob, eps):
    """Ct = -log(p + epsilon) (atlasProbabilityMapsRegularization3D.m:45-53),
    in float64 from the float32 inputs (the GPU rounds p + eps to float32)."""
    return -np.log(np.asarray(prob, F32).astype(np.float64) + float(eps))


def scaled255(img):
    """img_n = ((img - minI)/(maxI - minI)).*255.0 in single precision
    (interactiveGraphCutSegmentation3D.m:108-113)."""
    return (normalize(img) * F32(255.0)).astype(F32)


def histogram_counts(img, scribbles, L):
    """histc(img_n(lbl == 1), linspace(0,255,256)) for lbl = scribbles == l
    (interactiveGraphCutSegmentation3D.m:47-49, 116): bin k holds
    k <= x < k+1, the last bin also x == 255."""
    x = scaled255(img).ravel(order="F")
    s = np.asarray(scribbles).ravel(order="F")
    out = np.zeros((L, 256), np.int64)
    for l in range(1, L + 1):
        v = x[s == l]
        v = v[(v >= 0) & (v <= 255)]
        b = np.minimum(np.floor(v).astype(np.int64), 255)
        out[l - 1] = np.bincount(b, minlength=256)
    return out


def cost_histogram_ll(img, scribbles, L, eps=1e-10):
    """P = binCounts(uint16(img_n) + 1); cost = -log10(P + epsilon), the
    probabilities in double, the cost rounded to single
    (interactiveGraphCutSegmentation3D.m:119-122)."""
    counts = histogram_counts(img, scribbles, L)
    x = scaled255(img)
    idx = np.clip(np.floor(x.astype(np.float64) + 0.5), 0, 255).astype(np.int64)  # uint16()
    out = np.empty(x.shape + (L,), F32)
    with np.errstate(invalid="ignore", divide="ignore"):
        for l in range(L):
            p = counts[l] / counts[l].sum()
            table = (-np.log10(p + eps)).astype(F32)
            out[..., l] = table[idx]
    return out, counts


def alpha_contrast(img, a, b, c, squared=False, normalize_img=True):
    """alpha = a + b*exp(-c*|grad I|^p) with Matlab's gradient (central
    differences inside, one-sided at the ends), in float64
    (smoothManualSegmentations2D.m:82-91)."""
    x = (normalize(img) if normalize_img else np.asarray(img, F32)).astype(np.float64)
    grads = [np.gradient(x, axis=k) if x.shape[k] > 1 else np.zeros_like(x)
             for k in range(x.ndim)]
    g2 = sum(g * g for g in grads)
    t = g2 if squared else np.sqrt(g2)
    return a + b * np.exp(-c * t)
