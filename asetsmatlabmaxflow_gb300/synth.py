"""Seeded synthetic segmentation problems (numpy PCG64).

These stand in for real images/volumes at the shapes, sizes and value
distributions of the benchmark workloads; no public dataset is involved.
All arrays are float32 in Matlab column-major index order: a 3D volume has
shape (ny, nx, nz) and a multi-label array (ny, nx, [nz,] L), and is passed
to the solvers as np.asfortranarray (the reference's `g = z*Nx*Ny + x*Ny + y`
layout).
"""
from __future__ import annotations

import numpy as np


def rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def voronoi_labels(shape: tuple[int, ...], ncells: int, g: np.random.Generator) -> np.ndarray:
    """Index of the nearest of `ncells` uniform seeds, per pixel/voxel."""
    seeds = g.random((ncells, len(shape))) * np.array(shape, dtype=np.float64)
    return nearest_seed(shape, seeds)


def nearest_seed(shape: tuple[int, ...], seeds: np.ndarray) -> np.ndarray:
    from scipy.spatial import cKDTree

    tree = cKDTree(seeds)
    out = np.empty(int(np.prod(shape)), dtype=np.int32)
    grids = np.meshgrid(*[np.arange(n, dtype=np.float32) for n in shape], indexing="ij")
    pts = np.stack([gr.ravel(order="F") for gr in grids], axis=1)
    step = 1 << 21
    for s in range(0, pts.shape[0], step):
        _, idx = tree.query(pts[s:s + step], k=1)
        out[s:s + step] = idx
    return out.reshape(shape, order="F")


def voronoi_image(shape, ncells, values, sigma, g) -> np.ndarray:
    lab = voronoi_labels(shape, ncells, g)
    cell_val = g.choice(np.asarray(values, dtype=np.float64), size=ncells)
    img = cell_val[lab] + g.normal(0.0, sigma, size=shape)
    return np.asfortranarray(np.clip(img, 0.0, 1.0).astype(np.float32))


def contrast_alpha(img: np.ndarray) -> np.ndarray:
    """alpha = 0.1 + 0.9*exp(-10*|grad I|^2), central differences inside and
    one-sided at the borders (numpy.gradient, as Matlab's gradient)."""
    grads = np.gradient(img.astype(np.float64))
    if img.ndim == 1:
        grads = [grads]
    mag2 = sum(gr * gr for gr in grads)
    return np.asfortranarray((0.1 + 0.9 * np.exp(-10.0 * mag2)).astype(np.float32))


def binary2d(seed: int = 0, shape=(256, 256), alpha=0.5):
    """Binary 2D: 12-cell Voronoi, intensities {0.2, 0.8}, noise 0.15,
    Cs=|I-0.2|, Ct=|I-0.8|, constant alpha."""
    g = rng(seed)
    img = voronoi_image(shape, 12, (0.2, 0.8), 0.15, g)
    cs = np.abs(img - np.float32(0.2))
    ct = np.abs(img - np.float32(0.8))
    a = np.full(shape, alpha, dtype=np.float32, order="F")
    return np.asfortranarray(cs), np.asfortranarray(ct), a


def binary3d(seed: int = 0, shape=(256, 256, 256), ncells=40):
    """Binary 3D: 40-cell Voronoi, intensities {0.25, 0.75}, noise 0.2,
    Cs=|I-0.2|, Ct=|I-0.8| (the 2D cost terms), contrast-sensitive alpha."""
    g = rng(seed)
    img = voronoi_image(shape, ncells, (0.25, 0.75), 0.2, g)
    cs = np.asfortranarray(np.abs(img - np.float32(0.2)))
    ct = np.asfortranarray(np.abs(img - np.float32(0.8)))
    return cs, ct, contrast_alpha(img)


def potts3d(seed: int = 0, shape=(192, 192, 192), means=(0.1, 0.4, 0.6, 0.9), ncells=60,
            sigma=0.1, alpha=0.3):
    """Potts 3D: Voronoi with per-cell mean drawn from `means`, Ct_l=|I-c_l|."""
    g = rng(seed)
    img = voronoi_image(shape, ncells, means, sigma, g)
    L = len(means)
    ct = np.empty(shape + (L,), dtype=np.float32, order="F")
    for l, m in enumerate(means):
        ct[..., l] = np.abs(img - np.float32(m))
    a = np.full(shape + (L,), alpha, dtype=np.float32, order="F")
    return ct, a


def smooth_field(shape, ngauss: int, g: np.random.Generator) -> np.ndarray:
    grids = np.meshgrid(*[np.arange(n, dtype=np.float64) for n in shape], indexing="ij")
    f = np.zeros(shape)
    for _ in range(ngauss):
        c = g.random(len(shape)) * np.array(shape)
        w = (0.05 + 0.2 * g.random()) * min(shape)
        amp = g.uniform(-1.0, 1.0)
        r2 = sum((gr - ci) ** 2 for gr, ci in zip(grids, c))
        f += amp * np.exp(-r2 / (2 * w * w))
    f -= f.min()
    mx = f.max()
    return f / mx if mx > 0 else f


def ishikawa2d(seed: int = 0, shape=(1024, 1024), L=8, alpha=0.2, sigma=0.05):
    """Ishikawa 2D: sum of 16 Gaussians rescaled to [0,1] plus noise,
    Ct_l=|I-l/(L-1)|, alpha on every level boundary (L-1 slices)."""
    g = rng(seed)
    img = smooth_field(shape, 16, g) + g.normal(0.0, sigma, size=shape)
    img = img.astype(np.float32)
    ct = np.empty(shape + (L,), dtype=np.float32, order="F")
    for l in range(L):
        ct[..., l] = np.abs(img - np.float32(l / (L - 1)))
    a = np.full(shape + (L - 1,), alpha, dtype=np.float32, order="F")
    return ct, a


def potts_warmstart_draws(seed: int, shape=(128, 128, 128), L=6):
    """The random draws of one warm-start Potts problem, in generator order:
    label means U[0,1], 30-80 Voronoi cells, noise sigma U[0.05,0.2], alpha
    U[0.1,0.5], the cell seeds, each cell's mean, the noise field."""
    g = rng(seed)
    means = g.random(L)
    ncells = int(g.integers(30, 81))
    sigma = float(g.uniform(0.05, 0.2))
    alpha = float(g.uniform(0.1, 0.5))
    seeds = g.random((ncells, len(shape))) * np.array(shape, dtype=np.float64)
    cell_mean = means[g.integers(0, L, size=ncells)]
    noise = g.normal(0.0, sigma, size=shape)
    return means, seeds, cell_mean, alpha, noise


def potts_warmstart(seed: int, shape=(128, 128, 128), L=6):
    """Warm-start Potts problems: means U[0,1], 30-80 Voronoi cells, noise
    U[0.05,0.2], alpha U[0.1,0.5]; Ct_l=|I-c_l|, alpha on all L slices."""
    means, seeds, cell_mean, alpha, noise = potts_warmstart_draws(seed, shape, L)
    lab = nearest_seed(shape, seeds)
    img = np.clip(cell_mean[lab] + noise, 0.0, 1.0).astype(np.float32)
    ct = np.empty(shape + (L,), dtype=np.float32, order="F")
    for l in range(L):
        ct[..., l] = np.abs(img - np.float32(means[l]))
    a = np.full(shape + (L,), alpha, dtype=np.float32, order="F")
    return ct, a


def batch_problems(seed: int = 0, n2d: int = 48, n3d: int = 16):
    """Heterogeneous binary batch: n2d 2D problems with sides drawn from
    128..1024 (independently per axis) and n3d 3D volumes with sides from
    64..160, built like binary2d/binary3d with per-problem seeds, alpha a
    constant drawn from U[0.2, 0.8].  Returns [(Cs, Ct, alpha), ...]."""
    g = rng(seed)
    out = []
    for i in range(n2d):
        shape = (int(g.integers(128, 1025)), int(g.integers(128, 1025)))
        cs, ct, _ = binary2d(seed=1000 * (seed + 1) + i, shape=shape)
        a = np.full(shape, g.uniform(0.2, 0.8), np.float32, order="F")
        out.append((cs, ct, a))
    for i in range(n3d):
        shape = tuple(int(v) for v in g.integers(64, 161, size=3))
        cs, ct, _ = binary3d(seed=2000 * (seed + 1) + i, shape=shape, ncells=40)
        a = np.full(shape, g.uniform(0.2, 0.8), np.float32, order="F")
        out.append((cs, ct, a))
    return out
