"""Host-side checks of the HMF / DAG restatements' optional parts (no GPU):
the direction-field normalisation, the geodesic exemption's meaning, and
the pseudo-flow labels (maxflow/asetsHMF2D.m, asetsDAGMF2D.m)."""
import warnings

import numpy as np
import pytest

from oracle import dag as Dg
from oracle import hmf as H


def _hmf(shape, dtype, seed=1):
    g = np.random.default_rng(seed)
    img = g.random(shape).astype(dtype)
    L = [H.Node([], 0.15, np.abs(img - dtype(i / 3)).astype(dtype)) for i in range(4)]
    return H.Node([H.Node(L[:2], 0.2)] + L[2:], 0), L


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_normalised_directions_have_unit_length(dtype):
    g = np.random.default_rng(0)
    ls = [(g.random((30, 20)) - 0.5).astype(dtype) for _ in range(3)]
    ls[0][:3] = ls[1][:3] = ls[2][:3] = dtype(1e-4)      # length below the 0.001 cut
    out = H.normalize_dirs(ls, np.dtype(dtype))
    n = np.sqrt(sum(o.astype(np.float64) ** 2 for o in out))
    assert np.all(n[:3] == 0)
    assert np.allclose(n[3:], 1.0, atol=1e-6 if dtype == np.float32 else 1e-14)
    assert all(o.dtype == dtype for o in out)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_zero_directions_reproduce_the_isotropic_iteration(dtype):
    """All-zero fields: no exemption, so the geodesic branch gives the
    isotropic branch's states bit for bit."""
    a, _ = _hmf((13, 11), dtype)
    b, L = _hmf((13, 11), dtype)
    for leaf in L:
        leaf.lx = np.zeros((13, 11), dtype)
        leaf.ly = np.zeros((13, 11), dtype)
    a.max_full_flow(12, 0.1, 0.2)
    b.max_full_flow(12, 0.1, 0.2)
    for x, y in zip(H.preorder(a), H.preorder(b)):
        assert np.array_equal(x.u, y.u) and np.array_equal(x.div, y.div)
        assert all(np.array_equal(p, q) for p, q in zip(x.p, y.p))


def test_zero_directions_dag_3d():
    def graph(dirs):
        g = np.random.default_rng(4)
        img = g.random((6, 5, 4))
        L = [Dg.Node([], 0.15, np.abs(img - i / 3)) for i in range(4)]
        a = Dg.Node(L[:3], 0.2)
        b = Dg.Node(L[1:], 0.2)
        if dirs:
            for n in L + [a, b]:
                n.lx, n.ly, n.lz = (np.zeros((6, 5, 4)) for _ in range(3))
        return Dg.Node([a, b], 0)
    x, y = graph(False), graph(True)
    tx, ty = x.max_full_flow(8, 0.1, 0.25), y.max_full_flow(8, 0.1, 0.25)
    for p, q in zip(tx, ty):
        assert np.array_equal(p.u, q.u) and all(np.array_equal(s, t) for s, t in zip(p.p, q.p))


def test_flow_along_the_direction_is_exempt():
    """Rows of one pixel, lx = 1: a positive flow along +x leaves its cell
    along the cell's direction, so it is exempt and keeps its size past
    alpha; against lx = -1 the same flow is clipped to alpha."""
    D = (8, 1)
    p0 = [np.full((7, 1), 0.5), np.zeros((8, 0))]
    for lx, clipped in ((1.0, False), (-1.0, True)):
        ls = [np.full(D, lx), np.zeros(D)]
        q, e, a = H.exemption([x.copy() for x in p0], ls, D, np.dtype(np.float64))
        out, _, _ = H.project(q, 0.1, D, np.dtype(np.float64), e)
        if clipped:
            assert np.all(out[0] <= 0.1 + 1e-12)
        else:
            assert np.allclose(out[0], 0.5)


def test_pseudo_flow_labels():
    """Leaves' labels in [0, 1] summing to one per pixel, the inner nodes'
    the sum of their children's."""
    root, L = _hmf((17, 12), np.float64)
    for leaf in L:
        leaf.u = np.full((17, 12), 0.25)
    root.max_pseudo_flow(10, 0.05, 1.0)
    for leaf in L:
        assert leaf.u.min() >= 0 and leaf.u.max() <= 1
    assert np.allclose(root.u, 1.0, atol=1e-12)
    assert np.array_equal(root.C[0].u, L[0].u + L[1].u)


def test_pseudo_flow_from_zero_labels_is_nan():
    """A fresh tree's leaves hold u = 0: the normalisation divides 0 by 0,
    as the class does."""
    root, L = _hmf((5, 4), np.float64)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        root.max_pseudo_flow(2, 0.05, 1.0)
    assert all(np.isnan(leaf.u).all() for leaf in L)


def test_lx_without_ly_raises():
    root, L = _hmf((5, 4), np.float64)
    L[0].lx = np.ones((5, 4))
    with pytest.raises(ValueError):
        root.max_full_flow(1, 0.1, 0.2)
