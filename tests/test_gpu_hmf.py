"""Hierarchical max-flow on the GPU against the numpy restatement of
asetsHMF2D.m / asetsHMF3D.m (oracle/hmf.py): full flow with and without
direction fields, every state array bit for bit in float32 and float64,
costs to summation order; pseudo-flow to a stated tolerance (it passes
through exp); and the reference's linear-model test
(runTestHMFLinearModel.m) on a synthetic image."""
import ctypes

import numpy as np
import pytest

from oracle import hmf as H
from tests.gpu_helpers import require_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()


def _build(cls, shape, dtype, seed, nested, alpha_array):
    """The same tree for the oracle (H.Node) and the GPU class."""
    g = np.random.default_rng(seed)
    img = g.random(shape).astype(dtype)
    k = 5

    def leaf(make, i):
        a = (0.05 + 0.2 * g.random(shape)).astype(dtype) if (alpha_array and i == 1) else 0.15
        return make([], a, np.sqrt(np.abs(img - dtype(i / (k - 1)))).astype(dtype))

    def tree(make):
        g.bit_generator.state = np.random.default_rng(seed + 1).bit_generator.state
        leaves = [leaf(make, i) for i in range(k)]
        if nested:
            mid = make(leaves[:2], 0.2)
            root = make([mid] + leaves[2:], 0)
        else:
            root = make(leaves, 0)
        return root

    return tree(H.Node), tree(cls)


CASES = [
    ((37, 29), np.float64, False, False),
    ((37, 29), np.float32, True, True),
    ((1, 40), np.float64, False, False),
    ((11, 9, 7), np.float32, True, False),
    ((12, 10, 6), np.float64, False, True),
]


@pytest.mark.parametrize("shape,dtype,nested,alpha_array", CASES)
def test_full_flow_matches_restatement(shape, dtype, nested, alpha_array):
    from asetsmatlabmaxflow_gb300.hmf import asetsHMF2D, asetsHMF3D

    cls = asetsHMF2D if len(shape) == 2 else asetsHMF3D
    ref, gpu = _build(cls, shape, dtype, 3, nested, alpha_array)
    its, steps, cc = 25, 0.1, 0.2
    ref.max_full_flow(its, steps, cc)
    gpu.MaxFullFlow(its, steps, cc)
    bits = lambda a: np.ascontiguousarray(a).view(np.uint64 if a.dtype == np.float64 else np.uint32)  # noqa: E731
    for r, q in zip(H.preorder(ref), gpu._nodes()):
        for name in ("u", "pt", "div", "g"):
            assert np.array_equal(bits(getattr(q, name)), bits(getattr(r, name))), name
        for k, name in enumerate(("px", "py", "pz")[:len(shape)]):
            assert np.array_equal(bits(getattr(q, name)), bits(r.p[k])), name
        rt = 1e-9 if dtype == np.float64 else 1e-4
        assert np.isclose(q.dataCost, r.dataCost, rtol=rt, atol=1e-9)
        assert np.isclose(q.reguCost, r.reguCost, rtol=rt, atol=1e-6)


@pytest.mark.parametrize("dtype,nodes", [(np.float32, 15), (np.float32, 16), (np.float64, 7),
                                         (np.float64, 8)])
def test_full_flow_on_trees_either_side_of_the_staged_limit(dtype, nodes):
    """The per-pixel pass keeps every node of a pixel in shared memory up to
    15 nodes in float32 and 7 in float64, and reads them from global memory
    beyond: both forms against the restatement, bit for bit."""
    from asetsmatlabmaxflow_gb300.hmf import asetsHMF2D

    shape = (21, 18)
    g = np.random.default_rng(nodes)
    img = g.random(shape).astype(dtype)

    def tree(make):
        # root -> inner nodes of two or three leaves each, then leaves
        # under the root until `nodes` nodes
        count, kids, lab = 1, [], 0
        while count < nodes:
            room = nodes - count
            if room >= 4:
                n = 3 if room >= 5 else 2
                leaves = [make([], 0.15, np.sqrt(np.abs(img - dtype((lab + i) / 12))).astype(dtype))
                          for i in range(n)]
                lab += n
                kids.append(make(leaves, 0.2))
                count += 1 + n
            else:
                kids.append(make([], 0.1, np.abs(img - dtype(lab / 12)).astype(dtype)))
                lab += 1
                count += 1
        return make(kids, 0)

    ref, gpu = tree(H.Node), tree(asetsHMF2D)
    assert len(gpu._nodes()) == nodes
    ref.max_full_flow(15, 0.1, 0.2)
    gpu.MaxFullFlow(15, 0.1, 0.2)
    bits = lambda a: np.ascontiguousarray(a).view(np.uint64 if a.dtype == np.float64 else np.uint32)  # noqa: E731
    for r, q in zip(H.preorder(ref), gpu._nodes()):
        for name in ("u", "pt", "div", "g"):
            assert np.array_equal(bits(getattr(q, name)), bits(getattr(r, name))), name


def test_linear_model_denoises():
    """runTestHMFLinearModel.m: numLevels leaves with sqrt(|I - l/(L-1)|)
    costs under one root; the label-weighted reconstruction is closer to the
    clean image than the noisy input."""
    from asetsmatlabmaxflow_gb300 import synth
    from asetsmatlabmaxflow_gb300.hmf import asetsHMF2D

    g = synth.rng(7)
    clean = synth.smooth_field((96, 80), 6, g)
    noisy = clean + 0.15 * g.standard_normal(clean.shape)
    L = 16
    leaves = [asetsHMF2D([], 0.15, np.sqrt(np.abs(noisy - i / (L - 1)))) for i in range(L)]
    s = asetsHMF2D(leaves, 0)
    s.MaxFullFlow(200, 0.1, 1 / L)
    acc = sum(l.u for l in leaves)
    recon = sum(l.u * (i / (L - 1)) for i, l in enumerate(leaves)) / acc
    assert np.all(np.isfinite(recon))
    assert np.mean(np.abs(recon - clean)) < 0.6 * np.mean(np.abs(noisy - clean))


def test_bad_tree_is_rejected():
    from asetsmatlabmaxflow_gb300 import native as N

    par = np.array([-1, 2, 0], np.int32)  # child listed before its parent
    ct = (ctypes.c_void_p * 3)(None, None, None)
    st = N.lib().asets_hmf_full_flow(N.Context.default().handle, 8, 2, 4, 4, 1, 3,
                                     par.ctypes.data, ct, None, None, 1, 0.1, 0.2, None, None,
                                     None, None, None, None, None, None, None)
    assert st == N.ASETS_ERR_INVALID_ARG


def _dirs(shape, dtype, seed):
    """Direction fields with cells of zero length (below the 0.001 cut)."""
    g = np.random.default_rng(seed)
    ls = [(g.random(shape) - 0.5).astype(dtype) for _ in shape]
    dead = g.random(shape) < 0.1
    for l in ls:
        l[dead] = 0
    return ls


def _set_dirs(node, ls):
    node.lx, node.ly = ls[0].copy(), ls[1].copy()
    if len(ls) == 3:
        node.lz = ls[2].copy()


GEO_CASES = [
    ((29, 23), np.float32, True),
    ((29, 23), np.float64, False),
    ((9, 8, 7), np.float32, False),
    ((10, 7, 6), np.float64, True),
]


@pytest.mark.parametrize("shape,dtype,nested", GEO_CASES)
def test_geodesic_full_flow_matches_restatement(shape, dtype, nested):
    """The geodesic branch of UpdateSpatialFlows (direction fields on two
    leaves and, nested, on the inner node): every state array and the
    normalised fields bit for bit."""
    from asetsmatlabmaxflow_gb300.hmf import asetsHMF2D, asetsHMF3D

    cls = asetsHMF2D if len(shape) == 2 else asetsHMF3D
    ref, gpu = _build(cls, shape, dtype, 11, nested, False)
    for k, (r, q) in enumerate(zip(H.preorder(ref), gpu._nodes())):
        if k in (1, 3):
            ls = _dirs(shape, dtype, 20 + k)
            _set_dirs(r, ls)
            _set_dirs(q, ls)
    its, steps, cc = 25, 0.1, 0.2
    ref.max_full_flow(its, steps, cc)
    gpu.MaxFullFlow(its, steps, cc)
    for r, q in zip(H.preorder(ref), gpu._nodes()):
        for name in ("u", "pt", "div", "g"):
            assert np.array_equal(_bits_of(getattr(q, name)), _bits_of(getattr(r, name))), name
        for k, name in enumerate(("px", "py", "pz")[:len(shape)]):
            assert np.array_equal(_bits_of(getattr(q, name)), _bits_of(r.p[k])), name
        if r.lx is not None:
            for name in ("lx", "ly", "lz")[:len(shape)]:
                assert np.array_equal(_bits_of(getattr(q, name)), _bits_of(getattr(r, name))), name


def _bits_of(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint64 if a.dtype == np.float64 else np.uint32)


PSEUDO_CASES = [
    ((31, 27), np.float32, True, False),
    ((31, 27), np.float64, False, True),
    ((9, 8, 7), np.float32, False, True),
    ((10, 7, 6), np.float64, True, False),
]


@pytest.mark.parametrize("shape,dtype,nested,geodesic", PSEUDO_CASES)
def test_pseudo_flow_matches_restatement(shape, dtype, nested, geodesic):
    """MaxPseudoFlow from positive labels against the restatement.  The
    labels pass through exp, which the GPU's libm and numpy round
    differently in the last place, so the states agree to a tolerance:
    relative 1e-4 (float32) and 1e-10 (float64) of each array's range."""
    from asetsmatlabmaxflow_gb300.hmf import asetsHMF2D, asetsHMF3D

    cls = asetsHMF2D if len(shape) == 2 else asetsHMF3D
    ref, gpu = _build(cls, shape, dtype, 13, nested, False)
    g = np.random.default_rng(14)
    for r, q in zip(H.preorder(ref), gpu._nodes()):
        if not r.C:
            u0 = (0.2 + g.random(shape)).astype(dtype)
            r.u, q.u = u0.copy(), u0.copy()
    if geodesic:
        for k, (r, q) in enumerate(zip(H.preorder(ref), gpu._nodes())):
            if k == 2:
                ls = _dirs(shape, dtype, 30)
                _set_dirs(r, ls)
                _set_dirs(q, ls)
    its, steps, cc = 8, 0.05, 1.0
    ref.max_pseudo_flow(its, steps, cc)
    gpu.MaxPseudoFlow(its, steps, cc)
    tol = 1e-4 if dtype == np.float32 else 1e-10
    for r, q in zip(H.preorder(ref), gpu._nodes()):
        pairs = [("u", q.u, r.u), ("div", q.div, r.div), ("g", q.g, r.g)]
        pairs += [(nm, getattr(q, nm), r.p[k]) for k, nm in enumerate(("px", "py", "pz")[:len(shape)])]
        for name, a, b in pairs:
            assert a.dtype == b.dtype and a.shape == b.shape, name
            assert np.all(np.isfinite(b)), name
            scale = max(float(np.max(np.abs(b))), 1e-30)
            assert float(np.max(np.abs(a.astype(np.float64) - b))) <= tol * scale, name


def test_pseudo_flow_labels_partition_unity():
    """After MaxPseudoFlow the leaves' labels lie in [0, 1] and the root's
    (the sum over its children) is one per pixel."""
    from asetsmatlabmaxflow_gb300.hmf import asetsHMF2D

    g = np.random.default_rng(3)
    img = g.random((40, 33))
    leaves = [asetsHMF2D([], 0.2, np.abs(img - i / 3)) for i in range(4)]
    for l in leaves:
        l.u = np.full(img.shape, 0.25)
    root = asetsHMF2D([asetsHMF2D(leaves[:2], 0.3)] + leaves[2:], 0)
    root.MaxPseudoFlow(20, 0.05, 1.0)
    for l in leaves:
        assert l.u.min() >= 0 and l.u.max() <= 1
    assert np.allclose(root.u, 1.0, atol=1e-12)
    assert np.allclose(root.C[0].u, leaves[0].u + leaves[1].u, rtol=0, atol=0)


def test_lx_without_ly_is_rejected():
    from asetsmatlabmaxflow_gb300 import native as N
    from asetsmatlabmaxflow_gb300.hmf import asetsHMF2D

    leaves = [asetsHMF2D([], 0.1, np.ones((5, 4)) * i) for i in range(2)]
    leaves[0].lx = np.ones((5, 4))
    root = asetsHMF2D(leaves, 0)
    with pytest.raises(ValueError):
        root.MaxFullFlow(2, 0.1, 0.25)
    ct = (ctypes.c_void_p * 3)(None, leaves[0].Ct.ctypes.data, leaves[1].Ct.ctypes.data)
    lx = (ctypes.c_void_p * 3)(None, leaves[0].lx.ctypes.data, None)
    par = np.array([-1, 0, 0], np.int32)
    st = N.lib().asets_hmf_run(N.Context.default().handle, 0, 8, 2, 5, 4, 1, 3, par.ctypes.data,
                               ct, None, None, lx, None, None, 1, 0.1, 0.2, None, None, None,
                               None, None, None, None, None, None)
    assert st == N.ASETS_ERR_INVALID_ARG
