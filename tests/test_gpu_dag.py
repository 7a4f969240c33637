"""DAG max-flow (full flow) on the GPU against the numpy restatement of
asetsDAGMF2D.m / asetsDAGMF3D.m (oracle/dag.py): every state array bit for
bit, in float32 and float64, on graphs with shared children, with and
without direction fields."""
import numpy as np
import pytest

from oracle import dag as Dg
from tests.gpu_helpers import require_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()


def _graph(make, shape, dtype, seed, kind):
    g = np.random.default_rng(seed)
    img = g.random(shape).astype(dtype)
    al = (0.05 + 0.2 * g.random(shape)).astype(dtype)
    L = [make([], al if i == 2 else 0.15, np.abs(img - dtype(i / 3)).astype(dtype)) for i in range(4)]
    if kind == "shared":
        a = make([L[0], L[1], L[2]], 0.2)
        b = make([L[1], L[2], L[3]], 0.25)
        return make([a, b], 0), L
    if kind == "diamond":
        a = make([L[0], L[1]], 0.2)
        b = make([L[1], L[2]], 0.2)
        c = make([a, b, L[3]], 0.1)
        return make([c, L[2]], 0), L
    return make(L, 0), L  # flat: the Potts-like model


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint64 if a.dtype == np.float64 else np.uint32)


@pytest.mark.parametrize("shape,dtype,kind", [
    ((23, 19), np.float64, "shared"),
    ((23, 19), np.float32, "diamond"),
    ((30, 1), np.float64, "flat"),
    ((9, 8, 7), np.float32, "shared"),
    ((10, 7, 6), np.float64, "diamond"),
])
def test_full_flow_matches_restatement(shape, dtype, kind):
    from asetsmatlabmaxflow_gb300.hmf import asetsDAGMF2D, asetsDAGMF3D

    cls = asetsDAGMF2D if len(shape) == 2 else asetsDAGMF3D
    ref, _ = _graph(Dg.Node, shape, dtype, 5, kind)
    gpu, _ = _graph(cls, shape, dtype, 5, kind)
    its = 20
    ref.max_full_flow(its, 0.1, 0.25)
    gpu.MaxFullFlow(its, 0.1, 0.25)

    def order(root):  # the same discovery order on both graphs
        out, seen, st = [], set(), [root]
        while st:
            n = st.pop(0)
            if id(n) not in seen:
                seen.add(id(n))
                out.append(n)
                st.extend(n.C)
        return out

    for r, q in zip(order(ref), order(gpu)):
        for name in ("u", "pt", "div", "g"):
            assert np.array_equal(_bits(getattr(q, name)), _bits(getattr(r, name))), name
        for k, name in enumerate(("px", "py", "pz")[:len(shape)]):
            assert np.array_equal(_bits(getattr(q, name)), _bits(r.p[k])), name
        if len(r.P) > 1:
            assert np.array_equal(_bits(q.pn), _bits(r.pn))


def test_single_child_inner_node_is_rejected():
    from asetsmatlabmaxflow_gb300 import native as N
    from asetsmatlabmaxflow_gb300.hmf import asetsDAGMF2D

    leaf = asetsDAGMF2D([], 0.1, np.ones((4, 4)))
    mid = asetsDAGMF2D([leaf], 0.1)
    root = asetsDAGMF2D([mid, asetsDAGMF2D([], 0.1, np.ones((4, 4)))], 0)
    with pytest.raises(N.AsetsError):
        root.MaxFullFlow(2, 0.1, 0.25)


@pytest.mark.parametrize("shape,dtype,kind", [
    ((23, 19), np.float32, "shared"),
    ((23, 19), np.float64, "diamond"),
    ((9, 8, 7), np.float64, "shared"),
    ((10, 7, 6), np.float32, "diamond"),
])
def test_geodesic_full_flow_matches_restatement(shape, dtype, kind):
    """Direction fields on a shared leaf and an inner node (the geodesic
    branch of asetsDAGMF2D.m / 3D UpdateSpatialFlows): bit for bit."""
    from asetsmatlabmaxflow_gb300.hmf import asetsDAGMF2D, asetsDAGMF3D

    cls = asetsDAGMF2D if len(shape) == 2 else asetsDAGMF3D
    ref, Lr = _graph(Dg.Node, shape, dtype, 6, kind)
    gpu, Lg = _graph(cls, shape, dtype, 6, kind)
    g = np.random.default_rng(8)
    names = ("lx", "ly", "lz")[:len(shape)]
    for r, q in ((Lr[1], Lg[1]), (ref.C[0], gpu.C[0])):
        for nm in names:
            a = (g.random(shape) - 0.5).astype(dtype)
            a[g.random(shape) < 0.1] = 0
            setattr(r, nm, a.copy())
            setattr(q, nm, a.copy())
    ref.max_full_flow(15, 0.1, 0.25)
    gpu.MaxFullFlow(15, 0.1, 0.25)

    def order(root):
        out, seen, st = [], set(), [root]
        while st:
            n = st.pop(0)
            if id(n) not in seen:
                seen.add(id(n))
                out.append(n)
                st.extend(n.C)
        return out

    for r, q in zip(order(ref), order(gpu)):
        for name in ("u", "pt", "div", "g"):
            assert np.array_equal(_bits(getattr(q, name)), _bits(getattr(r, name))), name
        for k, name in enumerate(("px", "py", "pz")[:len(shape)]):
            assert np.array_equal(_bits(getattr(q, name)), _bits(r.p[k])), name
        if r.lx is not None:
            for nm in names:
                assert np.array_equal(_bits(getattr(q, nm)), _bits(getattr(r, nm))), nm


@pytest.mark.parametrize("dtype,nodes", [(np.float64, 4), (np.float64, 5), (np.float32, 9),
                                         (np.float32, 10)])
def test_full_flow_on_graphs_either_side_of_the_staged_limit(dtype, nodes):
    """The per-pixel pass keeps every node of a pixel in shared memory up to
    9 nodes in float32 and 4 in float64, and reads them from global memory
    beyond: both forms against the restatement, bit for bit."""
    from asetsmatlabmaxflow_gb300.hmf import asetsDAGMF2D

    shape = (19, 23)

    def graph(make):
        g = np.random.default_rng(nodes)
        img = g.random(shape).astype(dtype)
        if nodes <= 5:  # flat: root over nodes - 1 leaves
            return make([make([], 0.15, np.abs(img - dtype(i / 3)).astype(dtype))
                         for i in range(nodes - 1)], 0)
        # root over three inner nodes sharing leaves, leaves 0 .. nodes - 5
        L = [make([], 0.15, np.abs(img - dtype(i / 6)).astype(dtype)) for i in range(nodes - 4)]
        a = make([L[0], L[1]], 0.2)
        b = make([L[1], L[2]], 0.2)
        c = make(L[2:], 0.1)
        return make([a, b, c], 0)

    ref, gpu = graph(Dg.Node), graph(asetsDAGMF2D)
    ref.max_full_flow(15, 0.1, 0.25)
    gpu.MaxFullFlow(15, 0.1, 0.25)

    def order(root):
        out, seen, st = [], set(), [root]
        while st:
            n = st.pop(0)
            if id(n) not in seen:
                seen.add(id(n))
                out.append(n)
                st.extend(n.C)
        return out

    assert len(order(gpu)) == nodes
    for r, q in zip(order(ref), order(gpu)):
        for name in ("u", "pt", "div", "g"):
            assert np.array_equal(_bits(getattr(q, name)), _bits(getattr(r, name))), name
        if len(r.P) > 1:
            assert np.array_equal(_bits(q.pn), _bits(r.pn))
