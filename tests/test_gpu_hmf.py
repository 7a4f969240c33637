"""Hierarchical max-flow (full flow) on the GPU against the numpy
restatement of asetsHMF2D.m / asetsHMF3D.m (oracle/hmf.py): every state
array bit for bit in float32 and float64, costs to summation order; and the
reference's linear-model test (runTestHMFLinearModel.m) on a synthetic
image."""
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

    import ctypes
    par = np.array([-1, 2, 0], np.int32)  # child listed before its parent
    ct = (ctypes.c_void_p * 3)(None, None, None)
    st = N.lib().asets_hmf_full_flow(N.Context.default().handle, 8, 2, 4, 4, 1, 3,
                                     par.ctypes.data, ct, None, None, 1, 0.1, 0.2, None, None,
                                     None, None, None, None, None, None, None)
    assert st == N.ASETS_ERR_INVALID_ARG
