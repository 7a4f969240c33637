"""The Matlab-semantics solvers (the reference's .m twins) on the GPU
against their numpy restatement (oracle/mtwin.py): u bit for bit in float32
and float64, erriter to summation order, the same break iteration."""
import numpy as np
import pytest

from oracle import mtwin as M
from tests.gpu_helpers import require_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()


def _bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint64 if a.dtype == np.float64 else np.uint32)


def _check(got, ref, dtype):
    u, e, i, t = got
    ur, er, ir = ref
    assert i == ir
    assert u.dtype == dtype
    assert np.array_equal(_bits(u), _bits(ur))
    rt = 1e-12 if dtype == np.float64 else 2e-6
    assert np.allclose(e[:, 0].astype(np.float64), er.astype(np.float64), rtol=rt, atol=0)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("shape,beta", [((37, 29), 1e-12), ((40, 33), 5e-4), ((14, 11, 9), 1e-12)])
def test_binary(shape, beta, dtype):
    from asetsmatlabmaxflow_gb300 import matlab

    g = np.random.default_rng(1)
    img = g.random(shape).astype(dtype)
    cs, ct = np.abs(img - dtype(0.2)), np.abs(img - dtype(0.8))
    al = (0.2 + 0.3 * g.random(shape)).astype(dtype)
    its, cc = 60, 0.3
    steps = 0.16 if len(shape) == 2 else 0.11
    ref = M.binary(cs, ct, al, its, beta, cc, steps)
    if len(shape) == 2:
        got = matlab.asetsBinaryMF2D(cs, ct, al, [*shape, its, beta, cc, steps])
    else:
        got = matlab.asetsBinaryMF3D(cs, ct, al, [*shape, its, beta, cc, steps])
    _check(got, ref, dtype)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("shape,L,beta", [((31, 27), 4, 1e-12), ((12, 10, 7), 3, 1e-12),
                                          ((36, 30), 3, 2e-3)])
def test_potts(shape, L, beta, dtype):
    from asetsmatlabmaxflow_gb300 import matlab

    g = np.random.default_rng(2)
    ct = g.random(shape + (L,)).astype(dtype)
    ct[..., 1] = ct[..., 0]  # ties: the first minimum takes the label
    al = (0.1 + 0.3 * g.random(shape + (L,))).astype(dtype)
    its, cc = 40, 0.3
    steps = 0.16 if len(shape) == 2 else 0.11
    ref = M.potts(ct, al, its, beta, cc, steps)
    if len(shape) == 2:
        got = matlab.asetsPotts2D(ct, al, [*shape, L, its, beta, cc, steps])
    else:
        got = matlab.asetsPotts3D(ct, al, [*shape, L, its, beta, cc, steps])
    _check(got, ref, dtype)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("shape,L,beta", [((29, 23), 5, 1e-12), ((11, 9, 8), 4, 1e-12),
                                          ((30, 26), 2, 1e-3)])
def test_ishikawa(shape, L, beta, dtype):
    from asetsmatlabmaxflow_gb300 import matlab

    g = np.random.default_rng(3)
    ct = g.random(shape + (L,)).astype(dtype)
    al = (0.1 + 0.3 * g.random(shape + (L,))).astype(dtype)  # L slices given, L-1 used
    its, cc = 40, 0.3
    steps = 0.16 if len(shape) == 2 else 0.11
    ref = M.ishikawa(ct, al, its, beta, cc, steps)
    if len(shape) == 2:
        got = matlab.asetsIshikawa2D(ct, al, [*shape, L, its, beta, cc, steps])
    else:
        got = matlab.asetsIshikawa3D(ct, al, [*shape, L, its, beta, cc, steps])
    _check(got, ref, dtype)
