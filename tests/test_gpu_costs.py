"""Cost terms and regularisation weights on the GPU against the numpy
restatement of the reference's application code (oracle/costs.py)."""
import numpy as np
import pytest

from oracle import costs as C
from tests.gpu_helpers import require_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()


# (40, 36, 70): 16-byte paths (element count a multiple of 4) and several
# plane blocks of the alpha kernel; the others ragged
SHAPES = [(37, 29, 11), (64, 48), (5, 1, 3), (128, 1), (40, 36, 70)]


def _img(shape, seed):
    g = np.random.default_rng(seed)
    return np.asfortranarray((g.random(shape) * 700.0 - 120.0).astype(np.float32))


@pytest.mark.parametrize("shape", SHAPES)
def test_l1_cost_is_bit_exact(shape):
    from asetsmatlabmaxflow_gb300 import costs

    img = _img(shape, 1)
    models = [0.0, 0.25, 0.5, 0.9]
    got = costs.l1(img, models)
    assert np.array_equal(got.view(np.uint32), C.cost_l1(img, models).view(np.uint32))
    raw = costs.l1(img, [3.5, -1.0], normalize=False)
    assert np.array_equal(raw, C.cost_l1(img, [3.5, -1.0], normalize_img=False))


@pytest.mark.parametrize("shape", SHAPES[:2])
def test_neglog_cost(shape):
    from asetsmatlabmaxflow_gb300 import costs

    g = np.random.default_rng(2)
    p = np.asfortranarray(g.random(shape + (4,)).astype(np.float32))
    p.reshape(-1, order="F")[:7] = 0.0  # log(eps)
    got = costs.neglog(p, 1e-10).astype(np.float64)
    ref = C.cost_neglog(p, 1e-10)
    assert np.allclose(got, ref, rtol=2e-6, atol=2e-6)


@pytest.mark.parametrize("shape", SHAPES)
def test_histogram_ll_cost(shape):
    from asetsmatlabmaxflow_gb300 import costs

    img = _img(shape, 3)
    g = np.random.default_rng(4)
    L = 3
    scrib = np.asfortranarray(g.integers(0, L + 1, size=shape).astype(np.int32))
    scrib.reshape(-1, order="F")[:L] = np.arange(1, L + 1)  # every label scribbled
    ct, counts = costs.histogram_ll(img, scrib, L)
    ct_ref, counts_ref = C.cost_histogram_ll(img, scrib, L)
    assert np.array_equal(counts.astype(np.int64), counts_ref)
    assert np.array_equal(ct, ct_ref)


def test_histogram_bins_follow_histc_and_uint16():
    """A voxel at exactly 255 falls in the last bin, one at 254.6 is counted
    in bin 254 but looked up in bin 255 (floor for histc, rounding for
    uint16)."""
    from asetsmatlabmaxflow_gb300 import costs

    img = np.asfortranarray(np.array([0.0, 254.6, 255.0, 100.2, 100.5, 3.0], np.float32)
                            .reshape(6, 1))
    scrib = np.asfortranarray(np.array([1, 1, 1, 1, 1, 0], np.int32).reshape(6, 1))
    ct, counts = costs.histogram_ll(img, scrib, 1)
    assert counts[0, 254] == 1 and counts[0, 255] == 1 and counts[0, 0] == 1
    assert counts[0, 100] == 2 and counts.sum() == 5
    ct_ref, _ = C.cost_histogram_ll(img, scrib, 1)
    assert np.array_equal(ct, ct_ref)


@pytest.mark.parametrize("shape", SHAPES)
def test_contrast_alpha(shape):
    from asetsmatlabmaxflow_gb300 import costs

    img = _img(shape, 5)
    got = costs.alpha_contrast(img, 0.0, 0.2, 10.0, labels=3)
    ref = C.alpha_contrast(img, 0.0, 0.2, 10.0)
    for l in range(3):
        assert np.allclose(got[..., l], ref, rtol=1e-5, atol=1e-6)
    got2 = costs.alpha_contrast(img, 0.1, 0.9, 10.0, squared=True)
    assert np.allclose(got2, C.alpha_contrast(img, 0.1, 0.9, 10.0, squared=True),
                       rtol=1e-5, atol=1e-6)


def test_binary3d_workload_alpha_matches_synth():
    """The binary 3D workload's contrast-sensitive alpha (0.1 + 0.9 exp(-10
    |grad I|^2) on the raw image) built on the GPU."""
    from asetsmatlabmaxflow_gb300 import costs, synth

    g = synth.rng(0)
    img = synth.voronoi_image((48, 40, 24), 40, (0.25, 0.75), 0.2, g)
    got = costs.alpha_contrast(img, 0.1, 0.9, 10.0, squared=True, normalize=False)
    assert np.allclose(got, synth.contrast_alpha(img), rtol=1e-5, atol=1e-6)


def test_bad_arguments_are_rejected():
    from asetsmatlabmaxflow_gb300 import costs
    from asetsmatlabmaxflow_gb300 import native as N

    with pytest.raises(N.AsetsError):
        costs.l1(_img((8, 8), 0), list(range(33)))
