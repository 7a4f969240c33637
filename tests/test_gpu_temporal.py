"""The binary 2D kernel with two ALM iterations per pass (temporal
blocking, csrc/stencil2d_t2.cuh), selected explicitly, against the oracle on
fixed, even iteration counts: EXACT u bit-identical to the reference's
arithmetic, fast mode to the parity bar; odd and single-row shapes, columns
below one tile."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_helpers import assert_parity_bar, bits, require_gpu

pytestmark = pytest.mark.gpu

# positions (tile_config, 1-based) of the two-iteration variant in the
# binary 2D variant tables (csrc/binary2d_fast.cu, binary2d_exact.cu)
FAST_T2, EXACT_T2 = 5, 4


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()


def _rand(dims, seed):
    from scipy.ndimage import gaussian_filter

    g = np.random.default_rng(seed)
    sm = lambda: np.asfortranarray(gaussian_filter(g.random(dims), 1.0).astype(np.float32))  # noqa: E731
    return sm(), sm(), (0.1 + 0.6 * g.random(dims)).astype(np.float32)


@pytest.mark.parametrize("dims,maxit", [((301, 170), 40), ((224, 64), 30), ((57, 33), 24),
                                        ((1, 9), 10), ((450, 5), 20), ((1000, 333), 60)])
def test_two_iterations_per_pass_match_oracle(dims, maxit):
    from asetsmatlabmaxflow_gb300 import native as N

    cs, ct, alpha = _rand(dims, 17)
    cc, steps = 0.3, 0.16
    ref = O.solve("binary", dims, ct, alpha, cs=cs, max_it=maxit, err_bound=0.0, cc=cc,
                  steps=steps, erru_double=True)
    s = N.Solver(N.Context.default(), "binary", dims)
    s.set_inputs(ct, alpha, cs)
    assert s.run(maxit, 0.0, cc, steps, exact=True, tile_config=EXACT_T2) == maxit
    np.testing.assert_array_equal(bits(s.get_u()), bits(ref["u"]))
    np.testing.assert_allclose(s.get_cvg(), ref["cvg"], rtol=2e-5, atol=1e-12)
    ps, pt = s.get_flows()
    s.run(maxit, 0.0, cc, steps, exact=True)   # one iteration per pass
    ps1, pt1 = s.get_flows()
    np.testing.assert_array_equal(bits(ps), bits(ps1))
    np.testing.assert_array_equal(bits(pt), bits(pt1))
    assert s.run(maxit, 0.0, cc, steps, tile_config=FAST_T2) == maxit
    assert_parity_bar("binary", dims, 1, s.get_u().reshape(dims, order="F"),
                      ref["u"].reshape(dims, order="F"), s.get_cvg(), ref["cvg"])
    s.close()


def test_two_iteration_pass_flows_equal_single_iterations():
    """The spatial flows after a two-iteration-pass solve equal those of the
    one-iteration kernel (EXACT), so a saved state resumes identically."""
    from asetsmatlabmaxflow_gb300 import native as N

    dims = (260, 150)
    cs, ct, alpha = _rand(dims, 5)
    s = N.Solver(N.Context.default(), "binary", dims)
    s.set_inputs(ct, alpha, cs)
    s.run(16, 0.0, 0.3, 0.16, exact=True, tile_config=EXACT_T2)
    f2 = [a.copy() for a in s.get_spatial_flows() if a is not None]
    s.run(16, 0.0, 0.3, 0.16, exact=True)
    f1 = [a.copy() for a in s.get_spatial_flows() if a is not None]
    for a, b in zip(f2, f1):
        np.testing.assert_array_equal(bits(a), bits(b))
    s.close()
