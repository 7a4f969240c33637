"""GPU parity of the one-pass multi-label 2D kernel (stencil2d_labels.cuh):
the flows of every label and the per-pixel label update in one launch.

It is the first candidate (tile_config 1, and the default) of the Potts and
Ishikawa 2D solvers; tile_config 2 is the two-pass form (flow kernel +
label kernel).  EXACT results must be bit-identical to the oracle and to the
two-pass form (u, pt, ps and the spatial flows); the fast build meets the
parity bar; stopping runs stop where the oracle stops."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_helpers import assert_parity_bar, bits, require_gpu

pytestmark = pytest.mark.gpu

# tile_config of the one-pass forms: the label update in the flow warps,
# one label warp, two label warps, 16 x 16 tiles per iteration and for the
# whole solve; then the two-pass form
FUSED_FORMS = (1, 2, 3, 4, 5)
FUSED, TWO_PASS = 1, 6


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()


def _inputs(model, dims, L, seed):
    from scipy.ndimage import gaussian_filter

    g = np.random.default_rng(seed)
    ct = np.asfortranarray(gaussian_filter(g.random(dims + (L,)), (1.5, 1.5, 0)).astype(np.float32))
    la = L if model == "potts" else L - 1
    alpha = np.asfortranarray((0.05 + 0.4 * g.random(dims + (la,))).astype(np.float32))
    return ct, alpha


def _solve(model, dims, L, ct, alpha, max_it, eb, exact, tc, cc=0.3, steps=0.16):
    from asetsmatlabmaxflow_gb300 import native as N

    s = N.Solver(N.Context.default(), model, dims, L)
    s.set_inputs(ct, alpha)
    it = s.run(max_it, eb, cc, steps, exact=exact, tile_config=tc)
    u = s.get_u()
    ps, pt = s.get_flows()
    bx, by, _ = s.get_spatial_flows()
    cvg = s.get_cvg()
    _, launches = s.last_run_stats()
    s.close()
    return dict(it=it, u=u, ps=ps, pt=pt, bx=bx, by=by, cvg=cvg, launches=launches)


# (model, dims, labels): odd shapes, a single short column tile, one flow
# label, the largest label counts the kernel is built for
SHAPES = [
    ("potts", (97, 61), 4), ("potts", (7, 33), 2), ("potts", (130, 45), 8), ("potts", (61, 20), 1),
    ("ishikawa", (97, 61), 5), ("ishikawa", (7, 33), 2), ("ishikawa", (121, 40), 9),
    ("ishikawa", (60, 64), 3),
]


@pytest.mark.parametrize("model,dims,L", SHAPES)
def test_exact_fused_is_bit_identical_to_oracle_and_two_pass(model, dims, L):
    ct, alpha = _inputs(model, dims, L, 11)
    max_it = 13  # odd: the result is in the second parity
    ref = O.solve(model, dims, ct, alpha, nlab=L, max_it=max_it, err_bound=0.0, cc=0.3, steps=0.16,
                  want_state=True)
    f = _solve(model, dims, L, ct, alpha, max_it, 0.0, True, FUSED)
    t = _solve(model, dims, L, ct, alpha, max_it, 0.0, True, TWO_PASS)
    for tc in FUSED_FORMS[1:]:
        g = _solve(model, dims, L, ct, alpha, max_it, 0.0, True, tc)
        for k in ("u", "pt", "bx", "by"):
            np.testing.assert_array_equal(bits(g[k]), bits(t[k]), err_msg=f"{k} variant {tc}")
    assert f["it"] == t["it"] == ref["it"] == max_it
    np.testing.assert_array_equal(bits(f["u"]), bits(ref["u"]))
    np.testing.assert_array_equal(bits(f["pt"]), bits(ref["pt"]))
    if model == "potts":
        np.testing.assert_array_equal(bits(f["ps"]), bits(ref["ps"]))
        np.testing.assert_array_equal(bits(f["ps"]), bits(t["ps"]))
    for k in ("u", "pt", "bx", "by"):
        np.testing.assert_array_equal(bits(f[k]), bits(t[k]), err_msg=k)
    # erriter: the same terms, summed per tile instead of per label-kernel block
    np.testing.assert_allclose(f["cvg"], ref["cvg"], rtol=2e-5, atol=1e-12)
    # one launch per iteration instead of two
    assert f["launches"] * 2 == t["launches"]


# Potts with one label is solved from the start (u = 1): its erriter is
# rounding noise near 1e-8, which the EXACT test above covers bit for bit.
@pytest.mark.parametrize("model,dims,L", [c for c in SHAPES if c[2] > 1])
def test_fast_fused_meets_parity_bar(model, dims, L):
    ct, alpha = _inputs(model, dims, L, 12)
    max_it = 40
    ref = O.solve(model, dims, ct, alpha, nlab=L, max_it=max_it, err_bound=0.0, cc=0.3, steps=0.16)
    for tc in FUSED_FORMS:
        f = _solve(model, dims, L, ct, alpha, max_it, 0.0, False, tc)
        assert f["it"] == max_it
        assert_parity_bar(model, dims, L, f["u"], ref["u"], f["cvg"], ref["cvg"])


@pytest.mark.parametrize("model,L", [("potts", 4), ("ishikawa", 6)])
@pytest.mark.parametrize("exact", [True, False])
@pytest.mark.parametrize("tc", FUSED_FORMS)
def test_fused_stops_where_the_oracle_stops(model, L, exact, tc):
    dims = (150, 131)
    ct, alpha = _inputs(model, dims, L, 13)
    eb = 2e-4
    ref = O.solve(model, dims, ct, alpha, nlab=L, max_it=400, err_bound=eb, cc=0.3, steps=0.16)
    assert ref["it"] < 400
    f = _solve(model, dims, L, ct, alpha, 400, eb, exact, tc)
    assert f["it"] == ref["it"]
    n = min(ref["it"] + 1, 400)
    if exact:
        np.testing.assert_array_equal(bits(f["u"]), bits(ref["u"]))
    assert_parity_bar(model, dims, L, f["u"], ref["u"], f["cvg"], ref["cvg"], it=n)


@pytest.mark.parametrize("model,dims,L,launches", [
    ("potts", (2048, 1024), 4, 16), ("ishikawa", (1024, 1024), 8, 16),
    ("ishikawa", (1024, 1024), 3, 32), ("potts", (512, 512), 8, 32),
    ("potts", (256, 256), 4, 1), ("ishikawa", (200, 150), 6, 1), ("ishikawa", (128, 128), 8, 1),
    ("potts", (256, 256), 8, 1), ("potts", (512, 512), 4, 32)])
def test_default_form_by_size(model, dims, L, launches):
    """Without a tile_config the one-pass sweep kernel runs on two million
    pixels and more, and on half a million with six flow labels or more (one
    launch per iteration, one chunk of 16); images of up to 2^17 pixels run
    the whole solve in one cooperative launch (Potts 256^2 with eight labels
    two tiles per block); the rest the two-pass form (two launches per
    iteration)."""
    from asetsmatlabmaxflow_gb300 import native as N

    ct, alpha = _inputs(model, dims, L, 16)
    s = N.Solver(N.Context.default(), model, dims, L)
    s.set_inputs(ct, alpha)
    assert s.run(4, 0.0, 0.3, 0.16) == 4
    assert s.last_run_stats()[1] == launches
    s.close()


def test_a_batch_keeps_two_passes():
    """A 2D Potts problem in a batch (whose group shares one variant across
    label counts) runs the two-pass form, with the same EXACT result as the
    one-pass kernel alone."""
    from asetsmatlabmaxflow_gb300 import native as N

    dims, L = (90, 70), 3
    ct, alpha = _inputs("potts", dims, L, 14)
    lone = _solve("potts", dims, L, ct, alpha, 32, 0.0, True, FUSED)
    assert lone["launches"] == 32
    ctx = N.Context.default()
    s = N.Solver(ctx, "potts", dims, L)
    s.set_inputs(ct, alpha)
    b = N.Batch(ctx)
    b.add(s)
    b.run(32, 0.0, 0.3, 0.16, exact=True)
    np.testing.assert_array_equal(bits(s.get_u()), bits(lone["u"]))
    # and alone again afterwards: the one-pass kernel, same result
    assert s.run(32, 0.0, 0.3, 0.16, exact=True, tile_config=FUSED) == 32
    np.testing.assert_array_equal(bits(s.get_u()), bits(lone["u"]))
    assert s.last_run_stats()[1] == 32
    b.close()
    s.close()


def test_fused_warm_start_and_multilevel_match_two_pass():
    """Warm starts (initial u/pt/ps and flows) and the multilevel chain read
    the state from the right parity."""
    from asetsmatlabmaxflow_gb300 import native as N

    dims, L = (128, 96), 5
    ct, alpha = _inputs("ishikawa", dims, L, 15)
    ctx = N.Context.default()
    out = {}
    for tc in (FUSED, TWO_PASS):
        s = N.Solver(ctx, "ishikawa", dims, L)
        s.set_inputs(ct, alpha)
        s.run(7, 0.0, 0.3, 0.16, exact=True, tile_config=tc)
        u0 = s.get_u()
        _, pt0 = s.get_flows()
        bx, by, _ = s.get_spatial_flows()
        s.set_initial(u0=u0, pt0=pt0)
        s.set_initial_flows(bx=bx, by=by)
        s.run(9, 0.0, 0.3, 0.16, exact=True, tile_config=tc)
        warm = s.get_u()
        s.set_initial()
        it = s.run_multilevel(3, 50, 0.0, 0.3, 0.16, exact=True, tile_config=tc)
        out[tc] = (warm, s.get_u(), it)
        s.close()
    np.testing.assert_array_equal(bits(out[FUSED][0]), bits(out[TWO_PASS][0]))
    np.testing.assert_array_equal(bits(out[FUSED][1]), bits(out[TWO_PASS][1]))
    assert out[FUSED][2] == out[TWO_PASS][2]
