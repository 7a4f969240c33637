"""GPU parity of the binary 2D square-tile kernels (stencil2d_tile.cuh): one
whole iteration of a 32 x 32 or 16 x 16 tile per block, for small images,
one launch per iteration or every iteration in one cooperative launch.

They are selected with tile_config 6-9 (fast) and 5-8 (EXACT), after the
sweep variants: 32 x 32, 16 x 16, then the same as whole-solve launches.
EXACT results must be bit-identical to the oracle and to the sweep kernel
(u, ps, pt and the spatial flows), the fast build meets the parity bar,
stopping runs stop where the oracle stops, a batch of small images runs
the per-iteration form, and the whole-solve form takes several tiles per
block when they cannot all be resident."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_helpers import assert_parity_bar, bits, require_gpu

pytestmark = pytest.mark.gpu

TILE_FAST = (6, 7, 8, 9)
TILE_EXACT = (5, 6, 7, 8)
SWEEP = 1


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()


def _inputs(dims, seed):
    from scipy.ndimage import gaussian_filter

    g = np.random.default_rng(seed)
    sm = lambda: np.asfortranarray(gaussian_filter(g.random(dims), 1.2).astype(np.float32))  # noqa: E731
    return dict(Cs=sm(), Ct=sm(), alpha=np.asfortranarray((0.1 + 0.6 * g.random(dims)).astype(np.float32)))


def _solve(dims, inp, max_it, eb, exact, tc, cc=0.3, steps=0.16):
    from asetsmatlabmaxflow_gb300 import native as N

    s = N.Solver(N.Context.default(), "binary", dims)
    s.set_inputs(inp["Ct"], inp["alpha"], inp["Cs"])
    it = s.run(max_it, eb, cc, steps, exact=exact, tile_config=tc)
    u = s.get_u()
    ps, pt = s.get_flows()
    bx, by, _ = s.get_spatial_flows()
    out = dict(it=it, u=u, ps=ps, pt=pt, bx=bx, by=by, cvg=s.get_cvg())
    s.close()
    return out


# odd sizes, a single row or column, smaller than one tile, exact multiples
SHAPES = [(301, 170), (7, 33), (1, 9), (33, 1), (100, 257), (64, 64), (17, 16)]


@pytest.mark.parametrize("dims", SHAPES)
@pytest.mark.parametrize("tc", TILE_EXACT)
def test_exact_tile_is_bit_identical_to_oracle_and_sweep(dims, tc):
    inp = _inputs(dims, 21)
    max_it = 13  # odd: the result is in the second parity
    ref = O.solve("binary", dims, inp["Ct"], inp["alpha"], cs=inp["Cs"], max_it=max_it,
                  err_bound=0.0, cc=0.3, steps=0.16, want_state=True)
    t = _solve(dims, inp, max_it, 0.0, True, tc)
    w = _solve(dims, inp, max_it, 0.0, True, SWEEP)
    assert t["it"] == ref["it"] == max_it
    np.testing.assert_array_equal(bits(t["u"]), bits(ref["u"]))
    np.testing.assert_array_equal(bits(t["ps"]), bits(ref["ps"]))
    np.testing.assert_array_equal(bits(t["pt"]), bits(ref["pt"]))
    for k in ("u", "ps", "pt", "bx", "by"):
        np.testing.assert_array_equal(bits(t[k]), bits(w[k]), err_msg=k)
    np.testing.assert_allclose(t["cvg"], ref["cvg"], rtol=2e-5, atol=1e-12)


@pytest.mark.parametrize("dims", SHAPES)
@pytest.mark.parametrize("tc", TILE_FAST)
def test_fast_tile_meets_parity_bar(dims, tc):
    inp = _inputs(dims, 22)
    max_it = 60
    ref = O.solve("binary", dims, inp["Ct"], inp["alpha"], cs=inp["Cs"], max_it=max_it,
                  err_bound=0.0, cc=0.3, steps=0.16, erru_double=True)
    t = _solve(dims, inp, max_it, 0.0, False, tc)
    assert t["it"] == max_it
    assert_parity_bar("binary", dims, 1, t["u"].reshape(dims, order="F"),
                      ref["u"].reshape(dims, order="F"), t["cvg"], ref["cvg"])


@pytest.mark.parametrize("exact", [True, False])
@pytest.mark.parametrize("k", [0, 1, 2, 3])
def test_tile_stops_where_the_oracle_stops(exact, k):
    dims = (256, 256)
    inp = _inputs(dims, 23)
    free = O.solve("binary", dims, inp["Ct"], inp["alpha"], cs=inp["Cs"], max_it=400,
                   err_bound=0.0, cc=0.3, steps=0.16)
    # errBound just below every erriter of the first 120 iterations, and
    # clear of every erriter (1e-3 relative) so that rounding cannot move
    # the stop
    eb = float(np.min(free["cvg"][:120])) * 0.99
    ref = O.solve("binary", dims, inp["Ct"], inp["alpha"], cs=inp["Cs"], max_it=400,
                  err_bound=eb, cc=0.3, steps=0.16)
    assert 120 <= ref["it"] < 400
    if np.any(np.abs(free["cvg"][:ref["it"] + 1] / eb - 1.0) < 1e-3):
        pytest.skip("an erriter lies within rounding of errBound")
    t = _solve(dims, inp, 400, eb, exact, TILE_EXACT[k] if exact else TILE_FAST[k])
    assert t["it"] == ref["it"]
    if exact:
        np.testing.assert_array_equal(bits(t["u"]), bits(ref["u"]))


def test_batch_of_small_images_with_square_tiles():
    """A batch of small binary 2D images run with the 32 x 32 tile variant
    (the batch's 2D group variant) gives each member its lone EXACT result."""
    from asetsmatlabmaxflow_gb300 import native as N

    ctx = N.Context.default()
    shapes = [(96, 80), (130, 45), (64, 64), (200, 150)]
    solvers, lone = [], []
    for i, dims in enumerate(shapes):
        inp = _inputs(dims, 30 + i)
        lone.append(_solve(dims, inp, 300, 1e-4, True, SWEEP))
        s = N.Solver(ctx, "binary", dims)
        s.set_inputs(inp["Ct"], inp["alpha"], inp["Cs"])
        solvers.append(s)
    b = N.Batch(ctx)
    for s in solvers:
        b.add(s)
    its = b.run(300, 1e-4, 0.3, 0.16, exact=True, tile_config=TILE_EXACT[0])
    for s, ref, it in zip(solvers, lone, its):
        assert it == ref["it"]
        np.testing.assert_array_equal(bits(s.get_u()), bits(ref["u"]))
    b.close()
    for s in solvers:
        s.close()


@pytest.mark.parametrize("tc", TILE_EXACT[2:])
def test_whole_solve_launch_edges(tc):
    """maxIt 0 and 1, a warm start continued from a saved state (the second
    run equals an uninterrupted one), all in one cooperative launch each."""
    from asetsmatlabmaxflow_gb300 import native as N

    dims = (97, 83)
    inp = _inputs(dims, 40)
    ref = O.solve("binary", dims, inp["Ct"], inp["alpha"], cs=inp["Cs"], max_it=20,
                  err_bound=0.0, cc=0.3, steps=0.16)
    s = N.Solver(N.Context.default(), "binary", dims)
    s.set_inputs(inp["Ct"], inp["alpha"], inp["Cs"])
    assert s.run(0, 0.0, 0.3, 0.16, exact=True, tile_config=tc) == 0
    assert s.last_run_stats()[1] == 0
    assert s.run(1, 0.0, 0.3, 0.16, exact=True, tile_config=tc) == 1
    assert s.last_run_stats()[1] == 1
    s.run(12, 0.0, 0.3, 0.16, exact=True, tile_config=tc)
    u = s.get_u()
    ps, pt = s.get_flows()
    bx, by, _ = s.get_spatial_flows()
    s.set_initial(u0=u, ps0=ps, pt0=pt)
    s.set_initial_flows(bx=bx, by=by)
    assert s.run(8, 0.0, 0.3, 0.16, exact=True, tile_config=tc) == 8
    np.testing.assert_array_equal(bits(s.get_u()), bits(ref["u"]))
    s.close()


@pytest.mark.parametrize("tc", TILE_EXACT[2:])
def test_whole_solve_launch_with_more_tiles_than_blocks(tc):
    """1024 x 1000 in 16 x 16 or 32 x 32 tiles is more tiles than can be
    resident at once: each block takes several per iteration, with the same
    EXACT result as the sweep, in one launch."""
    dims = (1024, 1000)
    inp = _inputs(dims, 43)
    t = _solve(dims, inp, 11, 0.0, True, tc)
    w = _solve(dims, inp, 11, 0.0, True, SWEEP)
    assert t["it"] == w["it"] == 11
    for k in ("u", "ps", "pt", "bx", "by"):
        np.testing.assert_array_equal(bits(t[k]), bits(w[k]), err_msg=k)
    np.testing.assert_allclose(t["cvg"], w["cvg"], rtol=2e-5, atol=1e-12)


@pytest.mark.parametrize("dims,exact,launches", [
    ((256, 256), False, 1), ((301, 170), False, 1), ((512, 512), False, 1), ((1024, 1024), False, 16),
    ((1024, 1024), True, 1), ((2048, 2048), True, 32)])
def test_default_whole_solve_on_small_images(dims, exact, launches):
    """Without a tile_config a binary 2D image whose tiles can all be
    resident runs as one cooperative launch (EXACT: up to eight tiles per
    block); a larger one keeps the sweep (16 iterations per CUDA-graph
    chunk: fast two per launch, EXACT one)."""
    from asetsmatlabmaxflow_gb300 import native as N

    inp = _inputs(dims, 42)
    s = N.Solver(N.Context.default(), "binary", dims)
    s.set_inputs(inp["Ct"], inp["alpha"], inp["Cs"])
    assert s.run(20, 0.0, 0.3, 0.16, exact=exact) == 20
    assert s.last_run_stats()[1] == launches
    s.close()
