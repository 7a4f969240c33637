"""The binary 2D kernel with two ALM iterations per pass (temporal
blocking, csrc/stencil2d_t2.cuh; the fast default), against the oracle:
EXACT u bit-identical to the reference's arithmetic, fast mode to the parity
bar; odd and single-row shapes, columns below one tile; solves that stop at
the first iteration of a pass (errBound met there, odd maxIt), which re-run
that iteration alone; batches."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_helpers import assert_parity_bar, bits, require_gpu

pytestmark = pytest.mark.gpu

# positions (tile_config, 1-based) of the two-iteration variant in the
# binary 2D variant tables (csrc/binary2d_fast.cu, binary2d_exact.cu)
FAST_T2, EXACT_T2 = 1, 4


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


@pytest.mark.parametrize("dims", [(301, 170), (130, 90), (1, 9)])
def test_stopping_inside_a_pass_matches_oracle(dims):
    """errBound 1e-4 (the solve stops at whichever iteration meets it, the
    first or the second of a pass) and odd maxIt (the last pass runs one
    iteration too many): itNum, u (EXACT: bit-identical) and erriter as the
    oracle's, and the spatial flows as the one-iteration kernel's."""
    from asetsmatlabmaxflow_gb300 import native as N

    cs, ct, alpha = _rand(dims, 23)
    cc, steps = 0.3, 0.16
    s = N.Solver(N.Context.default(), "binary", dims)
    s.set_inputs(ct, alpha, cs)
    for max_it, eb in [(400, 1e-4), (401, 1e-4), (27, 0.0), (1, 0.0), (3, 0.0)]:
        ref = O.solve("binary", dims, ct, alpha, cs=cs, max_it=max_it, err_bound=eb, cc=cc,
                      steps=steps, erru_double=True)
        it = s.run(max_it, eb, cc, steps, exact=True, tile_config=EXACT_T2)
        assert it == ref["it"], (max_it, eb)
        n = min(it + 1, max_it)
        np.testing.assert_array_equal(bits(s.get_u()), bits(ref["u"]))
        cvg = s.get_cvg()
        np.testing.assert_allclose(cvg[:n], ref["cvg"][:n], rtol=2e-5, atol=1e-12)
        assert np.all(cvg[n:] == 0)
        f2 = [a.copy() for a in s.get_spatial_flows() if a is not None]
        assert s.run(max_it, eb, cc, steps, exact=True) == it   # one iteration per pass
        for a, b in zip(f2, [a for a in s.get_spatial_flows() if a is not None]):
            np.testing.assert_array_equal(bits(a), bits(b))
        it_f = s.run(max_it, eb, cc, steps)   # the fast default
        if eb == 0.0:
            assert it_f == max_it
    s.close()


@pytest.mark.parametrize("exact", [True, False])
def test_batch_with_two_iterations_per_pass_equals_single_solves(exact):
    """2D members of a batch on the two-iteration kernel, 3D members on the
    one-iteration one, each converging at its own iteration (odd or even):
    every member as when solved alone with the same kernel."""
    from asetsmatlabmaxflow_gb300 import native as N
    from asetsmatlabmaxflow_gb300 import synth

    ctx = N.Context.default()
    probs = []
    for i, shape in enumerate([(131, 77), (250, 256), (40, 33), (300, 120)]):
        cs, ct, _ = synth.binary2d(seed=70 + i, shape=shape)
        probs.append((shape, cs, ct, np.full(shape, 0.3 + 0.1 * i, np.float32, order="F")))
    cs, ct, _ = synth.binary3d(seed=90, shape=(40, 36, 30), ncells=8)
    probs.append(((40, 36, 30), cs, ct, np.full((40, 36, 30), 0.4, np.float32, order="F")))
    tc2 = EXACT_T2 if exact else FAST_T2
    solvers, ref = [], []
    for shape, cs, ct, alpha in probs:
        s = N.Solver(ctx, "binary", shape)
        s.set_inputs(ct, alpha, cs)
        it = s.run(400, 1e-4, 0.3, 0.16, exact=exact, tile_config=tc2 if len(shape) == 2 else 1)
        ref.append((it, s.get_u().copy()))
        solvers.append(s)
    b = N.Batch(ctx)
    for s in solvers:
        b.add(s)
    its = b.run(400, 1e-4, 0.3, 0.16, exact=exact, tile_config=tc2)
    assert len({i % 2 for i in its}) == 2 or len(set(its)) > 1
    for s, it, (it_ref, u_ref) in zip(solvers, its, ref):
        assert it == it_ref
        if exact:
            np.testing.assert_array_equal(bits(s.get_u()), bits(u_ref))
        else:
            assert float(np.max(np.abs(s.get_u() - u_ref))) <= 1e-5
    b.close()
    for s in solvers:
        s.close()
