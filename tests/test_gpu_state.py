"""Full iteration state (u, ps, pt and the spatial flows bx, by, bz) can be
saved after a run and restored: resuming from it reproduces an uninterrupted
run bit for bit (EXACT mode)."""
import numpy as np
import pytest

from tests.gpu_helpers import bits, require_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()


CASES = [
    ("binary", (37, 29, 11), 1, 0.35, 0.11),
    ("binary", (61, 45), 1, 0.3, 0.16),
    ("potts", (33, 20, 9), 4, 0.3, 0.11),
    ("potts", (50, 38), 3, 0.3, 0.16),
    ("ishikawa", (40, 27), 5, 0.3, 0.16),
    ("ishikawa", (21, 18, 10), 4, 0.3, 0.11),
]


def _inputs(model, dims, L, seed):
    g = np.random.default_rng(seed)
    n = int(np.prod(dims))
    if model == "binary":
        img = g.random(n).astype(np.float32)
        return dict(Cs=np.abs(img - 0.2).astype(np.float32), Ct=np.abs(img - 0.8).astype(np.float32),
                    alpha=(0.2 + 0.3 * g.random(n)).astype(np.float32))
    ct = g.random(n * L).astype(np.float32)
    al = L if model == "potts" else L - 1
    return dict(Cs=None, Ct=ct, alpha=(0.1 + 0.3 * g.random(n * al)).astype(np.float32))


@pytest.mark.parametrize("model,dims,L,cc,steps", CASES)
def test_resume_from_saved_state_is_bit_identical(model, dims, L, cc, steps):
    from asetsmatlabmaxflow_gb300 import native as N

    ctx = N.Context.default()
    inp = _inputs(model, dims, L, 5)
    k, m = 9, 14
    a = N.Solver(ctx, model, dims, L)
    a.set_inputs(inp["Ct"], inp["alpha"], inp["Cs"])
    a.run(k + m, 0.0, cc, steps, exact=True)
    u_full = a.get_u()
    ps_full, pt_full = a.get_flows()
    cvg_full = a.get_cvg(k + m)

    b = N.Solver(ctx, model, dims, L)
    b.set_inputs(inp["Ct"], inp["alpha"], inp["Cs"])
    b.run(k, 0.0, cc, steps, exact=True)
    u, (ps, pt), fl = b.get_u(), b.get_flows(), b.get_spatial_flows()
    assert all(np.all(np.isfinite(f)) for f in fl if f is not None)
    c = N.Solver(ctx, model, dims, L)
    c.set_inputs(inp["Ct"], inp["alpha"], inp["Cs"])
    c.set_initial(u, ps, pt)
    c.set_initial_flows(*fl)
    c.run(m, 0.0, cc, steps, exact=True)
    assert np.array_equal(bits(c.get_u()), bits(u_full))
    ps2, pt2 = c.get_flows()
    assert np.array_equal(bits(pt2), bits(pt_full))
    if ps2 is not None:
        assert np.array_equal(bits(ps2), bits(ps_full))
    assert np.array_equal(bits(c.get_cvg(m)), bits(cvg_full[k:]))
    # clearing returns to the cold start
    c.set_initial(None, None, None)
    c.run(k + m, 0.0, cc, steps, exact=True)
    assert np.array_equal(bits(c.get_u()), bits(u_full))
    for s in (a, b, c):
        s.close()


def test_border_faces_are_ignored():
    from asetsmatlabmaxflow_gb300 import native as N

    ctx = N.Context.default()
    dims, L = (24, 17, 6), 3
    inp = _inputs("potts", dims, L, 2)
    s = N.Solver(ctx, "potts", dims, L)
    s.set_inputs(inp["Ct"], inp["alpha"])
    s.run(5, 0.0, 0.3, 0.11, exact=True)
    u, (ps, pt), (bx, by, bz) = s.get_u(), s.get_flows(), s.get_spatial_flows()
    # flows at index 0 of each axis are border faces: always zero after a run
    ny, nx, nz = dims
    for f, ax in ((bx, 1), (by, 0), (bz, 2)):
        v = f.reshape((ny, nx, nz, L), order="F")
        assert not np.any(np.take(v, 0, axis=ax))
    ref = N.Solver(ctx, "potts", dims, L)
    ref.set_inputs(inp["Ct"], inp["alpha"])
    ref.set_initial(u, ps, pt)
    ref.set_initial_flows(bx, by, bz)
    ref.run(4, 0.0, 0.3, 0.11, exact=True)
    junk = [f.reshape((ny, nx, nz, L), order="F").copy() for f in (bx, by, bz)]
    junk[0][:, 0] = 7.0
    junk[1][0] = -3.0
    junk[2][:, :, 0] = 5.0
    s.set_initial(u, ps, pt)
    s.set_initial_flows(*[j.ravel(order="F") for j in junk])
    s.run(4, 0.0, 0.3, 0.11, exact=True)
    assert np.array_equal(bits(s.get_u()), bits(ref.get_u()))
    s.close()
    ref.close()


@pytest.mark.parametrize("model,dims,L", [("binary", (70, 52, 33), 1), ("potts", (40, 44, 30), 4),
                                          ("ishikawa", (130, 90), 5)])
def test_autotuned_solve_equals_default(model, dims, L):
    """ASETS_FLAG_AUTOTUNE on a single solve: the variants are timed from
    the problem's initial state, then the solve runs with the fastest --
    EXACT results bit-identical to the default variant's, fast results to
    the parity tolerance; a second call reuses the cached choice."""
    from asetsmatlabmaxflow_gb300 import native as N
    from tests.gpu_helpers import bits

    g = np.random.default_rng(3)
    n = int(np.prod(dims))
    ct = g.random(n * L).astype(np.float32)
    la = 1 if model == "binary" else (L if model == "potts" else L - 1)
    alpha = (0.1 + 0.3 * g.random(n * la)).astype(np.float32)
    cs = g.random(n).astype(np.float32) if model == "binary" else None
    steps = 0.11 if len(dims) == 3 else 0.16
    s = N.Solver(N.Context.default(), model, dims, L)
    s.set_inputs(ct, alpha, cs)
    for exact in (True, False):
        it0 = s.run(120, 1e-4, 0.3, steps, exact=exact)
        u0 = s.get_u().copy()
        for _ in range(2):
            it1 = s.run(120, 1e-4, 0.3, steps, exact=exact, autotune=True)
            u1 = s.get_u()
            if exact:
                assert it1 == it0
                np.testing.assert_array_equal(bits(u1), bits(u0))
            else:
                assert abs(it1 - it0) <= 1
                assert float(np.max(np.abs(u1 - u0))) <= 1e-3
    s.close()
