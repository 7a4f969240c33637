"""Multilevel (coarse-to-fine) solve: the grid transfers against the numpy
restatement (oracle/multilevel.py), bit for bit through EXACT-mode solves,
and the reduction of fine-grid iterations to errBound."""
import numpy as np
import pytest

from oracle import multilevel as M
from tests.gpu_helpers import bits, require_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()


CASES = [
    ("binary", (37, 29, 11), 1),
    ("binary", (61, 45), 1),
    ("potts", (33, 20, 9), 4),
    ("potts", (50, 38), 3),
    ("ishikawa", (40, 27), 5),
    ("ishikawa", (21, 18, 10), 4),
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


@pytest.mark.parametrize("model,dims,L", CASES)
def test_two_level_solve_equals_oracle_transfer(model, dims, L):
    from asetsmatlabmaxflow_gb300 import native as N

    ctx = N.Context.default()
    dim = len(dims)
    inp = _inputs(model, dims, L, 4)
    k, cc, steps = 7, 0.3, (0.11 if dim == 3 else 0.16)
    ml = N.Solver(ctx, model, dims, L)
    ml.set_inputs(inp["Ct"], inp["alpha"], inp["Cs"])
    ml.run_multilevel(2, k, 0.0, cc, steps, exact=True)
    its, _ = ml.multilevel_stats()
    assert its == [k, k]

    cd = M.coarse_dims(dims, dim)[:dim]
    co = N.Solver(ctx, model, cd, L)
    rs = lambda a, sc: None if a is None else M.restrict(a, dims, dim, sc)  # noqa: E731
    co.set_inputs(rs(inp["Ct"], 2.0), rs(inp["alpha"], 1.0), rs(inp["Cs"], 2.0))
    co.run(k, 0.0, cc, steps, exact=True)
    u, (ps, pt), fl = co.get_u(), co.get_flows(), co.get_spatial_flows()
    fine = N.Solver(ctx, model, dims, L)
    fine.set_inputs(inp["Ct"], inp["alpha"], inp["Cs"])
    pr = lambda a, sc=1.0, ax=None: M.prolong(a, cd, dims, dim, sc, ax)  # noqa: E731
    fine.set_initial(pr(u), None if ps is None else pr(ps, 0.5), pr(pt, 0.5))
    fine.set_initial_flows(*[pr(f, 1.0, ax) for f, ax in zip(fl, M.flow_axes(dim))])
    fine.run(k, 0.0, cc, steps, exact=True)
    assert np.array_equal(bits(ml.get_u()), bits(fine.get_u()))
    assert np.array_equal(bits(ml.get_cvg(k)), bits(fine.get_cvg(k)))
    _, ct_c, al_c = ml.level(1).get_inputs()
    assert np.array_equal(bits(ct_c), bits(rs(inp["Ct"], 2.0)))
    assert np.array_equal(bits(al_c), bits(rs(inp["alpha"], 1.0)))
    # the coarse level's own result is the oracle-restricted problem's
    assert np.array_equal(bits(ml.level(1).get_u()), bits(u))
    for s in (ml, co, fine):
        s.close()


def test_multilevel_needs_fewer_fine_iterations():
    from asetsmatlabmaxflow_gb300 import native as N, synth

    ctx = N.Context.default()
    ct, a = synth.potts3d(seed=3, shape=(64, 64, 64))
    L = ct.shape[-1]
    s = N.Solver(ctx, "potts", (64, 64, 64), L)
    s.set_inputs(ct, a)
    cold = s.run(3000, 1e-4, 0.3, 0.11)
    assert cold < 3000
    it = s.run_multilevel(3, 3000, 1e-4, 0.3, 0.11)
    its, _ = s.multilevel_stats()
    assert len(its) == 3 and its[0] == it
    assert all(i < 3000 for i in its)
    assert it < 0.75 * cold, (it, cold)
    # the coarsest level accepts an initial state through its handle
    top = s.level(2)
    assert (top.ny, top.nx, top.nz) == (16, 16, 16)
    s.close()


def test_level_handles_and_limits():
    from asetsmatlabmaxflow_gb300 import native as N

    ctx = N.Context.default()
    s = N.Solver(ctx, "binary", (20, 9, 40), 1)
    inp = _inputs("binary", (20, 9, 40), 1, 1)
    s.set_inputs(inp["Ct"], inp["alpha"], inp["Cs"])
    # 9 -> 5 -> 3 (< 4 cells): two levels at most
    assert s.multilevel_prepare(5) == 2
    with pytest.raises(N.AsetsError):
        s.level(2)
    s.close()


@pytest.mark.parametrize("exact", [True, False])
def test_batched_multilevel_equals_individual_multilevel(exact):
    """asets_batch_run_multilevel: members of uneven sizes (so with different
    level counts), Potts, Ishikawa and binary, 2D and 3D, solved level by
    level as batches, come out as their own multilevel solves -- the same
    itNum at every level, u bit-identical in EXACT mode."""
    from asetsmatlabmaxflow_gb300 import native as N

    ctx = N.Context.default()
    members = [("potts", (72, 64, 40), 4), ("potts", (33, 20, 9), 3), ("ishikawa", (90, 70), 5),
               ("binary", (96, 80, 48), 1), ("potts", (120, 100), 3)]
    levels, max_it, err = 3, 400, 1e-4
    solvers, ref = [], []
    for j, (model, dims, L) in enumerate(members):
        inp = _inputs(model, dims, L, 30 + j)
        steps = 0.11 if len(dims) == 3 else 0.16
        s = N.Solver(ctx, model, dims, L)
        s.set_inputs(inp["Ct"], inp["alpha"], inp["Cs"])
        # one cc and steps for the batch: the 3D value for all
        it = s.run_multilevel(levels, max_it, err, 0.3, 0.11, exact=exact)
        ref.append((it, s.multilevel_stats()[0], s.get_u().copy()))
        solvers.append(s)
    assert len({len(r[1]) for r in ref}) > 1  # members have different level counts
    b = N.Batch(ctx)
    for s in solvers:
        b.add(s)
    its = b.run_multilevel(levels, max_it, err, 0.3, 0.11, exact=exact)
    for s, it, (it_ref, lv_ref, u_ref) in zip(solvers, its, ref):
        assert it == it_ref
        assert s.multilevel_stats()[0] == lv_ref
        if exact:
            np.testing.assert_array_equal(bits(s.get_u()), bits(u_ref))
        else:
            assert float(np.max(np.abs(s.get_u() - u_ref))) <= 1e-5
    b.close()
    for s in solvers:
        s.close()
