"""Batched solver: every member must come out exactly as when solved alone
(same itNum, bit-identical u in EXACT mode, erriter up to summation order),
while problems of different sizes and dimensions converge at different
iterations inside one batch."""
import numpy as np
import pytest

from tests.gpu_helpers import bits, require_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()


def _problems():
    from asetsmatlabmaxflow_gb300 import synth

    out = []
    g = np.random.default_rng(5)
    for i, shape in enumerate([(131, 77), (64, 200), (250, 256), (40, 33)]):
        cs, ct, _ = synth.binary2d(seed=40 + i, shape=shape)
        alpha = np.full(shape, g.uniform(0.2, 0.8), np.float32, order="F")
        out.append((shape, cs, ct, alpha))
    for i, shape in enumerate([(64, 70, 66), (90, 64, 75), (33, 41, 29)]):
        cs, ct, _ = synth.binary3d(seed=60 + i, shape=shape, ncells=10)
        alpha = np.full(shape, g.uniform(0.2, 0.8), np.float32, order="F")
        out.append((shape, cs, ct, alpha))
    return out


@pytest.mark.parametrize("exact", [True, False])
def test_batch_members_equal_individual_solves(exact):
    from asetsmatlabmaxflow_gb300 import native as N

    ctx = N.Context.default()
    probs = _problems()
    max_it, err_bound = 400, 1e-4
    solvers = []
    ref = []
    for shape, cs, ct, alpha in probs:
        s = N.Solver(ctx, "binary", shape)
        s.set_inputs(ct, alpha, cs)
        cc, steps = (0.3, 0.16) if len(shape) == 2 else (0.35, 0.11)
        it = s.run(max_it, err_bound, 0.3, 0.11, exact=exact)
        ref.append((it, s.get_u().copy(), s.get_cvg()[:it + 1].copy()))
        solvers.append(s)
    b = N.Batch(ctx)
    for s in solvers:
        b.add(s)
    its = b.run(max_it, err_bound, 0.3, 0.11, exact=exact)
    assert len(set(its)) > 1  # members converge at different iterations
    for s, it, (it_ref, u_ref, cvg_ref) in zip(solvers, its, ref):
        assert it == it_ref
        u = s.get_u()
        if exact:
            np.testing.assert_array_equal(bits(u), bits(u_ref))
        else:
            assert float(np.max(np.abs(u - u_ref))) <= 1e-5
        np.testing.assert_allclose(s.get_cvg()[:it + 1], cvg_ref, rtol=1e-5)
    st = b.last_run_stats()
    assert st["iterations"] == sum(min(i + 1, max_it) for i in its)
    b.close()
    for s in solvers:
        s.close()


def test_batch_autotune_and_repeat_are_deterministic():
    from asetsmatlabmaxflow_gb300 import native as N

    ctx = N.Context.default()
    solvers = []
    for shape, cs, ct, alpha in _problems()[:5]:
        s = N.Solver(ctx, "binary", shape)
        s.set_inputs(ct, alpha, cs)
        solvers.append(s)
    b = N.Batch(ctx)
    for s in solvers:
        b.add(s)
    its1 = b.run(150, 1e-4, 0.3, 0.11, autotune=True)
    u1 = [s.get_u().copy() for s in solvers]
    st = b.last_run_stats()
    assert st["tile_config_2d"] >= 1 and st["tile_config_3d"] >= 1
    its2 = b.run(150, 1e-4, 0.3, 0.11, autotune=True)  # cached choice
    assert its1 == its2
    for s, u in zip(solvers, u1):
        np.testing.assert_array_equal(bits(s.get_u()), bits(u))
    b.close()


def _labelled_problems():
    """Potts and Ishikawa members of uneven sizes, 2D and 3D, with the
    parameters of the multi-region configurations."""
    from scipy.ndimage import gaussian_filter

    g = np.random.default_rng(21)
    out = []
    for model, dims, L in [("potts", (97, 130), 4), ("potts", (40, 36, 28), 5),
                           ("ishikawa", (120, 88), 6), ("ishikawa", (30, 34, 26), 4),
                           ("potts", (64, 48, 40), 3)]:
        ct = np.asfortranarray(gaussian_filter(g.random(dims + (L,)), 1.5).astype(np.float32))
        la = L if model == "potts" else L - 1
        alpha = np.asfortranarray((0.1 + 0.3 * g.random(dims + (la,))).astype(np.float32))
        out.append((model, dims, L, ct, alpha))
    return out


@pytest.mark.parametrize("exact", [True, False])
def test_mixed_batch_with_labelled_members_equals_individual_solves(exact):
    """Potts and Ishikawa problems (2D and 3D) batched with binary ones:
    every member as when solved alone -- same itNum, u bit-identical in
    EXACT mode -- while they converge at different iterations."""
    from asetsmatlabmaxflow_gb300 import native as N

    ctx = N.Context.default()
    max_it, err_bound, cc, steps = 300, 2e-4, 0.3, 0.11
    members = []
    for model, dims, L, ct, alpha in _labelled_problems():
        s = N.Solver(ctx, model, dims, L)
        s.set_inputs(ct, alpha)
        members.append(s)
    for shape, cs, ct, alpha in _problems()[:2] + _problems()[4:5]:
        s = N.Solver(ctx, "binary", shape)
        s.set_inputs(ct, alpha, cs)
        members.append(s)
    ref = []
    for s in members:
        it = s.run(max_it, err_bound, cc, steps, exact=exact)
        ref.append((it, s.get_u().copy(), s.get_cvg()[:it + 1].copy()))
    b = N.Batch(ctx)
    for s in members:
        b.add(s)
    its = b.run(max_it, err_bound, cc, steps, exact=exact)
    assert len(set(its)) > 2
    for s, it, (it_ref, u_ref, cvg_ref) in zip(members, its, ref):
        assert it == it_ref
        u = s.get_u()
        if exact:
            np.testing.assert_array_equal(bits(u), bits(u_ref))
        else:
            assert float(np.max(np.abs(u - u_ref))) <= 1e-5
        np.testing.assert_allclose(s.get_cvg()[:it + 1], cvg_ref, rtol=1e-5)
    st = b.last_run_stats()
    assert st["iterations"] == sum(min(i + 1, max_it) for i in its)
    b.close()
    for s in members:
        s.close()


@pytest.mark.parametrize("tile_config", [0, 2])
def test_member_solved_alone_after_a_batch(tile_config):
    """A member keeps its own single-solve layout through a batch run: solved
    alone afterwards (with the batch's kernel variant, or another one) it
    gives exactly what the batch gave it."""
    from asetsmatlabmaxflow_gb300 import native as N

    ctx = N.Context.default()
    solvers = []
    for shape, cs, ct, alpha in _problems():
        s = N.Solver(ctx, "binary", shape)
        s.set_inputs(ct, alpha, cs)
        solvers.append(s)
    b = N.Batch(ctx)
    for s in solvers:
        b.add(s)
    its = b.run(300, 1e-4, 0.3, 0.11, exact=True)
    got = [s.get_u().copy() for s in solvers]
    for s, it, u in zip(solvers, its, got):
        assert s.run(300, 1e-4, 0.3, 0.11, exact=True, tile_config=tile_config) == it
        np.testing.assert_array_equal(bits(s.get_u()), bits(u))
    b.close()
    for s in solvers:
        s.close()
