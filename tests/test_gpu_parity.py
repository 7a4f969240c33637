"""GPU parity: libasetscuda against the reference's golden vectors and the
oracle, through the C ABI (Python mirror of the mex functions) and through
the compiled drop-in mex files."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import golden_cases as G
from tests.gpu_helpers import assert_parity_bar, bits, require_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()


def _run_golden(case, exact, dropin=False):
    from asetsmatlabmaxflow_gb300 import solvers as S

    fn = S.mex_dropin(case["solver"]) if dropin else getattr(S, case["solver"])
    kw = {} if dropin else {"exact": exact}
    if case["model"] == "binary":
        return fn(case["Cs"], case["Ct"], case["alpha"], case["pars"], **kw)
    return fn(case["Ct"], case["alpha"], case["pars"], **kw)


@pytest.mark.parametrize("name", G.names())
def test_exact_mode_is_bit_identical_to_reference(name):
    case = G.load(name)
    u, cvg, it, timet = _run_golden(case, exact=True)
    assert int(it.ravel()[0]) == case["it"]
    assert u.shape == case["u"].shape
    np.testing.assert_array_equal(bits(u), bits(case["u"]))
    n = min(case["it"] + 1, case["max_it"])
    # erriter: same terms, parallel summation order
    np.testing.assert_allclose(cvg.ravel()[:n], case["cvg"][:n], rtol=2e-5, atol=1e-12)
    assert np.all(cvg.ravel()[n:] == 0)
    assert timet.dtype == np.float32 and it.dtype == np.uint16


@pytest.mark.parametrize("name", G.names())
def test_fast_mode_meets_parity_bar(name):
    case = G.load(name)
    u, cvg, it, _ = _run_golden(case, exact=False)
    assert int(it.ravel()[0]) == case["it"]
    n = min(case["it"] + 1, case["max_it"])
    assert_parity_bar(case["model"], case["dims"], case["nlab"], u, case["u"], cvg, case["cvg"], it=n)


@pytest.mark.parametrize("name", ["binary2d_reftest", "binary3d_odd", "potts2d_odd",
                                  "potts3d_conv", "ishikawa2d_conv", "ishikawa3d_odd"])
def test_dropin_mex_file_matches_reference(name):
    """The compiled GPU mex file, called through mexFunction like Matlab."""
    from asetsmatlabmaxflow_gb300.mexhost import MexFunction

    case = G.load(name)
    u, cvg, it, timet = _run_golden(case, exact=False, dropin=True)
    assert int(it.ravel()[0]) == case["it"]
    assert u.shape == case["u"].shape and cvg.shape == (case["max_it"], 1)
    assert it.dtype == np.uint16 and timet.dtype == np.float32 and timet.ravel()[0] > 0
    n = min(case["it"] + 1, case["max_it"])
    assert_parity_bar(case["model"], case["dims"], case["nlab"], u, case["u"], cvg, case["cvg"], it=n)
    assert "number of iterations" in MexFunction.last_print()


@pytest.mark.parametrize("dropin", [False, True])
def test_alpha_not_positive_raises_reference_message(dropin):
    from asetsmatlabmaxflow_gb300 import solvers as S
    from asetsmatlabmaxflow_gb300.mexhost import MexError

    case = G.load("binary3d_357")
    alpha = case["alpha"].copy()
    alpha[1, 2, 3] = 0.0
    fn = S.mex_dropin("asetsBinaryMF3D_mex") if dropin else S.asetsBinaryMF3D_mex
    with pytest.raises(MexError, match=r"alpha\(x\) must be positive. Exiting\.\.\."):
        fn(case["Cs"], case["Ct"], alpha, case["pars"])
    c2 = G.load("potts2d_ties")
    a2 = c2["alpha"].copy()
    a2[0, 0, 2] = -1.0
    fn2 = S.mex_dropin("asetsPotts2D_mex") if dropin else S.asetsPotts2D_mex
    with pytest.raises(MexError, match=r"alpha\(x,l\) must be positive"):
        fn2(c2["Ct"], a2, c2["pars"])
    # maxIt = 0 never reaches projStep: no error, init returned
    pars0 = case["pars"].copy()
    pars0[3] = 0
    u, cvg, it, _ = S.asetsBinaryMF3D_mex(case["Cs"], case["Ct"], alpha, pars0)
    assert int(it.ravel()[0]) == 0 and cvg.size == 0
    np.testing.assert_array_equal(u, (case["Cs"] - case["Ct"] >= 0).astype(np.float32))


# ------------------------------------------------------------------ oracle sizes

def _rand(model, dims, L, seed):
    from scipy.ndimage import gaussian_filter

    g = np.random.default_rng(seed)
    sm = lambda shp: np.asfortranarray(gaussian_filter(g.random(shp), 1.0).astype(np.float32))  # noqa: E731
    if model == "binary":
        return dict(Cs=sm(dims), Ct=sm(dims), alpha=(0.1 + 0.6 * g.random(dims)).astype(np.float32))
    la = L if model == "potts" else L - 1
    return dict(Ct=sm(dims + (L,)), alpha=(0.1 + 0.4 * g.random(dims + (la,))).astype(np.float32))


ORACLE_CASES = [
    ("binary", (200, 150), 1, 60, 0.3, 0.16),
    ("binary", (96, 80, 40), 1, 40, 0.35, 0.11),
    ("potts", (130, 97), 5, 40, 0.3, 0.16),
    ("potts", (48, 40, 20), 4, 30, 0.3, 0.11),
    ("ishikawa", (160, 120), 8, 40, 0.3, 0.16),
    ("ishikawa", (40, 33, 17), 4, 30, 0.3, 0.11),
]


@pytest.mark.parametrize("model,dims,L,maxit,cc,steps", ORACLE_CASES)
def test_against_oracle_at_larger_sizes(model, dims, L, maxit, cc, steps):
    from asetsmatlabmaxflow_gb300 import native as N

    inp = _rand(model, dims, L, 7)
    ref = O.solve(model, dims, inp["Ct"], inp["alpha"], cs=inp.get("Cs"), nlab=L, max_it=maxit,
                  err_bound=0.0, cc=cc, steps=steps)
    refd = O.solve(model, dims, inp["Ct"], inp["alpha"], cs=inp.get("Cs"), nlab=L, max_it=maxit,
                   err_bound=0.0, cc=cc, steps=steps, erru_double=True)
    s = N.Solver(N.Context.default(), model, dims, L)
    s.set_inputs(inp["Ct"], inp["alpha"], inp.get("Cs"))
    it = s.run(maxit, 0.0, cc, steps, exact=True)
    assert it == ref["it"]
    np.testing.assert_array_equal(bits(s.get_u()), bits(ref["u"]))
    np.testing.assert_allclose(s.get_cvg(), refd["cvg"], rtol=1e-5)
    it = s.run(maxit, 0.0, cc, steps, exact=False)
    u = s.get_u()
    shape = dims + ((L,) if model == "potts" else ((L - 1,) if model == "ishikawa" else ()))
    assert_parity_bar(model, dims, L, u.reshape(shape, order="F"),
                      ref["u"].reshape(shape, order="F"), s.get_cvg(), refd["cvg"])
    s.close()


def test_full_size_binary3d_first_iterations_match_oracle():
    """256^3 (the benchmark volume), a few iterations: u bit-exact in EXACT
    mode; erriter against the double-accumulating oracle (the reference's
    serial float sum drifts by ~1% at this size)."""
    from asetsmatlabmaxflow_gb300 import native as N
    from asetsmatlabmaxflow_gb300 import synth

    cs, ct, alpha = synth.binary3d(seed=3)
    dims = cs.shape
    refd = O.solve("binary", dims, ct, alpha, cs=cs, max_it=3, err_bound=0.0, cc=0.35,
                   steps=0.11, erru_double=True)
    s = N.Solver(N.Context.default(), "binary", dims)
    s.set_inputs(ct, alpha, cs)
    assert s.run(3, 0.0, 0.35, 0.11, exact=True) == 3
    np.testing.assert_array_equal(bits(s.get_u()), bits(refd["u"]))
    np.testing.assert_allclose(s.get_cvg(), refd["cvg"], rtol=1e-4)
    s.run(3, 0.0, 0.35, 0.11, exact=False)
    u = s.get_u()
    assert float(np.max(np.abs(u - refd["u"]))) <= 1e-3
    np.testing.assert_allclose(s.get_cvg(), refd["cvg"], rtol=1e-3)
    s.close()


def test_repeated_runs_are_deterministic_and_device_inputs_match():
    import torch

    from asetsmatlabmaxflow_gb300 import native as N

    inp = _rand("binary", (70, 66, 30), 1, 11)
    s = N.Solver(N.Context.default(), "binary", (70, 66, 30))
    s.set_inputs(inp["Ct"], inp["alpha"], inp["Cs"])
    s.run(25, 0.0, 0.3, 0.11)
    u1, c1 = s.get_u().copy(), s.get_cvg().copy()
    s.run(25, 0.0, 0.3, 0.11)
    np.testing.assert_array_equal(bits(s.get_u()), bits(u1))
    np.testing.assert_array_equal(bits(s.get_cvg()), bits(c1))
    dev = {k: torch.from_numpy(v.ravel(order="F").copy()).cuda() for k, v in inp.items()}
    torch.cuda.synchronize()
    s.set_inputs(dev["Ct"], dev["alpha"], dev["Cs"], where=N.DEVICE)
    s.run(25, 0.0, 0.3, 0.11)
    np.testing.assert_array_equal(bits(s.get_u()), bits(u1))
    out = torch.empty(70 * 66 * 30, dtype=torch.float32, device="cuda")
    s.get_u(out, where=N.DEVICE)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(bits(out.cpu().numpy()), bits(u1))
    s.close()


@pytest.mark.parametrize("model,dims,L", [("binary", (50, 40, 12), 1), ("potts", (60, 45), 3),
                                          ("ishikawa", (30, 28, 9), 4)])
def test_warm_start_matches_oracle_warm_start(model, dims, L):
    from asetsmatlabmaxflow_gb300 import native as N

    inp = _rand(model, dims, L, 21)
    kw = dict(cs=inp.get("Cs"), nlab=L, err_bound=0.0, cc=0.3, steps=0.11 if len(dims) == 3 else 0.16)
    first = O.solve(model, dims, inp["Ct"], inp["alpha"], max_it=15, want_state=True, **kw)
    cont = O.solve(model, dims, inp["Ct"], inp["alpha"], max_it=20, u0=first["u"],
                   ps0=first.get("ps"), pt0=first["pt"], **kw)
    s = N.Solver(N.Context.default(), model, dims, L)
    s.set_inputs(inp["Ct"], inp["alpha"], inp.get("Cs"))
    s.set_initial(first["u"], first.get("ps") if model != "ishikawa" else None, first["pt"])
    assert s.run(20, 0.0, kw["cc"], kw["steps"], exact=True) == cont["it"]
    np.testing.assert_array_equal(bits(s.get_u()), bits(cont["u"]))
    # the GPU's own final state continues the same way
    s.set_initial(None, None, None)
    s.run(15, 0.0, kw["cc"], kw["steps"], exact=True)
    ps, pt = s.get_flows()
    np.testing.assert_array_equal(bits(pt), bits(first["pt"]))
    if ps is not None:
        np.testing.assert_array_equal(bits(ps), bits(first["ps"]))
    s.close()


@pytest.mark.parametrize("tile_config", [1, 2, 3])
def test_every_binary3d_fast_variant_meets_parity_bar(tile_config):
    """Each compiled variant of the fast binary 3D kernel (28 x 28, 28 x 12
    and 28 x 8 tiles), selected explicitly, against the oracle."""
    from asetsmatlabmaxflow_gb300 import native as N

    model, dims, L, maxit, cc, steps = ORACLE_CASES[1]
    inp = _rand(model, dims, L, 9)
    ref = O.solve(model, dims, inp["Ct"], inp["alpha"], cs=inp["Cs"], nlab=L, max_it=maxit,
                  err_bound=0.0, cc=cc, steps=steps)
    refd = O.solve(model, dims, inp["Ct"], inp["alpha"], cs=inp["Cs"], nlab=L, max_it=maxit,
                   err_bound=0.0, cc=cc, steps=steps, erru_double=True)
    s = N.Solver(N.Context.default(), model, dims, L)
    s.set_inputs(inp["Ct"], inp["alpha"], inp["Cs"])
    s.run(maxit, 0.0, cc, steps, exact=False, tile_config=tile_config)
    assert_parity_bar(model, dims, L, s.get_u().reshape(dims, order="F"),
                      ref["u"].reshape(dims, order="F"), s.get_cvg(), refd["cvg"])
    s.close()


@pytest.mark.parametrize("dims", [(33, 41, 29), (61, 17, 9), (5, 7, 3), (121, 13, 6), (1, 9, 8)])
def test_odd_shapes_binary3d_against_oracle(dims):
    """Binary 3D volumes whose row count is odd, below one tile, or a single
    row: the default two-rows-per-thread kernel's last pair straddles the
    volume's end (one cell stored alone).  EXACT bit-exact, fast to the
    parity bar, both against the oracle."""
    from asetsmatlabmaxflow_gb300 import native as N

    inp = _rand("binary", dims, 1, 11)
    maxit, cc, steps = 30, 0.35, 0.11
    ref = O.solve("binary", dims, inp["Ct"], inp["alpha"], cs=inp["Cs"], max_it=maxit,
                  err_bound=0.0, cc=cc, steps=steps)
    refd = O.solve("binary", dims, inp["Ct"], inp["alpha"], cs=inp["Cs"], max_it=maxit,
                   err_bound=0.0, cc=cc, steps=steps, erru_double=True)
    s = N.Solver(N.Context.default(), "binary", dims)
    s.set_inputs(inp["Ct"], inp["alpha"], inp["Cs"])
    assert s.run(maxit, 0.0, cc, steps, exact=True) == ref["it"]
    np.testing.assert_array_equal(bits(s.get_u()), bits(ref["u"]))
    s.run(maxit, 0.0, cc, steps, exact=False)
    assert_parity_bar("binary", dims, 1, s.get_u().reshape(dims, order="F"),
                      ref["u"].reshape(dims, order="F"), s.get_cvg(), refd["cvg"])
    s.close()


@pytest.mark.parametrize("tile_config", [1, 2, 3, 4, 5, 6, 7, 8, 9])
def test_every_binary2d_fast_variant_meets_parity_bar(tile_config):
    """Each compiled variant of the fast binary 2D kernel (two iterations per
    pass with 224-row tiles; one per pass with 224- and 56-row tiles and two
    rows per thread with 240-row tiles and four or six stages; 32 x 32 and
    16 x 16 square tiles, per iteration and whole-solve), selected
    explicitly, against the oracle, on a
    column length that is not a multiple of any tile and is odd."""
    from asetsmatlabmaxflow_gb300 import native as N

    model, dims, L, maxit, cc, steps = "binary", (301, 170), 1, 60, 0.3, 0.16
    inp = _rand(model, dims, L, 13)
    ref = O.solve(model, dims, inp["Ct"], inp["alpha"], cs=inp["Cs"], nlab=L, max_it=maxit,
                  err_bound=0.0, cc=cc, steps=steps)
    refd = O.solve(model, dims, inp["Ct"], inp["alpha"], cs=inp["Cs"], nlab=L, max_it=maxit,
                   err_bound=0.0, cc=cc, steps=steps, erru_double=True)
    s = N.Solver(N.Context.default(), model, dims, L)
    s.set_inputs(inp["Ct"], inp["alpha"], inp["Cs"])
    s.run(maxit, 0.0, cc, steps, exact=False, tile_config=tile_config)
    assert_parity_bar(model, dims, L, s.get_u().reshape(dims, order="F"),
                      ref["u"].reshape(dims, order="F"), s.get_cvg(), refd["cvg"])
    s.close()
