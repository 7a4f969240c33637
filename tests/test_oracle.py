"""The oracle (C restatement) against the reference: golden vectors always,
the compiled reference mex solvers when the reference tree is present."""
import numpy as np
import pytest

from tests import golden_cases as G
from oracle import oracle as O


def _port(case, erru_double=False):
    return O.solve(case["model"], case["dims"], case["Ct"], case["alpha"], cs=case.get("Cs"),
                   nlab=case["nlab"], max_it=case["max_it"], err_bound=case["err_bound"],
                   cc=case["cc"], steps=case["steps"], erru_double=erru_double)


def _bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


@pytest.mark.parametrize("name", G.names())
def test_port_matches_golden_bit_exact(name):
    case = G.load(name)
    out = _port(case)
    assert out["it"] == case["it"]
    np.testing.assert_array_equal(_bits(out["u"]), _bits(case["u"].ravel(order="F")))
    np.testing.assert_array_equal(_bits(out["cvg"]), _bits(case["cvg"]))


@pytest.mark.parametrize("name", ["binary3d_odd", "potts3d_small", "ishikawa2d_reftest"])
def test_double_accumulated_erriter_is_close(name):
    case = G.load(name)
    f = _port(case)
    d = _port(case, erru_double=True)
    np.testing.assert_array_equal(_bits(f["u"]), _bits(d["u"]))
    n = min(f["it"], case["max_it"])
    np.testing.assert_allclose(d["cvg"][:n], f["cvg"][:n], rtol=1e-4)


needs_ref = pytest.mark.skipif(not O.reference_available() and not O._build.REF_SRC.is_dir(),
                               reason="reference sources not present on this machine")


def _rand_problem(model, dims, L, seed):
    g = np.random.default_rng(seed)
    if model == "binary":
        return dict(Cs=g.random(dims, dtype=np.float32), Ct=g.random(dims, dtype=np.float32),
                    alpha=(0.1 + g.random(dims)).astype(np.float32))
    la = L if model == "potts" else L - 1
    return dict(Ct=g.random(dims + (L,), dtype=np.float32),
                alpha=(0.1 + 0.5 * g.random(dims + (la,))).astype(np.float32))


SOLVERS = [("binary", (17, 12), 1), ("binary", (9, 11, 6), 1), ("potts", (15, 13), 5),
           ("potts", (8, 7, 5), 3), ("ishikawa", (16, 14), 4), ("ishikawa", (7, 9, 5), 3)]


@needs_ref
@pytest.mark.parametrize("model,dims,L", SOLVERS)
@pytest.mark.parametrize("seed", [0, 1])
def test_port_matches_compiled_reference(model, dims, L, seed):
    from tests.golden.make_golden import SOLVER

    inp = _rand_problem(model, dims, L, 100 + seed)
    maxit, errb, cc, steps = 25, 0.0, 0.3, 0.16 if len(dims) == 2 else 0.11
    fn = O.reference(SOLVER[(model, len(dims))])
    if model == "binary":
        pars = np.array(list(dims) + [maxit, errb, cc, steps], np.float32)
        ref = fn(inp["Cs"], inp["Ct"], inp["alpha"], pars)
    else:
        pars = np.array(list(dims) + [L, maxit, errb, cc, steps], np.float32)
        ref = fn(inp["Ct"], inp["alpha"], pars)
    out = O.solve(model, dims, inp["Ct"], inp["alpha"], cs=inp.get("Cs"), nlab=L, max_it=maxit,
                  err_bound=errb, cc=cc, steps=steps)
    np.testing.assert_array_equal(_bits(out["u"]), _bits(ref[0].ravel(order="F")))
    np.testing.assert_array_equal(_bits(out["cvg"]), _bits(ref[1].ravel()))
    assert int(ref[2].ravel()[0]) == out["it"]


@needs_ref
def test_reference_alpha_error_and_port_agree():
    from asetsmatlabmaxflow_gb300.mexhost import MexError

    inp = _rand_problem("binary", (6, 5), 1, 7)
    inp["alpha"][3, 2] = 0.0
    pars = np.array([6, 5, 10, 0.0, 0.3, 0.16], np.float32)
    with pytest.raises(MexError, match="alpha\\(x\\) must be positive"):
        O.reference("asetsBinaryMF2D_mex")(inp["Cs"], inp["Ct"], inp["alpha"], pars)
    with pytest.raises(O.OracleError, match="alpha"):
        O.solve("binary", (6, 5), inp["Ct"], inp["alpha"], cs=inp["Cs"], max_it=10,
                err_bound=0.0, cc=0.3, steps=0.16)


def test_port_maxit_zero_returns_init():
    inp = _rand_problem("ishikawa", (5, 4), 4, 3)
    out = O.solve("ishikawa", (5, 4), inp["Ct"], inp["alpha"], nlab=4, max_it=0,
                  err_bound=0.0, cc=0.3, steps=0.16)
    assert out["it"] == 0
    ct = inp["Ct"].reshape(-1, 4, order="F")
    first_min = np.argmin(ct, axis=1)
    u = out["u"].reshape(-1, 3, order="F")
    for l in range(3):
        np.testing.assert_array_equal(u[:, l], (l < first_min).astype(np.float32))


def test_warm_start_from_final_state_continues_the_solve():
    """Restarting from (u, ps, pt) with zero flows is the warm-start contract;
    with the flows reset it is not a bit-continuation, but must stay close."""
    inp = _rand_problem("potts", (12, 10), 3, 5)
    kw = dict(nlab=3, err_bound=0.0, cc=0.3, steps=0.16)
    a = O.solve("potts", (12, 10), inp["Ct"], inp["alpha"], max_it=30, want_state=True, **kw)
    b = O.solve("potts", (12, 10), inp["Ct"], inp["alpha"], max_it=5, u0=a["u"], ps0=a["ps"],
                pt0=a["pt"], **kw)
    assert b["it"] == 5 and np.isfinite(b["u"]).all()
