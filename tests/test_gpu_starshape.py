"""Star-shape Potts 2D on the GPU (FP64) against the float64 restatement of
maxflow/asetsPotts2D_starShape.m (oracle/starshape.py): u bit for bit,
erriter to summation order, the same break iteration."""
import numpy as np
import pytest

from oracle import starshape as S
from tests.gpu_helpers import require_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()


def _case(rows, cols, L, seed):
    g = np.random.default_rng(seed)
    ct = g.random((rows, cols, L))
    alpha = 0.1 + 0.3 * g.random((rows, cols, L))
    pts = [(int(g.integers(1, cols + 1)), int(g.integers(1, rows + 1))) for _ in range(L)]
    return ct, alpha, pts


@pytest.mark.parametrize("rows,cols,L,iters,beta", [
    (40, 33, 3, 40, 1e-12),   # runs all iterations
    (64, 48, 4, 300, 2e-3),   # breaks on erriter < beta
    (7, 5, 2, 25, 1e-12),
    (1, 17, 2, 10, 1e-12),
    (23, 1, 3, 10, 1e-12),
])
def test_matches_float64_restatement(rows, cols, L, iters, beta):
    from asetsmatlabmaxflow_gb300.starshape import asetsPotts2D_starShape

    ct, alpha, pts = _case(rows, cols, L, rows * 7 + cols)
    pars = [rows, cols, L, iters, beta, 0.25, 0.11, 0.05]
    u_ref, e_ref, i_ref = S.solve(ct, alpha, pars, pts)
    u, e, i, t = asetsPotts2D_starShape(ct, alpha, pars, np.array(pts))
    assert i == i_ref
    assert np.array_equal(u.view(np.uint64), u_ref.view(np.uint64))
    assert np.allclose(e[:, 0], e_ref, rtol=1e-12, atol=0)
    if i < iters:
        assert e_ref[i - 1] < beta and np.all(e[i:, 0] == 0)
    assert t > 0


def test_seed_points_keep_their_label():
    """The hard constraint at each seed makes that label win there."""
    from asetsmatlabmaxflow_gb300.starshape import asetsPotts2D_starShape

    ct, alpha, pts = _case(48, 40, 3, 9)
    u, e, i, t = asetsPotts2D_starShape(ct, alpha, [48, 40, 3, 200, 1e-5, 0.25, 0.11, 0.05],
                                        np.array(pts))
    for k, (x, y) in enumerate(pts):
        assert np.argmax(u[y - 1, x - 1, :]) == k


def test_bad_seed_is_rejected():
    from asetsmatlabmaxflow_gb300 import native as N
    from asetsmatlabmaxflow_gb300.starshape import asetsPotts2D_starShape

    ct, alpha, _ = _case(8, 8, 2, 1)
    with pytest.raises(N.AsetsError):
        asetsPotts2D_starShape(ct, alpha, [8, 8, 2, 5, 1e-5, 0.25, 0.11, 0.05],
                               np.array([[1, 1], [9, 2]]))
