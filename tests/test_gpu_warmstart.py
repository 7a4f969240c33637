"""The trained warm start (committed weights) on held-out problems: it
reaches errBound 1e-4 without the cold fallback, faster than the cold start,
and the learned coarsest-level state needs fewer iterations than the cold
coarsest start of the same multilevel solve."""
import pytest

from tests.gpu_helpers import require_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()


def test_trained_network_gains_over_the_method_without_it():
    from asetsmatlabmaxflow_gb300 import warmstart as W

    net, budget, level = W.load()
    assert level == W.LEVELS - 1 and 0 < budget < W.MAX_IT
    seeds = range(W.HELDOUT_SEED0 + 500, W.HELDOUT_SEED0 + 504)  # not in the reported set
    res = W.evaluate(net, budget, seeds, level=level, tight=False)
    s = W.summarize(res)
    assert s["fallbacks"] == 0 and s["regressions"] == 0
    # coarse-to-fine with the learned start: far fewer full-resolution
    # iterations and less wall time than the cold start
    assert s["warm_iters_mean"] < 0.3 * s["cold_iters_mean"]
    assert s["wall_ratio_cold_over_warm"] > 2.0
    # the network's own contribution: fewer coarsest-level iterations than
    # the same multilevel solve started cold
    assert s["coarsest_iters_learned_mean"] < s["coarsest_iters_cold_start_mean"]
    net.close()


def test_batched_warm_start_matches_single_solves(monkeypatch):
    """The batched warm-started solve (one batch per level) gives each
    problem the iterations of its own warm-started multilevel solve, and the
    cold batch each problem's cold itNum (default kernel variants on both
    sides: autotuning may pick different ones for a batch and a single
    solve)."""
    from asetsmatlabmaxflow_gb300 import warmstart as W

    monkeypatch.setattr(W, "AUTOTUNE", False)

    net, budget, level = W.load()
    seeds = [W.HELDOUT_SEED0 + 7, W.HELDOUT_SEED0 + 8, W.HELDOUT_SEED0 + 9]
    single = W.evaluate(net, budget, seeds, level=level, tight=False)
    batched = W.evaluate_batched(net, budget, seeds, level=level)
    assert batched["cold_iters"] == [r.cold_it for r in single]
    assert batched["warm_level_iters"] == [r.warm_its for r in single]
    assert batched["fallbacks"] == sum(r.fallback for r in single)
    assert batched["warm_batch_ms"] < batched["cold_batch_ms"]
    net.close()


def test_warm_solution_is_as_good_as_the_cold_one_where_labels_differ():
    """Label agreement between the warm and the cold 1e-4 solves is no
    measure of the warm path on this workload: two labels with nearly equal
    means swap whole regions, and the cold 1e-4 solve stops far from its own
    converged labelling.  What the warm path must keep is the solution's
    quality: its relaxed Potts energy at errBound 1e-4 is not above the cold
    solve's by more than 2e-3 (the largest excess on 200 held-out seeds was
    9.7e-4, below the cold solve's own energy drop from 1e-4 to 1e-5, which
    was at least 9.1e-4), and where the labels agree least the disagreement
    is concentrated on one pair of labels."""
    from asetsmatlabmaxflow_gb300 import warmstart as W

    net, _, level = W.load()
    seeds = [W.HELDOUT_SEED0 + 600, W.HELDOUT_SEED0 + 601, W.HELDOUT_SEED0 + 602]
    rows = W.diagnose(net, seeds, level=level)
    for r in rows:
        d4 = (r["warm4_E"] - r["cold4_E"]) / abs(r["cold4_E"])
        assert d4 <= 2e-3, (r["seed"], d4)
        # the cold 1e-4 solve is itself unconverged: its energy is above its 1e-5 one
        assert r["cold4_E"] > r["cold5_E"]
        assert r["warm4_it"] < r["cold4_it"]
        if r["agree4"] < 0.999:
            assert r["top_pair_share"] > 0.15  # of 30 ordered pairs (min 0.195 on 200 seeds)
    net.close()
