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
