"""Host-side pieces of the warm-start pipeline (no GPU)."""
import numpy as np

from asetsmatlabmaxflow_gb300 import synth, warmstart


def test_device_problem_generator_equals_synth():
    shape, L = (20, 14, 9), 6
    for seed in (0, 5, 1_000_003):
        ct, a1, af = warmstart.problem(seed, shape, L, device="cpu")
        ct_ref, a_ref = synth.potts_warmstart(seed, shape, L)
        n = int(np.prod(shape))
        assert np.array_equal(ct.numpy(), ct_ref.ravel(order="F"))
        assert np.array_equal(af.numpy(), a_ref.ravel(order="F"))
        assert np.array_equal(a1.numpy(), a_ref.ravel(order="F")[:n])


def test_summary_counts_fallback_iterations():
    R = warmstart.EvalResult
    res = [R(1, 300, 120.0, [40, 60, 200], 30.0, [38, 50, 90], 25.0, 1.0, False, 0.99, 0.98),
           R(2, 300, 120.0, [40, 60, 200], 30.0, [310, 50, 90], 250.0, 1.0, True, 1.0, 0.97)]
    s = warmstart.summarize(res)
    assert s["fallbacks"] == 1 and s["regressions"] == 0
    assert s["warm_iters_mean"] == (38 + 310 + 300) / 2
    assert s["coarsest_iters_learned_mean"] == 90 and s["coarsest_iters_cold_start_mean"] == 200
    assert abs(s["wall_ratio_cold_over_warm"] - 240 / 275) < 1e-12
    assert abs(s["wall_ratio_cold_over_multilevel"] - 4.0) < 1e-12
