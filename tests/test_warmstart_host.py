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
    res = [R(1, 300, 120.0, 100, 50.0, 2.0, False, 0.999),
           R(2, 300, 120.0, 300, 250.0, 2.0, True, 1.0)]
    s = warmstart.summarize(res)
    assert s["fallbacks"] == 1
    assert s["warm_iters_mean"] == (100 + 600) / 2
    assert abs(s["wall_ratio"] - 240 / 300) < 1e-12
