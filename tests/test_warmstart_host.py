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


def test_potts_energy_matches_a_direct_sum():
    """The relaxed Potts energy used to compare warm and cold solutions, on a
    small random u, against a loop over voxels and faces."""
    import numpy as np
    import torch

    from asetsmatlabmaxflow_gb300 import warmstart as W

    L, shape = 2, (3, 4, 2)
    ny, nx, nz = shape
    n = ny * nx * nz
    g = np.random.default_rng(0)
    u = torch.tensor(g.random(n * L), dtype=torch.float32)
    ct = torch.tensor(g.random(n * L), dtype=torch.float32)
    a = torch.full((n * L,), 0.25)
    U = u.numpy().reshape(L, nz, nx, ny).astype(np.float64)
    C = ct.numpy().reshape(L, nz, nx, ny)
    tot = float((U * C).sum())
    for l in range(L):
        for z in range(nz):
            for x in range(nx):
                for y in range(ny):
                    s = 0.0
                    for dz, dx, dy in ((1, 0, 0), (0, 1, 0), (0, 0, 1)):
                        for sg in (1, -1):
                            zz, xx, yy = z + sg * dz, x + sg * dx, y + sg * dy
                            if 0 <= zz < nz and 0 <= xx < nx and 0 <= yy < ny:
                                s += (U[l, zz, xx, yy] - U[l, z, x, y]) ** 2
                    tot += 0.25 * np.sqrt(0.5 * s)
    assert abs(W.potts_energy(ct, a, u, shape, L) - tot) < 1e-9 * max(1.0, abs(tot))
    oh = W.one_hot(torch.tensor([0, 1, 1]), 3, 2)
    assert oh.tolist() == [1.0, 0.0, 0.0, 0.0, 1.0, 1.0]
