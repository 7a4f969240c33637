"""The allocation-free binary 3D entry point (asets_binary_mf3d_noalloc).

It serves callers that cannot allocate device memory while they run (their
GPU memory is owned by another allocator, or allocation is forbidden after
start-up), so it takes device pointers and keeps its scratch in a fixed
device array.  Its results must equal the regular entry point's
(asets_binary_mf3d, which allocates per problem shape) on two calls in a row,
the second of which must not see the first call's leftover state.
Collected last so that a run stopping at the first failure has already run
every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem(shape, seed):
    from asetsmatlabmaxflow_gb300 import synth

    return synth.binary3d(seed=seed, shape=shape, ncells=12)


def _regular(cs, ct, alpha, max_it, err_bound, cc, steps):
    from asetsmatlabmaxflow_gb300 import native as N

    ny, nx, nz = cs.shape
    f = lambda a: np.ascontiguousarray(a.ravel(order="F"), dtype=np.float32)  # noqa: E731
    u = np.zeros(ny * nx * nz, np.float32)
    cvg = np.zeros(max_it, np.float32)
    it = ctypes.c_int()
    a, s, t = f(alpha), f(cs), f(ct)
    N.check(N.lib().asets_binary_mf3d(None, None, a.ctypes.data, s.ctypes.data, t.ctypes.data,
                                      nx, ny, nz, max_it, err_bound, cc, steps, u.ctypes.data,
                                      cvg.ctypes.data, ctypes.byref(it), None))
    return u, cvg, it.value


def _noalloc(cs, ct, alpha, max_it, err_bound, cc, steps):
    import torch

    from asetsmatlabmaxflow_gb300 import native as N

    ny, nx, nz = cs.shape
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).cuda()  # noqa: E731
    d_cs, d_ct, d_al = dev(cs), dev(ct), dev(alpha)
    d_u = torch.full((ny * nx * nz,), float("nan"), device="cuda")
    d_cvg = torch.full((max_it,), float("nan"), device="cuda")
    torch.cuda.synchronize()
    it = ctypes.c_int(-1)
    N.check(N.lib().asets_binary_mf3d_noalloc(None, d_al.data_ptr(), d_cs.data_ptr(),
                                              d_ct.data_ptr(), nx, ny, nz, max_it, err_bound, cc,
                                              steps, d_u.data_ptr(), d_cvg.data_ptr(),
                                              ctypes.byref(it), None))
    return d_u.cpu().numpy(), d_cvg.cpu().numpy(), it.value


def test_noalloc_matches_regular_entry_point_twice_in_a_row():
    cases = [((60, 52, 20), 1, 40, 0.0), ((33, 47, 17), 2, 300, 2e-3)]
    for shape, seed, max_it, err_bound in cases:
        cs, ct, alpha = _problem(shape, seed)
        u_ref, cvg_ref, it_ref = _regular(cs, ct, alpha, max_it, err_bound, 0.35, 0.11)
        u, cvg, it = _noalloc(cs, ct, alpha, max_it, err_bound, 0.35, 0.11)
        assert it == it_ref
        assert np.isfinite(u).all()
        assert float(np.max(np.abs(u - u_ref))) <= 1e-3
        n = min(it_ref + 1, max_it)
        np.testing.assert_allclose(cvg[:n], cvg_ref[:n], rtol=1e-3)
        assert np.all(cvg[n:] == 0)


def test_noalloc_rejects_problems_above_its_scratch_limit():
    import torch

    from asetsmatlabmaxflow_gb300 import native as N

    buf = torch.zeros(8, device="cuda")
    it = ctypes.c_int()
    p = buf.data_ptr()
    st = N.lib().asets_binary_mf3d_noalloc(None, p, p, p, 128, 128, 32, 1, 0.0, 0.3, 0.11, p, p,
                                           ctypes.byref(it), None)
    assert st == N.ASETS_ERR_INVALID_ARG
    assert b"limited to" in N.lib().asets_last_error()
