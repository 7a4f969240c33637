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


def _regular(cs, ct, alpha, max_it, err_bound, cc, steps, *, exact=False):
    from asetsmatlabmaxflow_gb300 import native as N

    ny, nx, nz = cs.shape
    f = lambda a: np.ascontiguousarray(a.ravel(order="F"), dtype=np.float32)  # noqa: E731
    u = np.zeros(ny * nx * nz, np.float32)
    cvg = np.zeros(max(max_it, 1), np.float32)
    it = ctypes.c_int()
    a, s, t = f(alpha), f(cs), f(ct)
    opt = N.Options(flags=N.FLAG_EXACT if exact else 0)
    N.check(N.lib().asets_binary_mf3d(None, ctypes.byref(opt), a.ctypes.data, s.ctypes.data,
                                      t.ctypes.data, nx, ny, nz, max_it, err_bound, cc, steps,
                                      u.ctypes.data, cvg.ctypes.data, ctypes.byref(it), None))
    return u, cvg[:max_it], it.value


def _device_buffers(cs, ct, alpha, max_it):
    import torch

    n = cs.size
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).cuda()  # noqa: E731
    bufs = {"cs": dev(cs), "ct": dev(ct), "alpha": dev(alpha),
            "u": torch.full((n,), float("nan"), device="cuda"),
            "cvg": torch.full((max(max_it, 1),), float("nan"), device="cuda")}
    torch.cuda.synchronize()
    return bufs


def _call_noalloc(bufs, shape, max_it, err_bound, cc, steps, *, exact=False, stream=None):
    """One call through the C ABI on device buffers; returns itNum."""
    from asetsmatlabmaxflow_gb300 import native as N

    ny, nx, nz = shape
    opt = N.Options(flags=N.FLAG_EXACT if exact else 0)
    it = ctypes.c_int(-1)
    N.check(N.lib().asets_binary_mf3d_noalloc(
        ctypes.byref(opt), bufs["alpha"].data_ptr(), bufs["cs"].data_ptr(), bufs["ct"].data_ptr(),
        nx, ny, nz, max_it, err_bound, cc, steps, bufs["u"].data_ptr(), bufs["cvg"].data_ptr(),
        ctypes.byref(it), stream))
    return it.value


def _noalloc(cs, ct, alpha, max_it, err_bound, cc, steps, *, exact=False, stream=None):
    bufs = _device_buffers(cs, ct, alpha, max_it)
    it = _call_noalloc(bufs, cs.shape, max_it, err_bound, cc, steps, exact=exact, stream=stream)
    return bufs["u"].cpu().numpy(), bufs["cvg"].cpu().numpy()[:max_it], it


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


def test_noalloc_exact_mode_is_bit_identical_to_regular_entry_point_and_oracle():
    """EXACT mode: u bit for bit equal to the regular entry point's and to the
    oracle's (the reference's float arithmetic), twice in a row."""
    from oracle import oracle as O

    for shape, seed, max_it in [((45, 38, 21), 3, 35), ((64, 40, 16), 4, 25)]:
        cs, ct, alpha = _problem(shape, seed)
        ref = O.solve("binary", shape, ct, alpha, cs=cs, max_it=max_it, err_bound=0.0, cc=0.35,
                      steps=0.11, erru_double=True)
        u_reg, _, it_reg = _regular(cs, ct, alpha, max_it, 0.0, 0.35, 0.11, exact=True)
        u, cvg, it = _noalloc(cs, ct, alpha, max_it, 0.0, 0.35, 0.11, exact=True)
        assert it == it_reg == ref["it"] == max_it
        np.testing.assert_array_equal(u.view(np.uint32), ref["u"].view(np.uint32))
        np.testing.assert_array_equal(u.view(np.uint32), u_reg.view(np.uint32))
        np.testing.assert_allclose(cvg, ref["cvg"], rtol=2e-5)


def test_noalloc_max_it_zero_returns_the_initial_labelling():
    cs, ct, alpha = _problem((20, 18, 7), 5)
    u, _, it = _noalloc(cs, ct, alpha, 0, 0.0, 0.35, 0.11)
    assert it == 0
    np.testing.assert_array_equal(u, (cs - ct >= 0).astype(np.float32).ravel(order="F"))


def test_noalloc_on_a_caller_stream_allocates_nothing():
    """A call on a non-default stream matches the default-stream call, and a
    second call leaves the device's free memory unchanged (the scratch was
    reserved by the first call on this device)."""
    import torch

    shape, max_it = (50, 44, 18), 30
    cs, ct, alpha = _problem(shape, 6)
    u_ref, cvg_ref, it_ref = _noalloc(cs, ct, alpha, max_it, 0.0, 0.35, 0.11)
    bufs = _device_buffers(cs, ct, alpha, max_it)
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    it = _call_noalloc(bufs, shape, max_it, 0.0, 0.35, 0.11, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before
    assert it == it_ref
    np.testing.assert_array_equal(bufs["u"].cpu().numpy(), u_ref)
    np.testing.assert_array_equal(bufs["cvg"].cpu().numpy()[:max_it], cvg_ref)
