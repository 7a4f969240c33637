"""Tensor-core 3x3x3 convolution (tcgen05) against a float64 reference on
the same BF16-rounded inputs."""
import numpy as np
import pytest

from tests.gpu_helpers import require_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()


def conv_ref(x, w, bias=None, flip=False):
    """x: [nz, nx, ny, 16] float64, w: [27, 16, 16]; zero padding."""
    nz, nx, ny, _ = x.shape
    xp = np.zeros((nz + 2, nx + 2, ny + 2, 16))
    xp[1:-1, 1:-1, 1:-1] = x
    out = np.zeros((nz, nx, ny, 16))
    for t in range(27):
        dz, dx, dy = t // 9, (t // 3) % 3, t % 3
        wt = w[26 - t].T if flip else w[t]
        out += np.einsum("zxyc,cd->zxyd", xp[dz:dz + nz, dx:dx + nx, dy:dy + ny], wt)
    if bias is not None:
        out += bias
    return out


def _bf16(a):
    import torch

    t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(torch.bfloat16)
    return t, t.float().numpy().astype(np.float64)


@pytest.mark.parametrize("shape,relu,fp32,flip,mask", [
    ((4, 5, 128), False, True, False, False),
    ((3, 4, 200), False, True, False, False),
    ((2, 3, 64), True, False, False, False),
    ((3, 3, 128), False, True, True, True),
])
def test_conv_matches_float64_reference(shape, relu, fp32, flip, mask):
    import torch

    from asetsmatlabmaxflow_gb300 import native as N

    nz, nx, ny = shape
    g = np.random.default_rng(sum(shape) + relu + 2 * flip)
    xt, x64 = _bf16(g.standard_normal((nz, nx, ny, 16)))
    wt, w64 = _bf16(0.2 * g.standard_normal((27, 16, 16)))
    bias = g.standard_normal(16).astype(np.float32)
    mt, m64 = _bf16(g.standard_normal((nz, nx, ny, 16)))
    dx, dw, db = xt.cuda(), wt.cuda(), torch.from_numpy(bias).cuda()
    dm = mt.cuda() if mask else None
    out = torch.empty((nz, nx, ny, 16), dtype=torch.float32 if fp32 else torch.bfloat16,
                      device="cuda")
    torch.cuda.synchronize()
    N.check(N.lib().asets_conv3d_bf16(N.Context.default().handle, dx.data_ptr(), dw.data_ptr(),
                                      db.data_ptr(), dm.data_ptr() if mask else None,
                                      out.data_ptr(), ny, nx, nz, int(relu), int(fp32),
                                      int(flip)))
    ref = conv_ref(x64, w64, bias, flip)
    if relu:
        ref = np.maximum(ref, 0)
    if mask:
        ref = np.where(m64 > 0, ref, 0.0)
    got = out.float().cpu().numpy().astype(np.float64)
    scale = conv_ref(np.abs(x64), np.abs(w64), np.abs(bias), flip)  # error scale per output
    tol = (1e-5 if fp32 else 8e-3) * (scale + 1e-3)
    bad = np.abs(got - ref) > tol
    assert not bad.any(), f"{bad.sum()} of {bad.size} outputs off; max err {np.abs(got-ref).max()}"


@pytest.fixture(scope="module")
def wgrad_lib(tmp_path_factory):
    import ctypes
    import subprocess
    from pathlib import Path

    from asetsmatlabmaxflow_gb300 import build

    root = Path(__file__).resolve().parent.parent
    out = tmp_path_factory.mktemp("wgradcheck") / "libwgradcheck.so"
    subprocess.run([build.nvcc(), *build.ARCH, *build.NVCC_FLAGS, f"-I{build.CSRC}",
                    f"-I{build.INCLUDE}", "-shared", "-o", str(out),
                    str(root / "tests" / "cuda" / "wgrad_check.cu"), "-lcuda"], check=True)
    lib = ctypes.CDLL(str(out))
    lib.wgrad_check.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                ctypes.POINTER(ctypes.c_double)]
    lib.wgrad_check.restype = ctypes.c_int
    return lib


@pytest.mark.parametrize("hp", [0, 1])
@pytest.mark.parametrize("dims", [(150, 3, 3), (128, 4, 5), (260, 2, 2), (37, 6, 3)])
def test_tensor_core_weight_gradient_matches_double_reference(wgrad_lib, dims, hp):
    """The tcgen05 weight and bias gradients (voxels as the GEMM's K, both
    operands MN-major) against a double-precision sum over the same BF16
    values, for channels-last and for padded half-planar operands: error
    within 1e-5 of the sum of |a * g| (FP32 accumulation)."""
    import ctypes

    worst = ctypes.c_double(1.0)
    assert wgrad_lib.wgrad_check(*dims, hp, ctypes.byref(worst)) == 0
    assert worst.value < 1e-5, worst.value
