"""Warm-start network: GPU loss and gradients against the float64 oracle
(oracle/wsnet.py), and a short training run that lowers the loss."""
import numpy as np
import pytest

from oracle import wsnet as W
from tests.gpu_helpers import require_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    require_gpu()


def _sample(dims, L, seed):
    g = np.random.default_rng(seed)
    n = int(np.prod(dims))
    ct = g.random(n * L).astype(np.float32)
    alpha = np.full(n, 0.3, np.float32)
    u = (g.random(n * L) > 0.5).astype(np.float32)
    ps = g.random(n).astype(np.float32)
    pt = g.random(n * L).astype(np.float32)
    return ct, alpha, u, ps, pt


def _to_net_layout(dims, L, ct, alpha, u, ps, pt):
    ny, nx, nz = dims
    n = ny * nx * nz
    x = np.zeros((nz, nx, ny, 16))
    tgt = np.zeros((nz, nx, ny, 16))
    vol = lambda a: a.reshape(nz, nx, ny)  # Matlab layout: y fastest  # noqa: E731
    for l in range(L):
        x[..., l] = vol(ct[l * n:(l + 1) * n])
        tgt[..., l] = vol(u[l * n:(l + 1) * n])
        tgt[..., L + 1 + l] = vol(pt[l * n:(l + 1) * n])
    x[..., L] = vol(alpha)
    tgt[..., L] = vol(ps)
    return x, tgt


def test_gradients_match_float64_oracle():
    import torch

    from asetsmatlabmaxflow_gb300 import native as N

    dims, L = (128, 3, 3), 6
    net = N.WarmStartNet(N.Context.default(), nlab=L, seed=7)
    params = net.get_params()
    host = _sample(dims, L, 3)
    dev = [torch.from_numpy(a).cuda() for a in host]
    torch.cuda.synchronize()
    loss, g = net.gradients(dims, *dev)
    x, tgt = _to_net_layout(dims, L, *host)
    loss_ref, g_ref, _ = W.loss_and_grads(params, x, tgt, L)
    assert abs(loss - loss_ref) <= 1e-3 * loss_ref
    for l in range(W.LAYERS):
        base = l * (W.NW + 16)
        for part in (slice(base, base + W.NW), slice(base + W.NW, base + W.NW + 16)):
            a, b = g[part].astype(np.float64), g_ref[part]
            err = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
            assert err < 2e-2, (l, part, err)
    net.close()


def test_training_lowers_the_loss():
    import torch

    from asetsmatlabmaxflow_gb300 import native as N

    dims, L = (128, 6, 5), 6
    net = N.WarmStartNet(N.Context.default(), nlab=L, seed=1)
    dev = [torch.from_numpy(a).cuda() for a in _sample(dims, L, 11)]
    torch.cuda.synchronize()
    first = net.train_step(dims, *dev, lr=3e-3)
    for _ in range(40):
        last = net.train_step(dims, *dev, lr=3e-3)
    assert last < 0.7 * first
    u0 = torch.empty(int(np.prod(dims)) * L, device="cuda")
    ps0 = torch.empty(int(np.prod(dims)), device="cuda")
    pt0 = torch.empty_like(u0)
    net.predict(dims, dev[0], dev[1], u0, ps0, pt0)
    torch.cuda.synchronize()
    assert torch.isfinite(u0).all() and float(u0.min()) >= 0 and float(u0.max()) <= 1
    net.close()
