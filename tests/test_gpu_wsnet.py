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
    """Ct, alpha, u, ps, pt, bx, by, bz (Matlab layout, label slowest)."""
    g = np.random.default_rng(seed)
    n = int(np.prod(dims))
    ct = g.random(n * L).astype(np.float32)
    alpha = (0.1 + 0.4 * g.random(n)).astype(np.float32)
    u = (g.random(n * L) > 0.5).astype(np.float32)
    ps = g.random(n).astype(np.float32)
    pt = g.random(n * L).astype(np.float32)
    fl = [(0.2 * g.standard_normal(n * L)).astype(np.float32) for _ in range(3)]
    return [ct, alpha, u, ps, pt] + fl


def _to_net_layout(dims, L, ct, alpha, u, ps, pt, bx, by, bz):
    ny, nx, nz = dims
    n = ny * nx * nz
    x = np.zeros((nz, nx, ny, 16))
    tgt = np.zeros((nz, nx, ny, 32))
    vol = lambda a: a.reshape(nz, nx, ny)  # Matlab layout: y fastest  # noqa: E731
    a = vol(alpha).astype(np.float32)
    for l in range(L):
        sl = slice(l * n, (l + 1) * n)
        x[..., l] = vol(ct[sl])
        tgt[..., l] = vol(u[sl])
        tgt[..., L + 1 + l] = vol(pt[sl])
        for k, b in enumerate((bx, by, bz)):
            tgt[..., 2 * L + 1 + k * L + l] = vol(b[sl]) * (np.float32(1) / a)
    x[..., L] = vol(alpha)
    tgt[..., L] = vol(ps)
    return x, tgt


@pytest.mark.parametrize("dims,L", [((128, 3, 3), 6), ((150, 2, 3), 3)])
def test_gradients_match_float64_oracle(dims, L):
    import torch

    from asetsmatlabmaxflow_gb300 import native as N

    net = N.WarmStartNet(N.Context.default(), nlab=L, seed=7)
    # non-zero output weights everywhere so every block carries a gradient
    params = net.get_params()
    params += np.random.default_rng(1).normal(0, 0.02, params.size).astype(np.float32)
    net.set_params(params)
    host = _sample(dims, L, 3)
    dev = [torch.from_numpy(a).cuda() for a in host]
    torch.cuda.synchronize()
    loss, g = net.gradients(dims, *dev)
    x, tgt = _to_net_layout(dims, L, *host)
    loss_ref, g_ref, _ = W.loss_and_grads(params, x, tgt, L)
    assert abs(loss - loss_ref) <= 1e-3 * loss_ref
    for b in range(W.BLOCKS):
        base = b * (W.NW + 16)
        for part in (slice(base, base + W.NW), slice(base + W.NW, base + W.NW + 16)):
            a, r = g[part].astype(np.float64), g_ref[part]
            err = np.linalg.norm(a - r) / max(np.linalg.norm(r), 1e-30)
            assert err < 2e-2, (b, part, err)
    net.close()


def test_prediction_layout_matches_oracle():
    import torch

    from asetsmatlabmaxflow_gb300 import native as N

    dims, L = (130, 4, 2), 6
    net = N.WarmStartNet(N.Context.default(), nlab=L, seed=3)
    params = net.get_params()
    host = _sample(dims, L, 9)
    n = int(np.prod(dims))
    ct, alpha = [torch.from_numpy(a).cuda() for a in host[:2]]
    outs = [torch.empty(s, device="cuda") for s in (n * L, n, n * L, n * L, n * L, n * L)]
    net.predict(dims, ct, alpha, *outs)
    torch.cuda.synchronize()
    x, tgt = _to_net_layout(dims, L, *host)
    _, _, out = W.loss_and_grads(params, x, tgt, L)  # [nz, nx, ny, 32]
    ny, nx, nz = dims
    flat = lambda v: np.ascontiguousarray(v).reshape(-1)  # noqa: E731  (z, x, y) = Matlab order
    a = host[1].astype(np.float64)
    exp_u = np.concatenate([np.clip(flat(out[..., l]), 0, 1) for l in range(L)])
    exp_ps = flat(out[..., L])
    exp_pt = np.concatenate([flat(out[..., L + 1 + l]) for l in range(L)])
    exp_b = [np.concatenate([flat(out[..., 2 * L + 1 + k * L + l]) * a for l in range(L)])
             for k in range(3)]
    got = [o.cpu().numpy().astype(np.float64) for o in outs]
    for e, gv in zip([exp_u, exp_ps, exp_pt] + exp_b, got):
        assert np.max(np.abs(e - gv)) <= 2e-2 * max(1.0, np.max(np.abs(e)))
    net.close()


def test_training_lowers_the_loss():
    import torch

    from asetsmatlabmaxflow_gb300 import native as N

    dims, L = (128, 6, 5), 6
    net = N.WarmStartNet(N.Context.default(), nlab=L, seed=1)
    ct, alpha = _sample(dims, L, 11)[:2]
    n = int(np.prod(dims))
    c = ct.reshape(L, n)
    # targets that are local functions of the input, so the loss can fall
    u = (c < 0.3).astype(np.float32).ravel()
    ps = c.min(0)
    fl = [(0.5 * alpha * (c - 0.5) * s).astype(np.float32).ravel() for s in (1.0, -0.5, 0.25)]
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in [ct, alpha, u, ps, ct] + fl]
    torch.cuda.synchronize()
    first = net.train_step(dims, *dev, lr=3e-3)
    for _ in range(40):
        last = net.train_step(dims, *dev, lr=3e-3)
    assert last < 0.7 * first
    net.close()
