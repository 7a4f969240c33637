"""Learned warm start for the Potts 3D solver: problem generation on the
device, solver-generated training pairs, training, and the warm-vs-cold
evaluation with its cold-start fallback.

The workload is Potts 3D, 128^3 voxels, L = 6 labels (cc = 0.3,
steps = 0.11): label means U[0,1], a Voronoi partition into 30-80 cells,
noise sigma U[0.05, 0.2], Ct_l = |I - c_l|, one alpha U[0.1, 0.5] per problem.
The network (asets_wsnet_*, four 3x3x3 convolutional layers with 16 hidden
channels) maps (Ct_1..Ct_6, alpha) to an initial solver state: u_1..u_6, ps,
pt_1..pt_6 and the spatial flows bx, by, bz.  It is trained on the states of
cold solves run to errBound 1e-5, one pair per seed, generated on the fly (a
replay buffer of recent pairs stays on the device).  The flows are part of
the prediction because the solver spends most of its iterations rebuilding
them: started from the exact converged (u, ps, pt) with zero flows, a solve
still needs 30-75% of the cold iterations, while noisy flows added to it
bring that down to about 10%.

Fallback: the warm solve gets the cold start's calibrated iteration budget
(the median iterations-to-errBound of cold solves of the training problems);
if it has not converged by then, the problem is solved again from the cold
start and that result is used.  The evaluation also solves every held-out
problem from the cold start, which judges the warm labelling (label
agreement).
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import native as N
from . import synth

WEIGHTS = Path(__file__).resolve().parent / "weights" / "potts3d_128_l6.npz"
SHAPE = (128, 128, 128)
LABELS = 6
CC, STEPS = 0.3, 0.11
TRAIN_ERR = 1e-5
EVAL_ERR = 1e-4
MAX_IT = 20000
HELDOUT_SEED0 = 1_000_000  # held-out seeds start here; training seeds below it


def problem(seed: int, shape=SHAPE, L: int = LABELS, device="cuda"):
    """One warm-start problem as torch tensors in Matlab layout (label
    slowest): Ct (N*L), alpha (N), alpha on all L slices (N*L).  The draws are
    synth.potts_warmstart's; the nearest-seed search and the cost terms run
    on `device` in the same float64/float32 arithmetic, so the result equals
    synth.potts_warmstart (up to exact distance ties)."""
    import torch

    means, seeds, cell_mean, alpha, noise = synth.potts_warmstart_draws(seed, shape, L)
    ny, nx, nz = shape
    n = ny * nx * nz
    dev = torch.device(device)
    sd = torch.from_numpy(seeds).to(dev)
    lab = torch.empty(n, dtype=torch.long, device=dev)
    chunk = 1 << 18
    for s0 in range(0, n, chunk):
        k = torch.arange(s0, min(n, s0 + chunk), device=dev)
        pts = torch.stack([k % ny, (k // ny) % nx, k // (ny * nx)], 1).to(torch.float64)
        d = ((pts[:, None, :] - sd[None, :, :]) ** 2).sum(-1)
        lab[s0:s0 + k.numel()] = d.argmin(1)
    cm = torch.from_numpy(cell_mean).to(dev)
    nz_ = torch.from_numpy(np.ascontiguousarray(noise.ravel(order="F"))).to(dev)
    img = (cm[lab] + nz_).clamp_(0.0, 1.0).to(torch.float32)
    mu = torch.from_numpy(means.astype(np.float32)).to(dev)
    ct = (img[None, :] - mu[:, None]).abs().reshape(-1)
    a1 = torch.full((n,), np.float32(alpha), dtype=torch.float32, device=dev)
    return ct.contiguous(), a1, a1.repeat(L)


def labels(u, n: int, L: int = LABELS):
    """argmax over labels of a Potts u (torch, Matlab layout)."""
    return u.view(L, n).argmax(0)


@dataclass
class Pair:
    ct: object
    alpha: object
    state: tuple  # u, ps, pt, bx, by, bz


class Runner:
    """One device-resident Potts solver for the warm-start shape."""

    def __init__(self, ctx: N.Context | None = None, shape=SHAPE, L: int = LABELS):
        import torch

        self.ctx = ctx or N.Context.default()
        self.shape, self.L = shape, L
        self.n = int(np.prod(shape))
        self.s = N.Solver(self.ctx, "potts", shape, L)
        self.u = torch.empty(self.n * L, device="cuda")
        self.ps = torch.empty(self.n, device="cuda")
        self.pt = torch.empty(self.n * L, device="cuda")
        self.b = [torch.empty(self.n * L, device="cuda") for _ in range(3)]

    def load(self, ct, alpha_full):
        self.s.set_inputs(ct, alpha_full, where=N.DEVICE)

    def cold(self, err: float, max_it: int = MAX_IT) -> int:
        self.s.set_initial(None, None, None)
        return self.s.run(max_it, err, CC, STEPS)

    def warm(self, state, err: float, max_it: int) -> int:
        u0, ps0, pt0, bx0, by0, bz0 = state
        self.s.set_initial(u0, ps0, pt0, where=N.DEVICE)
        self.s.set_initial_flows(bx0, by0, bz0, where=N.DEVICE)
        return self.s.run(max_it, err, CC, STEPS)

    @staticmethod
    def converged(it: int, max_it: int) -> bool:
        """itNum is the index of the iteration that met errBound, or maxIt
        when none did."""
        return it < max_it

    def first_below(self, it: int, err: float) -> int:
        """itNum a cold run with errBound `err` would have returned (the same
        trajectory; the Potts stopping rule is erriter <= errBound)."""
        c = self.s.get_cvg(min(it + 1, self.s.last_max_it))
        hit = np.nonzero(c <= err)[0]
        return int(hit[0]) if hit.size else -1

    def state(self):
        """Final (u, ps, pt, bx, by, bz) of the last run (device buffers)."""
        self.s.get_u(self.u, where=N.DEVICE)
        self.s.get_flows(self.ps, self.pt, where=N.DEVICE)
        self.s.get_spatial_flows(*self.b, where=N.DEVICE)
        return (self.u, self.ps, self.pt, *self.b)

    def close(self):
        self.s.close()


def train(train_seeds, *, steps_per_pair: int = 2, buffer: int = 24, lr: float = 2e-3,
          lr_final: float = 1e-4, seed: int = 0, log=print):
    """Train a fresh network on cold solutions (errBound 1e-5) of
    `train_seeds`.  Returns (net, info) where info holds the calibrated cold
    iteration budget for errBound 1e-4 and the loss history."""
    import torch

    run = Runner()
    net = N.WarmStartNet(run.ctx, nlab=LABELS, seed=seed)
    g = np.random.default_rng(seed)
    buf: list[Pair] = []
    cold_iters, losses = [], []
    total = len(train_seeds) * steps_per_pair
    k = 0
    t0 = time.time()
    for i, sd in enumerate(train_seeds):
        ct, a1, af = problem(sd)
        run.load(ct, af)
        it = run.cold(TRAIN_ERR)
        cold_iters.append(run.first_below(it, EVAL_ERR))
        buf.append(Pair(ct, a1, tuple(t.clone() for t in run.state())))
        if len(buf) > buffer:
            buf.pop(0)
        for _ in range(steps_per_pair):
            p = buf[int(g.integers(len(buf)))]
            frac = k / max(1, total - 1)
            lr_k = lr_final + 0.5 * (lr - lr_final) * (1 + np.cos(np.pi * frac))
            losses.append(net.train_step(run.shape, p.ct, p.alpha, *p.state, lr=lr_k))
            k += 1
        if log and (i % 50 == 0 or i == len(train_seeds) - 1):
            log(f"pair {i + 1}/{len(train_seeds)} seed {sd}: cold it(1e-5)={it} "
                f"it(1e-4)={cold_iters[-1]} loss={np.mean(losses[-2 * steps_per_pair:]):.5f} "
                f"{time.time() - t0:.0f}s")
    torch.cuda.synchronize()
    run.close()
    ci = np.array([c for c in cold_iters if c > 0])
    info = {"cold_budget": int(np.median(ci)), "cold_iters": np.array(cold_iters),
            "losses": np.array(losses, np.float32), "train_pairs": len(train_seeds),
            "steps_per_pair": steps_per_pair, "train_seconds": time.time() - t0}
    return net, info


def save(net: N.WarmStartNet, info: dict, path: Path = WEIGHTS) -> None:
    path.parent.mkdir(parents=True, exist_ok=True)
    np.savez(path, params=net.get_params(), cold_budget=info["cold_budget"],
             train_pairs=info["train_pairs"], steps_per_pair=info["steps_per_pair"],
             final_loss=float(np.mean(info["losses"][-50:])))


def load(ctx: N.Context | None = None, path: Path = WEIGHTS):
    """The trained network and its calibrated cold iteration budget."""
    d = np.load(path)
    net = N.WarmStartNet(ctx or N.Context.default(), nlab=LABELS, seed=0)
    net.set_params(d["params"])
    return net, int(d["cold_budget"])


@dataclass
class EvalResult:
    seed: int
    cold_it: int
    cold_ms: float          # wall time of the cold solve (init + iterations)
    warm_it: int            # iterations of the warm solve (its cap when it fell back)
    warm_ms: float          # net inference + warm solve (+ the cold solve on fallback)
    infer_ms: float
    fallback: bool
    agree_cold: float       # warm labels vs cold labels, both at errBound 1e-4
    agree_tight: float = float("nan")      # warm labels vs a 1e-5 cold solve
    cold_agree_tight: float = float("nan")  # cold 1e-4 labels vs the same
    extra: dict = field(default_factory=dict)


def _sync_ms(fn):
    import torch

    torch.cuda.synchronize()
    t = time.perf_counter()
    r = fn()
    torch.cuda.synchronize()
    return r, 1e3 * (time.perf_counter() - t)


def evaluate(net: N.WarmStartNet, cold_budget: int, seeds, *, tight: bool = True,
             run: Runner | None = None, log=None) -> list[EvalResult]:
    """Warm vs cold on held-out seeds, errBound 1e-4.  Each problem is solved
    cold first (also the judge), then warm with the fallback rule."""
    import torch

    own = run is None
    run = run or Runner()
    n, L = run.n, run.L
    pred = [torch.empty(n * L, device="cuda"), torch.empty(n, device="cuda")] + \
        [torch.empty(n * L, device="cuda") for _ in range(4)]
    out = []
    for sd in seeds:
        ct, a1, af = problem(sd)
        run.load(ct, af)
        cold_it, cold_ms = _sync_ms(lambda: run.cold(EVAL_ERR))
        lab_c = labels(run.state()[0], n).clone()

        def warm_path():
            net.predict(run.shape, ct, a1, *pred)
            t_inf = time.perf_counter()
            it = run.warm(pred, EVAL_ERR, cold_budget)
            fb = not run.converged(it, cold_budget)
            if fb:
                run.cold(EVAL_ERR)
            return it, fb, t_inf

        t0 = time.perf_counter()
        (warm_it, fb, t_inf), warm_ms = _sync_ms(warm_path)
        infer_ms = 1e3 * (t_inf - t0)
        lab_w = labels(run.state()[0], n)
        r = EvalResult(sd, cold_it, cold_ms, warm_it, warm_ms, infer_ms, fb,
                       float((lab_w == lab_c).float().mean()))
        if tight:
            run.cold(TRAIN_ERR)
            lab_t = labels(run.state()[0], n)
            r.agree_tight = float((lab_w == lab_t).float().mean())
            r.cold_agree_tight = float((lab_c == lab_t).float().mean())
        out.append(r)
        if log:
            log(f"seed {sd}: cold {cold_it} it {cold_ms:.1f} ms | warm {warm_it} it "
                f"{warm_ms:.1f} ms (net {infer_ms:.1f} ms){' FALLBACK' if fb else ''} | "
                f"agree cold {r.agree_cold:.5f} tight {r.agree_tight:.5f} "
                f"(cold vs tight {r.cold_agree_tight:.5f})")
    if own:
        run.close()
    return out


def summarize(res: list[EvalResult]) -> dict:
    c_it = np.array([r.cold_it for r in res], float)
    w_it = np.array([r.warm_it if not r.fallback else r.warm_it + r.cold_it for r in res], float)
    c_ms = np.array([r.cold_ms for r in res])
    w_ms = np.array([r.warm_ms for r in res])
    return {
        "problems": len(res),
        "cold_iters_mean": float(c_it.mean()), "warm_iters_mean": float(w_it.mean()),
        "cold_ms_mean": float(c_ms.mean()), "warm_ms_mean": float(w_ms.mean()),
        "infer_ms_mean": float(np.mean([r.infer_ms for r in res])),
        "iters_ratio": float(c_it.sum() / w_it.sum()),
        "wall_ratio": float(c_ms.sum() / w_ms.sum()),
        "fallbacks": int(sum(r.fallback for r in res)),
        "regressions": int(sum((not r.fallback) and r.warm_it >= r.cold_it for r in res)),
        "agree_cold_min": float(min(r.agree_cold for r in res)),
        "agree_cold_mean": float(np.mean([r.agree_cold for r in res])),
        "agree_tight_mean": float(np.nanmean([r.agree_tight for r in res])),
        "cold_agree_tight_mean": float(np.nanmean([r.cold_agree_tight for r in res])),
    }


def main(argv=None):
    """python -m asetsmatlabmaxflow_gb300.warmstart --train N --eval M"""
    import argparse
    import json

    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=2000, help="training pairs (seeds 0..N-1)")
    ap.add_argument("--eval", type=int, default=200, help="held-out seeds")
    ap.add_argument("--steps-per-pair", type=int, default=2)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--out", type=Path, default=WEIGHTS)
    ap.add_argument("--no-tight", action="store_true")
    ap.add_argument("--eval-only", action="store_true")
    a = ap.parse_args(argv)
    if a.eval_only:
        net, budget = load(path=a.out)
    else:
        net, info = train(range(a.train), steps_per_pair=a.steps_per_pair, lr=a.lr)
        save(net, info, a.out)
        budget = info["cold_budget"]
        print(json.dumps({"train_pairs": a.train, "cold_budget": budget,
                          "train_seconds": round(info["train_seconds"], 1),
                          "final_loss": float(np.mean(info["losses"][-50:]))}), flush=True)
    res = evaluate(net, budget, range(HELDOUT_SEED0, HELDOUT_SEED0 + a.eval),
                   tight=not a.no_tight, log=print)
    print(json.dumps(summarize(res)), flush=True)


if __name__ == "__main__":
    main()
