"""Learned warm start for the Potts 3D solver: problem generation on the
device, solver-generated training pairs, training, and the warm-vs-cold
evaluation with its cold-start fallback.

Workload: Potts 3D, 128^3 voxels, L = 6 labels (cc = 0.3, steps = 0.11):
label means U[0,1], a Voronoi partition into 30-80 cells, noise sigma
U[0.05, 0.2], Ct_l = |I - c_l|, one alpha U[0.1, 0.5] per problem.

The network (asets_wsnet_*: four 3x3x3 convolutional layers, 16 hidden
channels, BF16 on the tensor cores) maps (Ct_1..Ct_6, alpha) to an initial
solver state: u_1..u_6, ps, pt_1..pt_6 and the spatial flows bx, by, bz.  It
is trained on states of cold solves run to errBound 1e-5.

Where it is applied.  Measured on this workload, the state of a solve at
errBound 1e-4 depends on region-scale decisions far outside the network's
9^3 receptive field: started from the exact converged (u, ps, pt), a solve
still needs 30-75% of the cold iterations, and the network's prediction of
the full-resolution state (flows included) does not lower them.  The solve
therefore runs coarse to fine (asets_solver_run_multilevel, three levels:
32^3, 64^3, 128^3), and the network predicts the initial state of the
coarsest level, where the same receptive field covers a quarter of each
axis.  `level=0` trains and applies it at full resolution instead.

Fallback and judge: the warm solve is accepted when its full-resolution
iterations stay below the cold start's calibrated budget (the median
iterations-to-errBound of cold solves of training problems); otherwise the
problem is solved again from the cold start and that result is used.  The
evaluation solves every held-out problem from the cold start as well, which
judges the warm labelling (label agreement).
"""
from __future__ import annotations

import json
import time
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import native as N
from . import synth

WEIGHTS = Path(__file__).resolve().parent / "weights" / "potts3d_128_l6.npz"
SHAPE = (128, 128, 128)
LABELS = 6
LEVELS = 3
CC, STEPS = 0.3, 0.11
TRAIN_ERR = 1e-5
EVAL_ERR = 1e-4
MAX_IT = 20000
# every solve times the kernel variants for its size once (cached per
# process) and runs the fastest: the coarse levels gain from narrower tiles
AUTOTUNE = True
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


class Level:
    """Device buffers for one level's inputs and state."""

    def __init__(self, solver: N.Solver, L: int):
        import torch

        self.s = solver
        self.shape = (solver.ny, solver.nx, solver.nz)
        self.n = int(np.prod(self.shape))
        n = self.n
        self.ct = torch.empty(n * L, device="cuda")
        self.alpha_full = torch.empty(n * L, device="cuda")
        self.state = [torch.empty(n * L, device="cuda"), torch.empty(n, device="cuda")] + \
            [torch.empty(n * L, device="cuda") for _ in range(4)]  # u, ps, pt, bx, by, bz

    @property
    def alpha(self):
        return self.alpha_full[:self.n]

    def read_inputs(self):
        self.s.get_inputs(None, self.ct, self.alpha_full, where=N.DEVICE)

    def read_state(self):
        """Final (u, ps, pt, bx, by, bz) of this level's last run."""
        u, ps, pt, bx, by, bz = self.state
        self.s.get_u(u, where=N.DEVICE)
        self.s.get_flows(ps, pt, where=N.DEVICE)
        self.s.get_spatial_flows(bx, by, bz, where=N.DEVICE)
        return self.state

    def set_initial(self, st=None):
        if st is None:
            self.s.set_initial(None, None, None)
            return
        u0, ps0, pt0, bx0, by0, bz0 = st
        self.s.set_initial(u0, ps0, pt0, where=N.DEVICE)
        self.s.set_initial_flows(bx0, by0, bz0, where=N.DEVICE)


class Runner:
    """The full-resolution Potts solver and its multilevel chain."""

    def __init__(self, ctx: N.Context | None = None, shape=SHAPE, L: int = LABELS,
                 levels: int = LEVELS):
        self.ctx = ctx or N.Context.default()
        self.shape, self.L = shape, L
        self.n = int(np.prod(shape))
        self.s = N.Solver(self.ctx, "potts", shape, L)
        self.levels = levels
        self.lv: list[Level] = []

    def load(self, ct, alpha_full):
        self.s.set_inputs(ct, alpha_full, where=N.DEVICE)
        got = self.s.multilevel_prepare(self.levels)
        if not self.lv:
            self.lv = [Level(self.s.level(k), self.L) for k in range(got)]
        self.top = self.lv[-1]
        for lv in self.lv:
            lv.read_inputs()

    def cold(self, err: float, max_it: int = MAX_IT) -> int:
        self.lv[0].set_initial(None)
        return self.s.run(max_it, err, CC, STEPS, autotune=AUTOTUNE)

    def warm(self, state, err: float, max_it: int) -> int:
        """Full-resolution solve from `state`."""
        self.lv[0].set_initial(state)
        return self.s.run(max_it, err, CC, STEPS, autotune=AUTOTUNE)

    def multilevel(self, err: float, max_it: int = MAX_IT, top_state=None):
        """Coarse-to-fine solve; the coarsest level starts from `top_state`
        (or cold).  Returns (full-resolution itNum, per-level itNum)."""
        self.top.set_initial(top_state)
        it = self.s.run_multilevel(len(self.lv), max_it, err, CC, STEPS, autotune=AUTOTUNE)
        return it, self.s.multilevel_stats()[0]

    def close(self):
        self.s.close()


def train(train_seeds, *, level: int = LEVELS - 1, epochs: int = 16, lr: float = 2e-3,
          lr_final: float = 1e-4, calib: int = 50, seed: int = 0, log=print):
    """Train a fresh network on cold solutions (errBound 1e-5) of
    `train_seeds` at multilevel `level` (0 = full resolution; pairs kept on
    the device).  The first `calib` seeds also get a full-resolution cold
    solve at errBound 1e-4 for the fallback budget."""
    import torch

    run = Runner()
    net = N.WarmStartNet(run.ctx, nlab=LABELS, seed=seed)
    pairs, cold_iters = [], []
    t0 = time.time()
    for i, sd in enumerate(train_seeds):
        ct, a1, af = problem(sd)
        run.load(ct, af)
        lv = run.lv[level]
        if i < calib:
            cold_iters.append(run.cold(EVAL_ERR))
        lv.set_initial(None)
        lv.s.run(MAX_IT, TRAIN_ERR, CC, STEPS)
        st = [t.clone() for t in lv.read_state()]
        pairs.append((lv.ct.clone(), lv.alpha.clone(), st))
        if log and (i % 250 == 0 or i == len(train_seeds) - 1):
            log(f"pair {i + 1}/{len(train_seeds)} {time.time() - t0:.0f}s")
    gen_s = time.time() - t0
    g = np.random.default_rng(seed)
    total = epochs * len(pairs)
    losses = []
    t1 = time.time()
    order = None
    for k in range(total):
        if k % len(pairs) == 0:
            order = g.permutation(len(pairs))
        ct, a1, st = pairs[order[k % len(pairs)]]
        lr_k = lr_final + 0.5 * (lr - lr_final) * (1 + np.cos(np.pi * k / max(1, total - 1)))
        losses.append(net.train_step(run.lv[level].shape, ct, a1, *st, lr=lr_k))
        if log and (k % 2000 == 0 or k == total - 1):
            log(f"step {k + 1}/{total} loss {np.mean(losses[-200:]):.5f} {time.time() - t1:.0f}s")
    torch.cuda.synchronize()
    run.close()
    info = {"cold_budget": int(np.median(cold_iters)) if cold_iters else MAX_IT,
            "losses": np.array(losses, np.float32), "train_pairs": len(pairs),
            "epochs": epochs, "level": level, "gen_seconds": gen_s,
            "train_seconds": time.time() - t1}
    return net, info


def save(net: N.WarmStartNet, info: dict, path: Path = WEIGHTS) -> None:
    path.parent.mkdir(parents=True, exist_ok=True)
    np.savez(path, params=net.get_params(), cold_budget=info["cold_budget"],
             train_pairs=info["train_pairs"], epochs=info["epochs"], level=info["level"],
             final_loss=float(np.mean(info["losses"][-200:])))


def load(ctx: N.Context | None = None, path: Path = WEIGHTS):
    """(network, cold iteration budget, level it was trained for)."""
    d = np.load(path)
    net = N.WarmStartNet(ctx or N.Context.default(), nlab=LABELS, seed=0)
    net.set_params(d["params"])
    return net, int(d["cold_budget"]), int(d["level"])


@dataclass
class EvalResult:
    seed: int
    cold_it: int
    cold_ms: float              # wall time of the cold solve (init + iterations)
    ml_its: list                # per-level itNum, multilevel with a cold coarsest level
    ml_ms: float
    warm_its: list              # per-level itNum with the learned initial state
    warm_ms: float              # net inference + solve (+ the cold solve on fallback)
    infer_ms: float
    fallback: bool
    agree_cold: float           # warm labels vs cold labels, both at errBound 1e-4
    agree_ml: float             # multilevel (cold coarsest) labels vs cold labels
    agree_tight: float = float("nan")       # warm labels vs a 1e-5 cold solve
    cold_agree_tight: float = float("nan")  # cold 1e-4 labels vs the same
    extra: dict = field(default_factory=dict)


def _sync_ms(fn):
    import torch

    torch.cuda.synchronize()
    t = time.perf_counter()
    r = fn()
    torch.cuda.synchronize()
    return r, 1e3 * (time.perf_counter() - t)


def evaluate(net: N.WarmStartNet, cold_budget: int, seeds, *, level: int = LEVELS - 1,
             tight: bool = True, run: Runner | None = None, log=None) -> list[EvalResult]:
    """Cold vs multilevel vs learned warm start on held-out seeds, errBound
    1e-4.  level = the multilevel level the network predicts (0 = a direct
    full-resolution warm start without the coarse levels)."""
    own = run is None
    run = run or Runner()
    n = run.n
    out = []
    for sd in seeds:
        ct, a1, af = problem(sd)
        run.load(ct, af)
        lv = run.lv[level]
        cold_it, cold_ms = _sync_ms(lambda: run.cold(EVAL_ERR))
        lab_c = labels(run.lv[0].read_state()[0], n).clone()
        (_, ml_its), ml_ms = _sync_ms(lambda: run.multilevel(EVAL_ERR))
        lab_m = labels(run.lv[0].read_state()[0], n).clone()

        def warm_path():
            net.predict(lv.shape, lv.ct, lv.alpha, *lv.state)
            t_inf = time.perf_counter()
            if level == 0:
                it = run.warm(lv.state, EVAL_ERR, cold_budget)
                its = [it]
            else:
                it, its = run.multilevel(EVAL_ERR, MAX_IT, lv.state)
            fb = it >= cold_budget
            if fb:
                run.cold(EVAL_ERR)
            return its, fb, t_inf

        t0 = time.perf_counter()
        (w_its, fb, t_inf), warm_ms = _sync_ms(warm_path)
        lab_w = labels(run.lv[0].read_state()[0], n)
        r = EvalResult(sd, cold_it, cold_ms, ml_its, ml_ms, w_its, warm_ms,
                       1e3 * (t_inf - t0), fb, float((lab_w == lab_c).float().mean()),
                       float((lab_m == lab_c).float().mean()))
        if tight:
            # both solved to errBound 1e-5 as well: time and label agreement
            it_t, ms_t = _sync_ms(lambda: run.cold(TRAIN_ERR))
            lab_t = labels(run.lv[0].read_state()[0], n).clone()
            r.agree_tight = float((lab_w == lab_t).float().mean())
            r.cold_agree_tight = float((lab_c == lab_t).float().mean())
            r.extra["ml_agree_tight"] = float((lab_m == lab_t).float().mean())
            if level > 0:
                def warm_tight():
                    net.predict(lv.shape, lv.ct, lv.alpha, *lv.state)
                    return run.multilevel(TRAIN_ERR, MAX_IT, lv.state)
                (_, its5), ms5 = _sync_ms(warm_tight)
                lab5 = labels(run.lv[0].read_state()[0], n)
                r.extra.update(cold5_it=it_t, cold5_ms=ms_t, warm5_its=its5, warm5_ms=ms5,
                               agree5=float((lab5 == lab_t).float().mean()))
        out.append(r)
        if log:
            log(f"seed {sd}: cold {cold_it} it {cold_ms:.1f} ms | multilevel {ml_its} "
                f"{ml_ms:.1f} ms | learned {w_its} {warm_ms:.1f} ms (net {r.infer_ms:.1f} ms)"
                f"{' FALLBACK' if fb else ''} | agree cold {r.agree_cold:.4f} "
                f"(multilevel {r.agree_ml:.4f}) tight {r.agree_tight:.4f} "
                f"(cold {r.cold_agree_tight:.4f})")
    if own:
        run.close()
    return out


def evaluate_batched(net: N.WarmStartNet, cold_budget: int, seeds, *, level: int = LEVELS - 1,
                     runs: list | None = None) -> dict:
    """The batched form on held-out seeds: every problem solved in one batch
    (asets_batch_*), cold -- one batch of the full-resolution solvers --
    against the learned warm start -- the network's coarsest-level state for
    each problem, then one batch per level (asets_batch_run_multilevel),
    members whose full-resolution iterations reach the cold budget solved
    again cold as one batch.  Wall times of the whole batch, per-member
    iterations and label agreement with the cold batch's labels."""
    own = runs is None
    runs = runs or [Runner() for _ in seeds]
    for run, sd in zip(runs, seeds):
        ct, a1, af = problem(sd)
        run.load(ct, af)
    ctx = runs[0].ctx
    cold = N.Batch(ctx)
    for run in runs:
        run.lv[0].set_initial(None)
        cold.add(run.s)
    cold_its, cold_ms = _sync_ms(lambda: cold.run(MAX_IT, EVAL_ERR, CC, STEPS, autotune=AUTOTUNE))
    lab_c = [labels(run.lv[0].read_state()[0], run.n).clone() for run in runs]
    cold.close()

    warm = N.Batch(ctx)
    for run in runs:
        warm.add(run.s)

    def warm_path():
        for run in runs:
            lv = run.lv[level]
            net.predict(lv.shape, lv.ct, lv.alpha, *lv.state)
            lv.set_initial(lv.state)
        its = warm.run_multilevel(len(runs[0].lv), MAX_IT, EVAL_ERR, CC, STEPS,
                                  autotune=AUTOTUNE)
        fb = [i for i, it in enumerate(its) if it >= cold_budget]
        if fb:
            again = N.Batch(ctx)
            for i in fb:
                runs[i].lv[0].set_initial(None)
                again.add(runs[i].s)
            again.run(MAX_IT, EVAL_ERR, CC, STEPS, autotune=AUTOTUNE)
            again.close()
        return its, fb

    (warm_its, fb), warm_ms = _sync_ms(warm_path)
    level_its = [run.s.multilevel_stats()[0] for run in runs]
    agree = [float((labels(run.lv[0].read_state()[0], run.n) == lc).float().mean())
             for run, lc in zip(runs, lab_c)]
    warm.close()
    if own:
        for run in runs:
            run.close()
    return {"problems": len(runs), "cold_batch_ms": cold_ms, "warm_batch_ms": warm_ms,
            "wall_ratio_cold_over_warm": cold_ms / warm_ms,
            "cold_iters": list(cold_its), "warm_iters": list(warm_its),
            "warm_level_iters": level_its, "fallbacks": len(fb),
            "agree_cold_mean": float(np.mean(agree)), "agree_cold_min": float(min(agree))}


def potts_energy(ct, alpha_full, u, shape, L: int = LABELS) -> float:
    """Relaxed Potts energy of a labelling function u (torch, Matlab layout,
    label slowest), in float64: sum over labels and voxels of u_l Ct_l plus
    alpha_l times the per-voxel gradient norm sqrt(0.5 * sum of the squared
    differences across the voxel's 2*dim faces), the norm the solver's
    projection bounds the flows with (|p| <= alpha,
    maxflow/asetsPotts3D_mex.c:342-374); faces on the volume's border carry
    no difference.  A one-hot u gives the discrete Potts energy of its
    labelling."""
    ny, nx, nz = shape
    U = u.reshape(L, nz, nx, ny).double()
    data = float((U * ct.reshape(L, nz, nx, ny).double()).sum())
    g2 = U.new_zeros(U.shape)
    for d in (1, 2, 3):
        if U.shape[d] < 2:
            continue
        f2 = U.diff(dim=d) ** 2
        n = U.shape[d]
        g2.narrow(d, 0, n - 1).add_(f2)
        g2.narrow(d, 1, n - 1).add_(f2)
    tv = float((alpha_full.reshape(L, nz, nx, ny).double() * (0.5 * g2).sqrt()).sum())
    return data + tv


def one_hot(lab, n: int, L: int = LABELS):
    """Labels (n,) -> a one-hot u in Matlab layout (label slowest)."""
    import torch

    return torch.nn.functional.one_hot(lab, L).T.reshape(-1).float()


def diagnose(net: N.WarmStartNet, seeds, *, level: int = LEVELS - 1, run: Runner | None = None,
             log=None) -> list[dict]:
    """Per held-out problem: why the warm-started labelling differs from the
    cold one.  Solves cold and warm (learned coarsest state, coarse to fine)
    to errBound 1e-4 and to 1e-5, and reports for each of the four results
    the relaxed Potts energy of u and the discrete energy of its argmax
    labelling, with the label agreements, the smallest gap between two label
    means, the share of voxels whose cold top-two u margin exceeds 0.1 and
    the agreement on them, and the label pair that accounts for most of the
    disagreement."""
    import torch

    own = run is None
    run = run or Runner()
    n, L = run.n, run.L
    out = []
    for sd in seeds:
        means = synth.potts_warmstart_draws(sd)[0]
        ct, a1, af = problem(sd)
        run.load(ct, af)
        lv = run.lv[level]
        res = {}
        for err, tag in ((EVAL_ERR, "4"), (TRAIN_ERR, "5")):
            it_c = run.cold(err)
            u_c = run.lv[0].read_state()[0].clone()
            net.predict(lv.shape, lv.ct, lv.alpha, *lv.state)
            it_w, _ = run.multilevel(err, MAX_IT, lv.state)
            u_w = run.lv[0].read_state()[0].clone()
            res[tag] = (it_c, u_c, it_w, u_w)
        r = {"seed": int(sd), "alpha": float(a1[0]),
             "means": [round(float(m), 4) for m in means],
             "min_mean_gap": float(np.min(np.diff(np.sort(means))))}
        labs = {}
        for tag, (it_c, u_c, it_w, u_w) in res.items():
            lc, lw = labels(u_c, n, L), labels(u_w, n, L)
            labs["c" + tag], labs["w" + tag] = lc, lw
            r[f"cold{tag}_it"], r[f"warm{tag}_it"] = int(it_c), int(it_w)
            r[f"cold{tag}_E"] = potts_energy(ct, af, u_c, run.shape, L)
            r[f"warm{tag}_E"] = potts_energy(ct, af, u_w, run.shape, L)
            r[f"cold{tag}_Elab"] = potts_energy(ct, af, one_hot(lc, n, L), run.shape, L)
            r[f"warm{tag}_Elab"] = potts_energy(ct, af, one_hot(lw, n, L), run.shape, L)
            r[f"agree{tag}"] = float((lc == lw).float().mean())
        r["cold4_vs_cold5"] = float((labs["c4"] == labs["c5"]).float().mean())
        r["warm4_vs_cold5"] = float((labs["w4"] == labs["c5"]).float().mean())
        top2 = res["4"][1].view(L, n).topk(2, dim=0).values
        conf = (top2[0] - top2[1]) > 0.1
        r["confident_share"] = float(conf.float().mean())
        r["agree4_confident"] = float((labs["c4"] == labs["w4"])[conf].float().mean()) \
            if bool(conf.any()) else float("nan")
        diff = labs["c4"] != labs["w4"]
        if bool(diff.any()):
            pair = labs["c4"][diff] * L + labs["w4"][diff]
            cnt = torch.bincount(pair, minlength=L * L)
            k = int(cnt.argmax())
            a, b = divmod(k, L)
            r["top_pair"] = [a, b]
            r["top_pair_share"] = float(cnt[k]) / float(diff.sum())
            r["top_pair_gap"] = float(abs(means[a] - means[b]))
        out.append(r)
        if log:
            log(json.dumps(r))
    if own:
        run.close()
    return out


def summarize(res: list[EvalResult]) -> dict:
    c_it = np.array([r.cold_it for r in res], float)
    w_it = np.array([r.warm_its[0] + (r.cold_it if r.fallback else 0) for r in res], float)
    m_it = np.array([r.ml_its[0] for r in res], float)
    c_ms = np.array([r.cold_ms for r in res])
    w_ms = np.array([r.warm_ms for r in res])
    m_ms = np.array([r.ml_ms for r in res])
    top_m = np.array([r.ml_its[-1] for r in res], float)
    top_w = np.array([r.warm_its[-1] for r in res], float)
    return {
        "problems": len(res),
        "cold_iters_mean": float(c_it.mean()),
        "multilevel_iters_mean": float(m_it.mean()),
        "warm_iters_mean": float(w_it.mean()),
        "coarsest_iters_cold_start_mean": float(top_m.mean()),
        "coarsest_iters_learned_mean": float(top_w.mean()),
        "cold_ms_mean": float(c_ms.mean()), "multilevel_ms_mean": float(m_ms.mean()),
        "warm_ms_mean": float(w_ms.mean()),
        "infer_ms_mean": float(np.mean([r.infer_ms for r in res])),
        "wall_ratio_cold_over_warm": float(c_ms.sum() / w_ms.sum()),
        "wall_ratio_cold_over_multilevel": float(c_ms.sum() / m_ms.sum()),
        "wall_ratio_multilevel_over_warm": float(m_ms.sum() / w_ms.sum()),
        "fallbacks": int(sum(r.fallback for r in res)),
        "regressions": int(sum((not r.fallback) and r.warm_its[0] >= r.cold_it for r in res)),
        "agree_cold_mean": float(np.mean([r.agree_cold for r in res])),
        "agree_cold_min": float(min(r.agree_cold for r in res)),
        "agree_cold_ge_999": int(sum(r.agree_cold >= 0.999 for r in res)),
        "agree_ml_mean": float(np.mean([r.agree_ml for r in res])),
        **_summary_tight(res),
        **_summary_1e5(res),
    }


def _summary_tight(res) -> dict:
    t = [r for r in res if np.isfinite(r.agree_tight)]
    if not t:
        return {}
    return {"agree_tight_mean": float(np.mean([r.agree_tight for r in t])),
            "cold_agree_tight_mean": float(np.mean([r.cold_agree_tight for r in t]))}


def _summary_1e5(res) -> dict:
    ex = [r.extra for r in res if "warm5_ms" in r.extra]
    if not ex:
        return {}
    c = np.array([e["cold5_ms"] for e in ex])
    w = np.array([e["warm5_ms"] for e in ex])
    return {"err1e5_cold_ms_mean": float(c.mean()), "err1e5_warm_ms_mean": float(w.mean()),
            "err1e5_cold_iters_mean": float(np.mean([e["cold5_it"] for e in ex])),
            "err1e5_warm_iters_mean": float(np.mean([e["warm5_its"][0] for e in ex])),
            "err1e5_wall_ratio": float(c.sum() / w.sum()),
            "err1e5_agree_mean": float(np.mean([e["agree5"] for e in ex])),
            "err1e5_agree_min": float(min(e["agree5"] for e in ex)),
            "err1e5_agree_ge_999": int(sum(e["agree5"] >= 0.999 for e in ex))}


def main(argv=None):
    """python -m asetsmatlabmaxflow_gb300.warmstart --train N --eval M"""
    import argparse

    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=2000, help="training pairs (seeds 0..N-1)")
    ap.add_argument("--eval", type=int, default=200, help="held-out seeds")
    ap.add_argument("--level", type=int, default=LEVELS - 1)
    ap.add_argument("--epochs", type=int, default=16)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--out", type=Path, default=WEIGHTS)
    ap.add_argument("--no-tight", action="store_true")
    ap.add_argument("--eval-only", action="store_true")
    ap.add_argument("--results", type=Path, default=None, help="per-seed results (JSON)")
    ap.add_argument("--diagnose", action="store_true",
                    help="per-seed energies and agreements of cold and warm solves "
                         "(committed weights)")
    a = ap.parse_args(argv)
    if a.diagnose:
        net, budget, level = load(path=a.out)
        rows = diagnose(net, range(HELDOUT_SEED0, HELDOUT_SEED0 + a.eval), level=level,
                        log=print)
        if a.results:
            a.results.write_text(json.dumps(rows, indent=1))
        return
    if a.eval_only:
        net, budget, level = load(path=a.out)
    else:
        net, info = train(range(a.train), level=a.level, epochs=a.epochs, lr=a.lr)
        save(net, info, a.out)
        budget, level = info["cold_budget"], a.level
        print(json.dumps({"train_pairs": a.train, "level": level, "cold_budget": budget,
                          "gen_seconds": round(info["gen_seconds"], 1),
                          "train_seconds": round(info["train_seconds"], 1),
                          "final_loss": float(np.mean(info["losses"][-200:]))}), flush=True)
    res = evaluate(net, budget, range(HELDOUT_SEED0, HELDOUT_SEED0 + a.eval), level=level,
                   tight=not a.no_tight, log=print)
    summary = summarize(res)
    print(json.dumps(summary), flush=True)
    if a.results:
        from dataclasses import asdict

        a.results.write_text(json.dumps({"summary": summary,
                                         "per_seed": [asdict(r) for r in res]}, indent=1))


if __name__ == "__main__":
    main()
