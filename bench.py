"""Benchmark: binary continuous max-flow 3D, 256^3 float32, 200 fixed ALM
iterations per step (the throughput run of the binary 3D workload).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

One JSON line on rank 0.  `value` is whole-job Gvoxel-iter/s with inputs
resident in HBM; `e2e` the same through the C ABI one-shot call
(asets_binary_mf3d) from pinned host buffers, host<->device copies included.
`roofline` relates the fused iteration kernel's algorithmic bytes (60 B per
voxel-iteration: 6 state arrays read+written, 3 inputs read) to the measured
HBM copy bandwidth.  `--impl reference` times the CPU restatement of the
reference C solver (bit-identical to it) on all host cores, one independent
solve per core.  Under torchrun each rank solves its own volume (weak
scaling, replicas only: the path has no exchange between problems).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Gvoxel-iter/s (binary 3D 256^3); time-to-errBound, learned warm vs cold start"
UNIT = "Gvoxel-iter/s"
SHAPE = (256, 256, 256)
ITERS = 200
CC, STEPS = 0.35, 0.11
BYTES_PER_VOXEL_ITER = 60  # 6 state arrays x (read + write) x 4 B + 3 inputs x 4 B
WORKLOAD = "binary3d_256^3_200it"


def workload_config(world: int) -> dict:
    """The `config` of both arms' JSON lines (the same dict, so the two lines
    name the same workload)."""
    return {"workload": WORKLOAD, "model": "binary continuous max-flow 3D",
            "shape": list(SHAPE), "iterations_per_step": ITERS, "cc": CC, "steps": STEPS,
            "err_bound": 0.0, "parallelism": f"replicas{world}",
            "l2": "working set ~1 GB per iteration, larger than L2; no flush",
            "voronoi_cells": 40, "intensities": [0.25, 0.75], "noise": 0.2}


def host_cores() -> int:
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-solver measurement")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the binary 2D / Potts 3D / Ishikawa 2D workloads")
    ap.add_argument("--no-next", action="store_true",
                    help="skip the hierarchical/DAG, Matlab-semantics, star-shape and cost-term "
                         "measurements")
    ap.add_argument("--warm-seeds", type=int, default=4,
                    help="held-out Potts problems for the warm-start comparison (0: skip)")
    ap.add_argument("--profile-iters", type=int, default=0,
                    help="run one solve of N iterations of the workload and exit (for ncu)")
    ap.add_argument("--shape", default="256,256,256", help="volume for --profile-iters")
    ap.add_argument("--tile-config", type=int, default=0, help="kernel variant for --profile-iters")
    ap.add_argument("--profile-model", default="binary",
                    choices=["binary", "potts", "potts192", "ishikawa1024", "potts2048", "hmf",
                             "dag", "costs", "matlab3d", "starshape"],
                    help="model for --profile-iters (potts: the warm-start workload, seed 1000000; "
                         "potts192: Potts 3D 192^3 L=4; ishikawa1024: Ishikawa 2D 1024^2 L=8; "
                         "potts2048: Potts 2D 2048^2 L=4 (the Ishikawa field's Ct, alpha 0.2); "
                         "hmf / dag: the 1024^2 six-node tree / graph of the `next` entries; "
                         "costs: N pairs of L1-cost and contrast-alpha calls on 256^3; "
                         "matlab3d: Matlab-semantics binary 3D 256^3; starshape: 512^2 L=4)")
    ap.add_argument("--profile-conv", type=int, default=0,
                    help="run the warm-start network's forward pass on an S^3 volume and exit")
    return ap.parse_args()


def profile_conv(args):
    """Five forward passes of the warm-start network (committed weights) on
    an S^3 volume of 6 labels, for profilers."""
    import torch

    from asetsmatlabmaxflow_gb300 import warmstart as W

    net, _, _ = W.load()
    n = args.profile_conv ** 3
    dims = (args.profile_conv,) * 3
    g = torch.Generator(device="cuda").manual_seed(0)
    ct = torch.rand(n * 6, device="cuda", generator=g)
    a = torch.full((n,), 0.3, device="cuda")
    outs = [torch.empty(n * 6, device="cuda"), torch.empty(n, device="cuda")] + \
        [torch.empty(n * 6, device="cuda") for _ in range(4)]
    net.predict(dims, ct, a, *outs)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(5):
        net.predict(dims, ct, a, *outs)
    torch.cuda.synchronize()
    ms = 1e3 * (time.perf_counter() - t0) / 5
    print(json.dumps({"profile_conv": list(dims), "conv_launches": 5 * 5,
                      "predict_ms": ms}))


def profile_run(args):
    """One solve of the benchmark problem (or a smaller volume) for profilers."""
    from asetsmatlabmaxflow_gb300 import native as N
    from asetsmatlabmaxflow_gb300 import synth

    if args.profile_model == "potts":
        from asetsmatlabmaxflow_gb300 import warmstart as W

        run = W.Runner()
        ct6, a1, af = W.problem(W.HELDOUT_SEED0)
        run.load(ct6, af)
        it = run.s.run(args.profile_iters, 0.0, W.CC, W.STEPS, tile_config=args.tile_config)
        ms, n = run.s.last_run_stats()
        print(json.dumps({"profile_run": "potts 128^3 L=6", "iterations": it,
                          "ms_per_iteration": ms / max(args.profile_iters, 1)}))
        return
    if args.profile_model in ("hmf", "dag"):
        from asetsmatlabmaxflow_gb300 import hmf as HM

        make = _hmf_tree if args.profile_model == "hmf" else _dag_graph
        cls = HM.asetsHMF2D if args.profile_model == "hmf" else HM.asetsDAGMF2D
        make(cls, (1024, 1024), np.float32, 0).MaxFullFlow(args.profile_iters, 0.1, 0.25)
        print(json.dumps({"profile_run": f"{args.profile_model} 1024x1024, 6 nodes",
                          "iterations": args.profile_iters}))
        return
    if args.profile_model == "matlab3d":
        from asetsmatlabmaxflow_gb300 import matlab as M

        cs, ct, al = synth.binary3d(seed=0, shape=(256, 256, 256))
        M.asetsBinaryMF3D(cs, ct, al, [256, 256, 256, args.profile_iters, 0.0, 0.35, 0.11])
        print(json.dumps({"profile_run": "matlab binary 3D 256^3", "iterations": args.profile_iters}))
        return
    if args.profile_model == "starshape":
        from asetsmatlabmaxflow_gb300 import starshape as SS

        g = np.random.default_rng(0)
        ct = g.random((512, 512, 4))
        al = 0.1 + 0.3 * g.random((512, 512, 4))
        pts = np.array([[64, 64], [448, 64], [64, 448], [448, 448]])
        SS.asetsPotts2D_starShape(ct, al, [512, 512, 4, args.profile_iters, 0.0, 0.25, 0.11, 0.05],
                                  pts)
        print(json.dumps({"profile_run": "star-shape Potts 2D 512^2 L=4",
                          "iterations": args.profile_iters}))
        return
    if args.profile_model == "costs":
        import torch

        cs, ct, al = synth.binary3d(seed=0, shape=(256, 256, 256))
        img = torch.from_numpy(ct.ravel(order="F").copy()).cuda()
        out = torch.empty(img.numel() * 4, device="cuda")
        models = np.array([0.2, 0.4, 0.6, 0.8], np.float32)
        h = N.Context.default().handle
        for _ in range(args.profile_iters):
            N.check(N.lib().asets_cost_l1(h, N.DEVICE, img.data_ptr(), img.numel(),
                                          models.ctypes.data, 4, 1, out.data_ptr()))
            N.check(N.lib().asets_alpha_contrast(h, N.DEVICE, img.data_ptr(), 256, 256, 256, 1,
                                                 0.1, 0.9, 10.0, 1, 1, out.data_ptr()))
        torch.cuda.synchronize()
        print(json.dumps({"profile_run": "costs 256^3", "calls": args.profile_iters}))
        return
    if args.profile_model in ("potts192", "ishikawa1024", "potts2048"):
        # the multi-region configurations: cc 0.3, steps 0.11 (3D) / 0.16 (2D)
        if args.profile_model == "potts192":
            ct, a = synth.potts3d(seed=0)
            model, dims, L, steps = "potts", ct.shape[:3], ct.shape[3], 0.11
        elif args.profile_model == "potts2048":
            ct, _ = synth.ishikawa2d(seed=0, shape=(2048, 2048), L=4)
            a = np.full(ct.shape, 0.2, np.float32, order="F")
            model, dims, L, steps = "potts", ct.shape[:2], ct.shape[2], 0.16
        else:
            ct, a = synth.ishikawa2d(seed=0)
            model, dims, L, steps = "ishikawa", ct.shape[:2], ct.shape[2], 0.16
        s = N.Solver(N.Context.default(), model, dims, L)
        s.set_inputs(ct, a)
        it = s.run(args.profile_iters, 0.0, 0.3, steps, tile_config=args.tile_config)
        ms, n = s.last_run_stats()
        print(json.dumps({"profile_run": f"{model} {'x'.join(map(str, dims))} L={L}",
                          "iterations": it, "ms_per_iteration": ms / max(args.profile_iters, 1)}))
        return
    shape = tuple(int(x) for x in args.shape.split(","))
    cs, ct, alpha = synth.binary3d(seed=0, shape=shape)
    s = N.Solver(N.Context.default(), "binary", shape)
    s.set_inputs(ct, alpha, cs)
    it = s.run(args.profile_iters, 0.0, CC, STEPS, tile_config=args.tile_config)
    ms, n = s.last_run_stats()
    print(json.dumps({"profile_run": list(shape), "tile_config": args.tile_config,
                      "iterations": it, "ms_per_launch": ms / max(n, 1)}))


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
        pg = dist
    return world, rank, local, pg


def max_over_ranks(pg, x: float) -> float:
    if pg is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def barrier(pg):
    if pg is not None:
        pg.barrier()


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except (KeyError, ValueError):
            pass
    return 6800.0, "fallback"


def traffic_per_launch():
    """DRAM bytes of one fused iteration launch on this workload, from the
    committed ncu summary (profiles/), or None."""
    p = ROOT / "profiles" / "binary3d_256_traffic.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["dram_bytes_per_launch"])
        except (KeyError, ValueError):
            return None
    return None


def batch_run(ctx, cpu: bool) -> dict:
    """Batched workload: 48 binary 2D (sides 128..1024) + 16 binary 3D (sides
    64..160) problems, alpha ~ U[0.2, 0.8], errBound 1e-4, one persistent
    launch per dimension and iteration, autotuned tile variant."""
    from asetsmatlabmaxflow_gb300 import native as N
    from asetsmatlabmaxflow_gb300 import synth

    probs = synth.batch_problems(seed=0)
    solvers = []
    for cs, ct, alpha in probs:
        s = N.Solver(ctx, "binary", cs.shape)
        s.set_inputs(ct, alpha, cs)
        solvers.append(s)
    b = N.Batch(ctx)
    for s in solvers:
        b.add(s)
    cc_, steps_ = 0.3, 0.16
    b.run(2000, 1e-4, cc_, steps_, autotune=True)  # tune + warm-up
    its = b.run(2000, 1e-4, cc_, steps_, autotune=True)
    st = b.last_run_stats()
    vox = sum(float(np.prod(p[0].shape)) * (i + 1) for p, i in zip(probs, its))
    out = {"workload": "48 binary 2D (128..1024 per side) + 16 binary 3D (64..160 per side), "
                       "errBound 1e-4, cc 0.3, steps 0.16",
           "unit": "Gvoxel-iter/s",
           "problems": len(probs), "ms_to_errbound_all": st["ms"],
           "iterations_summed": st["iterations"], "max_iterations": max(its) + 1,
           "gvoxel_iter_per_s": vox / (st["ms"] * 1e-3) / 1e9,
           "tile_config_2d": st["tile_config_2d"], "tile_config_3d": st["tile_config_3d"],
           "launches": st["launches"]}
    b.close()
    for s in solvers:
        s.close()
    if cpu:
        out["cpu_baseline"] = batch_cpu_baseline(probs, cc_, steps_)
    return out


def batch_cpu_baseline(probs, cc_: float, steps_: float, iters: int = 20) -> dict:
    """The batch on the host: every problem solved by the oracle (the
    reference's C solver restated, bit-identical to it) for `iters`
    iterations, one single-thread solve per host core at a time; aggregate
    voxel-iterations per second over all cores."""
    from concurrent.futures import ThreadPoolExecutor

    from oracle import oracle as O

    cores = host_cores()

    def one(p):
        cs, ct, alpha = p
        O.solve("binary", cs.shape, ct, alpha, cs=cs, max_it=iters, err_bound=0.0, cc=cc_,
                steps=steps_)

    O.lib()
    order = sorted(probs, key=lambda p: -p[0].size)  # largest first: even finish
    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=cores) as ex:
        list(ex.map(one, order))
    dt = time.perf_counter() - t0
    vox = sum(float(p[0].size) for p in probs) * iters
    return {"value": vox / dt / 1e9, "unit": "Gvoxel-iter/s", "cores": cores, "kind": "port",
            "seconds": dt,
            "sample": f"all {len(probs)} problems, {iters} iterations each incl. init, "
                      f"{cores} concurrent single-thread solves (C restatement)"}


def config_cpu_baseline(model, dims, L, inputs, steps_, iters) -> dict:
    """One single-thread oracle solve of a `configs` workload, `iters`
    iterations (init included); inputs are (Ct, alpha[, Cs])."""
    from oracle import oracle as O

    ct, alpha = inputs[0], inputs[1]
    cs = inputs[2] if len(inputs) > 2 else None
    t0 = time.perf_counter()
    O.solve(model, dims, ct, alpha, cs=cs, nlab=L, max_it=iters, err_bound=0.0, cc=0.3,
            steps=steps_)
    dt = time.perf_counter() - t0
    nvox = float(np.prod(dims))
    return {"value": nvox * iters / dt / 1e9, "unit": "Gvoxel-iter/s", "cores": 1,
            "kind": "port", "seconds": dt,
            "sample": f"{iters} iterations incl. init, 1 thread, same input "
                      "(C restatement, bit-identical to the reference C)"}


def configs_run(ctx, cpu: bool) -> list:
    """The other workloads of the metric, each on its own solver: binary 2D
    256^2 (pars [256,256,300,1e-4,0.3,0.16]), Potts 3D 192^3 L=4 and
    Ishikawa 2D 1024^2 L=8 (cc 0.3, steps 0.11 / 0.16).  Per workload: 100
    fixed iterations (errBound 0) give the device time per iteration (both
    passes of a labelled iteration) and its algorithmic-byte roofline, then
    one solve to errBound 1e-4.  Variants autotuned (ASETS_FLAG_AUTOTUNE)."""
    from asetsmatlabmaxflow_gb300 import native as N
    from asetsmatlabmaxflow_gb300 import synth

    peak, peak_kind = peaks()
    rows = []
    cs2, ct2, a2 = synth.binary2d(seed=0)
    ct3, a3 = synth.potts3d(seed=0)
    cti, ai = synth.ishikawa2d(seed=0)
    # name, model, dims, labels, inputs, steps, maxIt, bytes per voxel-iteration,
    # iterations of the single-thread CPU sample
    table = (
        ("binary2d_256^2", "binary", cs2.shape, 1, (ct2, a2, cs2), 0.16, 300, 52, 300),
        ("potts3d_192^3_L4", "potts", ct3.shape[:3], ct3.shape[3], (ct3, a3), 0.11, 2000,
         48 * ct3.shape[3] + 8, 4),
        ("ishikawa2d_1024^2_L8", "ishikawa", cti.shape[:2], cti.shape[2], (cti, ai), 0.16, 2000,
         (4 * cti.shape[2] - 3) * 8 + (2 * cti.shape[2] - 1) * 4, 20),
    )
    fixed = 100
    for name, model, dims, L, inputs, steps_, max_it, bpv, cpu_its in table:
        s = N.Solver(ctx, model, dims, L) if model != "binary" else N.Solver(ctx, model, dims)
        s.set_inputs(*inputs)
        nvox = int(np.prod(dims))
        s.run(fixed, 0.0, 0.3, steps_, autotune=True)  # tune + warm-up
        s.run(fixed, 0.0, 0.3, steps_, autotune=True)
        ms, _ = s.last_run_stats()
        it_ms = ms / fixed
        achieved = bpv * nvox / (it_ms * 1e-3) / 1e9
        it = s.run(max_it, 1e-4, 0.3, steps_, autotune=True)
        conv_ms, _ = s.last_run_stats()
        rows.append({"workload": name, "voxels": nvox, "labels": L,
                     "gvoxel_iter_per_s": nvox / (it_ms * 1e-3) / 1e9,
                     "ms_per_iteration": it_ms, "bytes_per_voxel_iter": bpv,
                     "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                                  "unit": "GB/s", "frac": achieved / peak,
                                  "peak_kind": peak_kind},
                     "err_bound": 1e-4, "max_it": max_it, "itnum": it,
                     "ms_to_errbound": conv_ms})
        if cpu:
            rows[-1]["cpu_baseline"] = config_cpu_baseline(model, dims, L, inputs, steps_,
                                                            cpu_its)
        s.close()
    return rows


def _per_iteration_s(solve, n: int) -> float:
    """Seconds per iteration of a synchronous host-array solve: the slope of
    the wall time of n-, 2n- and 4n-iteration solves (best of three each;
    copies and set-up do not depend on the iteration count).  While the
    iterations are not at least twice the fixed part of the n-iteration
    solve's time, or the slope is not positive, n grows fourfold (at most
    three times), so that host copy noise cannot swamp the iteration time."""
    import torch

    def wall(k):
        best = float("inf")
        for _ in range(3):
            torch.cuda.synchronize()
            t = time.perf_counter()
            solve(k)
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - t)
        return best

    solve(2)  # warm-up
    for _ in range(4):
        ks = np.array([n, 2 * n, 4 * n], float)
        ts = np.array([wall(int(k)) for k in ks])
        slope = float(np.polyfit(ks, ts, 1)[0])
        if slope > 0 and slope * n >= 2.0 * (ts[0] - slope * n):
            break
        n *= 4
    if slope <= 0:
        # not resolved above host noise: the longest call's time per
        # iteration, fixed costs included, bounds it from above
        return float(ts[2] / ks[2])
    return slope


def _hmf_tree(make, shape, dt, seed):
    """Five leaves (Ct = sqrt|I - i/4|), the first two under an inner node."""
    g = np.random.default_rng(seed)
    img = g.random(shape).astype(dt)
    leaves = [make([], 0.15, np.sqrt(np.abs(img - dt(i / 4))).astype(dt)) for i in range(5)]
    return make([make(leaves[:2], 0.2)] + leaves[2:], 0)


def _dag_graph(make, shape, dt, seed):
    """Four leaves, two inner nodes sharing two of them."""
    g = np.random.default_rng(seed)
    img = g.random(shape).astype(dt)
    L = [make([], 0.15, np.abs(img - dt(i / 3)).astype(dt)) for i in range(4)]
    return make([make([L[0], L[1], L[2]], 0.2), make([L[1], L[2], L[3]], 0.25)], 0)


def next_rows_run(ctx, stream, cpu: bool) -> list:
    """The solvers beside the mex path (hierarchical / DAG max-flow, the
    Matlab-semantics solvers, star-shape Potts 2D) and the cost-term kernels:
    device time per iteration (host-array solves: difference of two solve
    lengths; cost kernels: CUDA events on device arrays), rate against the
    algorithmic bytes, and (cpu) the numpy restatement timed on one core for
    a few iterations of the same problem, after every GPU row is timed (a
    numpy restatement's large temporaries disturbed the next host-array
    timing).  `stream` is the context's stream."""
    import torch

    from asetsmatlabmaxflow_gb300 import costs as K
    from asetsmatlabmaxflow_gb300 import hmf as HM
    from asetsmatlabmaxflow_gb300 import matlab as M
    from asetsmatlabmaxflow_gb300 import native as N
    from asetsmatlabmaxflow_gb300 import starshape as SS
    from asetsmatlabmaxflow_gb300 import synth

    peak, peak_kind = peaks()
    rows = []
    pending_cpu = []

    def row(name, units, unit_name, bytes_per_unit, bytes_note, sec_per_it, cpu_fn=None,
            cpu_its=0, dtype="f32"):
        r = {"workload": name, "dtype": dtype, "ms_per_iteration": 1e3 * sec_per_it,
             f"g{unit_name}_per_s": units / sec_per_it / 1e9,
             "bytes_per_unit": bytes_per_unit, "bytes": bytes_note,
             "roofline": {"bound": "hbm", "achieved": units * bytes_per_unit / sec_per_it / 1e9,
                          "peak": peak, "unit": "GB/s",
                          "frac": units * bytes_per_unit / sec_per_it / 1e9 / peak,
                          "peak_kind": peak_kind}}
        if cpu and cpu_fn is not None:
            pending_cpu.append((r, cpu_fn, cpu_its, units, unit_name))
        rows.append(r)

    shape2 = (1024, 1024)
    npix = shape2[0] * shape2[1]
    # hierarchical max-flow, float32: 6 nodes below the root (5 leaves)
    state = {}

    def hmf(k):
        if "h" not in state:
            state["h"] = _hmf_tree(HM.asetsHMF2D, shape2, np.float32, 0)
        state["h"].MaxFullFlow(k, 0.1, 0.25, ctx=ctx)

    def hmf_cpu(k):
        from oracle import hmf as OH
        _hmf_tree(OH.Node, shape2, np.float32, 0).max_full_flow(k, 0.1, 0.25)

    row("hmf2d_1024^2_6nodes_full_flow", 6 * npix, "node-pixel-iter", 32 + 4 * 5 / 6 + 8 / 6,
        "per node-pixel: px, py, pt, u read+written; Ct of the 5 leaves and the root's pt",
        _per_iteration_s(hmf, 20), hmf_cpu, 2)

    def dag(k):
        if "d" not in state:
            state["d"] = _dag_graph(HM.asetsDAGMF2D, shape2, np.float32, 0)
        state["d"].MaxFullFlow(k, 0.1, 0.25, ctx=ctx)

    def dag_cpu(k):
        from oracle import dag as OD
        _dag_graph(OD.Node, shape2, np.float32, 0).max_full_flow(k, 0.1, 0.25)

    row("dag2d_1024^2_6nodes_full_flow", 6 * npix, "node-pixel-iter", 32 + 4 * 4 / 6 + 8 / 6,
        "per node-pixel: px, py, pt, u read+written; Ct of the 4 leaves and the root's pt "
        "(the shared children's pn not counted)", _per_iteration_s(dag, 20), dag_cpu, 2)

    # Matlab-semantics binary 3D, float32, 256^3 (never breaks: errBound 0, '<' rule)
    cs, ct, al = synth.binary3d(seed=0, shape=(256, 256, 256))
    nvox = cs.size

    def mt3(k):
        M.asetsBinaryMF3D(cs, ct, al, [256, 256, 256, k, 0.0, 0.35, 0.11], ctx=ctx)

    def mt3_cpu(k):
        from oracle import mtwin as OM
        OM.binary(cs, ct, al, k, 0.0, 0.35, 0.11)

    row("matlab_binary3d_256^3", nvox, "voxel-iter", 60,
        "bx, by, bz, ps, pt, u read+written, Cs, Ct, alpha read (fp32)",
        _per_iteration_s(mt3, 20), mt3_cpu, 2)

    # Matlab-semantics Potts 2D, float64, 1024^2 L=4
    g = np.random.default_rng(0)
    ctp = g.random(shape2 + (4,))
    alp = np.full(shape2 + (4,), 0.3)

    def mp2(k):
        M.asetsPotts2D(ctp, alp, [1024, 1024, 4, k, 0.0, 0.3, 0.16], ctx=ctx)

    def mp2_cpu(k):
        from oracle import mtwin as OM
        OM.potts(ctp, alp, k, 0.0, 0.3, 0.16)

    row("matlab_potts2d_1024^2_L4_f64", npix, "pixel-iter", (4 * 4 + 1) * 16 + 2 * 4 * 8,
        "(4L+1) state arrays read+written, Ct and alpha read (fp64)",
        _per_iteration_s(mp2, 20), mp2_cpu, 2, dtype="f64")

    # star-shape Potts 2D, float64, 512^2 L=4
    ss = (512, 512)
    cts = g.random(ss + (4,))
    als = 0.1 + 0.3 * g.random(ss + (4,))
    pts = np.array([[64, 64], [448, 64], [64, 448], [448, 448]])

    def star(k):
        SS.asetsPotts2D_starShape(cts, als, [512, 512, 4, k, 0.0, 0.25, 0.11, 0.05], pts, ctx=ctx)

    def star_cpu(k):
        from oracle import starshape as OS
        OS.solve(cts, als, [512, 512, 4, k, 0.0, 0.25, 0.11, 0.05], [tuple(p) for p in pts])

    row("starshape_potts2d_512^2_L4_f64", ss[0] * ss[1], "pixel-iter",
        (5 * 4 + 1) * 16 + 4 * 4 * 8,
        "px, py, pt, u, v per label and ps read+written; Ct, alpha, two direction fields read (fp64)",
        _per_iteration_s(star, 20), star_cpu, 2, dtype="f64")

    # cost terms on device arrays, 256^3: CUDA events on the context's stream
    img = torch.from_numpy(np.asfortranarray(ct).ravel(order="F").copy()).cuda()
    out = torch.empty(nvox * 4, device="cuda")
    models = np.array([0.2, 0.4, 0.6, 0.8], np.float32)

    def events(fn, n=10):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(n):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) * 1e-3 / n

    row("cost_l1_256^3_L4", nvox, "voxel", 8 + 16,
        "image read twice (range, then costs), 4 costs written", events(
            lambda: N.check(N.lib().asets_cost_l1(ctx.handle, N.DEVICE, img.data_ptr(), nvox,
                                                  models.ctypes.data, 4, 1, out.data_ptr()))))
    row("alpha_contrast_256^3", nvox, "voxel", 12,
        "image read twice (range, then gradient), alpha written", events(
            lambda: N.check(N.lib().asets_alpha_contrast(ctx.handle, N.DEVICE, img.data_ptr(),
                                                         256, 256, 256, 1, 0.1, 0.9, 10.0, 1, 1,
                                                         out.data_ptr()))))
    for r, cpu_fn, cpu_its, units, unit_name in pending_cpu:
        t = time.perf_counter()
        cpu_fn(cpu_its)
        sec = (time.perf_counter() - t) / cpu_its
        r["cpu_baseline"] = {"value": units / sec / 1e9, "unit": f"G{unit_name}/s", "cores": 1,
                             "kind": "port",
                             "sample": f"{cpu_its} iterations incl. initialisation, numpy, "
                                       "same problem"}
    return rows


def warm_start_run(ctx, nseeds: int) -> dict:
    """Potts 3D 128^3, L = 6, errBound 1e-4 on held-out seeds: cold start vs
    the multilevel solve vs the multilevel solve whose coarsest level starts
    from the trained network (committed weights)."""
    from asetsmatlabmaxflow_gb300 import warmstart as W

    net, budget, level = W.load(ctx)
    run = W.Runner(ctx)
    W.evaluate(net, budget, [W.HELDOUT_SEED0 + 900], level=level, tight=False, run=run)  # warm-up
    seeds = list(range(W.HELDOUT_SEED0, W.HELDOUT_SEED0 + nseeds))
    res = W.evaluate(net, budget, seeds, level=level, tight=False, run=run)
    run.close()
    # the same problems as one batch: cold batch against warm-started batch
    runs = [W.Runner(ctx) for _ in seeds]
    W.evaluate_batched(net, budget, seeds, level=level, runs=runs)  # warm-up
    batched = W.evaluate_batched(net, budget, seeds, level=level, runs=runs)
    for r in runs:
        r.close()
    net.close()
    out = W.summarize(res)
    out["batched"] = batched
    out["workload"] = ("Potts 3D 128^3 L=6 (means U[0,1], Voronoi 30-80 cells, noise U[.05,.2], "
                       "alpha U[.1,.5]), cc 0.3, steps 0.11, errBound 1e-4, held-out seeds "
                       f"{W.HELDOUT_SEED0}..{W.HELDOUT_SEED0 + nseeds - 1}; wall ms per solve")
    out["levels"] = W.LEVELS
    return out


def cpu_baseline_sample(cs, ct, alpha, iters: int) -> dict:
    """Single-core oracle solve of the same volume for `iters` iterations
    (init included, as the reference's timet)."""
    from oracle import oracle as O

    t0 = time.perf_counter()
    O.solve("binary", SHAPE, ct, alpha, cs=cs, max_it=iters, err_bound=0.0, cc=CC, steps=STEPS)
    dt = time.perf_counter() - t0
    return {"value": float(np.prod(SHAPE)) * iters / dt / 1e9, "unit": UNIT, "cores": 1,
            "kind": "port", "seconds": dt,
            "sample": f"256^3 binary 3D, {iters} iterations incl. init, 1 thread "
                      "(C restatement, bit-identical to maxflow/asetsBinaryMF3D_mex.c)"}


def run_reference(args, rank, pg):
    """CPU arm: the reference C path on all host cores, one solve per core."""
    if rank != 0:
        return
    from concurrent.futures import ThreadPoolExecutor

    from asetsmatlabmaxflow_gb300 import synth
    from oracle import oracle as O

    cs, ct, alpha = synth.binary3d(seed=0, shape=SHAPE)
    cores = host_cores()
    # per core per step: a bounded sample of the 200-iteration run; at 32
    # iterations the per-call allocation and init (as in the reference's own
    # call) are about 3% of it
    iters = 32

    def one(_):
        O.solve("binary", SHAPE, ct, alpha, cs=cs, max_it=iters, err_bound=0.0, cc=CC, steps=STEPS)

    O.lib()
    with ThreadPoolExecutor(max_workers=cores) as ex:
        for _ in range(args.warmup):
            list(ex.map(one, range(cores)))
        t0 = time.perf_counter()
        for _ in range(args.steps):
            list(ex.map(one, range(cores)))
        dt = time.perf_counter() - t0
    value = float(np.prod(SHAPE)) * iters * cores * args.steps / dt / 1e9
    sample = (f"256^3 binary 3D, {iters} iterations incl. init per core per step, "
              f"{cores} concurrent single-thread solves")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(args.gpus),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.profile_iters:
        profile_run(args)
        return
    if args.profile_conv:
        profile_conv(args)
        return
    world, rank, local, pg = dist_setup()
    if args.impl == "reference":
        run_reference(args, rank, pg)
        return
    import torch

    from asetsmatlabmaxflow_gb300 import native as N
    from asetsmatlabmaxflow_gb300 import synth

    torch.cuda.set_device(local)
    stream = torch.cuda.Stream()
    ctx = N.Context(local)
    ctx.set_stream(stream.cuda_stream)
    cs, ct, alpha = synth.binary3d(seed=rank, shape=SHAPE)
    nvox = int(np.prod(SHAPE))

    # ---- value: device-resident inputs, one step = one 200-iteration solve
    s = N.Solver(ctx, "binary", SHAPE)
    s.set_inputs(ct, alpha, cs)
    for _ in range(args.warmup):
        s.run(ITERS, 0.0, CC, STEPS)
    kernel_ms = []
    launches = 0
    barrier(pg)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            it = s.run(ITERS, 0.0, CC, STEPS)
            ms, nl = s.last_run_stats()
            kernel_ms.append(ms / ITERS)  # device time per executed iteration launch
            launches += nl + 1  # iteration launches (graph chunks) + the init kernel
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier(pg)
    t_ms = max_over_ranks(pg, ev0.elapsed_time(ev1))
    value = world * nvox * ITERS * args.steps / (t_ms * 1e-3) / 1e9

    # ---- roofline of the fused iteration kernel
    peak, peak_kind = peaks()
    per_launch_ms = statistics.median(kernel_ms)
    achieved = BYTES_PER_VOXEL_ITER * nvox / (per_launch_ms * 1e-3) / 1e9
    traffic = traffic_per_launch()

    # ---- time to errBound 1e-4 (convergence run): cold start, and the
    # multilevel (coarse-to-fine) solve; wall time of the synchronous call
    def timed(fn):
        torch.cuda.synchronize()
        t = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return r, 1e3 * (time.perf_counter() - t)

    s.run(2000, 1e-4, CC, STEPS)
    conv_it, conv_wall = timed(lambda: s.run(2000, 1e-4, CC, STEPS))
    conv_ms, _ = s.last_run_stats()
    u_cold = s.get_u()
    s.run_multilevel(3, 2000, 1e-4, CC, STEPS)
    ml_it, ml_wall = timed(lambda: s.run_multilevel(3, 2000, 1e-4, CC, STEPS))
    ml_its, ml_dev = s.multilevel_stats()
    ml_agree = float(np.mean((s.get_u() > 0.5) == (u_cold > 0.5)))
    s.close()

    # ---- e2e: the C ABI one-shot call from pinned host buffers
    h_cs = torch.from_numpy(cs.ravel(order="F").copy()).pin_memory()
    h_ct = torch.from_numpy(ct.ravel(order="F").copy()).pin_memory()
    h_al = torch.from_numpy(alpha.ravel(order="F").copy()).pin_memory()
    h_u = torch.empty(nvox, dtype=torch.float32).pin_memory()
    h_cvg = torch.empty(ITERS, dtype=torch.float32).pin_memory()
    lib = N.lib()
    import ctypes

    itn = ctypes.c_int(0)

    def e2e_call():
        st = lib.asets_binary_mf3d(ctx.handle, None, h_al.data_ptr(), h_cs.data_ptr(),
                                   h_ct.data_ptr(), SHAPE[1], SHAPE[0], SHAPE[2], ITERS, 0.0, CC,
                                   STEPS, h_u.data_ptr(), h_cvg.data_ptr(), ctypes.byref(itn), None)
        N.check(st)

    for _ in range(max(1, args.warmup)):
        e2e_call()
    barrier(pg)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_call()
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(pg, time.perf_counter() - t0)
    e2e_value = world * nvox * ITERS * args.steps / e2e_s / 1e9
    ok = bool(np.isfinite(h_u.numpy()).all())

    cpu_on = rank == 0 and not args.no_cpu_baseline
    batch = None if args.no_batch else batch_run(ctx, cpu_on)
    configs = configs_run(ctx, cpu_on) if (rank == 0 and not args.no_configs) else None
    warm = warm_start_run(ctx, args.warm_seeds) if (rank == 0 and args.warm_seeds > 0) else None
    nxt = next_rows_run(ctx, stream, not args.no_cpu_baseline) \
        if (rank == 0 and not args.no_next) else None

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline_sample(cs, ct, alpha, 8)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": workload_config(world),
            "e2e": {"value": e2e_value, "unit": UNIT,
                    "h2d_bytes_per_step": 3 * nvox * 4, "d2h_bytes_per_step": nvox * 4 + ITERS * 4},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "peak_kind": peak_kind, "kernel": "stencil_col_kernel<3, 16 warps, 2 rows per thread (60x12 tile), 5 stages, refill in Z, binary, fast>",
                         "bytes_per_voxel_iter": BYTES_PER_VOXEL_ITER,
                         "launch_ms": per_launch_ms},
            "time_to_errbound": {"err_bound": 1e-4, "iterations": conv_it, "ms": conv_ms,
                                 "wall_ms": conv_wall,
                                 "multilevel": {"levels": len(ml_its), "iterations": ml_its,
                                                "device_ms": ml_dev, "wall_ms": ml_wall,
                                                "label_agreement_with_cold": ml_agree}},
            "warm_start": warm,
            "clocks": clk.summary(),
            "gpu_launches": launches,
            "batch": batch,
            "configs": configs,
            "next": nxt,
            "finite": ok,
        }
        if cpu is not None:
            line["cpu_baseline"] = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
