"""bench.py's multi-rank plumbing on CPU: world_size-2 gloo ranks set up the
process group from the torchrun environment, meet at the barrier, and take
the maximum of their timings (each rank solves its own replica; the path
has no data exchange)."""
import multiprocessing as mp
import socket
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q) -> None:
    import os

    os.environ.update(WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench

    w, r, local, pg = bench.dist_setup()
    bench.barrier(pg)
    t = bench.max_over_ranks(pg, 10.0 + rank)  # this rank's elapsed ms
    bench.barrier(pg)
    q.put((r, w, local, t))
    pg.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_max_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    assert all(o[1] == 2 for o in out)
    assert all(o[3] == 11.0 for o in out)  # both ranks report the slowest rank's time


def test_single_process_needs_no_group(monkeypatch):
    sys.path.insert(0, str(ROOT))
    import bench

    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    w, r, local, pg = bench.dist_setup()
    assert (w, r, local, pg) == (1, 0, 0, None)
    assert bench.max_over_ranks(pg, 3.5) == 3.5
