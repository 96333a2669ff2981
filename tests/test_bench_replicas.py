"""The multi-rank path of bench.py on CPU: two gloo ranks, as torchrun starts them.

Paths are independent, so N GPUs run N replicas of the frame with no data-path
collective; the ranks only meet in barriers around the timed region and in the max over
ranks of its time. Rank 0 alone runs the reference arm; the other ranks return without
work."""
import multiprocessing as mp
import os
import socket
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    sys.path.insert(0, str(ROOT))
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench
    w, r, local = bench.dist_setup(None)
    bench.barrier(w)
    # each rank's timed-region length differs; every rank must see the slowest one
    m = bench.all_max(w, 10.0 + 5.0 * r)
    bench.barrier(w)
    # the reference arm: ranks other than 0 return before touching the scene
    if r != 0:
        bench.run_reference(None, w, r)
    import torch.distributed as dist
    dist.destroy_process_group()
    out.put((r, w, local, m))


def test_two_gloo_ranks_share_max_time():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 2, 0, 15.0), (1, 2, 1, 15.0)]


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.all_max(1, 3.5) == 3.5
    bench.barrier(1)
