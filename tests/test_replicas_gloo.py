"""The N > 1 path of bench.py (independent replicas, one per rank): process-group setup from
the torchrun environment, the barriers around the timed region and the max over ranks of the
step time, run as two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench

    w, r, local = bench.dist_init()
    assert (w, r, local) == (world, rank, rank)
    bench.barrier(w)
    # each rank's step time differs; every rank gets the largest
    t = bench.max_over_ranks(w, 0.010 * (rank + 1))
    bench.barrier(w)
    out.put((rank, t))
    import torch.distributed as dist

    dist.destroy_process_group()


def test_two_gloo_ranks_share_the_max_step_time():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    res = dict(q.get(timeout=10) for _ in range(2))
    assert res == {0: pytest.approx(0.020), 1: pytest.approx(0.020)}
