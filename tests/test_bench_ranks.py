"""The N > 1 path of bench.py (independent replicas, one process per GPU):
rank set-up, the barrier and the max-over-ranks timing, run as two gloo
ranks on the CPU."""
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port),
                       "CUDA_VISIBLE_DEVICES": ""})
    sys.path.insert(0, ROOT)
    import bench
    r, w = bench.dist_init(world)
    bench.barrier(w)
    t = bench.max_over_ranks(1.5 + r, w)      # each rank's own time; the max is reported
    bench.barrier(w)
    import torch.distributed as dist
    dist.destroy_process_group()
    q.put((r, w, t))


def test_two_gloo_ranks_report_the_slowest():
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
    assert out == [(0, 2, 2.5), (1, 2, 2.5)]
