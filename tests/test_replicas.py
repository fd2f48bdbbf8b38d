"""Replica aggregation of bench.py --gpus N (independent sweeps per rank; the step
timing is the slowest rank's and the work is summed) on a world-size-2 gloo group."""
import os
import socket

import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import bench
    d = bench.Dist()
    try:
        d.barrier()
        step_s = 1.0 + rank          # rank 1 is the slower replica
        tasks = 100.0 * (rank + 1)
        q.put((rank, d.allreduce(step_s, "max"), d.allreduce(tasks, "sum"), d.local))
    finally:
        d.close()


def test_two_rank_aggregation():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    results = sorted(q.get(timeout=10) for _ in range(2))
    for rank, max_s, total, local in results:
        assert max_s == 2.0 and total == 300.0 and local == rank
