"""The N>1 path of bench.py on CPU: two gloo ranks (127.0.0.1) agree on the max-over-ranks
times and the whole-job rate (sum of all ranks' points over the slowest rank's time)."""
import os
import socket
import sys

import torch
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks([10.0 + 5 * rank, 3.0 - rank, 7.0])  # rank 1 is slower on the first
        rate = bench.whole_job_rate(1000, 4, world, ms[0])
        out.put((rank, ms, rate))
    finally:
        torch.distributed.destroy_process_group()


def test_two_gloo_ranks_agree_on_max_times_and_job_rate():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, rate in res:
        assert ms == [15.0, 3.0, 7.0], (rank, ms)
        assert abs(rate - 1000 * 4 * 2 / 0.015) < 1e-6 * rate


def test_single_process_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks([1, 2.5]) == [1.0, 2.5]
