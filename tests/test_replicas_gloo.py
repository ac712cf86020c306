"""The multi-GPU path runs independent replicas; its only cross-rank step is the timing
aggregation (max over ranks). Exercised here with two gloo ranks on the CPU."""
import os
import socket

import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import sys
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms, value = bench.aggregate_ranks(10.0 + 5.0 * rank, world)
    out[rank] = (ms, value)
    dist.destroy_process_group()


def test_replica_timing_takes_the_slowest_rank():
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    for r in range(2):
        ms, value = res[r]
        assert ms == 15.0
        assert abs(value - 2 * 1000.0 / 15.0) < 1e-9
