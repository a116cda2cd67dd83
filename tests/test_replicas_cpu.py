"""The multi-GPU path is replicas only (every rank renders its own copy of
the workload; no data-path collective): its host logic, the max-over-ranks
step time and the whole-job throughput, on world_size-2 gloo ranks on the
CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import sys
    import torch.distributed as dist
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.max_over_ranks(1.0 + rank, world, "cpu")  # rank 1 is the slower replica
    v = bench.job_throughput(bench.N_TRIS, world, ms)
    q.put((rank, ms, v))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_timing_is_max_over_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    import bench
    for rank, ms, v in res:
        assert ms == 2.0
        assert v == pytest.approx(2 * bench.N_TRIS / 2e-3 / 1e6)
