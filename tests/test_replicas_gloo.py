"""Multi-GPU is replicas only: each rank advances its own copy of the workload and the
benchmark reports the slowest rank's time and all ranks' cell-updates.  The aggregation
runs here on CPU ranks over gloo (world size 2, 127.0.0.1)."""
import os
import socket

import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t, cells = bench.job_aggregate(10.0 + rank, 1000 * (rank + 1), "cpu")
    out[rank] = (t, cells)
    dist.barrier()
    dist.destroy_process_group()


def test_job_aggregate_two_ranks():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0] == (11.0, 3000.0) and out[1] == (11.0, 3000.0)


def test_job_aggregate_single_process_is_identity():
    import bench
    assert bench.job_aggregate(5.0, 42, "cpu") == (5.0, 42)
