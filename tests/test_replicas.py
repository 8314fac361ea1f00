"""Multi-GPU is replicas only: N independent engine runs, no data-path
collective.  The whole-job figure is units over all ranks / the slowest rank's
time (max over ranks).  Checked here with two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        # rank r "took" r + 1 seconds for 1000 units
        value, seconds = bench.replica_throughput(1000, float(rank + 1))
        q.put((rank, value, seconds))
    finally:
        dist.destroy_process_group()


def test_replica_throughput_takes_the_slowest_rank():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, seconds in got:
        assert seconds == pytest.approx(2.0)
        assert value == pytest.approx(1000 * world / 2.0)


def test_single_process_is_its_own_job():
    import bench
    value, seconds = bench.replica_throughput(500, 0.25)
    assert (value, seconds) == (2000.0, 0.25)
