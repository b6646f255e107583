"""bench.py --gpus N runs N independent replicas (one solver per rank, no
data exchange); the job's time is the slowest rank's and its value the sum
over ranks.  The rank logic is checked here with two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.replica_time_ms(10.0 + 5.0 * rank, world, device="cpu")
        value = bench.replica_value(1000, 5, 4, ms, world)
        out.put((rank, ms, value, bench.env_rank()))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, value, env in res:
        assert ms == pytest.approx(15.0)              # the slowest rank's time
        assert value == pytest.approx(2 * 1000 * 5 * 4 / 15e-3)
        assert env == (rank, 2, rank)


def test_single_replica_is_local():
    import bench
    assert bench.replica_time_ms(7.5, 1) == 7.5
    assert bench.replica_value(10, 5, 2, 1.0, 1) == pytest.approx(10 * 5 * 2 / 1e-3)
