"""The multi-GPU form of the bench is replicas (each rank steps its own world; no data
path collective): the per-rank figure is reduced to the job's with a MAX over ranks.
Checked here with two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, values, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    dist.barrier()
    out[rank] = bench.replica_max(values[rank], dist)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_max_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    values = [0.25, 0.31]
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, values, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0] == out[1] == pytest.approx(0.31)


def test_replica_max_single_rank_is_identity():
    import bench
    assert bench.replica_max(0.42) == pytest.approx(0.42)
