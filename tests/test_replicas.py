"""The bench's multi-GPU path (independent replicas, max-over-ranks time)
with two gloo ranks on the CPU."""
import os
import socket

import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, lr = bench.dist_info()
    assert (r, w, lr) == (rank, world, rank)
    t = bench.replica_max(10.0 + 5.0 * rank, w, torch.device("cpu"))  # ranks time 10 ms and 15 ms
    out[rank] = t
    dist.barrier()
    dist.destroy_process_group()


def test_replica_max_two_ranks():
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
    assert dict(out) == {0: 15.0, 1: 15.0}


def test_replica_max_single_rank():
    import bench
    assert bench.replica_max(3.5, 1, torch.device("cpu")) == 3.5
