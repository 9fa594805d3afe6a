"""Multi-rank replica logic of bench.py on CPU (world_size 2, gloo, 127.0.0.1).

k-points shard across ranks with no data-path collective; the only exchange is
the max over ranks of the timed region."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from hybridhsdla_gb300 import synth
    s = synth.make_system("t1")
    mine = bench.shard_kpoints(list(range(len(s.kpoints))), rank, world)
    got = [None] * world
    dist.all_gather_object(got, mine)
    t = bench._max_over_ranks(world, float(10 * (rank + 1)))
    if rank == 0:
        q.put((got, t))
    dist.destroy_process_group()


def test_kpoint_shards_and_max_over_ranks():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got, t = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    flat = sorted(i for part in got for i in part)
    assert flat == [0, 1, 2]                     # disjoint and complete
    assert set(got[0]).isdisjoint(got[1])
    assert t == 20.0                             # max over ranks
