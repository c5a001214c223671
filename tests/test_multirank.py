"""The N>1 path on CPU with gloo, world size 2.  Simulations are independent,
so ranks share nothing on the data path: each rank takes its round-robin share
(as the reference deals files to devices) and only the timing is reduced."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    items = list(range(11))
    mine = bench.shard(items, rank, world)
    dev_s = 1.0 + rank                      # rank 1 is slower
    vsteps = 100 * len(mine)
    t, v = bench.reduce_timing(dist, dev_s, vsteps)
    q.put((rank, mine, t, v))
    dist.destroy_process_group()


def test_two_rank_sharding_and_timing_reduction():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, m0, t0, v0), (r1, m1, t1, v1) = out
    assert m0 == [0, 2, 4, 6, 8, 10] and m1 == [1, 3, 5, 7, 9]
    assert sorted(m0 + m1) == list(range(11)) and not set(m0) & set(m1)
    assert t0 == t1 == 2.0                  # max over ranks
    assert v0 == v1 == 1100                 # whole-job voxel-steps
