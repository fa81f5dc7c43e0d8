"""Multi-rank host logic of the replica path on the CPU: two gloo ranks."""
import os
import socket

import pytest

from umbreon_gb300 import replicas


def test_partition_covers_every_item_once():
    for n in (0, 1, 7, 64, 65):
        for world in (1, 2, 3, 8):
            seen = [i for r in range(world) for i in replicas.partition(n, r, world)]
            assert seen == list(range(n))
            sizes = [len(replicas.partition(n, r, world)) for r in range(world)]
            assert max(sizes) - min(sizes) <= (1 if n else 0)


def test_single_process_reduction_is_identity():
    units_s, ms = replicas.job_throughput(1000.0, 2.0)
    assert ms == 2.0 and units_s == 1000.0 / 2e-3


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ws, r, local = replicas.env_ranks()
        mine = replicas.partition(64, r, ws)
        # each rank "renders" its frames: 1,000 rays and (rank + 1) ms per frame
        units_s, ms = replicas.job_throughput(1000.0 * len(mine), float(len(mine) * (r + 1)))
        dist.barrier()
        q.put((r, list(mine), units_s, ms))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_slowest_rank_sets_the_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, f0, u0, ms0), (r1, f1, u1, ms1) = out
    assert f0 + f1 == list(range(64))
    # slowest rank: 32 frames x 2 ms; all ranks: 64,000 rays
    assert ms0 == ms1 == 64.0
    assert u0 == u1 == pytest.approx(64000.0 / 0.064)
