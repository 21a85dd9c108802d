"""The N > 1 host path of the replicas (one process per GPU, independent units, no
data-path collective) on CPU with the gloo backend, world size 2."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank), LOCAL_RANK=str(rank))
    import torch.distributed as dist
    from sfhgpu import replicas as R
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w, r, lr = R.dist_env()
        R.barrier(w)
        mx = R.max_over_ranks(w, 10.0 + r)
        tot = R.sum_over_ranks(w, len(R.shard(1200, w, r)))
        # each rank evaluates its own shard of independent units (here: a sum of squares)
        mine = sum(u * u for u in R.shard(1200, w, r))
        allsum = R.sum_over_ranks(w, mine)
        q.put((r, w, lr, mx, tot, allsum))
    finally:
        dist.destroy_process_group()


def test_replicas_world_size_two_gloo():
    import torch.multiprocessing as mp
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
    assert [o[0] for o in out] == [0, 1]
    for r, w, lr, mx, tot, allsum in out:
        assert (w, lr) == (2, r)
        assert mx == 11.0
        assert tot == 1200
        assert allsum == sum(u * u for u in range(1200))


@pytest.mark.parametrize("n,world", [(1200, 2), (7, 3), (0, 4), (5, 8)])
def test_shard_covers_units_once(n, world):
    from sfhgpu.replicas import shard
    parts = [shard(n, world, r) for r in range(world)]
    flat = [u for p in parts for u in p]
    assert flat == list(range(n))
    assert max(len(p) for p in parts) - min(len(p) for p in parts) <= 1
    with pytest.raises(ValueError):
        shard(n, world, world)
