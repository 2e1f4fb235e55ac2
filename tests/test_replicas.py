"""The multi-GPU path is replicas only: state points are split across ranks
with no exchange on the data path, ranks meet only for timing (barrier, max of
the elapsed time) and the final tallies. Checked here with 2 gloo ranks on CPU."""
import os

import pytest

torch = pytest.importorskip("torch")


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from classicaldft_gb300 import statepoints as sp
    pts = sp.sample_state_points(16, seed=2024)
    mine = sp.shard(pts, rank, world)
    # every rank reports its indices and its cost; the max-over-ranks reduction of the bench
    idx = torch.full((16,), -1, dtype=torch.int64)
    idx[: len(mine)] = torch.tensor(mine, dtype=torch.int64)
    gathered = [torch.zeros(16, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(gathered, idx)
    t = torch.tensor([float(rank + 1)])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    if rank == 0:
        out.put(([g[g >= 0].tolist() for g in gathered], float(t.item())))
    dist.destroy_process_group()


def test_sweep_shards_across_two_ranks():
    import socket
    import torch.multiprocessing as mp
    from classicaldft_gb300 import statepoints as sp
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    shards, tmax = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert tmax == 2.0
    assert sorted(shards[0] + shards[1]) == list(range(16))
    assert not set(shards[0]) & set(shards[1])
    pts = sp.sample_state_points(16, seed=2024)
    cost = [sum(p["n"] ** 3 for p in (pts[i] for i in sh)) for sh in shards]
    assert max(cost) <= 1.35 * min(cost)  # balanced by N^3 cost
    assert shards == [sp.shard(pts, r, 2) for r in range(2)]
