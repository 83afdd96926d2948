"""Host-side multi-rank logic on CPU (gloo, world size 2)."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from lassie_gb300 import sharding


def test_weak_shards_are_disjoint():
    a, b = sharding.weak_shard(2048, 0), sharding.weak_shard(2048, 1)
    assert len(a) == len(b) == 2048 and set(a).isdisjoint(b)


def test_cost_shard_balances_and_covers():
    sizes = [32 + (q * 37) % 481 for q in range(300)]
    parts = sharding.cost_shard(sizes, 4)
    assert sorted(q for p in parts for q in p) == list(range(300))
    loads = [sum(sizes[q] ** 3 for q in p) for p in parts]
    assert max(loads) / min(loads) < 1.05


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ids = list(sharding.weak_shard(8, rank))
    elapsed = 1.0 + rank  # rank 1 is slower
    done = 3 + rank  # completed instances on this rank
    q.put((rank, ids, sharding.max_over_ranks(elapsed), sharding.sum_over_ranks(done)))
    dist.destroy_process_group()


def test_gloo_max_over_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][2] == res[1][2] == 2.0
    assert res[0][3] == res[1][3] == 7.0
    assert set(res[0][1]).isdisjoint(res[1][1])


def test_strong_split_of_the_batched_workload():
    """bench.py --scaling strong: the 2048-instance batch split over 8 ranks
    by cost covers every instance once, with the N^3 loads within 1 %."""
    from lassie_gb300 import synth
    sizes = synth.c4_sizes(2048)
    assert sizes[:5] == [synth.make_c4_instance(q).n_species for q in range(5)]
    for world in (2, 4, 8):
        parts = sharding.cost_shard(sizes, world)
        assert sorted(q for p in parts for q in p) == list(range(2048))
        loads = [sum(sizes[q] ** 3 for q in p) for p in parts]
        assert max(loads) / min(loads) < 1.01
