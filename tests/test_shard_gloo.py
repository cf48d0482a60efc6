"""Multi-rank path on CPU (gloo, world size 2): the ensemble is split into
one shard per rank, greedy by mesh size, every member in exactly one shard
and the shards balanced; no collective touches the data path, and the
timing/throughput reductions of bench.py are max/sum over ranks."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK="0",
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    # bench.dist_init selects the GPU of the rank; on CPU only the process
    # group part is exercised here
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from pycathy_wrapper_gb300.shard import member_nodes
    cases = bench._cases(6, rank, 600.0, precond=2, world=world)
    names = [c.name for c in cases]
    seeds_dem = [float(c.dem.dem.sum()) for c in cases]
    load = float(sum(member_nodes(cases)))
    shards = [None] * world
    dist.all_gather_object(shards, names)  # test-side check only
    t = bench.allmax(1.0 + rank, world)
    s = bench.allsum(10.0 * (rank + 1), world)
    loads = [bench.allmax(load if r == rank else 0.0, world) for r in range(world)]
    bench.barrier(world)
    q.put((rank, names, seeds_dem, t, s, shards, loads))
    dist.destroy_process_group()


@pytest.mark.timeout(300)
def test_two_ranks_shard_members_and_reduce_scalars():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=240) for _ in ps)
    for p in ps:
        p.join(60)
        assert p.exitcode == 0
    (r0, n0, d0, t0, s0, sh0, l0), (r1, n1, d1, t1, s1, sh1, l1) = res
    assert (r0, r1) == (0, 1)
    assert t0 == t1 == 2.0            # max over ranks of the timed region
    assert s0 == s1 == 30.0           # total simulated seconds of all ranks
    assert set(d0).isdisjoint(d1)     # each rank has its own members
    assert sh0 == sh1 == [n0, n1]     # every rank derives the same split
    # one ensemble of 12 members, each in exactly one shard
    assert sorted(n0 + n1) == sorted(f"member{m}" for m in range(12))
    from pycathy_wrapper_gb300.inputs import config2_members
    from pycathy_wrapper_gb300.shard import member_nodes
    biggest = max(member_nodes(config2_members(12, tmax=600.0)))
    assert abs(l0[0] - l0[1]) <= biggest  # greedy bound on the imbalance


def test_shard_members_covers_once_and_balances():
    sys.path.insert(0, ROOT)
    import numpy as np
    from pycathy_wrapper_gb300.shard import shard_members
    rng = np.random.default_rng(3)
    costs = rng.integers(10_000, 140_000, size=256)
    for nr in (1, 2, 3, 8):
        sh = shard_members(costs, nr)
        allm = sorted(m for s in sh for m in s)
        assert allm == list(range(256))
        loads = [int(costs[s].sum()) for s in sh]
        assert max(loads) - min(loads) <= costs.max()
        assert all(s == sorted(s) for s in sh)
