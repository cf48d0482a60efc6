"""Multi-rank path of bench.py on CPU (gloo, world size 2): each rank owns
its own ensemble shard (seeds offset by 256 per rank), no collective touches
the data path, and the timing/throughput reductions are max/sum over ranks."""
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
    cases = bench._cases(3, rank, 600.0, precond=2)
    names = [c.name for c in cases]
    seeds_dem = [float(c.dem.dem.sum()) for c in cases]
    t = bench.allmax(1.0 + rank, world)
    s = bench.allsum(10.0 * (rank + 1), world)
    bench.barrier(world)
    q.put((rank, names, seeds_dem, t, s))
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
    (r0, n0, d0, t0, s0), (r1, n1, d1, t1, s1) = res
    assert (r0, r1) == (0, 1)
    assert t0 == t1 == 2.0            # max over ranks of the timed region
    assert s0 == s1 == 30.0           # total simulated seconds of all ranks
    assert set(d0).isdisjoint(d1)     # each rank has its own members
